"""Adjoints on the GPU: the backend's autograd Functions against central finite
differences (torch.autograd.gradcheck, eps 1e-6 as in tests/tensor/test_svd.py:414-464)
and against the reference's own autograd gradients (golden vectors)."""
import numpy as np
import pytest
import torch

import oracle
from yastn_gb300 import backend as B
from yastn_gb300 import ops
from yastn_gb300.workloads import load_trace

pytestmark = pytest.mark.gpu


def dev(x):
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def _first(trace, fn):
    return [c for c in load_trace(trace)['calls'] if c['fn'] == fn and not np.iscomplexobj(c['args'][0])][0]


def test_gradcheck_merge_unmerge(cuda_device):
    c = _first('tensordot_fuse_to_matrix', 'transpose_and_merge')
    data, order, mn, mm, Dsize = c['args']
    x = dev(data).requires_grad_(True)
    assert torch.autograd.gradcheck(lambda t: B.transpose_and_merge(t, order, mn, mm, Dsize), (x,), eps=1e-6,
                                    atol=1e-8)
    u = _first('tensordot_fuse_to_matrix', 'unmerge')
    d, meta = u['args']
    y = dev(d).requires_grad_(True)
    assert torch.autograd.gradcheck(lambda t: B.unmerge(t, meta), (y,), eps=1e-6, atol=1e-8)


@pytest.mark.parametrize('name', ['tensordot_fuse_to_matrix', 'tensordot_fuse_contracted'])
def test_gradcheck_dot(name, cuda_device):
    c = _first(name, 'dot')
    A, Bm, meta, Dsize = c['args']
    a = dev(A).requires_grad_(True)
    b = dev(Bm).requires_grad_(True)
    assert torch.autograd.gradcheck(lambda x, y: B.dot(x, y, meta, Dsize), (a, b), eps=1e-6, atol=1e-7)


def test_gradcheck_transpose_dot_sum(cuda_device):
    c = _first('tensordot_no_fusion', 'transpose_dot_sum')
    A, Bm, meta, Ar, Br, Ao, Bo, Dsize = c['args']
    a = dev(A).requires_grad_(True)
    b = dev(Bm).requires_grad_(True)
    assert torch.autograd.gradcheck(lambda x, y: B.transpose_dot_sum(x, y, meta, Ar, Br, Ao, Bo, Dsize), (a, b),
                                    eps=1e-6, atol=1e-7)


def test_gradcheck_apply_mask(cuda_device):
    c = [c for c in load_trace('svd')['calls'] if c['fn'] == 'apply_mask' and not np.iscomplexobj(c['args'][0])][0]
    A, mask, meta, Dsize, axis, ndim = c['args']
    dmask = {k: dev(np.asarray(v, dtype=np.int64)) for k, v in mask.items()}
    a = dev(A).requires_grad_(True)
    assert torch.autograd.gradcheck(lambda x: B.apply_mask(x, dmask, meta, Dsize, axis, ndim), (a,), eps=1e-6,
                                    atol=1e-8)


def _svd_meta(shapes):
    meta, off, oU, oS, oV = [], 0, 0, 0, 0
    for m, n in shapes:
        k = min(m, n)
        meta.append(((off, off + m * n), (m, n), (oU, oU + m * k), (m, k), (oS, oS + k), (oV, oV + k * n), (k, n)))
        off += m * n; oU += m * k; oS += k; oV += k * n
    return tuple(meta), off, (oU, oS, oV)


def test_gradcheck_svd(cuda_device):
    """A gauge-invariant loss (as in test_svd.py:414-464): S-norm plus U S Vh contractions."""
    meta, n, sizes = _svd_meta([(4, 4), (5, 3), (2, 6)])
    rng = np.random.default_rng(3)
    x = dev(rng.normal(size=n)).requires_grad_(True)
    wU = dev(rng.normal(size=sizes[0]))
    wV = dev(rng.normal(size=sizes[2]))

    def f(t):
        U, S, V = B.svd(t, meta, sizes)
        out = S.norm()
        # (U diag(S) Vh) contracted with a fixed tensor is gauge invariant
        for sl, D, slU, DU, slS, slV, DV in meta:
            u = U[slU[0]:slU[1]].view(DU)
            v = V[slV[0]:slV[1]].view(DV)
            s = S[slS[0]:slS[1]]
            out = out + ((u * s) @ v).pow(2).sum() * 0.1
        return out
    assert torch.autograd.gradcheck(f, (x,), eps=1e-6, atol=1e-6)


@pytest.mark.parametrize('cplx', [False, True])
def test_svd_adjoint_matches_reference_autograd(cplx, cuda_device):
    tr = load_trace('adjoints')
    A = tr['_arrays']
    calls = [c for c in tr['calls'] if c['fn'] == 'svd_backward']
    c = [c for c in calls if np.iscomplexobj(A[c['data']]) == cplx][0]
    dA = ops.svd_backward(dev(A[c['U']]), dev(A[c['S']]), dev(A[c['V']]), dev(A[c['gU']]), dev(A[c['gS']]),
                          dev(A[c['gV']]), c['meta'], A[c['data']].size, dev(A[c['data']]).dtype)
    assert rel(dA.cpu().numpy(), A[c['grad']]) <= 1e-10


def test_svd_adjoint_matches_oracle_random(cuda_device):
    meta, n, sizes = _svd_meta([(7, 7), (9, 4), (3, 8), (1, 4)])
    rng = np.random.default_rng(11)
    data = rng.normal(size=n)
    U, S, V = oracle.svd(data, meta, sizes)
    gU, gS, gV = rng.normal(size=sizes[0]), rng.normal(size=sizes[1]), rng.normal(size=sizes[2])
    ref = oracle.svd_backward(U, S, V, gU, gS, gV, meta, n, np.float64)
    got = ops.svd_backward(dev(U), dev(S), dev(V), dev(gU), dev(gS), dev(gV), meta, n, torch.float64)
    assert rel(got.cpu().numpy(), ref) <= 1e-10
    # only gS (the sigma term), as when a loss depends on S alone
    ref = oracle.svd_backward(U, S, V, None, gS, None, meta, n, np.float64)
    got = ops.svd_backward(dev(U), dev(S), dev(V), None, dev(gS), None, meta, n, torch.float64)
    assert rel(got.cpu().numpy(), ref) <= 1e-10


def test_fix_signs_adjoint_real(cuda_device):
    meta, n, sizes = _svd_meta([(5, 5), (6, 3)])
    rng = np.random.default_rng(12)
    U, S, V = oracle.svd(rng.normal(size=n), meta, sizes)
    u = dev(U).requires_grad_(True)
    v = dev(V).requires_grad_(True)
    assert torch.autograd.gradcheck(lambda a, b: B.fix_svd_signs(a, b, meta), (u, v), eps=1e-6, atol=1e-8)


def test_eigh_adjoint_matches_reference_autograd(cuda_device):
    """The eigh adjoint on the reference's own U, S and cotangents (SYMEIG path and
    torch.linalg.eigh path, real and complex, a degenerate pair included)."""
    import json, os
    from yastn_gb300 import ops
    from yastn_gb300.workloads import GOLDEN, _decode
    with open(os.path.join(GOLDEN, 'eigh_adjoint.json')) as f:
        calls = json.load(f)['calls']
    z = np.load(os.path.join(GOLDEN, 'eigh_adjoint.npz'))
    for c in calls:
        meta = _decode(c['meta'], None)
        U, S, gU, gS, ref = (torch.from_numpy(z[c[k]]).cuda() for k in ('U', 'S', 'gU', 'gS', 'grad'))
        g = ops.eigh_backward(U, S, gU, gS, meta, ref.numel(), ref.dtype, c['order_by_magnitude']).cpu().numpy()
        r = ref.cpu().numpy()
        assert np.abs(g - r).max() <= 1e-10 * np.abs(r).max(), c['order_by_magnitude']


@pytest.mark.parametrize('by_mag', [False, True])
def test_gradcheck_eigh(by_mag, cuda_device):
    """Finite differences of a gauge-invariant loss through the backend's eigh."""
    from yastn_gb300 import backend as BK
    rng = np.random.default_rng(4)
    meta, off, offU, offS, parts = [], 0, 0, 0, []
    for d in (4, 6):
        a = rng.normal(size=(d, d))
        parts.append((a + a.T).ravel())
        meta.append(((off, off + d * d), (d, d), (offU, offU + d * d), (d, d), (offS, offS + d)))
        off += d * d; offU += d * d; offS += d
    meta = tuple(meta)
    data = torch.from_numpy(np.concatenate(parts)).cuda().requires_grad_(True)
    w = torch.from_numpy(rng.normal(size=offS)).cuda()

    def loss(x):
        S, U = BK.eigh(x, meta, (offS, offU), order_by_magnitude=by_mag)
        # eigenvalues and a gauge-invariant function of the eigenvectors (|U|^4)
        return (S * w).sum() + (U.abs() ** 4).sum()

    def sym(x):  # keep the perturbation symmetric per block
        out = []
        for sl, D, *_ in meta:
            b = x[sl[0]:sl[1]].view(D)
            out.append(((b + b.T) / 2).reshape(-1))
        return torch.cat(out)
    assert torch.autograd.gradcheck(lambda x: loss(sym(x)), (data,), eps=1e-6, atol=1e-6, rtol=1e-5)
