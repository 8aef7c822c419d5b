"""Family (c) on the GPU: block SVD / eigh (Jacobi), truncation, gauge fix, masks.

Singular values and eigenvalues: max |S - S_ref| <= 1e-12 * max S_ref (FP64,
norm-wise). Singular vectors are checked through gauge-invariant quantities:
reconstruction |U S Vh - A| <= 1e-12 |A| and orthonormality <= 1e-12 (the reference
checks reconstruction at 1e-10, tests/tensor/test_svd.py:22). Truncation masks and
kept dimensions must match exactly.
"""
import json
import os

import numpy as np
import pytest
import torch

import oracle
from yastn_gb300 import ops
from yastn_gb300.workloads import load_trace, GOLDEN

pytestmark = pytest.mark.gpu
TOL = 1e-12


def dev(x):
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


def host(t):
    return t.detach().cpu().numpy()


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)) if b.size else 0.0


def check_svd(data, meta, U, S, V, S_ref):
    assert rel(S, S_ref) <= TOL
    for sl, D, slU, DU, slS, slV, DV in meta:
        a = data[sl[0]:sl[1]].reshape(D)
        u = U[slU[0]:slU[1]].reshape(DU)
        s = S[slS[0]:slS[1]]
        vh = V[slV[0]:slV[1]].reshape(DV)
        if a.size == 0:
            continue
        assert np.all(np.diff(s) <= 0), "singular values not descending"
        assert np.all(s >= 0)
        scale = max(np.abs(a).max(), 1e-300)
        assert np.abs((u * s) @ vh - a).max() <= TOL * scale * max(1, min(D))
        k = DU[1]
        assert np.abs(u.conj().T @ u - np.eye(k)).max() <= TOL * max(10, k)
        assert np.abs(vh @ vh.conj().T - np.eye(k)).max() <= TOL * max(10, k)


@pytest.mark.parametrize('name', ['svd', 'svd_ill', 'fix_signs'])
def test_svd_on_reference_calls(name, cuda_device):
    tr = load_trace(name)
    n = 0
    for c in tr['calls']:
        if c['fn'] != 'svd':
            continue
        data, meta, sizes = c['args'][:3]
        U, S, V = (host(x) for x in ops.svd(dev(data), meta, sizes))
        check_svd(data, meta, U, S, V, c['out'][1])
        n += 1
    if name != 'fix_signs':
        assert n > 0


def test_svd_vectors_match_oracle_after_gauge_fix(cuda_device):
    """With distinct singular values the vectors agree with LAPACK's up to the gauge."""
    rng = np.random.default_rng(7)
    shapes = [(12, 12), (20, 7), (5, 16), (1, 1), (3, 1)]
    meta, off, oU, oS, oV = [], 0, 0, 0, 0
    for m, n in shapes:
        k = min(m, n)
        meta.append(((off, off + m * n), (m, n), (oU, oU + m * k), (m, k), (oS, oS + k), (oV, oV + k * n), (k, n)))
        off += m * n; oU += m * k; oS += k; oV += k * n
    meta = tuple(meta)
    data = rng.normal(size=off)
    U, S, V = ops.svd(dev(data), meta, (oU, oS, oV))
    Uf, Vf, _ = ops.fix_svd_signs(U, V, meta)
    Ur, Sr, Vr = oracle.svd(data, meta, (oU, oS, oV))
    Urf, Vrf = oracle.fix_svd_signs(Ur, Vr, meta)
    assert rel(host(S), Sr) <= TOL
    assert rel(host(Uf), Urf) <= 1e-9 and rel(host(Vf), Vrf) <= 1e-9


def test_svd_rank_deficient_and_zero_blocks(cuda_device):
    """Zero singular values: vectors completed to orthonormal sets (LAPACK behaviour)."""
    rng = np.random.default_rng(8)
    blocks = [np.zeros((4, 6)), np.outer(rng.normal(size=5), rng.normal(size=3)),
              rng.normal(size=(6, 2)) @ rng.normal(size=(2, 6)), np.zeros((3, 3))]
    meta, off, oU, oS, oV, parts = [], 0, 0, 0, 0, []
    for a in blocks:
        m, n = a.shape
        k = min(m, n)
        meta.append(((off, off + m * n), (m, n), (oU, oU + m * k), (m, k), (oS, oS + k), (oV, oV + k * n), (k, n)))
        off += m * n; oU += m * k; oS += k; oV += k * n
        parts.append(a.ravel())
    meta = tuple(meta)
    data = np.concatenate(parts)
    U, S, V = (host(x) for x in ops.svd(dev(data), meta, (oU, oS, oV)))
    _, Sr, _ = oracle.svd(data, meta, (oU, oS, oV))
    assert np.abs(S - Sr).max() <= TOL * max(1.0, np.abs(Sr).max())
    check_svd(data, meta, U, S, V, Sr)


@pytest.mark.parametrize('qr,blocked64', [(True, True), (True, False), (False, True), (False, False)])
@pytest.mark.parametrize('cplx', [False, True])
def test_svd_start_and_fp64_phase_variants(qr, blocked64, cplx, cuda_device):
    """Every combination of the start (QR-preconditioned or from A's rows) and of the FP64
    phase (4-row super-vectors in shared memory, or one pair per warp) on random, graded,
    rank-deficient, tall, wide and tiny blocks."""
    rng = np.random.default_rng(31)
    f = lambda *sh: rng.normal(size=sh) + (1j * rng.normal(size=sh) if cplx else 0)
    q1, _ = np.linalg.qr(f(120, 120))
    q2, _ = np.linalg.qr(f(120, 120))
    blocks = [f(70, 50), f(33, 90), f(1, 5), f(6, 1), (q1 * np.logspace(0, -13, 120)) @ q2,
              f(64, 20) @ f(20, 64), np.zeros((7, 9))]
    meta, off, oU, oS, oV, parts = [], 0, 0, 0, 0, []
    for a in blocks:
        m, n = a.shape
        k = min(m, n)
        meta.append(((off, off + m * n), (m, n), (oU, oU + m * k), (m, k), (oS, oS + k), (oV, oV + k * n), (k, n)))
        off += m * n; oU += m * k; oS += k; oV += k * n
        parts.append(a.ravel())
    meta = tuple(meta)
    data = np.concatenate(parts)
    saved = ops.SVD_QR[0], ops.BLOCKED_FP64[0]
    ops.SVD_QR[0], ops.BLOCKED_FP64[0] = qr, blocked64
    try:
        U, S, V = (host(x) for x in ops.svd(dev(data), meta, (oU, oS, oV)))
    finally:
        ops.SVD_QR[0], ops.BLOCKED_FP64[0] = saved
    _, Sr, _ = oracle.svd(data, meta, (oU, oS, oV))
    check_svd(data, meta, U, S, V, Sr)


@pytest.mark.parametrize('cplx', [False, True])
def test_svd_large_rank_deficient_blocks(cplx, cuda_device):
    """Blocks of low numerical rank (products of thin factors, as the projector blocks of a
    corner transfer matrix step): the rounding-noise rows are left out of the rotations and
    their vectors completed, so Jacobi converges and the factorisation stays orthonormal."""
    rng = np.random.default_rng(21)
    specs = [(432, 432, 100), (300, 120, 40), (80, 250, 30), (256, 256, 200), (64, 64, 64)]
    blocks = []
    for m, n, r in specs:
        f = lambda *sh: rng.normal(size=sh) + (1j * rng.normal(size=sh) if cplx else 0)
        blocks.append((f(m, r) * np.logspace(0, -6, r)) @ f(r, n))
    meta, off, oU, oS, oV, parts = [], 0, 0, 0, 0, []
    for a in blocks:
        m, n = a.shape
        k = min(m, n)
        meta.append(((off, off + m * n), (m, n), (oU, oU + m * k), (m, k), (oS, oS + k), (oV, oV + k * n), (k, n)))
        off += m * n; oU += m * k; oS += k; oV += k * n
        parts.append(a.ravel())
    meta = tuple(meta)
    data = np.concatenate(parts)
    U, S, V = (host(x) for x in ops.svd(dev(data), meta, (oU, oS, oV)))
    _, Sr, _ = oracle.svd(data, meta, (oU, oS, oV))
    check_svd(data, meta, U, S, V, Sr)


@pytest.mark.parametrize('blocked,rows', [(False, None), (True, 4), (True, 8), (True, 16)])
def test_svd_fp32_phase_variants(blocked, rows, cuda_device):
    """Both FP32 phases (one pair per warp; super-vectors of 4/8/16 rows in shared memory)
    give LAPACK's singular values and an orthonormal factorisation."""
    rng = np.random.default_rng(11)
    shapes = [(200, 150), (64, 300), (37, 37), (5, 3), (1, 9), (90, 90)]
    meta, off, oU, oS, oV = [], 0, 0, 0, 0
    for m, n in shapes:
        k = min(m, n)
        meta.append(((off, off + m * n), (m, n), (oU, oU + m * k), (m, k), (oS, oS + k), (oV, oV + k * n), (k, n)))
        off += m * n; oU += m * k; oS += k; oV += k * n
    meta = tuple(meta)
    data = rng.normal(size=off)
    # a graded block: singular values over 12 decades
    a = meta[5][0][0]
    q1, _ = np.linalg.qr(rng.normal(size=(90, 90)))
    q2, _ = np.linalg.qr(rng.normal(size=(90, 90)))
    data[a:a + 8100] = ((q1 * np.logspace(0, -12, 90)) @ q2).ravel()
    saved = ops.BLOCKED_FP32[0], ops.ROWS_PER_SUPER[0]
    ops.BLOCKED_FP32[0], ops.ROWS_PER_SUPER[0] = blocked, rows
    try:
        U, S, V = (host(x) for x in ops.svd(dev(data), meta, (oU, oS, oV)))
    finally:
        ops.BLOCKED_FP32[0], ops.ROWS_PER_SUPER[0] = saved
    _, Sr, _ = oracle.svd(data, meta, (oU, oS, oV))
    check_svd(data, meta, U, S, V, Sr)


@pytest.mark.parametrize('blocked,rows', [(False, None), (True, 8), (True, 16)])
def test_complex_svd_and_eigh(blocked, rows, cuda_device):
    """complex128 blocks (wide, tall, square, rank-deficient, graded): LAPACK's singular
    values, U S Vh = A, unitary factors; Hermitian eigh with the same kernels."""
    rng = np.random.default_rng(13)
    shapes = [(120, 70), (33, 150), (40, 40), (6, 2), (1, 5)]
    blocks = [rng.normal(size=sh) + 1j * rng.normal(size=sh) for sh in shapes]
    q1, _ = np.linalg.qr(rng.normal(size=(50, 50)) + 1j * rng.normal(size=(50, 50)))
    q2, _ = np.linalg.qr(rng.normal(size=(50, 50)) + 1j * rng.normal(size=(50, 50)))
    blocks.append((q1 * np.logspace(0, -11, 50)) @ q2)                          # graded
    blocks.append(np.outer(rng.normal(size=7) + 1j, rng.normal(size=9) - 2j))   # rank one
    meta, off, oU, oS, oV, parts = [], 0, 0, 0, 0, []
    for a in blocks:
        m, n = a.shape
        k = min(m, n)
        meta.append(((off, off + m * n), (m, n), (oU, oU + m * k), (m, k), (oS, oS + k), (oV, oV + k * n), (k, n)))
        off += m * n; oU += m * k; oS += k; oV += k * n
        parts.append(a.ravel())
    meta = tuple(meta)
    data = np.concatenate(parts)
    saved = ops.BLOCKED_FP32[0], ops.ROWS_PER_SUPER[0]
    ops.BLOCKED_FP32[0], ops.ROWS_PER_SUPER[0] = blocked, rows
    try:
        U, S, V = (host(x) for x in ops.svd(dev(data), meta, (oU, oS, oV)))
        # Hermitian eigh on H = B + B^H of the square blocks
        hs = [a + a.conj().T for a in blocks if a.shape[0] == a.shape[1]]
        hmeta, ho, hu, hsz = [], 0, 0, 0
        for h in hs:
            d = h.shape[0]
            hmeta.append(((ho, ho + d * d), (d, d), (hu, hu + d * d), (d, d), (hsz, hsz + d)))
            ho += d * d; hu += d * d; hsz += d
        hdata = np.concatenate([h.ravel() for h in hs])
        E, Q = (host(x) for x in ops.eigh(dev(hdata), tuple(hmeta), (hsz, hu)))
    finally:
        ops.BLOCKED_FP32[0], ops.ROWS_PER_SUPER[0] = saved
    _, Sr, _ = oracle.svd(data, meta, (oU, oS, oV))
    assert np.abs(S - Sr).max() <= TOL * max(1.0, np.abs(Sr).max())
    check_svd(data, meta, U, S, V, Sr)
    for h, (sl, D, slU, DU, slS) in zip(hs, hmeta):
        e, q = E[slS[0]:slS[1]], Q[slU[0]:slU[1]].reshape(DU)
        assert np.abs(e - np.linalg.eigvalsh(h)).max() <= TOL * np.abs(h).max() * D[0]
        assert np.abs((q * e) @ q.conj().T - h).max() <= TOL * np.abs(h).max() * D[0]


def test_svd_empty(cuda_device):
    U, S, V = ops.svd(torch.zeros(0, dtype=torch.float64, device='cuda'), (), (0, 0, 0))
    assert U.numel() == S.numel() == V.numel() == 0


def test_eigh_on_reference_calls(cuda_device):
    tr = load_trace('eigh')
    n = 0
    for c in tr['calls']:
        data, meta, sizes = c['args']
        S, U = (host(x) for x in ops.eigh(dev(data), meta, sizes))
        assert rel(S, c['out'][0]) <= TOL
        for sl, D, slU, DU, slS in meta:
            a = data[sl[0]:sl[1]].reshape(D)
            u = U[slU[0]:slU[1]].reshape(DU)
            s = S[slS[0]:slS[1]]
            assert np.all(np.diff(s) >= 0)
            assert np.abs((u * s) @ u.conj().T - a).max() <= TOL * max(1, np.abs(a).max()) * D[0]
            assert np.abs(u.conj().T @ u - np.eye(DU[1])).max() <= TOL * max(10, DU[1])
        n += 1
    assert n > 0


@pytest.mark.parametrize('cplx', [False, True])
def test_eigh_rank_deficient_psd_blocks_reconstruct(cplx, cuda_device):
    """Gram matrices F F^H of wide-rowed F (rank-deficient, positive semidefinite, the
    eigenvalues of the shifted block clustered near the shift): U diag(S) U^H reproduces
    every block to the rounding level (relative 1e-13) and U is unitary, over many draws
    (YASTN's test_fuse_hard.py::test_hard_split meets such blocks)."""
    rng = np.random.default_rng(5)
    for trial in range(12):
        shapes = [(86, 19), (91, 120), (30, 40), (7, 3)]
        blocks, meta, off_a, off_u, off_s = [], [], 0, 0, 0
        for n, r in shapes:
            F = rng.normal(size=(n, r)) + (1j * rng.normal(size=(n, r)) if cplx else 0)
            G = F @ F.conj().T
            blocks.append(G)
            meta.append(((off_a, off_a + n * n), (n, n), (off_u, off_u + n * n), (n, n), (off_s, off_s + n)))
            off_a += n * n; off_u += n * n; off_s += n
        data = np.concatenate([b.ravel() for b in blocks])
        S, U = (host(x) for x in ops.eigh(dev(data), tuple(meta), (off_s, off_u)))
        for G, (sl, D, slU, DU, slS) in zip(blocks, meta):
            u = U[slU[0]:slU[1]].reshape(DU)
            s = S[slS[0]:slS[1]]
            assert np.linalg.norm((u * s) @ u.conj().T - G) <= 1e-13 * np.linalg.norm(G), (trial, D)
            assert np.abs(u.conj().T @ u - np.eye(DU[1])).max() <= 1e-13 * DU[1]


def test_eigh_order_by_magnitude(cuda_device):
    rng = np.random.default_rng(9)
    a = rng.normal(size=(9, 9)); a = a + a.T
    meta = (((0, 81), (9, 9), (0, 81), (9, 9), (0, 9)),)
    S, U = (host(x) for x in ops.eigh(dev(a.ravel()), meta, (9, 81), order_by_magnitude=True))
    ref = np.linalg.eigvalsh(a)
    ref = ref[np.argsort(-np.abs(ref), kind='stable')]
    assert rel(S, ref) <= TOL


def _decode_opts(opts):
    out = {}
    for k, v in opts.items():
        if isinstance(v, dict) and '__dict__' in v:
            v = {tuple(kk): vv for kk, vv in v['__dict__']}
        out[k] = v
    return out


def test_device_truncation_matches_reference_masks(cuda_device):
    with open(os.path.join(GOLDEN, 'truncation.json')) as f:
        cases = json.load(f)['cases']
    for case in cases:
        S = np.array(case['S'])
        charges = [tuple(c) for c in case['charges']]
        mask, kept = ops.truncation_mask_data(dev(S), case['slices'], charges, **_decode_opts(case['opts']))
        ref = np.array(case['mask'], dtype=bool)
        np.testing.assert_array_equal(host(mask), ref)
        assert kept == [int(ref[lo:hi].sum()) for lo, hi in case['slices']]


def test_fix_signs_golden_matrix(cuda_device):
    """test_svd.py:159-186 golden gauge-fixed U (complex blocks) from oracle U, V."""
    tr = load_trace('fix_signs')
    svd_call = [c for c in tr['calls'] if c['fn'] == 'svd'][0]
    fix_call = [c for c in tr['calls'] if c['fn'] == 'fix_svd_signs'][0]
    Ui, Vi, meta = fix_call['args']
    Uo, Vo, _ = ops.fix_svd_signs(dev(Ui), dev(Vi), meta)
    assert rel(host(Uo), fix_call['out'][0]) <= TOL and rel(host(Vo), fix_call['out'][1]) <= TOL
    gold = {k: np.array(v)[:, 0::2] + 1j * np.array(v)[:, 1::2] for k, v in tr['Ufixed'].items()}
    Uo = host(Uo)
    blocks = [Uo[m[2][0]:m[2][1]].reshape(m[3]) for m in meta]
    assert any(b.shape == (3, 2) and np.abs(b - gold['(0,0)']).max() < TOL for b in blocks)


def test_fix_signs_real_vs_oracle(cuda_device):
    tr = load_trace('svd')
    for c in tr['calls']:
        if c['fn'] == 'fix_svd_signs' and not np.iscomplexobj(c['args'][0]):
            Ui, Vi, meta = c['args']
            Uo, Vo, _ = ops.fix_svd_signs(dev(Ui), dev(Vi), meta)
            assert rel(host(Uo), c['out'][0]) <= TOL and rel(host(Vo), c['out'][1]) <= TOL


@pytest.mark.parametrize('name', ['svd', 'svd_ill'])
def test_apply_mask_on_reference_calls(name, cuda_device):
    tr = load_trace(name)
    n = 0
    for c in tr['calls']:
        if c['fn'] != 'apply_mask':
            continue
        A, mask, meta, Dsize, axis, ndim = c['args']
        dmask = {k: dev(np.asarray(v, dtype=np.int64)) for k, v in mask.items()}
        got = host(ops.apply_mask(dev(A), dmask, meta, Dsize, axis, ndim))
        np.testing.assert_array_equal(got, c['out'][0])
        g = np.random.default_rng(0).normal(size=Dsize).astype(A.dtype)
        back = host(ops.apply_mask(dev(g), dmask, meta, None, axis, ndim, scatter_size=A.size))
        np.testing.assert_array_equal(back, oracle.apply_mask_backward(g, mask, meta, A.size, axis, ndim))
        n += 1
    assert n > 0


@pytest.mark.parametrize('cplx', [False, True])
def test_fix_signs_adjoint_vs_reference_autograd(cplx, cuda_device):
    """yb_fix_signs_adjoint against torch's autograd of the reference's fix_svd_signs
    (fixture) and the oracle: real, and complex with the gradient through the phases."""
    import json, os
    from yastn_gb300.workloads import GOLDEN, _decode
    with open(os.path.join(GOLDEN, 'fix_signs_adjoint.json')) as f:
        calls = json.load(f)['calls']
    z = np.load(os.path.join(GOLDEN, 'fix_signs_adjoint.npz'))
    c = [c for c in calls if np.iscomplexobj(z[c['U']]) == cplx][0]
    meta = _decode(c['meta'], None)
    U, V, gU, gV = (z[c[k]] for k in ('U', 'V', 'gU', 'gV'))
    dU, dV = (host(x) for x in ops.fix_svd_signs_backward(dev(U), dev(V), dev(gU), dev(gV), meta))
    assert rel(dU, z[c['dU']]) <= 1e-12 and rel(dV, z[c['dV']]) <= 1e-12


def test_fix_signs_autograd_gradcheck_complex(cuda_device):
    """torch.autograd.gradcheck of the backend's complex fix_svd_signs (the phases of the
    columns' largest entries carry a gradient); U, Vh from a complex SVD, so no near-ties."""
    from yastn_gb300 import backend as BK
    rng = np.random.default_rng(8)
    meta, offU, offS, offV, Us, Vs = [], 0, 0, 0, [], []
    for m, n in ((5, 5), (6, 3), (2, 4)):
        k = min(m, n)
        u, _, vh = np.linalg.svd(rng.normal(size=(m, n)) + 1j * rng.normal(size=(m, n)), full_matrices=False)
        Us.append(u.ravel()); Vs.append(vh.ravel())
        meta.append(((0, 0), (m, n), (offU, offU + m * k), (m, k), (offS, offS + k), (offV, offV + k * n), (k, n)))
        offU += m * k; offS += k; offV += k * n
    meta = tuple(meta)
    U = dev(np.concatenate(Us)).requires_grad_(True)
    V = dev(np.concatenate(Vs)).requires_grad_(True)
    assert torch.autograd.gradcheck(lambda a, b: BK.fix_svd_signs(a, b, meta), (U, V), eps=1e-7, atol=1e-6)


def _qr_checks(data, meta, Q, R, Qr=None, Rr=None):
    for sl, D, slQ, DQ, slR, DR in meta:
        a = data[sl[0]:sl[1]].reshape(D)
        q, r = Q[slQ[0]:slQ[1]].reshape(DQ), R[slR[0]:slR[1]].reshape(DR)
        scale = max(np.abs(a).max(), 1e-300)
        assert np.abs(q @ r - a).max() <= TOL * scale * max(D)
        assert np.abs(q.conj().T @ q - np.eye(DQ[1])).max() <= TOL * max(10, DQ[1])
        assert np.abs(np.tril(r[:, :DR[0]], -1)).max(initial=0) == 0
        assert (np.real(np.diag(r)) >= 0).all() and np.abs(np.imag(np.diag(r))).max(initial=0) == 0
        if Qr is not None and np.linalg.cond(a) < 1e6:  # a well-conditioned block's factors are unique
            assert rel(q, Qr[slQ[0]:slQ[1]].reshape(DQ)) <= 1e-10
            assert rel(r, Rr[slR[0]:slR[1]].reshape(DR)) <= 1e-10


def test_qr_on_reference_calls(cuda_device):
    """Batched Householder QR with R's diagonal made positive against the reference's NumPy
    backend (tall, square, wide, complex, rank-deficient blocks), and the adjoint (real and
    complex) against the reference torch backend's autograd gradient."""
    tr = load_trace('qr')
    n = 0
    for c in tr['calls']:
        if c['fn'] != 'qr':
            continue
        data, meta, sizes = c['args']
        Q, R = (host(x) for x in ops.qr(dev(data), meta, sizes))
        _qr_checks(data, meta, Q, R, *c['out'])
        full = all(np.linalg.matrix_rank(data[sl[0]:sl[1]].reshape(D)) == min(D) for sl, D, *_ in meta)
        if 'adjoint' in c and full:
            adj = c['adjoint']
            g = host(ops.qr_backward(dev(c['out'][0]), dev(c['out'][1]), dev(adj['gQ']), dev(adj['gR']), dev(data),
                                     meta))
            assert rel(g, adj['grad']) <= 1e-10
        n += 1
    assert n == 5


@pytest.mark.parametrize('cplx', [False, True])
def test_qr_large_blocks(cplx, cuda_device):
    """Blocks of 432 x 432, 600 x 200, 100 x 900, 2000 x 16 and a graded one against the
    oracle; the adjoint (real and complex, the four ungraded blocks) against the oracle's."""
    rng = np.random.default_rng(41)
    f = lambda *sh: rng.normal(size=sh) + (1j * rng.normal(size=sh) if cplx else 0)
    q1, _ = np.linalg.qr(f(150, 150))
    blocks = [f(432, 432), f(600, 200), f(100, 900), f(2000, 16), (q1 * np.logspace(0, -10, 150)) @ f(150, 150)]
    meta, off, oQ, oR, parts = [], 0, 0, 0, []
    for a in blocks:
        m, n = a.shape
        k = min(m, n)
        meta.append(((off, off + m * n), (m, n), (oQ, oQ + m * k), (m, k), (oR, oR + k * n), (k, n)))
        off += m * n; oQ += m * k; oR += k * n
        parts.append(a.ravel())
    meta = tuple(meta)
    data = np.concatenate(parts)
    Q, R = (host(x) for x in ops.qr(dev(data), meta, (oQ, oR)))
    Qr, Rr = oracle.qr(data, meta, (oQ, oR))
    _qr_checks(data, meta, Q, R, Qr, Rr)
    gQ, gR = f(oQ), f(oR)
    meta_w = meta[:4]  # the graded block's adjoint amplifies by 1e10
    g = host(ops.qr_backward(dev(Qr), dev(Rr), dev(gQ), dev(gR), dev(data), meta_w))
    ref = oracle.qr_backward(Qr, Rr, gQ, gR, data, meta_w)
    assert rel(g, ref) <= 1e-10


@pytest.mark.parametrize('cplx', [False, True])
def test_qr_autograd_gradcheck(cplx, cuda_device):
    """torch.autograd.gradcheck of the backend's qr Function (central differences; complex
    inputs are checked by torch in its Wirtinger convention)."""
    from yastn_gb300 import backend as BK
    rng = np.random.default_rng(2)
    shapes = [(5, 3), (4, 4), (2, 6)]
    meta, off, oQ, oR = [], 0, 0, 0
    for m, n in shapes:
        k = min(m, n)
        meta.append(((off, off + m * n), (m, n), (oQ, oQ + m * k), (m, k), (oR, oR + k * n), (k, n)))
        off += m * n; oQ += m * k; oR += k * n
    meta = tuple(meta)
    x = dev(rng.normal(size=off) + (1j * rng.normal(size=off) if cplx else 0)).requires_grad_(True)
    assert torch.autograd.gradcheck(lambda d: BK.qr(d, meta, (oQ, oR)), (x,), eps=1e-6, atol=1e-7)
