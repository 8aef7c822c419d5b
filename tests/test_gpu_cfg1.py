"""The benchmark workload end to end on the GPU, through the backend module exactly as
YASTN drives it (the recorded call sequence of tensordot + svd_with_truncation on the
U(1) D=64 rank-4 tensors, regenerated from seed 0), against the oracle and the
reference's recorded spectrum and truncation."""
import numpy as np
import pytest
import torch

import oracle
from yastn_gb300 import backend as BK
from yastn_gb300 import ops
from yastn_gb300.workloads import load_trace, cfg1_inputs

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def test_cfg1_tensordot_svd_truncation(cuda_device):
    tr = load_trace('cfg1')
    calls = tr['calls']
    A, B = cfg1_inputs(tr)
    dA, dB = torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda()
    # tensordot: merge A, merge B, dot, unmerge
    c0, c1, c2, c3 = calls[:4]
    Am = BK.transpose_and_merge(dA, *c0['args'][1:])
    Bm = BK.transpose_and_merge(dB, *c1['args'][1:])
    Cm = BK.dot(Am, Bm, *c2['args'][2:])
    C = BK.unmerge(Cm, c3['args'][1])
    Cref = oracle.unmerge(oracle.dot(oracle.transpose_and_merge(A, *c0['args'][1:]),
                                     oracle.transpose_and_merge(B, *c1['args'][1:]), *c2['args'][2:]),
                          c3['args'][1])
    Ch = C.cpu().numpy()
    assert rel(Ch, Cref) <= 1e-12
    assert abs(float(Ch.sum()) - tr['C_checksum']['sum0']) <= 1e-9 * tr['C_checksum']['abs0']
    # svd_with_truncation: merge C, svd, unmerge U and V
    c4, c5, c6, c7 = calls[4:8]
    M = BK.transpose_and_merge(C, *c4['args'][1:])
    meta_svd, sizes = c5['args'][1], c5['args'][2]
    U, S, V = BK.svd(M, meta_svd, sizes)
    Sh = S.cpu().numpy()
    assert rel(Sh, np.array(tr['S_full'])) <= 1e-12
    Uu = BK.unmerge(U, c6['args'][1])
    Vu = BK.unmerge(V, c7['args'][1])
    # truncation D_total=64 by global ranking: kept sectors (-1, 0, 1) with (11, 41, 12)
    slices = [m[4] for m in meta_svd]
    order = np.argsort([sl[0] for sl in slices])
    s_slices = [tuple(slices[i]) for i in order]
    mask, kept = ops.truncation_mask_data(S, s_slices, None, D_total=64)
    assert sum(kept) == 64
    ref_mask = oracle.truncation_mask(np.array(tr['S_full']), s_slices, None, D_total=64)
    np.testing.assert_array_equal(mask.cpu().numpy(), ref_mask)
    np.testing.assert_allclose(np.sort(Sh[mask.cpu().numpy()])[::-1], np.sort(tr['S_kept'])[::-1], rtol=1e-12)
    assert sorted(k for k in kept if k) == sorted(d[0] for d in tr['S_kept_D'])
    # apply the recorded masks (same kept indices) to U, S, V
    for c, data in zip(calls[8:11], (Uu, S, Vu)):
        Ain, mask_r, meta, Dsize, axis, ndim = c['args']
        dmask = {k: torch.as_tensor(np.asarray(v, dtype=np.int64)).cuda() for k, v in mask_r.items()}
        out = BK.apply_mask(data, dmask, meta, Dsize, axis, ndim)
        assert out.numel() == Dsize
        if data is S:  # U and V are compared through the gauge-free spectrum only
            np.testing.assert_allclose(out.cpu().numpy(), np.array(tr['S_kept']), rtol=1e-12)


@pytest.mark.parametrize('mode', ['fp64', 'emulated'])
def test_heff2_lanczos_on_gpu(mode, cuda_device):
    """The DMRG Heff2 matvec (10 backend calls, 772 sector GEMMs) and YASTN's 30-step
    Lanczos on the GPU: the matvec within 1e-12 of the oracle replay, the lowest Ritz value
    within 1e-10 of the reference's own eigs result."""
    from yastn_gb300.workloads import Heff2Workload, lanczos, ritz_lowest
    wl = Heff2Workload()
    BK.set_gemm_mode(mode)
    try:
        env = wl.env(lambda x: torch.from_numpy(x).cuda())
        mv = lambda v: wl.matvec(v, env, BK.dot, BK.transpose_and_merge, lambda x, f: x * f)
        out = mv(torch.from_numpy(wl.data['AA']).cuda()).cpu().numpy()
        envh = wl.env(lambda x: x)
        ref = wl.matvec(wl.data['AA'], envh, oracle.dot, oracle.transpose_and_merge, lambda x, f: x * f)
        assert rel(out, ref) <= 1e-12
        V, al, be = lanczos(mv, torch.from_numpy(wl.data['AA']).cuda(), 30, torch.dot, torch.linalg.vector_norm)
        lam, _ = ritz_lowest(al, be)
        assert abs(lam - wl.tr['lanczos_lowest']) <= 1e-10 * abs(wl.tr['lanczos_lowest'])
    finally:
        BK.set_gemm_mode('fp64')
