"""U(1)xU(1) complex128 workload on the GPU (595 uneven blocks per tensor): the tensordot
(two merges, 595 complex sector GEMMs in one launch) against the oracle per sector and the
reference's checksum; the truncated block SVD of C (34 complex sectors up to 1661) against
the reference's spectrum checksum, the kept dimensions exactly, and U S Vh = C."""
import numpy as np
import pytest
import torch

import oracle
from yastn_gb300 import backend as BK, ops
from yastn_gb300.workloads import load_trace, cfg3_inputs

pytestmark = pytest.mark.gpu
TOL = 1e-12


@pytest.fixture(scope='module')
def cfg3():
    tr = load_trace('cfg3')
    A, B = cfg3_inputs(tr)
    return tr, A, B


@pytest.mark.parametrize('mode', ['fp64', 'emulated'])
def test_cfg3_tensordot(mode, cfg3, cuda_device):
    tr, A, B = cfg3
    c0, c1, c2 = tr['calls'][:3]
    Am = oracle.transpose_and_merge(A, *c0['args'][1:])
    Bm = oracle.transpose_and_merge(B, *c1['args'][1:])
    ref = oracle.dot(Am, Bm, *c2['args'][2:])
    dAm = BK.transpose_and_merge(torch.from_numpy(A).cuda(), *c0['args'][1:])
    dBm = BK.transpose_and_merge(torch.from_numpy(B).cuda(), *c1['args'][1:])
    np.testing.assert_array_equal(dAm.cpu().numpy(), Am)
    saved = BK.get_gemm_mode()
    BK.set_gemm_mode(mode)
    try:
        got = BK.dot(dAm, dBm, *c2['args'][2:]).cpu().numpy()
    finally:
        BK.set_gemm_mode(saved)
    for slc, Dc, *_ in c2['args'][2]:
        r, g = ref[slc[0]:slc[1]], got[slc[0]:slc[1]]
        if r.size:
            assert np.abs(g - r).max() <= TOL * np.abs(r).max(), Dc
    chk = tr['C_checksum']
    assert abs(float(got.real.sum()) - chk['sum0']) <= 1e-10 * chk['abs0']


def test_cfg3_svd_with_truncation(cfg3, cuda_device):
    tr, A, B = cfg3
    c = tr['calls']
    Am = oracle.transpose_and_merge(A, *c[0]['args'][1:])
    Bm = oracle.transpose_and_merge(B, *c[1]['args'][1:])
    C = oracle.dot(Am, Bm, *c[2]['args'][2:])
    M = BK.transpose_and_merge(torch.from_numpy(C).cuda(), *c[3]['args'][1:])
    meta, sizes = c[4]['args'][1:3]
    U, S, V = BK.svd(M, meta, sizes)
    Sh = S.cpu().numpy()
    chk = c[4]['out'][1].checksum
    assert abs(float(Sh.sum()) - chk['sum0']) <= 1e-10 * chk['abs0']
    assert abs(float((Sh * Sh).sum()) - chk['sq0']) <= 1e-10 * chk['sq0']
    slices = [tuple(m[4]) for m in meta]
    mask, kept = ops.truncation_mask_data(S, slices, None, tol=1e-8)
    assert sorted(k for k in kept if k) == sorted(d[0] for d in tr['S_kept_D'])
    Mh, Uh, Vh = M.cpu().numpy(), U.cpu().numpy(), V.cpu().numpy()
    for sl, D, slU, DU, slS, slV, DV in meta:
        a = Mh[sl[0]:sl[1]].reshape(D)
        u, s, v = Uh[slU[0]:slU[1]].reshape(DU), Sh[slS[0]:slS[1]], Vh[slV[0]:slV[1]].reshape(DV)
        assert np.abs((u * s) @ v - a).max() <= TOL * np.abs(a).max() * max(1, min(D))
