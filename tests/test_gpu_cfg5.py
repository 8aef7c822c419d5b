"""Precision-study workload on the GPU: U(1) rank-4 tensors with D=128 per leg over
t=-16..16 and every block scaled by 10^u, u ~ U(-4, 0); tensordot A(2,3) x B(0,1) under
fuse_to_matrix (sector GEMMs up to 946^3). Native FP64 and the emulated (BF16 digit
slices) sector GEMMs are both held to 1e-12 relative per sector result against the FP64
oracle, and the unmerged result to the reference's checksum."""
import numpy as np
import pytest
import torch

import oracle
from yastn_gb300 import backend as BK
from yastn_gb300.workloads import load_trace, cfg5_inputs

pytestmark = pytest.mark.gpu
TOL = 1e-12


@pytest.fixture(scope='module')
def cfg5():
    tr = load_trace('cfg5')
    A, B = cfg5_inputs(tr)
    c0, c1, c2, c3 = tr['calls']
    Am = oracle.transpose_and_merge(A, *c0['args'][1:])
    Bm = oracle.transpose_and_merge(B, *c1['args'][1:])
    ref = oracle.dot(Am, Bm, *c2['args'][2:])
    return tr, A, B, ref


@pytest.mark.parametrize('mode', ['fp64', 'emulated'])
def test_cfg5_per_sector_error(mode, cfg5, cuda_device):
    tr, A, B, ref = cfg5
    c0, c1, c2, c3 = tr['calls']
    saved = BK.get_gemm_mode()
    BK.set_gemm_mode(mode)
    try:
        dA, dB = torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda()
        Am = BK.transpose_and_merge(dA, *c0['args'][1:])
        Bm = BK.transpose_and_merge(dB, *c1['args'][1:])
        Cm = BK.dot(Am, Bm, *c2['args'][2:])
        C = BK.unmerge(Cm, c3['args'][1]).cpu().numpy()
        got = Cm.cpu().numpy()
    finally:
        BK.set_gemm_mode(saved)
    for slc, Dc, *_ in c2['args'][2]:
        r, g = ref[slc[0]:slc[1]], got[slc[0]:slc[1]]
        if r.size:
            assert np.abs(g - r).max() <= TOL * np.abs(r).max(), (mode, Dc)
    chk = tr['C_checksum']
    assert abs(float(C.sum()) - chk['sum0']) <= 1e-10 * chk['abs0']
