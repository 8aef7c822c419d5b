"""The allocation-free emulated dot (yb_ozaki_dot_static) against the allocating one and
the oracle.

Some callers cannot allocate device memory at the moment they call into this library:
a host framework that owns the whole device memory budget and forbids allocations after
start-up, or a caller for which an allocation would synchronise the device in the middle
of its stream work. For them the library offers one entry point whose scratch lives in a
device array built into the library (16 MiB, shared by all calls). This test calls it
through the C ABI on two calls in a row, with different shapes and data, and checks each
result against the regular entry point (scratch from the caller) and against the oracle,
within the 1e-12 tolerance of the other sector-GEMM tests. The shapes include sectors the
emulation leaves to the native FP64 kernel (K < 16; at most 8 rows and more than 64
columns), which the call computes too. It also checks the size limit and that complex
data is refused.
"""
import ctypes

import numpy as np
import pytest
import torch

import oracle
from yastn_gb300 import _native as N
from yastn_gb300 import _plans as P
from yastn_gb300 import ops

pytestmark = pytest.mark.gpu
TOL = 1e-12


def _problem(shapes, rng):
    """Random sector GEMMs C_k = A_k B_k laid out as YASTN's dot metadata."""
    meta, oa, ob, oc, As, Bs = [], 0, 0, 0, [], []
    for m, k, n in shapes:
        meta.append(((oc, oc + m * n), (m, n), (oa, oa + m * k), (m, k), (ob, ob + k * n), (k, n)))
        As.append(rng.normal(size=m * k))
        Bs.append(rng.normal(size=k * n))
        oa += m * k; ob += k * n; oc += m * n
    return tuple(meta), np.concatenate(As), np.concatenate(Bs), oc


def _dev(x):
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def _call_static(A, B, meta, Dsize, s=8, dtype=N.YB_F64):
    plan = P.ozaki_dot_plan(meta, s)
    nat = plan.native_direct
    arrs = [_dev(x) for x in (plan.split_recs, plan.split_groups, plan.outs, plan.tiles,
                              nat.outs, nat.terms, nat.tiles)]
    C = torch.zeros(Dsize, dtype=torch.float64, device='cuda')
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    st = N.lib().yb_ozaki_dot_static(
        _p(A), _p(B), _p(C), dtype, _p(arrs[0]), _p(arrs[1]), len(plan.split_groups), _p(arrs[2]), _p(arrs[3]),
        len(plan.tiles), _p(arrs[4]), _p(arrs[5]), _p(arrs[6]), len(nat.tiles), s, plan.a_size, plan.b_size,
        plan.a_exps, plan.b_exps, stream)
    torch.cuda.synchronize()
    return st, C


def test_static_scratch_dot_matches_allocating_entry_point_and_oracle(cuda_device):
    rng = np.random.default_rng(17)
    # second list: a K < 16 sector (48 x 8 x 70) and a skinny one (5 x 300 x 200), native
    for shapes in ([(40, 70, 30), (64, 64, 64), (16, 200, 20)],
                   [(130, 90, 77), (17, 33, 250), (48, 8, 70), (5, 300, 200), (48, 16, 16)]):
        meta, A, B, Dsize = _problem(shapes, rng)
        plan = P.ozaki_dot_plan(meta, 8)
        assert len(plan.tiles) > 0
        if len(shapes) > 3:
            assert len(plan.native_direct.tiles) > 0  # the native sectors are part of this call
        dA, dB = _dev(A), _dev(B)
        st, got = _call_static(dA, dB, meta, Dsize)
        assert st == N.YB_OK
        ref = ops.dot_ozaki(dA, dB, meta, Dsize)
        err = float((got - ref).abs().max() / ref.abs().max())
        assert err <= TOL, err
        want = oracle.dot(A, B, meta, Dsize)
        g = got.cpu().numpy()
        for slc, Dc, *_ in meta:
            r = want[slc[0]:slc[1]]
            assert np.abs(g[slc[0]:slc[1]] - r).max() <= TOL * np.abs(r).max(), Dc


def test_static_scratch_rejects_problems_beyond_its_size_and_complex_data(cuda_device):
    rng = np.random.default_rng(18)
    meta, A, B, Dsize = _problem([(900, 900, 900)], rng)  # 2 x (2 x 8 x 900 x 912) bytes of digits > 16 MiB
    st, _ = _call_static(_dev(A), _dev(B), meta, Dsize)
    assert st == N.YB_ERR_TOO_LARGE
    meta, A, B, Dsize = _problem([(32, 32, 32)], rng)
    st, _ = _call_static(_dev(A), _dev(B), meta, Dsize, dtype=N.YB_C128)
    assert st == N.YB_ERR_INVALID
