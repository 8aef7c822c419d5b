"""The allocation-free emulated dot (yb_ozaki_dot_static) against the allocating one.

Some callers cannot allocate device memory at the moment they call into this library:
a host framework that owns the whole device memory budget and forbids allocations after
start-up, or a caller for which an allocation would synchronise the device in the middle
of its stream work. For them the library offers one entry point whose scratch lives in a
device array built into the library (16 MiB, shared by all calls). This test calls it
through the C ABI on two calls in a row, with different shapes and data, and checks each
result against the regular entry point (scratch from the caller) within the 1e-12
tolerance of the other sector-GEMM tests; it also checks the size limit.
"""
import ctypes

import numpy as np
import pytest
import torch

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


def _call_static(A, B, meta, Dsize, s=8):
    plan = P.ozaki_dot_plan(meta, s)
    bt_tasks, bt_items = plan.bT.packed(False)
    arrs = [_dev(x) for x in (plan.a_recs, plan.b_recs, bt_tasks, bt_items, plan.outs, plan.tiles)]
    C = torch.zeros(Dsize, dtype=torch.float64, device='cuda')
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    st = N.lib().yb_ozaki_dot_static(
        _p(A), _p(B), _p(C), _p(arrs[0]), len(plan.a_recs), plan.a_rows, _p(arrs[1]), len(plan.b_recs), plan.b_rows,
        _p(arrs[2]), len(bt_tasks), _p(arrs[3]), len(bt_items), _p(arrs[4]), _p(arrs[5]), len(plan.tiles), s,
        plan.a_size, plan.b_size, plan.a_exps, plan.b_exps, plan.bT_size, stream)
    torch.cuda.synchronize()
    return st, C


def test_static_scratch_dot_matches_allocating_entry_point(cuda_device):
    rng = np.random.default_rng(17)
    for shapes in ([(40, 70, 30), (64, 64, 64), (16, 200, 20)],
                   [(130, 90, 77), (17, 33, 250), (48, 16, 16)]):
        meta, A, B, Dsize = _problem(shapes, rng)
        dA, dB = _dev(A), _dev(B)
        st, got = _call_static(dA, dB, meta, Dsize)
        assert st == N.YB_OK
        ref = ops.dot_ozaki(dA, dB, meta, Dsize)
        err = float((got - ref).abs().max() / ref.abs().max())
        assert err <= TOL, err


def test_static_scratch_rejects_problems_beyond_its_size(cuda_device):
    rng = np.random.default_rng(18)
    meta, A, B, Dsize = _problem([(900, 900, 900)], rng)  # 2 x 8 x 900 x 912 bf16 + B^T > 16 MiB
    st, _ = _call_static(_dev(A), _dev(B), meta, Dsize)
    assert st == N.YB_ERR_TOO_LARGE
