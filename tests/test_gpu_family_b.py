"""Family (b) on the GPU: grouped sector GEMMs (dot, transpose_dot_sum) and adjoints.

Tolerance: max |C - C_ref| <= 1e-12 * max |C_ref| (FP64, norm-wise relative), the
reference tests' 1e-12 (tests/tensor/test_tensordot.py:21).
"""
import json
import os

import numpy as np
import pytest
import torch

import oracle
from yastn_gb300 import ops
from yastn_gb300.workloads import load_trace, cfg1_inputs, GOLDEN, _decode

pytestmark = pytest.mark.gpu
TOL = 1e-12


def dev(x):
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


def host(t):
    return t.detach().cpu().numpy()


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)) if b.size else 0.0


@pytest.mark.parametrize('name', ['tensordot_fuse_to_matrix', 'tensordot_fuse_contracted', 'tensordot_no_fusion'])
def test_dot_and_tds_on_reference_calls(name, cuda_device):
    tr = load_trace(name)
    n = 0
    for c in tr['calls']:
        if c['fn'] == 'dot':
            A, B, meta, Dsize = c['args']
            got = host(ops.dot(dev(A), dev(B), meta, Dsize))
            assert got.dtype == c['out'][0].dtype
            assert rel(got, c['out'][0]) <= TOL
            n += 1
        elif c['fn'] == 'transpose_dot_sum':
            A, B, meta, Ar, Br, Ao, Bo, Dsize = c['args']
            got = host(ops.transpose_dot_sum(dev(A), dev(B), meta, Ar, Br, Ao, Bo, Dsize))
            assert rel(got, c['out'][0]) <= TOL
            n += 1
    assert n > 0


@pytest.mark.parametrize('name', ['tensordot_fuse_to_matrix', 'tensordot_fuse_contracted'])
def test_dot_adjoint_matches_oracle(name, cuda_device):
    tr = load_trace(name)
    rng = np.random.default_rng(5)
    for c in tr['calls']:
        if c['fn'] != 'dot':
            continue
        A, B, meta, Dsize = c['args']
        dtype = np.promote_types(A.dtype, B.dtype)
        Cb = rng.normal(size=Dsize).astype(dtype)
        if np.iscomplexobj(Cb):
            Cb = Cb + 1j * rng.normal(size=Dsize)
        Ab, Bb = ops.dot_backward(dev(Cb), dev(A), dev(B), meta)
        Ar, Br = oracle.dot_backward(Cb, A, B, meta)
        assert rel(host(Ab), Ar) <= TOL and rel(host(Bb), Br) <= TOL


def test_dot_golden_adjoint(cuda_device):
    tr = load_trace('adjoints')
    A = tr['_arrays']
    c = [c for c in tr['calls'] if c['fn'] == 'dot_backward'][0]
    Ab, Bb = ops.dot_backward(dev(A[c['Cb']]), dev(A[c['A']]), dev(A[c['B']]), c['meta'])
    assert rel(host(Ab), A[c['Ab']]) <= TOL and rel(host(Bb), A[c['Bb']]) <= TOL


def test_tds_golden_adjoint(cuda_device):
    with open(os.path.join(GOLDEN, 'tds_adjoint.json')) as f:
        args = json.load(f)['args']
    meta, Ar, Br, Ao, Bo, _ = (_decode(a, None) for a in args)
    z = np.load(os.path.join(GOLDEN, 'tds_adjoint.npz'))
    Ab, Bb = ops.transpose_dot_sum_backward(dev(z['Cb']), dev(z['A']), dev(z['B']), meta, Ar, Br, Ao, Bo)
    assert rel(host(Ab), z['Ab']) <= TOL and rel(host(Bb), z['Bb']) <= TOL


def test_dot_empty_and_zero_k(cuda_device):
    """Sectors with an empty contracted dimension give zero blocks; no sectors give an empty output."""
    meta = (((0, 6), (2, 3), (0, 0), (2, 0), (0, 0), (0, 3)),)
    A = torch.zeros(1, dtype=torch.float64, device='cuda')
    B = torch.zeros(1, dtype=torch.float64, device='cuda')
    got = host(ops.dot(A, B, meta, 6))
    np.testing.assert_array_equal(got, np.zeros(6))
    assert ops.dot(A, B, (), 0).numel() == 0


@pytest.mark.parametrize('cplx', [False, True])
def test_split_k_dots(cplx, cuda_device):
    """Outputs with few tiles and a long contracted dimension (split-K: chunk products and
    an ordered reduction) against the oracle, forward and adjoint, real and complex."""
    from yastn_gb300 import _plans as P
    rng = np.random.default_rng(12)
    shapes = [(1, 373248, 1), (3, 3000, 2000), (100, 1500, 100), (5, 7, 9)]
    meta, oa, ob, oc = [], 0, 0, 0
    for m, k, n in shapes:
        meta.append(((oc, oc + m * n), (m, n), (oa, oa + m * k), (m, k), (ob, ob + k * n), (k, n)))
        oa += m * k; ob += k * n; oc += m * n
    meta = tuple(meta)
    assert P.dot_plan(meta).split is not None
    f = lambda n: rng.normal(size=n) + (1j * rng.normal(size=n) if cplx else 0)
    A, B, Cb = f(oa), f(ob), f(oc)
    got = host(ops.dot(dev(A), dev(B), meta, oc))
    assert rel(got, oracle.dot(A, B, meta, oc)) <= TOL
    Ab, Bb = ops.dot_backward(dev(Cb), dev(A), dev(B), meta)
    Ar, Br = oracle.dot_backward(Cb, A, B, meta)
    assert rel(host(Ab), Ar) <= TOL and rel(host(Bb), Br) <= TOL


@pytest.mark.parametrize('cplx', [False, True])
def test_skinny_tile_kinds(cplx, cuda_device):
    """Outputs with 1..16 rows (skinny tiles up to the kernel's bound of 16) and with 1..16
    columns (64x64 tiles; their adjoints make skinny outputs) against the oracle, forward
    and adjoint."""
    from yastn_gb300 import _plans as P
    rng = np.random.default_rng(13)
    shapes = [(r, 37, 700) for r in range(1, 17)] + [(700, 29, c) for c in range(1, 17)] + \
             [(2592, 18, 9), (9, 9, 9), (64, 64, 64)]
    meta, oa, ob, oc = [], 0, 0, 0
    for m, k, n in shapes:
        meta.append(((oc, oc + m * n), (m, n), (oa, oa + m * k), (m, k), (ob, ob + k * n), (k, n)))
        oa += m * k; ob += k * n; oc += m * n
    meta = tuple(meta)
    f = lambda n: rng.normal(size=n) + (1j * rng.normal(size=n) if cplx else 0)
    A, B, Cb = f(oa), f(ob), f(oc)
    saved = P.SKINNY_ROWS
    P.SKINNY_ROWS = 16
    try:
        got = host(ops.dot(dev(A), dev(B), meta, oc))
        Ab, Bb = ops.dot_backward(dev(Cb), dev(A), dev(B), meta)
    finally:
        P.SKINNY_ROWS = saved
        P.CACHE.by_id.clear(); P.CACHE.by_val.clear()
    assert rel(got, oracle.dot(A, B, meta, oc)) <= TOL
    Ar, Br = oracle.dot_backward(Cb, A, B, meta)
    assert rel(host(Ab), Ar) <= TOL and rel(host(Bb), Br) <= TOL


@pytest.mark.parametrize('cplx', [False, True])
def test_tall_and_wide_skinny_tiles(cplx, cuda_device):
    """Default plans: outputs of at most 16 columns and many rows (tall tiles: 256 rows x all
    columns, one row per thread) and of 9..16 rows at least 4096 wide (skinny tiles), as the
    double-layer contraction's sector GEMMs are, against the oracle: forward, adjoint, and
    alpha/beta."""
    from yastn_gb300 import _plans as P
    rng = np.random.default_rng(14)
    shapes = [(3000, 18, 9), (700, 5, 16), (65, 40, 1), (9, 36, 5000), (16, 7, 4096), (12, 3, 4500),
              (2600, 70, 3), (64, 9, 9)]
    meta, oa, ob, oc = [], 0, 0, 0
    for m, k, n in shapes:
        meta.append(((oc, oc + m * n), (m, n), (oa, oa + m * k), (m, k), (ob, ob + k * n), (k, n)))
        oa += m * k; ob += k * n; oc += m * n
    meta = tuple(meta)
    plan = P.dot_plan(meta)
    assert {1, 3} <= set(int(t[3]) for t in plan.tiles)
    f = lambda n: rng.normal(size=n) + (1j * rng.normal(size=n) if cplx else 0)
    A, B, Cb, C0 = f(oa), f(ob), f(oc), f(oc)
    got = host(ops.dot(dev(A), dev(B), meta, oc))
    ref = oracle.dot(A, B, meta, oc)
    assert rel(got, ref) <= TOL
    Ab, Bb = ops.dot_backward(dev(Cb), dev(A), dev(B), meta)
    Ar, Br = oracle.dot_backward(Cb, A, B, meta)
    assert rel(host(Ab), Ar) <= TOL and rel(host(Bb), Br) <= TOL
    c = dev(C0)
    ops.run_gemm(plan, dev(A), dev(B), c, alpha=0.5, beta=2.0)
    assert rel(host(c), 0.5 * ref + 2.0 * C0) <= TOL


def test_cfg1_full_size_dot(cuda_device):
    """The benchmark's 13 sector GEMMs (n up to 822, 3.25 GFLOP) vs numpy BLAS."""
    tr = load_trace('cfg1')
    A, B = cfg1_inputs(tr)
    c0, c1, c2 = tr['calls'][:3]
    Am = oracle.transpose_and_merge(A, *c0['args'][1:])
    Bm = oracle.transpose_and_merge(B, *c1['args'][1:])
    _, _, meta, Dsize = c2['args']
    got = host(ops.dot(dev(Am), dev(Bm), meta, Dsize))
    ref = oracle.dot(Am, Bm, meta, Dsize)
    assert rel(got, ref) <= TOL
    chk = c2['out'][0].checksum
    assert abs(float(got.sum()) - chk['sum0']) <= 1e-9 * chk['abs0']


@pytest.mark.parametrize('name', ['tensordot_fuse_to_matrix', 'tensordot_fuse_contracted'])
def test_dot_ozaki_on_reference_calls(name, cuda_device):
    """Emulated FP64 (8 BF16 digit slices) within 1e-12 of the reference products."""
    tr = load_trace(name)
    n = 0
    for c in tr['calls']:
        if c['fn'] != 'dot' or np.iscomplexobj(c['args'][0]) or np.iscomplexobj(c['args'][1]):
            continue
        A, B, meta, Dsize = c['args']
        got = host(ops.dot_ozaki(dev(A), dev(B), meta, Dsize))
        assert rel(got, c['out'][0]) <= TOL
        n += 1
    assert n > 0


@pytest.mark.parametrize('tc', [64, 32, False])
def test_hold_constant_operands(tc, cuda_device):
    """Inside ops.hold_constant_operands an unchanged operand's merge and digit planes are
    computed once: results stay bit-identical to calls outside the scope, a held operand
    modified in place (version counter) or a held merge output modified in place is
    recomputed, and nothing is held across the scope's end."""
    tr = load_trace('cfg1')
    A, B = cfg1_inputs(tr)
    c0, c1, c2 = tr['calls'][:3]
    _, _, meta, Dsize = c2['args']
    Am = oracle.transpose_and_merge(A, *c0['args'][1:])
    Bg = dev(B)
    saved = ops.OZAKI_TC[0]
    ops.OZAKI_TC[0] = tc
    try:
        rng = np.random.default_rng(21)
        As = [dev(Am * (1.0 + 0.1 * i) + 1e-3 * rng.normal(size=Am.size)) for i in range(3)]
        want = [host(ops.dot_ozaki(a, ops.merge(Bg, *c1['args'][1:]), meta, Dsize)) for a in As]
        with ops.hold_constant_operands():
            Bm1 = ops.merge(Bg, *c1['args'][1:])
            Bm2 = ops.merge(Bg, *c1['args'][1:])
            assert Bm2 is Bm1  # the held merge
            got = [host(ops.dot_ozaki(a, ops.merge(Bg, *c1['args'][1:]), meta, Dsize)) for a in As]
            assert all(np.array_equal(g, w) for g, w in zip(got, want))
            assert len(ops._HOLD['split']) >= 1 and len(ops._HOLD['merge']) == 1
            # the source changes in place: merge and digits are recomputed
            Bg.mul_(2.0)
            Bm3 = ops.merge(Bg, *c1['args'][1:])
            assert Bm3 is not Bm1
            g2 = host(ops.dot_ozaki(As[0], Bm3, meta, Dsize))
            assert np.array_equal(g2, 2.0 * want[0])
            # the held output changes in place: the merge is recomputed from the source
            Bm3.zero_()
            Bm4 = ops.merge(Bg, *c1['args'][1:])
            assert Bm4 is not Bm3 and float(Bm4.abs().max()) > 0
        assert not ops._HOLD['split'] and not ops._HOLD['merge']
    finally:
        ops.OZAKI_TC[0] = saved


def test_cfg1_full_size_dot_ozaki(cuda_device):
    """The benchmark's 13 sector GEMMs emulated: error vs the FP64 oracle per slice count."""
    tr = load_trace('cfg1')
    A, B = cfg1_inputs(tr)
    c0, c1, c2 = tr['calls'][:3]
    Am = oracle.transpose_and_merge(A, *c0['args'][1:])
    Bm = oracle.transpose_and_merge(B, *c1['args'][1:])
    _, _, meta, Dsize = c2['args']
    ref = oracle.dot(Am, Bm, meta, Dsize)
    errs = {}
    for s in (6, 7, 8):
        errs[s] = rel(host(ops.dot_ozaki(dev(Am), dev(Bm), meta, Dsize, slices=s)), ref)
    assert errs[8] <= TOL, errs
    assert errs[7] <= 1e-10 and errs[6] <= 1e-8, errs


def test_dot_ozaki_wide_dynamic_range(cuda_device):
    """Per-block scales 10^U(-4,0) (the precision-study inputs): per-row exponents keep it exact."""
    rng = np.random.default_rng(9)
    shapes = [(40, 70, 30), (64, 64, 64), (3, 200, 5)]
    meta, oa, ob, oc, As, Bs = [], 0, 0, 0, [], []
    for m, k, n in shapes:
        a = rng.normal(size=(m, k)) * 10 ** rng.uniform(-4, 0)
        b = rng.normal(size=(k, n)) * 10 ** rng.uniform(-4, 0)
        meta.append(((oc, oc + m * n), (m, n), (oa, oa + m * k), (m, k), (ob, ob + k * n), (k, n)))
        oa += m * k; ob += k * n; oc += m * n
        As.append(a.ravel()); Bs.append(b.ravel())
    meta = tuple(meta)
    A, B = np.concatenate(As), np.concatenate(Bs)
    ref = oracle.dot(A, B, meta, oc)
    got = host(ops.dot_ozaki(dev(A), dev(B), meta, oc))
    for slc, Dc, *_ in meta:
        r, g = ref[slc[0]:slc[1]], got[slc[0]:slc[1]]
        assert np.abs(g - r).max() <= TOL * np.abs(r).max()


SMALL_SHAPES = [(1, 16, 1), (1, 40, 1), (7, 33, 3), (15, 17, 129), (70, 20, 2), (9, 160, 34), (130, 50, 9),
                (3, 5, 2000), (5, 8, 100), (64, 3, 64), (66, 15, 65), (33, 1, 31)]


def _small_sector_problem(seed, cplx=False):
    rng = np.random.default_rng(seed)
    meta, oa, ob, oc = [], 0, 0, 0
    for m, k, n in SMALL_SHAPES:
        meta.append(((oc, oc + m * n), (m, n), (oa, oa + m * k), (m, k), (ob, ob + k * n), (k, n)))
        oa += m * k; ob += k * n; oc += m * n
    A, B = rng.normal(size=oa), rng.normal(size=ob)
    if cplx:
        A, B = A + 1j * rng.normal(size=oa), B - 1j * rng.normal(size=ob)
    return tuple(meta), A, B, oc


@pytest.mark.parametrize('emulated', [False, True])
@pytest.mark.parametrize('cplx', [False, True])
def test_dot_small_and_ragged_sectors(emulated, cplx, cuda_device):
    """Sectors with m or n below a warp's share of a tile (skipped warps), K not a multiple of
    the K-step, skinny and tall outputs: native and emulated (complex: two real products with
    doubled K), both GEMM kernels, against the oracle per sector."""
    meta, A, B, oc = _small_sector_problem(21, cplx)
    ref = oracle.dot(A, B, meta, oc)
    saved = ops.OZAKI_TC[0]
    try:
        for tc in ((64, 32, False) if emulated else (None,)):
            ops.OZAKI_TC[0] = tc
            f = ops.dot_ozaki if emulated else ops.dot
            got = host(f(dev(A), dev(B), meta, oc))
            for slc, Dc, *_ in meta:
                r, g = ref[slc[0]:slc[1]], got[slc[0]:slc[1]]
                assert np.abs(g - r).max() <= TOL * max(np.abs(r).max(), 1e-300), (Dc, tc)
    finally:
        ops.OZAKI_TC[0] = saved


@pytest.mark.parametrize('name', ['cfg1', 'small'])
def test_ozaki_tcgen05_matches_mma_sync(name, cuda_device):
    """The tcgen05/TMEM kernel (128 x 64 and 128 x 32 tiles) and the mma.sync kernel form the
    same exact diagonal sums and the same folds: their products agree bit for bit; no CTA
    reports a failed wait."""
    if name == 'cfg1':
        tr = load_trace('cfg1')
        A, B = cfg1_inputs(tr)
        c0, c1, c2 = tr['calls'][:3]
        A = oracle.transpose_and_merge(A, *c0['args'][1:])
        B = oracle.transpose_and_merge(B, *c1['args'][1:])
        _, _, meta, Dsize = c2['args']
    else:
        meta, A, B, Dsize = _small_sector_problem(22)
    saved = ops.OZAKI_TC[0]
    try:
        got_tc = {}
        for tn in (64, 32):  # 128 x 64 tiles; 128 x 32 tiles with two alternating TMEM buffers
            ops.OZAKI_TC[0] = tn
            assert ops.ozaki_device_error(reset=True) == 0
            got_tc[tn] = host(ops.dot_ozaki(dev(A), dev(B), meta, Dsize))
            assert ops.ozaki_device_error(reset=True) == 0
        ops.OZAKI_TC[0] = False
        got_mma = host(ops.dot_ozaki(dev(A), dev(B), meta, Dsize))
    finally:
        ops.OZAKI_TC[0] = saved
    np.testing.assert_array_equal(got_tc[64], got_mma)
    np.testing.assert_array_equal(got_tc[32], got_mma)
    ref = oracle.dot(A, B, meta, Dsize)
    assert rel(got_mma, ref) <= TOL


@pytest.mark.parametrize('cplx', [False, True])
@pytest.mark.parametrize('slices', [6, 7, 8])
def test_ozaki_split_matches_digit_model(cplx, slices, cuda_device):
    """yb_ozaki_split in both layouts (digit planes and the tcgen05 tile layout), A by rows
    and B by columns in place, against the NumPy digit model bit for bit: every BF16 digit
    (padding zeros included) and every row exponent. The data spans many binades, with a
    zero row, a subnormal row and exact ties of the last digit."""
    import ctypes
    from yastn_gb300 import _native as N
    from yastn_gb300 import _plans as P
    import plan_interp as PI
    rng = np.random.default_rng(31 + slices + 10 * cplx)
    shapes = [(40, 30, 20), (16, 16, 17), (130, 20, 70), (6, 300, 200), (33, 17, 65), (20, 130, 129)]
    meta, oa, ob, oc = [], 0, 0, 0
    for m, k, n in shapes:
        meta.append(((oc, oc + m * n), (m, n), (oa, oa + m * k), (m, k), (ob, ob + k * n), (k, n)))
        oa += m * k; ob += k * n; oc += m * n
    meta = tuple(meta)
    A = rng.normal(size=oa) * np.exp(rng.normal(size=oa) * 4)
    B = rng.normal(size=ob) * np.exp(rng.normal(size=ob) * 4)
    A[:30] = 0.0                                   # the first row of the first block
    A[30:60] = rng.normal(size=30) * 1e-310        # a subnormal row
    # exact ties of the last digit: row maximum 1 (e = 1), the rest (2j + 1) 2^{-7s}
    A[60] = 1.0
    A[61:90] = (2.0 * rng.integers(0, 2 ** 30, size=29) + 1.0) * 2.0 ** (-7 * slices) * rng.choice([-1, 1], 29)
    if cplx:
        A = A + 1j * rng.normal(size=oa)
        B = B + 1j * rng.normal(size=ob)
    plan = P.ozaki_dot_plan(meta, slices, cplx)
    dA, dB = dev(A), dev(B)
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for recs, groups, sizes in ((plan.split_recs, plan.split_groups, (plan.a_size, plan.b_size)),
                                (plan.split_recs_tc, plan.split_groups_tc, (plan.a_size_tc, plan.b_size_tc)),
                                (plan.split_recs_tc32, plan.split_groups_tc32, (plan.a_size_tc32, plan.b_size_tc32))):
        want, want_e = PI.ozaki_split(recs, groups, A, B, slices, sizes, (plan.a_exps, plan.b_exps))
        a_sl = torch.full((sizes[0],), 7.0, dtype=torch.bfloat16, device='cuda')  # nonzero: padding must be written
        b_sl = torch.full((sizes[1],), 7.0, dtype=torch.bfloat16, device='cuda')
        a_ex = torch.zeros(plan.a_exps, dtype=torch.int32, device='cuda')
        b_ex = torch.zeros(plan.b_exps, dtype=torch.int32, device='cuda')
        drec, dgrp = dev(recs), dev(groups)
        N.call('yb_ozaki_split', ctypes.c_void_p(dA.data_ptr()), ctypes.c_void_p(dB.data_ptr()),
               ctypes.c_void_p(a_sl.data_ptr()), ctypes.c_void_p(b_sl.data_ptr()), ctypes.c_void_p(a_ex.data_ptr()),
               ctypes.c_void_p(b_ex.data_ptr()), ctypes.c_void_p(drec.data_ptr()), ctypes.c_void_p(dgrp.data_ptr()),
               len(groups), slices, st)
        torch.cuda.synchronize()
        for got, got_e, w, we in ((a_sl, a_ex, want[0], want_e[0]), (b_sl, b_ex, want[1], want_e[1])):
            np.testing.assert_array_equal(host(got.float()).astype(np.int64), w)
            np.testing.assert_array_equal(host(got_e).astype(np.int64), we)


def test_short_skinny_gemm_values_and_nan(cuda_device):
    """The short skinny kernel (one term, m <= 8, K <= 8): values match the oracle, and an
    infinity or NaN in B meeting a zero of A gives NaN, as in the reference's NumPy product."""
    from yastn_gb300 import _plans as P
    rng = np.random.default_rng(41)
    shapes = [(3, 4, 1500), (2, 3, 700), (1, 4, 65)]
    meta, oa, ob, oc = [], 0, 0, 0
    for m, k, n in shapes:
        meta.append(((oc, oc + m * n), (m, n), (oa, oa + m * k), (m, k), (ob, ob + k * n), (k, n)))
        oa += m * k; ob += k * n; oc += m * n
    meta = tuple(meta)
    assert P.dot_plan(meta).all_short
    A = rng.normal(size=oa)
    A[::3] = 0.0
    B = rng.normal(size=ob)
    got = host(ops.dot(dev(A), dev(B), meta, oc))
    ref = oracle.dot(A, B, meta, oc)
    assert rel(got, ref) <= TOL
    B2 = B.copy()
    B2[5] = np.inf
    B2[ob - 3] = np.nan
    with np.errstate(invalid='ignore', over='ignore'):
        ref2 = oracle.dot(A, B2, meta, oc)
    got2 = host(ops.dot(dev(A), dev(B2), meta, oc))
    np.testing.assert_array_equal(np.isnan(got2), np.isnan(ref2))
    np.testing.assert_array_equal(np.isinf(got2), np.isinf(ref2))
    ok = np.isfinite(ref2)
    assert np.abs(got2[ok] - ref2[ok]).max() <= TOL * np.abs(ref2[ok]).max()


def test_short_skinny_gemm_alpha_beta_complex_and_eight_rows(cuda_device):
    """The short skinny kernel's other compiled forms: alpha/beta (C = alpha A B + beta C, the
    form the decompositions call), complex128 strips, and sectors of 5..8 rows or K of 5..8
    (A read per use, columns in passes), all against the oracle."""
    from yastn_gb300 import _plans as P
    rng = np.random.default_rng(43)
    shapes = [(3, 4, 1500), (8, 7, 900), (5, 2, 513), (2, 8, 1030), (1, 1, 40)]
    meta, oa, ob, oc = [], 0, 0, 0
    for m, k, n in shapes:
        meta.append(((oc, oc + m * n), (m, n), (oa, oa + m * k), (m, k), (ob, ob + k * n), (k, n)))
        oa += m * k; ob += k * n; oc += m * n
    meta = tuple(meta)
    plan = P.dot_plan(meta)
    assert plan.all_short
    for cplx in (False, True):
        A, B, C0 = rng.normal(size=oa), rng.normal(size=ob), rng.normal(size=oc)
        if cplx:
            A = A + 1j * rng.normal(size=oa)
            B = B + 1j * rng.normal(size=ob)
            C0 = C0 + 1j * rng.normal(size=oc)
        ref = oracle.dot(A, B, meta, oc)
        got = host(ops.dot(dev(A), dev(B), meta, oc))
        assert rel(got, ref) <= TOL
        got_ab = host(ops.run_gemm(plan, dev(A), dev(B), dev(C0), alpha=-0.5, beta=1.5))
        assert rel(got_ab, -0.5 * ref + 1.5 * C0) <= TOL
        # beta = 0 with alpha != 1 never reads C: a NaN there does not reach the result
        Cn = np.full(oc, np.nan, dtype=C0.dtype)
        got_a = host(ops.run_gemm(plan, dev(A), dev(B), dev(Cn), alpha=2.0, beta=0.0))
        assert rel(got_a, 2.0 * ref) <= TOL
