"""Host plan compiler, checked on the CPU by interpreting the packed records with numpy.

The records are exactly what the CUDA kernels read; interpreting them reproduces the
oracle on the reference's recorded calls (bit-exact for data movement).
"""
import numpy as np
import pytest

import oracle
from yastn_gb300 import _plans as P
from yastn_gb300.workloads import load_trace
import plan_interp as PI

TRACES = ['tensordot_fuse_to_matrix', 'tensordot_fuse_contracted', 'tensordot_no_fusion', 'svd', 'cfg1']


def test_fast_division_constants():
    rng = np.random.default_rng(0)
    for d in list(range(1, 70)) + list(rng.integers(1, 2 ** 31 - 1, size=200)):
        m, s = P.fast_div_consts(int(d))
        n = np.concatenate([rng.integers(0, 2 ** 31, size=2000), [0, 2 ** 31 - 1, int(d) - 1, int(d)]])
        np.testing.assert_array_equal(PI.fast_div_np(n, m, s), n // int(d))


@pytest.mark.parametrize('name', TRACES)
@pytest.mark.parametrize('vec', [False, True])
def test_copy_plans_reproduce_reference(name, vec):
    tr = load_trace(name)
    n = 0
    for c in tr['calls']:
        if c['fn'] == 'transpose_and_merge':
            data, order, mn, mm, Dsize = c['args']
            if not isinstance(data, np.ndarray):
                continue
            plan = P.merge_plan(order, mn, mm, Dsize)
            tasks, items = plan.packed(vec and data.dtype == np.float64)
            out = PI.run_copy(tasks, items, data, np.zeros(Dsize, dtype=data.dtype))
            np.testing.assert_array_equal(out, c['out'][0])
            # adjoint: the swapped plan scatters back exactly onto the source positions
            inv = plan.swapped(data.size)
            ti, it = inv.packed(vec and data.dtype == np.float64)
            back = PI.run_copy(ti, it, out, np.zeros(data.size, dtype=data.dtype))
            np.testing.assert_array_equal(back, oracle.transpose_and_merge_backward(out, order, mn, mm, data.size))
            n += 1
        elif c['fn'] == 'unmerge':
            data, meta = c['args']
            if not isinstance(data, np.ndarray):
                continue
            plan = P.unmerge_plan(meta, data.size)
            assert plan.full
            tasks, items = plan.packed(vec and data.dtype == np.float64)
            out = PI.run_copy(tasks, items, data, np.zeros(data.size, dtype=data.dtype))
            np.testing.assert_array_equal(out, c['out'][0])
            n += 1
    if name != 'cfg1':
        assert n > 0


def test_cfg1_merge_plan_shape():
    """The benchmark merge: 231 source blocks into 13 fused sectors, full coverage."""
    tr = load_trace('cfg1')
    c = tr['calls'][0]
    _, order, mn, mm, Dsize = c['args']
    plan = P.merge_plan(order, mn, mm, Dsize)
    assert len(plan.tasks_list) == 231 and len(mn) == 13 and plan.full
    tasks, items = plan.packed(True)
    assert tasks[:, P.CP_NDIM].max() <= 2  # identity order: rows of the block, one strided dim
    rng = np.random.default_rng(1)
    data = rng.normal(size=Dsize)
    out = PI.run_copy(tasks, items, data, np.zeros(Dsize))
    np.testing.assert_array_equal(out, oracle.transpose_and_merge(data, order, mn, mm, Dsize))


@pytest.mark.parametrize('name', ['tensordot_fuse_to_matrix', 'tensordot_fuse_contracted'])
def test_dot_plans_reproduce_reference(name):
    tr = load_trace(name)
    n = 0
    for c in tr['calls']:
        if c['fn'] != 'dot':
            continue
        A, B, meta, Dsize = c['args']
        plan = P.dot_plan(meta)
        dtype = np.promote_types(A.dtype, B.dtype)
        out = PI.run_gemm(plan, A.astype(dtype), B.astype(dtype), np.zeros(Dsize, dtype=dtype))
        ref = c['out'][0]
        assert np.abs(out - ref).max() <= 1e-12 * max(1.0, np.abs(ref).max())
        # adjoint plans against the oracle adjoint
        rng = np.random.default_rng(3)
        Cb = rng.normal(size=Dsize).astype(dtype)
        pa, pb = P.dot_backward_plans(meta)
        Ab = PI.run_gemm(pa, Cb, B.astype(dtype), np.zeros(A.size, dtype=dtype))
        Bb = PI.run_gemm(pb, A.astype(dtype), Cb, np.zeros(B.size, dtype=dtype))
        Ab_r, Bb_r = oracle.dot_backward(Cb, A, B, meta)
        assert np.abs(Ab - Ab_r).max() <= 1e-12 * max(1.0, np.abs(Ab_r).max())
        assert np.abs(Bb - Bb_r).max() <= 1e-12 * max(1.0, np.abs(Bb_r).max())
        n += 1
    assert n > 0


def _meta_dot(shapes):
    meta, oa, ob, oc = [], 0, 0, 0
    for m, k, n in shapes:
        meta.append(((oc, oc + m * n), (m, n), (oa, oa + m * k), (m, k), (ob, ob + k * n), (k, n)))
        oa += m * k; ob += k * n; oc += m * n
    return tuple(meta), oa, ob, oc


@pytest.mark.parametrize('shapes', [
    [(1, 20000, 1)],                                   # a long dot product: one tile, K cut in chunks
    [(3, 3000, 2000), (100, 1500, 100), (5, 7, 9)],    # skinny and square long-K outputs beside a short one
    [(200, 1200, 150), (200, 1200, 150)],              # two dense blocks, 24 tiles: K cut in five
])
def test_split_k_plans_cover_and_reproduce(shapes):
    """Plans with few tiles and long K split the K range: the chunks cover the workspace,
    the reduction tasks cover every output, and the result is the product (dot and adjoint)."""
    meta, oa, ob, oc = _meta_dot(shapes)
    plan = P.dot_plan(meta)
    assert plan.split is not None
    rng = np.random.default_rng(4)
    A, B = rng.normal(size=oa), rng.normal(size=ob)
    out = PI.run_gemm(plan, A, B, np.zeros(oc))
    ref = oracle.dot(A, B, meta, oc)
    assert np.abs(out - ref).max() <= 1e-12 * np.abs(ref).max() * np.sqrt(max(k for _, k, _ in shapes))
    # alpha/beta applied once, by the reduction
    c0 = rng.normal(size=oc)
    out2 = PI.run_gemm(plan, A, B, c0.copy(), alpha=-0.5, beta=1.5)
    assert np.abs(out2 - (-0.5 * ref + 1.5 * c0)).max() <= 1e-11 * np.abs(ref).max()
    Cb = rng.normal(size=oc)
    pa, pb = P.dot_backward_plans(meta)
    Ab = PI.run_gemm(pa, Cb, B, np.zeros(oa))
    Bb = PI.run_gemm(pb, A, Cb, np.zeros(ob))
    Ab_r, Bb_r = oracle.dot_backward(Cb, A, B, meta)
    assert np.abs(Ab - Ab_r).max() <= 1e-11 * np.abs(Ab_r).max()
    assert np.abs(Bb - Bb_r).max() <= 1e-11 * np.abs(Bb_r).max()


def test_skinny_tile_kinds_cover_and_reproduce():
    """Outputs with at most 16 rows (skinny tiles, 1024 or 256 columns wide) beside 64x64
    tiles: coverage and values, forward and adjoint, real and complex."""
    shapes = [(3, 40, 300), (12, 20, 700), (16, 9, 2000), (500, 30, 5), (2592, 18, 9), (70, 7, 13),
              (9, 9, 9), (64, 64, 64)]
    meta, oa, ob, oc = _meta_dot(shapes)
    saved = P.SKINNY_ROWS
    P.SKINNY_ROWS = 16  # the kernel's bound (the default plans stop at 8 rows)
    try:
        plan = P.dot_plan(meta)
    finally:
        P.SKINNY_ROWS = saved
    P.CACHE.by_id.clear(); P.CACHE.by_val.clear()
    kinds = set(int(t[3]) for t in plan.tiles)
    assert kinds == {0, 1, 3}  # (500, 30, 5) and (2592, 18, 9) take tall tiles
    rng = np.random.default_rng(8)
    for cplx in (False, True):
        f = lambda n: rng.normal(size=n) + (1j * rng.normal(size=n) if cplx else 0)
        A, B, Cb = f(oa), f(ob), f(oc)
        out = PI.run_gemm(plan, A, B, np.zeros(oc, dtype=A.dtype))
        ref = oracle.dot(A, B, meta, oc)
        assert np.abs(out - ref).max() <= 1e-12 * np.abs(ref).max()
        pa, pb = P.dot_backward_plans(meta)
        Ab = PI.run_gemm(pa, Cb, B, np.zeros(oa, dtype=A.dtype))
        Bb = PI.run_gemm(pb, A, Cb, np.zeros(ob, dtype=A.dtype))
        Ab_r, Bb_r = oracle.dot_backward(Cb, A, B, meta)
        assert np.abs(Ab - Ab_r).max() <= 1e-12 * np.abs(Ab_r).max()
        assert np.abs(Bb - Bb_r).max() <= 1e-12 * np.abs(Bb_r).max()
    P.CACHE.by_id.clear(); P.CACHE.by_val.clear()


def test_tall_and_wide_skinny_tiles_cover_and_reproduce():
    """Default plans: outputs of at most 16 columns and more than 64 rows take tall tiles
    (256 rows x all columns, kind 3), outputs of 9..16 rows at least 4096 wide take skinny
    tiles (kind 1); the double-layer contraction's sector GEMMs (93312 x 18 by 18 x 9 and
    9 x 36 by 36 x 93312 at chi=144) are such outputs. Coverage and values, forward and
    adjoint, real and complex, on smaller instances."""
    shapes = [(3000, 18, 9), (700, 5, 16), (65, 40, 1), (9, 36, 5000), (16, 7, 4096), (12, 3, 4500),
              (64, 9, 9), (15, 20, 300)]
    meta, oa, ob, oc = _meta_dot(shapes)
    plan = P.dot_plan(meta)
    kinds = [int(t[3]) for t in plan.tiles]
    by_out = {}
    for oi, tr, tc, kd in plan.tiles:
        by_out.setdefault(int(oi), set()).add(int(kd))
    assert [by_out[i] for i in range(len(shapes))] == [{3}, {3}, {3}, {1}, {1}, {1}, {0}, {0}]
    assert kinds.count(3) == 12 + 3 + 1
    rng = np.random.default_rng(9)
    for cplx in (False, True):
        f = lambda n: rng.normal(size=n) + (1j * rng.normal(size=n) if cplx else 0)
        A, B, Cb = f(oa), f(ob), f(oc)
        out = PI.run_gemm(plan, A, B, np.zeros(oc, dtype=A.dtype))
        ref = oracle.dot(A, B, meta, oc)
        assert np.abs(out - ref).max() <= 1e-12 * np.abs(ref).max()
        pa, pb = P.dot_backward_plans(meta)
        Ab = PI.run_gemm(pa, Cb, B, np.zeros(oa, dtype=A.dtype))
        Bb = PI.run_gemm(pb, A, Cb, np.zeros(ob, dtype=A.dtype))
        Ab_r, Bb_r = oracle.dot_backward(Cb, A, B, meta)
        assert np.abs(Ab - Ab_r).max() <= 1e-12 * np.abs(Ab_r).max()
        assert np.abs(Bb - Bb_r).max() <= 1e-12 * np.abs(Bb_r).max()
    P.CACHE.by_id.clear(); P.CACHE.by_val.clear()


def test_short_skinny_tiles_cover_and_reproduce():
    """Outputs of one term with at most 8 rows and K <= 8 (the contractions with a small MPO
    block) take short skinny tiles of 512 columns; a plan made
    of them alone runs on the short kernel (all_short). Coverage and values, real and
    complex; the Heff2 workload's two MPO contractions are such plans."""
    shapes = [(3, 4, 1500), (1, 1, 65), (8, 8, 513), (2, 3, 4000), (2, 4, 7)]
    meta, oa, ob, oc = _meta_dot(shapes)
    plan = P.dot_plan(meta)
    assert set(int(t[3]) for t in plan.tiles) == {2} and plan.all_short
    mixed = P.dot_plan(_meta_dot(shapes + [(3, 9, 300), (64, 64, 64)])[0])
    assert set(int(t[3]) for t in mixed.tiles) == {0, 1, 2} and not mixed.all_short
    rng = np.random.default_rng(9)
    for cplx in (False, True):
        f = lambda n: rng.normal(size=n) + (1j * rng.normal(size=n) if cplx else 0)
        A, B = f(oa), f(ob)
        out = PI.run_gemm(plan, A, B, np.zeros(oc, dtype=A.dtype))
        ref = oracle.dot(A, B, meta, oc)
        assert np.abs(out - ref).max() <= 1e-12 * np.abs(ref).max()
    from yastn_gb300.workloads import Heff2Workload
    dots = [c['args'][2] for c in Heff2Workload().calls if c['fn'] == 'dot']
    assert [P.dot_plan(m).all_short for m in dots] == [False, True, True, False]


def test_split_k_not_used_when_tiles_fill_the_gpu():
    meta, *_ = _meta_dot([(64, 4096, 64)] * 400)
    assert P.dot_plan(meta).split is None


def test_tds_plans_reproduce_reference():
    import yastn_gb300._plans as PP
    tr = load_trace('tensordot_no_fusion')
    n = 0
    for c in tr['calls']:
        if c['fn'] != 'transpose_dot_sum':
            continue
        A, B, meta, Ar, Br, Ao, Bo, Dsize = c['args']
        dtype = np.promote_types(A.dtype, B.dtype)

        def permute(data, reshape, order):
            tasks, offs, low = [], [], 0
            for sl, Di, Dl, Dr in reshape:
                sst = PP.row_major_strides(Di)
                Dt = [Di[o] for o in order]
                tasks.append((sl[0], low, Dt, [sst[o] for o in order], PP.row_major_strides(Dt)))
                offs.append(low)
                low += Dl * Dr
            cp = PP.CopyPlan(tasks, low, low)
            t, it = cp.packed(False)
            return PI.run_copy(t, it, data.astype(dtype), np.zeros(low, dtype=dtype)), offs
        Ap, Aoffs = permute(A, Ar, Ao)
        Bp, Boffs = permute(B, Br, Bo)
        plan = PP.tds_plan(meta, Ar, Br, tuple(Aoffs), tuple(Boffs))
        out = PI.run_gemm(plan, Ap, Bp, np.zeros(Dsize, dtype=dtype))
        ref = c['out'][0]
        assert np.abs(out - ref).max() <= 1e-12 * max(1.0, np.abs(ref).max())
        n += 1
    assert n > 0


@pytest.mark.parametrize('dtype', [np.float64, np.complex128])
def test_svd_adjoint_decomposition_matches_oracle(dtype):
    """P/Q GEMMs + K/TR core + finishing GEMMs == torch_svd_gesdd.py:296-428 restated."""
    rng = np.random.default_rng(4)
    shapes = [(6, 6), (9, 4), (3, 8), (1, 5), (5, 1)]
    meta, off, oU, oS, oV = [], 0, 0, 0, 0
    for m, n in shapes:
        k = min(m, n)
        meta.append(((off, off + m * n), (m, n), (oU, oU + m * k), (m, k), (oS, oS + k), (oV, oV + k * n), (k, n)))
        off += m * n; oU += m * k; oS += k; oV += k * n
    meta = tuple(meta)
    data = rng.normal(size=off).astype(dtype)
    if dtype == np.complex128:
        data = data + 1j * rng.normal(size=off)
    U, S, V = oracle.svd(data, meta, (oU, oS, oV))
    gU = rng.normal(size=oU).astype(dtype)
    gV = rng.normal(size=oV).astype(dtype)
    gS = rng.normal(size=oS)
    if dtype == np.complex128:
        gU = gU + 1j * rng.normal(size=oU)
        gV = gV + 1j * rng.normal(size=oV)
    plan = P.svd_adjoint_plan(meta)
    Pm = PI.run_gemm(plan.gP, U, gU, np.zeros(plan.kk, dtype=dtype))
    Qm = PI.run_gemm(plan.gQ, V, gV, np.zeros(plan.kk, dtype=dtype))
    K, TR = PI.svd_adjoint_core(plan, Pm, Qm, S, gS, gU, gV, dtype)
    PI.run_gemm(plan.gT, K, V, TR, beta=1.0)
    PI.run_gemm(plan.gR, U, K, TR, beta=1.0)
    dA = np.zeros(off, dtype=dtype)
    PI.run_gemm(plan.gA1, U, TR, dA)
    PI.run_gemm(plan.gA2, TR, V, dA)
    ref = oracle.svd_backward(U, S, V, gU, gS, gV, meta, off, dtype)
    assert np.abs(dA - ref).max() <= 1e-10 * max(1.0, np.abs(ref).max())


def test_svd_plan_pairs_cover_all_pairs():
    """Circle-method ordering: N-1 rounds of disjoint pairs cover every pair once."""
    for k in (1, 2, 3, 7, 8, 13):
        N = k + (k % 2)
        seen = set()
        for rd in range(N - 1):
            used = set()
            for pi in range(N // 2):
                if pi == 0:
                    p, q = N - 1, rd
                else:
                    p, q = (rd + pi) % (N - 1), (rd - pi + (N - 1)) % (N - 1)
                assert p not in used and q not in used
                used |= {p, q}
                if p < k and q < k:
                    seen.add((min(p, q), max(p, q)))
        assert seen == {(i, j) for i in range(k) for j in range(i + 1, k)}


def test_mask_plan_diagonal_records():
    """Diagonal tensors give (sln, Dn:int, sla, Da:int, tm) records (yastn/tensor/_merging.py:577-579)."""
    meta = (((0, 2), 2, (3, 6), 3, (0,)), ((2, 3), 1, (0, 3), 3, (1,)))
    recs, items, total = P.mask_plan(meta, 0, {(0,): (0, 2), (1,): (2, 1)})
    assert total == 3 and recs[:, 2].tolist() == [1, 1] and recs[:, 5].tolist() == [1, 1]


@pytest.mark.parametrize('rows_per_super', [0, 4])
def test_mixed_precision_jacobi_schedule_on_plan_layout(rows_per_super):
    """FP32 sweeps (one pair per warp, or blocked on super-vectors) -> widen -> Newton-Schulz
    (grouped GEMM plans) -> X = W X_0 (plan) -> FP64 sweeps, on the plan's workspace offsets,
    reproduces LAPACK's singular values."""
    rng = np.random.default_rng(0)
    shapes = [(30, 30), (40, 17), (13, 35), (1, 5), (6, 6)]
    meta, off, oU, oS, oV = [], 0, 0, 0, 0
    for m, n in shapes:
        k = min(m, n)
        meta.append(((off, off + m * n), (m, n), (oU, oU + m * k), (m, k), (oS, oS + k), (oV, oV + k * n), (k, n)))
        off += m * n; oU += m * k; oS += k; oV += k * n
    meta = tuple(meta)
    data = rng.normal(size=off)
    data[meta[4][0][0]:meta[4][0][1]] = 0  # an all-zero block
    plan = P.svd_plan(meta, rows_per_super if rows_per_super else None)
    w32 = np.zeros(plan.n32, np.float32)
    w64 = np.zeros(plan.n64)
    for r in plan.blocks:
        a, m, n, k, L = int(r[0]), int(r[1]), int(r[2]), int(r[9]), int(r[10])
        A = data[a:a + m * n].reshape(m, n)
        X0 = A.T if m > n else A
        w32[int(r[13]):int(r[13]) + k * L] = X0.ravel().astype(np.float32)
        w32[int(r[14]):int(r[14]) + k * k] = np.eye(k, dtype=np.float32).ravel()
    if rows_per_super:
        assert plan.rows_per_super == rows_per_super
        assert plan.blocks[:, 15].tolist() == [8, 6, 4, 2, 2]  # ceil(k / 4) rounded up to even
        assert plan.super_rounds == 7 and len(plan.super_items) == 11
        nsw, conv = PI.block_jacobi_sweeps(w32, w32, plan.blocks, rows_per_super, 3, 1e-4, 40)
    else:
        nsw, conv = PI.jacobi_sweeps(w32, w32, plan.blocks, np.float32, 1e-4, 40)
    assert all(conv)
    for r in plan.blocks:
        k = int(r[9])
        w64[int(r[7]):int(r[7]) + k * k] = w32[int(r[14]):int(r[14]) + k * k]
    w0, t0, n0, ws = plan.w_range
    for _ in range(2):
        w64[n0:n0 + ws] = w64[w0:w0 + ws]
        PI.run_gemm(plan.gram, w64, w64, w64)
        PI.run_gemm(plan.ns, w64, w64, w64, alpha=-0.5, beta=1.5)
        w64[w0:w0 + ws] = w64[n0:n0 + ws]
    for r in plan.blocks:
        k = int(r[9])
        Wb = w64[int(r[7]):int(r[7]) + k * k].reshape(k, k)
        assert np.abs(Wb @ Wb.T - np.eye(k)).max() < 1e-14
    PI.run_gemm(plan.xform, w64, data, w64)
    nsw, conv = PI.jacobi_sweeps(w64, w64, plan.blocks, np.float64, 1e-8, 20)
    assert all(conv) and max(nsw) <= 4
    U, S, V = oracle.svd(data, meta, (oU, oS, oV))
    for r, mt in zip(plan.blocks, meta):
        k, L = int(r[9]), int(r[10])
        X = w64[int(r[6]):int(r[6]) + k * L].reshape(k, L)
        s = np.sort(np.linalg.norm(X, axis=1))[::-1]
        sr = S[mt[4][0]:mt[4][1]]
        assert np.abs(s - sr).max() <= 1e-13 * max(sr.max(), 1.0)


@pytest.mark.parametrize('cplx', [False, True])
def test_qr_preconditioned_jacobi_on_plan_layout(cplx):
    """The QR-preconditioned SVD on the plan layout: Householder QR of M = X_0^T (records
    [16..22]), FP32 phase on R's rows, Newton-Schulz, X = W R by the xform plan, FP64
    phase, the finalize rules and the closing GEMMs (Vh = conj(W) Q^T for wide blocks,
    U = conj(Q) W^T for tall ones) give LAPACK's singular values and A = U S Vh with
    orthonormal factors, on random and graded blocks."""
    rng = np.random.default_rng(9)
    shapes = [(24, 24), (31, 12), (9, 26), (1, 4), (5, 1), (40, 40)]
    meta, off, oU, oS, oV = [], 0, 0, 0, 0
    for m, n in shapes:
        k = min(m, n)
        meta.append(((off, off + m * n), (m, n), (oU, oU + m * k), (m, k), (oS, oS + k), (oV, oV + k * n), (k, n)))
        off += m * n; oU += m * k; oS += k; oV += k * n
    meta = tuple(meta)
    f = lambda *sh: rng.normal(size=sh) + (1j * rng.normal(size=sh) if cplx else 0)
    data = f(off)
    q1, _ = np.linalg.qr(f(40, 40))
    q2, _ = np.linalg.qr(f(40, 40))
    a5 = meta[5][0][0]
    data[a5:a5 + 1600] = ((q1 * np.logspace(0, -12, 40)) @ q2).ravel()   # graded over 12 decades
    plan = P.svd_plan(meta, None, cplx, qr=True)
    assert plan.qr and all(int(r[10]) == int(r[9]) for r in plan.blocks)
    ct, rt = (np.complex128, np.complex64) if cplx else (np.float64, np.float32)
    w32 = np.zeros(plan.n32, rt)
    w64 = np.zeros(plan.n64, ct)
    scale = []
    for r in plan.blocks:
        A = data[int(r[0]):int(r[0]) + int(r[1]) * int(r[2])]
        scale.append(2.0 ** -np.frexp(np.linalg.norm(A))[1])
    PI.qr_precondition(w64, w32, plan.blocks, data, scale)
    nsw, conv = PI.jacobi_sweeps(w32, w32, plan.blocks, rt, 1e-4, 40)
    assert all(conv)
    for r in plan.blocks:
        k = int(r[9])
        w64[int(r[7]):int(r[7]) + k * k] = w32[int(r[14]):int(r[14]) + k * k]
    w0, t0, n0, ws = plan.w_range
    for _ in range(2):
        w64[n0:n0 + ws] = w64[w0:w0 + ws]
        PI.run_gemm(plan.gram, w64, w64, w64)
        PI.run_gemm(plan.ns, w64, w64, w64, alpha=-0.5, beta=1.5)
        w64[w0:w0 + ws] = w64[n0:n0 + ws]
    PI.run_gemm(plan.xform, w64, w64, w64)
    nsw, conv = PI.jacobi_sweeps(w64, w64, plan.blocks, ct, 1e-8, 20)
    assert all(conv) and max(nsw) <= 4, nsw
    U, S, V = np.zeros(oU, ct), np.zeros(oS), np.zeros(oV, ct)
    PI.finalize_qr(w64, plan.blocks, U, S, V)
    PI.run_gemm(plan.qfin_v, w64, w64, V)
    PI.run_gemm(plan.qfin_u, w64, w64, U)
    _, Sr, _ = oracle.svd(data, meta, (oU, oS, oV))
    assert np.abs(S - Sr).max() <= 1e-13 * np.abs(Sr).max()
    for sl, D, slU, DU, slS, slV, DV in meta:
        u = U[slU[0]:slU[1]].reshape(DU)
        vh = V[slV[0]:slV[1]].reshape(DV)
        s = S[slS[0]:slS[1]]
        a = data[sl[0]:sl[1]].reshape(D)
        assert np.abs((u * s) @ vh - a).max() <= 1e-13 * max(np.abs(a).max(), 1e-300)
        k = DU[1]
        assert np.abs(u.conj().T @ u - np.eye(k)).max() <= 1e-13
        assert np.abs(vh @ vh.conj().T - np.eye(k)).max() <= 1e-13


def test_qr_adjoint_plan_reproduces_oracle():
    """The QR adjoint's grouped-GEMM plans, the copyltu/back-substitution records and the copy
    into dA (numpy statement of the two elementwise kernels) give the oracle's adjoint on
    tall, square and wide blocks."""
    rng = np.random.default_rng(6)
    shapes = [(9, 4), (5, 5), (3, 8), (1, 6), (12, 1)]
    meta, off, oQ, oR = [], 0, 0, 0
    for m, n in shapes:
        k = min(m, n)
        meta.append(((off, off + m * n), (m, n), (oQ, oQ + m * k), (m, k), (oR, oR + k * n), (k, n)))
        off += m * n; oQ += m * k; oR += k * n
    meta = tuple(meta)
    data = rng.normal(size=off)
    Q, R = oracle.qr(data, meta, (oQ, oR))
    gQ, gR = rng.normal(size=oQ), rng.normal(size=oR)
    plan = P.qr_plan(meta)
    Bw = gQ.copy()
    M = np.zeros(plan.m_size)
    PI.run_gemm(plan.w1, data, gR, Bw, beta=1.0)
    PI.run_gemm(plan.m1, R, gR, M)
    PI.run_gemm(plan.m2, Bw, Q, M, alpha=-1.0, beta=1.0)
    for mo, k, b0, rows, ldb, r0, ldr, _ in plan.adj:
        Mb = M[mo:mo + k * k].reshape(k, k)
        Mb[:] = np.tril(Mb) + np.tril(Mb, -1).T
    PI.run_gemm(plan.s1, Q, M, Bw, beta=1.0)
    for mo, k, b0, rows, ldb, r0, ldr, _ in plan.adj:
        Bb = Bw[b0:b0 + rows * ldb].reshape(rows, ldb)[:, :k]
        U = np.stack([R[r0 + i * ldr: r0 + i * ldr + k] for i in range(k)])
        Bb[:] = np.linalg.solve(np.triu(U), Bb.T).T
    dA = np.zeros(off)
    for so, do, sizes, ss, ds in plan.copies:
        for i in range(sizes[0]):
            dA[do + i * ds[0]: do + i * ds[0] + sizes[1]] = Bw[so + i * ss[0]: so + i * ss[0] + sizes[1]]
    PI.run_gemm(plan.y1, Q, gR, dA)
    ref = oracle.qr_backward(Q, R, gQ, gR, data, meta)
    assert np.abs(dA - ref).max() <= 1e-12 * np.abs(ref).max()


@pytest.mark.parametrize('qr_start', [False, True])
def test_completion_plans_orthonormal_completion(qr_start):
    """The blocked completion's records (candidate fill, the two projection GEMMs, the QR of
    the candidates, the copy into the factor) applied with numpy: the factor's last nz
    vectors of each block become orthonormal and orthogonal to the earlier ones, which stay
    untouched."""
    rng = np.random.default_rng(10)
    shapes = [(30, 12), (9, 26), (20, 20), (7, 3)]
    meta, oU, oS, oV, off = [], 0, 0, 0, 0
    for m, n in shapes:
        k = min(m, n)
        meta.append(((off, off + m * n), (m, n), (oU, oU + m * k), (m, k), (oS, oS + k), (oV, oV + k * n), (k, n)))
        off += m * n; oU += m * k; oS += k; oV += k * n
    meta = tuple(meta)
    plan = P.svd_plan(meta, None, False, qr=qr_start)
    nz = [5, 4, 20, 1]  # the third block: every vector completed
    U, V = np.zeros(oU), np.zeros(oV)
    for r, z in zip(plan.blocks, nz):  # orthonormal leading vectors, zeros at the completed ones
        m, n, k, tall, from_r = int(r[1]), int(r[2]), int(r[9]), bool(r[12]), bool(r[16])
        to_u = tall != from_r
        Lv = m if to_u else n
        q, _ = np.linalg.qr(rng.normal(size=(Lv, k)))
        q[:, k - z:] = 0
        if to_u:
            U[int(r[3]):int(r[3]) + m * k] = q.ravel()
        else:
            V[int(r[5]):int(r[5]) + k * n] = q.T.ravel()
    U0, V0 = U.copy(), V.copy()
    for cp in P.completion_plans(plan.blocks, nz):
        F = U if cp.to_u else V
        G = np.zeros(cp.G)
        for g0, cnt in cp.fill:
            G[g0:g0 + cnt] = rng.uniform(-1, 1, size=cnt)
        C = np.zeros(max(cp.C, 1))
        for _ in range(2):
            PI.run_gemm(cp.g1, F, G, C)
            PI.run_gemm(cp.g2, F, C, G, alpha=-1.0, beta=1.0)
        Qc = np.zeros(cp.Q)
        for sl, D, slQ, DQ, slR, DR in cp.meta:
            q, _ = np.linalg.qr(G[sl[0]:sl[1]].reshape(D))
            Qc[slQ[0]:slQ[1]] = q.ravel()
        for so, do, sizes, ss, ds in cp.copy.tasks_list:
            for i in range(sizes[0]):
                for j in range(sizes[1]):
                    F[do + i * ds[0] + j * ds[1]] = Qc[so + i * ss[0] + j * ss[1]]
    for r, z, (sl, D, slU, DU, slS, slV, DV) in zip(plan.blocks, nz, meta):
        u, vh = U[slU[0]:slU[1]].reshape(DU), V[slV[0]:slV[1]].reshape(DV)
        u0, vh0 = U0[slU[0]:slU[1]].reshape(DU), V0[slV[0]:slV[1]].reshape(DV)
        k = DU[1]
        to_u = bool(r[12]) != bool(r[16])
        f, f0 = (u, u0) if to_u else (vh.T, vh0.T)
        assert np.abs(f.T @ f - np.eye(k)).max() < 1e-13
        np.testing.assert_array_equal(f[:, :k - z], f0[:, :k - z])


@pytest.mark.parametrize('cplx', [False, True])
def test_qr_plan_layout_reproduces_oracle(cplx):
    """yb_qr's records ([16] = 2) and the grouped GEMM of R's right part, applied with numpy
    (the kernel's Householder steps and sign fix), give the oracle's Q and R."""
    rng = np.random.default_rng(12)
    shapes = [(9, 4), (5, 5), (3, 8), (1, 6), (12, 1)]
    meta, off, oQ, oR = [], 0, 0, 0
    for m, n in shapes:
        k = min(m, n)
        meta.append(((off, off + m * n), (m, n), (oQ, oQ + m * k), (m, k), (oR, oR + k * n), (k, n)))
        off += m * n; oQ += m * k; oR += k * n
    meta = tuple(meta)
    data = rng.normal(size=off) + (1j * rng.normal(size=off) if cplx else 0)
    plan = P.qr_plan(meta, cplx)
    assert all(int(r[16]) == 2 for r in plan.blocks)
    dt = np.complex128 if cplx else np.float64
    Q, R = np.zeros(oQ, dt), np.zeros(oR, dt)
    PI.qr_plain(np.zeros(plan.n64, dt), plan.blocks, data, Q, R)
    PI.run_gemm(plan.right, Q, data, R)
    Qr, Rr = oracle.qr(data, meta, (oQ, oR))
    assert np.abs(Q - Qr).max() < 1e-12 and np.abs(R - Rr).max() < 1e-12


def test_mixed_precision_jacobi_schedule_complex():
    """Complex blocks: FP32 phase on complex64 rows with phase-aligned rotations, widen,
    Newton-Schulz with T = W^H W, X = W X_0 (X_0 = A^H for tall blocks), FP64 phase; the
    finalize rules (wide: U = W^H, Vh rows = x_i / s_i; tall: U columns = conj(x_i) / s_i,
    Vh = W) reproduce LAPACK's singular values and A."""
    rng = np.random.default_rng(3)
    shapes = [(20, 20), (31, 12), (9, 26), (1, 4)]
    meta, off, oU, oS, oV = [], 0, 0, 0, 0
    for m, n in shapes:
        k = min(m, n)
        meta.append(((off, off + m * n), (m, n), (oU, oU + m * k), (m, k), (oS, oS + k), (oV, oV + k * n), (k, n)))
        off += m * n; oU += m * k; oS += k; oV += k * n
    meta = tuple(meta)
    data = rng.normal(size=off) + 1j * rng.normal(size=off)
    plan = P.svd_plan(meta, None, True)
    w32 = np.zeros(plan.n32, np.complex64)
    w64 = np.zeros(plan.n64, np.complex128)
    for r in plan.blocks:
        a, m, n, k, L = int(r[0]), int(r[1]), int(r[2]), int(r[9]), int(r[10])
        A = data[a:a + m * n].reshape(m, n)
        X0 = A.conj().T if m > n else A
        w32[int(r[13]):int(r[13]) + k * L] = X0.ravel().astype(np.complex64)
        w32[int(r[14]):int(r[14]) + k * k] = np.eye(k, dtype=np.complex64).ravel()
    nsw, conv = PI.jacobi_sweeps(w32, w32, plan.blocks, np.complex64, 1e-4, 40)
    assert all(conv)
    for r in plan.blocks:
        k = int(r[9])
        w64[int(r[7]):int(r[7]) + k * k] = w32[int(r[14]):int(r[14]) + k * k]
    w0, t0, n0, ws = plan.w_range
    for _ in range(2):
        w64[n0:n0 + ws] = w64[w0:w0 + ws]
        PI.run_gemm(plan.gram, w64, w64, w64)
        PI.run_gemm(plan.ns, w64, w64, w64, alpha=-0.5, beta=1.5)
        w64[w0:w0 + ws] = w64[n0:n0 + ws]
    PI.run_gemm(plan.xform, w64, data, w64)
    nsw, conv = PI.jacobi_sweeps(w64, w64, plan.blocks, np.complex128, 1e-8, 20)
    assert all(conv)
    _, Sr, _ = oracle.svd(data, meta, (oU, oS, oV))
    for r, mt in zip(plan.blocks, meta):
        a, m, n, k, L = int(r[0]), int(r[1]), int(r[2]), int(r[9]), int(r[10])
        X = w64[int(r[6]):int(r[6]) + k * L].reshape(k, L)
        Wb = w64[int(r[7]):int(r[7]) + k * k].reshape(k, k)
        s = np.linalg.norm(X, axis=1)
        if m > n:
            U, Vh = (X.conj() / s[:, None]).T, Wb
        else:
            U, Vh = Wb.conj().T, X / s[:, None]
        A = data[a:a + m * n].reshape(m, n)
        assert np.abs((U * s) @ Vh - A).max() <= 1e-13 * np.abs(A).max()
        assert np.abs(np.sort(s)[::-1] - Sr[mt[4][0]:mt[4][1]]).max() <= 1e-13 * max(s.max(), 1.0)


def _split_rows_view(src, rec):
    """The real rows yb_ozaki_split reads for one record: element k of row i at source
    offset rec[0] + i*rec[3] + k*rec[8] (FP64 or complex elements by mode)."""
    s0, rows, K, rs, mode = (int(x) for x in rec[:5])
    ks = int(rec[8])
    if mode == 0:
        return np.stack([src[s0 + r * rs + ks * np.arange(K)] for r in range(rows)])
    half = K // 2
    out = []
    for r in range(rows):
        z = src[s0 + r * rs + ks * np.arange(half)]
        out.append({1: np.concatenate([z.real, z.imag]), 2: np.concatenate([z.real, -z.imag]),
                    3: np.concatenate([z.imag, z.real])}[mode])
    return np.stack(out)


def _recs_of(plan, op, tc=False):
    recs = plan.split_recs_tc if tc else plan.split_recs
    return recs[(recs[:, 9] & 1) == op]


def test_ozaki_complex_plan_reproduces_complex_products():
    """Complex sectors as two real products with doubled K: A rows [re | im], B^T rows
    [re | -im] and [im | re], outputs interleaved with column stride 2."""
    rng = np.random.default_rng(17)
    shapes = [(40, 30, 20), (16, 16, 17), (5, 40, 9), (3, 8, 100)]
    meta, oa, ob, oc = [], 0, 0, 0
    for m, k, n in shapes:
        meta.append(((oc, oc + m * n), (m, n), (oa, oa + m * k), (m, k), (ob, ob + k * n), (k, n)))
        oa += m * k; ob += k * n; oc += m * n
    meta = tuple(meta)
    A = rng.normal(size=oa) + 1j * rng.normal(size=oa)
    B = rng.normal(size=ob) + 1j * rng.normal(size=ob)
    plan = P.ozaki_dot_plan(meta, 8, True)
    assert len(plan.outs) == 2 * 3 and len(plan.native.outs) == 1       # (3, 8, 100) is short: native
    assert sorted(set(int(r[4]) for r in _recs_of(plan, 0))) == [1]
    assert sorted(int(r[4]) for r in _recs_of(plan, 1)) == [2, 2, 2, 3, 3, 3]
    a_rows = {int(r[5]): _split_rows_view(A, r) for r in _recs_of(plan, 0)}
    b_rows = {int(r[5]): _split_rows_view(B, r) for r in _recs_of(plan, 1)}  # B's columns, in place
    Cd = np.zeros(2 * oc)
    for o in plan.outs:
        c_off, m, n, ldc, ao, _, bo, _, Kr, Kp, cs = (int(x) for x in o[:11])
        part = a_rows[ao] @ b_rows[bo].T
        for i in range(m):
            Cd[c_off + i * ldc + cs * np.arange(n)] = part[i]
    C = Cd[0::2] + 1j * Cd[1::2]
    for (slc, Dc, sla, Da, slb, Db), o in zip(meta[:3], range(3)):
        ref = A[sla[0]:sla[1]].reshape(Da) @ B[slb[0]:slb[1]].reshape(Db)
        np.testing.assert_allclose(C[slc[0]:slc[1]].reshape(Dc), ref, rtol=1e-12, atol=1e-12)


def test_eigh_adjoint_plan_reproduces_reference_autograd():
    """X = op(U)^T gU, the inner matrix, T = U K, dA = T op(U)^T on the packed records
    reproduce the reference's eigh gradients (SYMEIG and torch.linalg.eigh, real and complex)."""
    import json, os
    from yastn_gb300.workloads import GOLDEN, _decode
    with open(os.path.join(GOLDEN, 'eigh_adjoint.json')) as f:
        calls = json.load(f)['calls']
    z = np.load(os.path.join(GOLDEN, 'eigh_adjoint.npz'))
    for c in calls:
        meta = _decode(c['meta'], None)
        U, S, gU, gS, ref = (z[c[k]] for k in ('U', 'S', 'gU', 'gS', 'grad'))
        plan = P.eigh_adjoint_plan(meta, c['order_by_magnitude'], np.iscomplexobj(U))
        X = PI.run_gemm(plan.gX, U, gU, np.zeros(plan.kk, dtype=U.dtype))
        K = PI.eigh_adjoint_core(X, S, gS, plan.recs, c['order_by_magnitude'])
        T = PI.run_gemm(plan.gT, U, K, np.zeros(plan.kk, dtype=U.dtype))
        dA = PI.run_gemm(plan.gA, T, U, np.zeros(ref.size, dtype=ref.dtype))
        assert np.abs(dA - ref).max() <= 1e-10 * np.abs(ref).max(), c['order_by_magnitude']


def _ozaki_digits(x, s):
    """NumPy restatement of the split of csrc/yb_ozaki.cu (rows of x): balanced base-128
    digits of Q = rint(x 2^{7s-e}) extracted from the low end with integer arithmetic."""
    mx = np.abs(x).max(axis=1)
    e = np.where(mx > 0, np.frexp(mx)[1], 0)
    q = np.rint(np.ldexp(x, 7 * s - e[:, None])).astype(np.int64)
    digits = [None] * s
    for t in range(s - 1, 0, -1):
        r = ((q + 64) & 127) - 64
        digits[t] = r.astype(np.float64)
        q = (q - r) >> 7
    digits[0] = q.astype(np.float64)
    return e, digits


def _ozaki_digits_bits(x, s):
    """The integer-only split of csrc/yb_ozaki.cu restated with numpy int64: row exponent
    from the bit patterns, Q = rint(x 2^{7s-e}) by a round-half-even shift of the
    mantissa, digits from U = Q + 64 (1 + 128 + ... + 128^{s-2})."""
    bits = np.ascontiguousarray(x).view(np.int64)
    mag = bits & np.int64(0x7fffffffffffffff)
    mx = mag.max(axis=1)
    e = np.zeros(len(x), dtype=np.int64)
    normal = mx >= (1 << 52)
    e[normal] = (mx[normal] >> 52) - 1022
    sub = (~normal) & (mx > 0)
    e[sub] = np.frexp(mx[sub].view(np.float64))[1]
    E = mag >> 52
    M = mag & np.int64((1 << 52) - 1)
    ex = np.where(E != 0, E - 1075, -1074)
    M = np.where(E != 0, M | np.int64(1 << 52), M)
    up = ex + 7 * s - e[:, None]
    q = np.zeros_like(M)
    left = up >= 0
    q[left] = M[left] << up[left]
    sh = np.minimum(-up, 63)
    r = ~left
    qr = M[r] >> sh[r]
    rem = M[r] & ((np.int64(1) << sh[r]) - 1)
    half = np.int64(1) << (sh[r] - 1)
    qr = qr + ((rem > half) | ((rem == half) & ((qr & 1) == 1)))
    q[r] = qr
    q = np.where(mag == 0, 0, q)
    q = np.where(bits < 0, -q, q)
    bias = 0
    for _ in range(s - 1):
        bias = (bias << 7) | 64
    u = q + np.int64(bias)
    digits = [((u >> (7 * (s - 1 - t))) & 127) - 64 for t in range(1, s)]
    return e, [(u >> (7 * (s - 1))).astype(np.float64)] + [d.astype(np.float64) for d in digits]


@pytest.mark.parametrize('s', [6, 7, 8])
def test_ozaki_integer_split_matches_rint_split(s):
    """The bit-level split (no FP64 arithmetic) gives exactly the digits of rint(x 2^{7s-e}):
    normal, subnormal, zero and negative entries, and exact rounding ties."""
    rng = np.random.default_rng(12)
    x = rng.normal(size=(6, 40)) * 10.0 ** rng.uniform(-30, 30, size=(6, 1))
    x[1, :5] = 0.0
    x[2] = rng.normal(size=40) * 1e-310           # a subnormal row
    x[3, 7] = -x[3, 7]
    e = np.frexp(np.abs(x[4]).max())[1]
    x[4, 10] = (2 ** 40 + 0.5) * 2.0 ** (e - 7 * s)   # ties at the last digit
    x[4, 11] = (2 ** 40 + 1.5) * 2.0 ** (e - 7 * s)
    x[4, 12] = -(2 ** 40 + 0.5) * 2.0 ** (e - 7 * s)
    x[5] = 0.0                                     # an all-zero row
    e_ref, d_ref = _ozaki_digits(x, s)
    e_bit, d_bit = _ozaki_digits_bits(x, s)
    np.testing.assert_array_equal(e_ref, e_bit)
    for a, b in zip(d_ref, d_bit):
        np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize('s', [6, 7, 8])
def test_ozaki_split_and_slice_products(s):
    """Digits are BF16-exact integers; the kept slice pairs reproduce A @ B to the bound."""
    rng = np.random.default_rng(6)
    A = rng.normal(size=(37, 150)) * 10.0 ** rng.uniform(-4, 0, size=(37, 1))
    B = rng.normal(size=(150, 29))
    ea, da = _ozaki_digits(A, s)
    eb, db = _ozaki_digits(B.T, s)
    for d in da + db:
        assert np.all(np.abs(d) <= 128) and np.all(d == np.rint(d))
        # exact in bfloat16: at most 8 significant bits
        m, _ = np.frexp(np.abs(d[d != 0]))
        assert np.all((m * 256) == np.rint(m * 256))
    rec = sum(d * 2.0 ** (-7 * (t + 1)) for t, d in enumerate(da)) * 2.0 ** ea[:, None]
    # remainder after s digits: |v_s| <= 1/2 at weight 2^{-7s}, row scale 2^{e_i}
    assert np.all(np.abs(rec - A).max(axis=1) <= 0.5 * 2.0 ** (-7 * s) * 2.0 ** ea)
    C = np.zeros((37, 29))
    for ta in range(s):
        for tb in range(s - ta):
            P = da[ta] @ db[tb].T  # exact integers (< 2^53)
            C += P * 2.0 ** (-7 * (ta + tb))
    C *= 2.0 ** (ea[:, None] + eb[None, :] - 14)
    ref = A @ B
    # truncation of the dropped digits + FP64 rounding of both summations (K = 150)
    bound = ((s + 2) * 2.0 ** (-7 * s) + 2 * 150 * 2.0 ** -53) * (np.abs(A) @ np.abs(B)).max()
    assert np.abs(C - ref).max() <= bound


def test_ozaki_plan_records():
    rng = np.random.default_rng(8)
    shapes = [(40, 70, 30), (16, 16, 16), (3, 200, 5), (64, 20, 33), (5, 8, 100), (4, 40, 300)]
    meta, oa, ob, oc = [], 0, 0, 0
    for m, k, n in shapes:
        meta.append(((oc, oc + m * n), (m, n), (oa, oa + m * k), (m, k), (ob, ob + k * n), (k, n)))
        oa += m * k; ob += k * n; oc += m * n
    meta = tuple(meta)
    A, B = rng.normal(size=oa), rng.normal(size=ob)
    plan = P.ozaki_dot_plan(meta, 8)
    # short contractions (K < 16) and skinny outputs (m <= 8 < 64 < n) go to the native
    # kernel, the rest (small m or n included) are split
    assert len(plan.outs) == 4 and len(plan.native.outs) == 2
    a_recs, b_recs = _recs_of(plan, 0), _recs_of(plan, 1)
    assert len({tuple(r[:1]) for r in a_recs}) == len(a_recs)  # each A block split once
    assert all(r[7] % 16 == 0 and r[7] >= r[2] for r in plan.split_recs)
    assert all(int(r[5]) % 16 == 0 for r in plan.split_recs)
    big = [mt for mt in meta if mt[3][1] >= 16 and not (mt[3][0] <= 8 and mt[5][1] > 64)]
    for rec, (slc, Dc, sla, Da, slb, Db) in zip(a_recs, big):
        np.testing.assert_array_equal(_split_rows_view(A, rec), A[sla[0]:sla[1]].reshape(Da))
    # B blocks are split by columns read in place: the rows of B^T
    for rec, (slc, Dc, sla, Da, slb, Db) in zip(b_recs, big):
        np.testing.assert_array_equal(_split_rows_view(B, rec), B[slb[0]:slb[1]].reshape(Db).T)
    # 8-row groups cover every record's rows once
    cover = sorted((int(g[0]), int(g[1]) + i) for g in plan.split_groups for i in range(P.OZ_SPLIT_ROWS)
                   if int(g[1]) + i < int(plan.split_recs[int(g[0])][1]))
    assert cover == [(ri, i) for ri, r in enumerate(plan.split_recs) for i in range(int(r[1]))]
    # the native part reproduces its sector
    out = PI.run_gemm(plan.native, A, B, np.zeros(oc))
    for slc, Dc, sla, Da, slb, Db in meta[4:]:
        np.testing.assert_allclose(out[slc[0]:slc[1]].reshape(Dc),
                                   A[sla[0]:sla[1]].reshape(Da) @ B[slb[0]:slb[1]].reshape(Db), rtol=1e-13)


@pytest.mark.parametrize('tn', [64, 32])
def test_ozaki_tiled_records_and_tiles(tn):
    """Records of the tcgen05 kernel: every operand block gets s * ceil(rows / tile) * tile * Kp
    digits in the tile layout (128 rows for A, the tile width 64 or 32 for B's columns),
    without overlap and in block order; the 8-row groups cover the padded rows; the output
    records point at the remapped blocks; tiles cover every output once by decreasing K."""
    sfx = '_tc' if tn == 64 else '_tc32'
    at = lambda plan, name: getattr(plan, name + sfx)
    rng = np.random.default_rng(23)
    shapes = [(40, 30, 20), (16, 16, 17), (130, 20, 70), (5, 40, 9), (3, 8, 100), (6, 300, 200)]
    meta, oa, ob, oc = [], 0, 0, 0
    for m, k, n in shapes:
        meta.append(((oc, oc + m * n), (m, n), (oa, oa + m * k), (m, k), (ob, ob + k * n), (k, n)))
        oa += m * k; ob += k * n; oc += m * n
    meta = tuple(meta)
    for cplx in (False, True):
        plan = P.ozaki_dot_plan(meta, 8, cplx)
        recs_t = at(plan, 'split_recs')
        for op, th, size in ((0, 128, at(plan, 'a_size')), (1, tn, at(plan, 'b_size'))):
            end = 0
            for r in recs_t:
                if int(r[9]) & 1 != op:
                    continue
                assert int(r[5]) == end and int(r[9]) == op | (th << 8)
                end += 8 * (-(-int(r[1]) // th) * th) * int(r[7])
            assert end == size
        groups = [(int(g[0]), int(g[1])) for g in at(plan, 'split_groups')]
        want = {(ri, g) for ri, r in enumerate(recs_t)
                for g in range(0, -(-int(r[1]) // (int(r[9]) >> 8)) * (int(r[9]) >> 8), P.OZ_SPLIT_ROWS)}
        assert set(groups) == want and len(groups) == len(want)
        ga, gb = getattr(plan, 'split_groups' + sfx + '_ab')
        assert sorted(map(tuple, np.concatenate([ga, gb]).tolist())) == sorted(groups)
        assert all(int(recs_t[g[0]][9]) & 1 == 0 for g in ga) and all(int(recs_t[g[0]][9]) & 1 == 1 for g in gb)
        # the same blocks in both layouts
        assert np.array_equal(np.delete(plan.split_recs, [5, 9], axis=1), np.delete(recs_t, [5, 9], axis=1))
        new = {(int(r[9]) & 1, int(r[5])): int(t[5]) for r, t in zip(plan.split_recs, recs_t)}
        for o, t in zip(plan.outs, at(plan, 'outs')):
            assert int(t[4]) == new[(0, int(o[4]))] and int(t[6]) == new[(1, int(o[6]))]
            assert np.array_equal(np.delete(o, [4, 6]), np.delete(t, [4, 6]))
        want = {(oi, tr, tc) for oi, o in enumerate(at(plan, 'outs'))
                for tr in range(-(-int(o[1]) // 128)) for tc in range(-(-int(o[2]) // tn))}
        got = [tuple(int(x) for x in t[:3]) for t in at(plan, 'tiles')]
        assert len(got) == len(want) and set(got) == want
        ks = [int(at(plan, 'outs')[t[0]][8]) for t in at(plan, 'tiles')]
        assert ks == sorted(ks, reverse=True)


def test_ozaki_split_model_reconstructs_the_operands():
    """The digit model of yb_ozaki_split (both layouts, real and complex records): every
    record's digits and exponents rebuild its rows to within half a unit of the last digit,
    the records tile the digit arrays without overlap, and the leading digit stays within
    [-128, 128], the others within [-64, 63]."""
    rng = np.random.default_rng(29)
    shapes = [(40, 30, 20), (16, 16, 17), (130, 20, 70), (6, 300, 200), (33, 17, 65)]
    meta, oa, ob, oc = [], 0, 0, 0
    for m, k, n in shapes:
        meta.append(((oc, oc + m * n), (m, n), (oa, oa + m * k), (m, k), (ob, ob + k * n), (k, n)))
        oa += m * k; ob += k * n; oc += m * n
    meta = tuple(meta)
    for cplx in (False, True):
        A = rng.normal(size=oa) * np.exp(rng.normal(size=oa) * 3)
        B = rng.normal(size=ob) * np.exp(rng.normal(size=ob) * 3)
        if cplx:
            A = A + 1j * rng.normal(size=oa)
            B = B + 1j * rng.normal(size=ob)
        for s in (6, 8):
            plan = P.ozaki_dot_plan(meta, s, cplx)
            for recs, groups, sizes in ((plan.split_recs, plan.split_groups, (plan.a_size, plan.b_size)),
                                        (plan.split_recs_tc, plan.split_groups_tc, (plan.a_size_tc, plan.b_size_tc)),
                                        (plan.split_recs_tc32, plan.split_groups_tc32,
                                         (plan.a_size_tc32, plan.b_size_tc32))):
                dig, exps = PI.ozaki_split(recs, groups, A, B, s, sizes, (plan.a_exps, plan.b_exps))
                for op in (0, 1):
                    d = dig[op]
                    assert d.min() >= -128 and d.max() <= 128
                for rec in recs:
                    op, th = int(rec[9]) & 1, int(rec[9]) >> 8
                    rows, K, Kp, dst, eo = int(rec[1]), int(rec[2]), int(rec[7]), int(rec[5]), int(rec[6])
                    rows_p = -(-rows // th) * th if th else rows
                    x = PI.split_rows(B if op else A, rec)
                    e = exps[op][eo:eo + rows]
                    r = np.arange(rows)[:, None]
                    k = np.arange(K)[None, :]
                    if th == 0:
                        off = r * Kp + k
                    else:
                        off = (r // th) * (Kp // 16) * th * 16 + (k // 16) * th * 16 + ((r % th) // 8) * 128 + \
                            ((k % 16) // 8) * 64 + (r % 8) * 8 + k % 8
                    val = sum(dig[op][dst + t * rows_p * Kp + off].astype(float) * 2.0 ** (-7 * (t + 1))
                              for t in range(s))
                    rebuilt = np.ldexp(val, e[:, None])
                    assert np.all(np.abs(rebuilt - x) <= np.ldexp(0.5 + 1e-9, (e - 7 * s)[:, None]))
                    lead = dig[op][dst + off]
                    assert np.all(np.abs(lead) <= 128)


def test_ozaki_tc_schedule_covers_tiles_once_and_balances():
    """The tcgen05 kernel's per-CTA schedule: every tile exactly once, CTA ranges contiguous,
    no CTA above the SM count, and the largest CTA load within one tile of the balanced mean
    (longest-processing-time assignment) on the DMRG workload's two emulated dots."""
    from yastn_gb300.workloads import Heff2Workload
    dots = [c['args'][2] for c in Heff2Workload().calls if c['fn'] == 'dot']
    for meta, tn in ((dots[0], 64), (dots[3], 64), (dots[0], 32), (dots[3], 32)):
        plan = P.ozaki_dot_plan(meta, 8)
        tiles_t = plan.tiles_tc if tn == 64 else plan.tiles_tc32
        outs_t = plan.outs_tc if tn == 64 else plan.outs_tc32
        for sms in (152, 37):
            tiles, offs = P.ozaki_tc_schedule(plan, sms, tn)
            assert offs[0] == 0 and offs[-1] == len(tiles_t) and len(offs) == min(sms, len(tiles_t)) + 1
            assert np.all(np.diff(offs) >= 0)
            key = lambda a: sorted(map(tuple, a.tolist()))
            assert key(tiles) == key(tiles_t)
            steps = lambda t: int(outs_t[t[0]][9]) // 16 + P.OZ_TC_FOLD_STEPS
            loads = [sum(steps(t) for t in tiles[offs[b]:offs[b + 1]]) for b in range(len(offs) - 1)]
            biggest = max(steps(t) for t in tiles)
            assert max(loads) <= sum(loads) / len(loads) + biggest


def test_fix_signs_plan_takes_truncated_and_partial_svd_records():
    """The gauge fix's records accept U (m x k), Vh (k x n) of any k (truncated or partial
    SVDs, where YASTN may pass no S slice) and keep the fields its kernels read."""
    meta = (((0, 12), (3, 4), (0, 6), (3, 2), (0, 2), (0, 8), (2, 4)),
            ((12, 32), (4, 5), (6, 18), (4, 3), None, (8, 23), (3, 5)),
            ((32, 32), (0, 3), (18, 18), (0, 0), (2, 2), (23, 23), (0, 3)))
    plan = P.fix_signs_plan(meta)
    assert plan.max_k == 3 and len(plan.blocks) == 2
    r0, r1 = plan.blocks
    assert [int(r0[i]) for i in (1, 2, 3, 4, 5, 9)] == [3, 4, 0, 0, 0, 2]
    assert [int(r1[i]) for i in (1, 2, 3, 4, 5, 9)] == [4, 5, 6, 2, 8, 3]
    with pytest.raises(P.PlanError):
        P.fix_signs_plan((((0, 12), (3, 4), (0, 6), (3, 2), (0, 3), (0, 8), (2, 4)),))


def test_plan_cache_save_and_load(tmp_path):
    """Plans written by save_cache and read back by load_cache (without their device state)
    are found by value: rebuilding them from the same metadata is a cache hit, no build, and
    every packed array is equal to the original's."""
    from yastn_gb300.workloads import Heff2Workload
    w = Heff2Workload()
    P.CACHE.by_id.clear(); P.CACHE.by_val.clear()
    built = []
    for fn, keys, args, okey in w.steps:
        if fn == 'dot':
            built.append(('dot', args[2], P.dot_plan(args[2])))
            built.append(('ozaki', args[2], P.ozaki_dot_plan(args[2], 8)))
        else:
            plan = P.merge_plan(*args[1:])
            plan.packed(True)
            plan._dev['x'] = (object(),)  # stands in for device copies, which are not written
            built.append(('merge', args[1:], plan))
    P.ozaki_tc_schedule(built[1][2], 152)
    path = tmp_path / 'plans.pkl'
    n = P.save_cache(str(path))
    assert n == len(P.CACHE.by_val) >= len(built) - 3
    P.CACHE.by_id.clear(); P.CACHE.by_val.clear()
    assert P.load_cache(str(path)) == n
    misses = P.CACHE.misses
    for kind, key, old in built:
        new = {'dot': lambda: P.dot_plan(key), 'ozaki': lambda: P.ozaki_dot_plan(key, 8),
               'merge': lambda: P.merge_plan(*key)}[kind]()
        assert new is not old and new._dev == {}
        if kind == 'merge':
            for v in (True, False):
                for a, b in zip(new.packed(v), old.packed(v)):
                    assert np.array_equal(a, b)
        elif kind == 'dot':
            assert np.array_equal(new.tiles, old.tiles) and np.array_equal(new.outs, old.outs)
        else:
            assert np.array_equal(new.split_recs_tc, old.split_recs_tc) and new.prefer_tc == old.prefer_tc
            assert np.array_equal(new.native.tiles, old.native.tiles)
            assert not hasattr(new, 'tuned_tc')
    assert P.CACHE.misses == misses  # every plan came from the file
    bad = tmp_path / 'bad.pkl'
    import pickle
    bad.write_bytes(pickle.dumps({'version': 0, 'entries': []}))
    with pytest.raises(P.PlanError):
        P.load_cache(str(bad))
    P.CACHE.by_id.clear(); P.CACHE.by_val.clear()


@pytest.mark.parametrize('seed', [0, 1, 2])
def test_random_sector_shapes_every_tile_kind(seed):
    """Seeded random sector shapes spanning every tile kind (64 x 64, skinny, short skinny,
    tall skinny) and the split-K path: tile coverage and values of the packed records,
    forward and both adjoints, real and complex, against the oracle."""
    rng = np.random.default_rng(100 + seed)
    shapes = []
    for _ in range(14):
        kind = rng.integers(0, 5)
        if kind == 0:
            shapes.append((int(rng.integers(1, 200)), int(rng.integers(1, 200)), int(rng.integers(1, 200))))
        elif kind == 1:  # few rows, wide
            shapes.append((int(rng.integers(1, 17)), int(rng.integers(1, 60)), int(rng.integers(65, 5000))))
        elif kind == 2:  # few rows, short K
            shapes.append((int(rng.integers(1, 9)), int(rng.integers(1, 9)), int(rng.integers(1, 3000))))
        elif kind == 3:  # few columns, tall
            shapes.append((int(rng.integers(65, 3000)), int(rng.integers(1, 80)), int(rng.integers(1, 17))))
        else:  # long K
            shapes.append((int(rng.integers(1, 40)), int(rng.integers(500, 4000)), int(rng.integers(1, 40))))
    meta, oa, ob, oc = _meta_dot(shapes)
    plan = P.dot_plan(meta)
    for cplx in (False, True):
        f = lambda n: rng.normal(size=n) + (1j * rng.normal(size=n) if cplx else 0)
        A, B, Cb = f(oa), f(ob), f(oc)
        out = PI.run_gemm(plan, A, B, np.zeros(oc, dtype=A.dtype))
        ref = oracle.dot(A, B, meta, oc)
        assert np.abs(out - ref).max() <= 1e-12 * max(np.abs(ref).max(), 1.0)
        pa, pb = P.dot_backward_plans(meta)
        Ab = PI.run_gemm(pa, Cb, B, np.zeros(oa, dtype=A.dtype))
        Bb = PI.run_gemm(pb, A, Cb, np.zeros(ob, dtype=A.dtype))
        Ab_r, Bb_r = oracle.dot_backward(Cb, A, B, meta)
        assert np.abs(Ab - Ab_r).max() <= 1e-12 * max(np.abs(Ab_r).max(), 1.0)
        assert np.abs(Bb - Bb_r).max() <= 1e-12 * max(np.abs(Bb_r).max(), 1.0)
    P.CACHE.by_id.clear(); P.CACHE.by_val.clear()
