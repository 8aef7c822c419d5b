"""NumPy interpreter of the packed C-ABI records (test helper).

Executes copy / grouped-GEMM / SVD-adjoint records exactly as the CUDA kernels read
them (including the 32-bit fast-division constants), so the host plan compiler can be
checked against the oracle on the CPU.
"""
import numpy as np

from yastn_gb300 import _plans as P


def fast_div_np(n, magic, shift):
    n = np.asarray(n, dtype=np.uint64)
    return ((((n * np.uint64(magic)) >> np.uint64(32)) + n) >> np.uint64(shift)).astype(np.int64)


def run_copy(tasks, items, src, dst):
    """Apply copy tasks from src to dst (1-D numpy arrays of the same dtype)."""
    covered = {}
    for ti, first in items:
        covered.setdefault(int(ti), []).append(int(first))
    for ti, rec in enumerate(tasks):
        ndim, count, vec = int(rec[P.CP_NDIM]), int(rec[P.CP_COUNT]), int(rec[P.CP_VEC])
        firsts = sorted(covered.get(ti, []))
        if rec[P.CP_KIND] == 1:
            assert firsts == list(range(0, count, P.COPY_ITEM_TILES)), "items do not tile the task"
            _run_tiles(rec, src, dst)
            continue
        assert firsts == list(range(0, count, P.COPY_ITEM_UNITS)), "items do not tile the task"
        idx = np.arange(count, dtype=np.int64)
        so = np.full(count, rec[P.CP_SRC], dtype=np.int64)
        do = np.full(count, rec[P.CP_DST], dtype=np.int64)
        for d in range(ndim - 1, -1, -1):
            size = int(rec[P.CP_SIZE + d])
            q = fast_div_np(idx, int(rec[P.CP_MAGIC + d]), int(rec[P.CP_SHIFT + d]))
            assert np.array_equal(q, idx // size), "fast division constants are wrong"
            r = idx - q * size
            so += r * rec[P.CP_SSTR + d]
            do += r * rec[P.CP_DSTR + d]
            idx = q
        if vec:
            for j in (0, 1):
                dst[2 * do + j] = src[2 * so + j]
        else:
            dst[do] = src[so]
    return dst


def _run_tiles(rec, src, dst):
    """A kind-1 (tiled transpose) record: tile index -> (outer dims, tile y, tile x) by the
    record's fast-division constants, then the elements of the tile clipped to (NY, NX)."""
    T = P.COPY_TILE
    ndim, count = int(rec[P.CP_NDIM]), int(rec[P.CP_COUNT])
    nx, ny = int(rec[P.CP_NX]), int(rec[P.CP_NY])
    ss_x, ds_y = int(rec[P.CP_SSTR + ndim - 1]) // T, int(rec[P.CP_DSTR + ndim - 2]) // T
    assert rec[P.CP_SSTR + ndim - 2] == T and rec[P.CP_DSTR + ndim - 1] == T
    for t in range(count):
        idx, so, do, pos = t, int(rec[P.CP_SRC]), int(rec[P.CP_DST]), {}
        for d in range(ndim - 1, -1, -1):
            size = int(rec[P.CP_SIZE + d])
            q = int(fast_div_np(idx, int(rec[P.CP_MAGIC + d]), int(rec[P.CP_SHIFT + d])))
            assert q == idx // size, "fast division constants are wrong"
            r = idx - q * size
            so += r * int(rec[P.CP_SSTR + d]); do += r * int(rec[P.CP_DSTR + d]); pos[d] = r
            idx = q
        ex, ey = min(T, nx - pos[ndim - 1] * T), min(T, ny - pos[ndim - 2] * T)
        xi, yi = np.meshgrid(np.arange(ex), np.arange(ey), indexing='ij')
        dst[do + yi * ds_y + xi] = src[so + xi * ss_x + yi]


def run_gemm(plan, a, b, c, alpha=1.0, beta=0.0):
    """Grouped sum-of-products GEMM records applied with numpy (the direct outputs, then the
    split-K partial products into a workspace and their ordered reduction)."""
    _run_outs(plan.outs, plan.terms, plan.tiles, a, b, c, alpha, beta)
    sp = getattr(plan, 'split', None)
    if sp is not None:
        ws = np.full(sp.ws, np.nan, dtype=c.dtype)
        _run_outs(sp.outs, sp.terms, sp.tiles, a, b, ws, 1.0, 0.0)
        assert not np.isnan(ws).any(), "split-K chunks do not cover the workspace"
        items = {}
        for ri, it in sp.tasks:
            items.setdefault(int(ri), set()).add(int(it))
        for ri, r in enumerate(sp.red):
            c_off, m, n, ldc, p_off, chunks = (int(x) for x in r[:6])
            assert items.get(ri, set()) == set(range((m * n + 1023) // 1024)), "reduction tasks do not cover"
            acc = np.zeros(m * n, dtype=c.dtype)
            for ch in range(chunks):
                acc += ws[p_off + ch * m * n: p_off + (ch + 1) * m * n]
            rows = c_off + np.arange(m)[:, None] * ldc + np.arange(n)[None, :]
            c[rows] = alpha * acc.reshape(m, n) + (beta * c[rows] if beta != 0 else 0)
    return c


def _run_outs(outs, terms, tiles, a, b, c, alpha, beta):
    plan = type('Recs', (), {'outs': outs, 'terms': terms, 'tiles': tiles})
    seen = {}
    for oi, tr, tc, kind in plan.tiles:
        seen.setdefault(int(oi), set()).add((int(tr), int(tc), int(kind)))
    for oi, o in enumerate(plan.outs):
        c_off, m, n, ldc, t0, t1 = (int(x) for x in o[:6])
        if m == 0 or n == 0:
            continue
        if any(kd == 1 for _, _, kd in seen.get(oi, ())):  # skinny: all rows x 1024 columns (256 above 8 rows)
            assert m <= 16, "skinny tiles take at most 16 rows"
            w = P.skinny_cols(m)
            want = {(0, j, 1) for j in range((n + w - 1) // w)}
        elif any(kd == 3 for _, _, kd in seen.get(oi, ())):  # tall skinny: 256 rows x all n <= 16 columns
            assert n <= 16, "tall tiles take at most 16 columns"
            want = {(i, 0, 3) for i in range((m + 255) // 256)}
        elif any(kd == 2 for _, _, kd in seen.get(oi, ())):  # short skinny: m <= 8, one term, K <= 8
            assert m <= 8 and t1 - t0 == 1 and int(plan.terms[t0][2]) <= 8, "short tiles: m <= 8, one term, K <= 8"
            want = {(t0, j, 2) for j in range((n + 511) // 512)}  # tile row: the term index
        else:
            want = {(i, j, 0) for i in range((m + 63) // 64) for j in range((n + 63) // 64)}
        assert seen.get(oi, set()) == want, "tiles do not cover the output"
        acc = np.zeros((m, n), dtype=c.dtype)
        for t in range(t0, t1):
            a_off, b_off, k, ars, acs, brs, bcs, fl = (int(x) for x in plan.terms[t])
            ii, ll = np.meshgrid(np.arange(m), np.arange(k), indexing='ij')
            At = a[a_off + ii * ars + ll * acs]
            ll2, jj = np.meshgrid(np.arange(k), np.arange(n), indexing='ij')
            Bt = b[b_off + ll2 * brs + jj * bcs]
            if fl & 1:
                At = At.conj()
            if fl & 2:
                Bt = Bt.conj()
            acc += At @ Bt
        rows = c_off + np.arange(m)[:, None] * ldc + np.arange(n)[None, :]
        c[rows] = alpha * acc + (beta * c[rows] if beta != 0 else 0)
    return c


def rinv(x):
    return x / (x * x + 1e-12)


def svd_adjoint_core(plan, Pm, Qm, S, gS, gU, gV, dtype):
    """The K / TR formulas of csrc/yb_adjoint.cu, restated with numpy."""
    K = np.zeros(plan.kk, dtype=dtype)
    TR = np.zeros(max(plan.tr, 1), dtype=dtype)
    for r in plan.recs:
        a_off, m, n, uo, so, vo, kko, tro, k, kind = (int(x) for x in r[:10])
        s = S[so:so + k]
        Pb = Pm[kko:kko + k * k].reshape(k, k)
        Qb = Qm[kko:kko + k * k].reshape(k, k)
        F = rinv(s[None, :] - s[:, None])
        G = rinv(s[None, :] + s[:, None])
        np.fill_diagonal(F, 0)
        np.fill_diagonal(G, 0)
        Kb = 0.5 * (F + G) * (Pb - Pb.conj().T) + 0.5 * (F - G) * (Qb - Qb.conj().T)
        d = np.zeros(k, dtype=dtype)
        if gS is not None:
            d = d + gS[so:so + k]
        if np.iscomplexobj(Pb):
            d = d + 1j * np.diagonal(Pb).imag * rinv(s)
        Kb[np.arange(k), np.arange(k)] = d
        if kind == 1:
            Kb = Kb - rinv(s)[:, None] * Qb.conj().T
        elif kind == 2:
            Kb = Kb - Pb * rinv(s)[None, :]
        K[kko:kko + k * k] = Kb.ravel()
        if kind == 1:
            TR[tro:tro + k * n] = (rinv(s)[:, None] * gV[vo:vo + k * n].reshape(k, n)).ravel()
        elif kind == 2:
            TR[tro:tro + m * k] = (gU[uo:uo + m * k].reshape(m, k) * rinv(s)[None, :]).ravel()
    return K, TR


def jacobi_sweeps(X, W, blocks, dtype, tol_stop, max_sweeps):
    """The round-robin one-sided Jacobi of csrc/yb_svd.cu (svd_sweeps_kernel), restated
    sequentially with numpy on the plan's workspace layout. Returns (sweeps, converged)."""
    eps = 2.0 ** -24 if dtype in (np.float32, np.complex64) else 2.0 ** -53
    return _sweeps(X, W, blocks, dtype, tol_stop, max_sweeps, eps)


def block_jacobi_sweeps(X, W, blocks, br, inner_sweeps, tol_stop, max_sweeps):
    """The blocked FP32 Jacobi of csrc/yb_svd.cu (svd_block_sweeps_kernel), restated
    sequentially: super-vectors of ``br`` rows paired by the circle method, up to
    ``inner_sweeps`` sweeps among the 2*br rows of a pair with the rotations accumulated in
    Q, then W rows <- Q W rows. Returns (sweeps, converged)."""
    eps = 2.0 ** -24
    r2 = 2 * br
    nb = len(blocks); conv = [False] * nb; nsw = [0] * nb
    max_rounds = max(int(r[15]) - 1 for r in blocks)
    for sw in range(max_sweeps):
        maxcos = [0.0] * nb
        for rd in range(max_rounds):
            for b, r in enumerate(blocks):
                k, L, NS = int(r[9]), int(r[10]), int(r[15])
                if conv[b] or rd >= NS - 1:
                    continue
                xo, wo = int(r[13]), int(r[14])
                Xb = X[xo:xo + k * L].reshape(k, L)
                Wb = W[wo:wo + k * k].reshape(k, k)
                for pi in range(NS // 2):
                    P_, Q_ = (NS - 1, rd) if pi == 0 else ((rd + pi) % (NS - 1), (rd - pi + NS - 1) % (NS - 1))
                    grow = [sv * br + i for sv in (P_, Q_) for i in range(br)]
                    grow = [g if g < k else -1 for g in grow]
                    Xs = np.zeros((r2, L), np.float32)
                    for i, g in enumerate(grow):
                        if g >= 0:
                            Xs[i] = Xb[g]
                    Qs = np.eye(r2, dtype=np.float32)
                    any_rot = False
                    for _ in range(inner_sweeps):
                        rot = False
                        for ir in range(r2 - 1):
                            for w in range(br):
                                p, q = (r2 - 1, ir) if w == 0 else ((ir + w) % (r2 - 1), (ir - w + r2 - 1) % (r2 - 1))
                                p, q = min(p, q), max(p, q)
                                if grow[p] < 0 or grow[q] < 0:
                                    continue
                                xp, xq = Xs[p].astype(np.float64), Xs[q].astype(np.float64)
                                al, be, ga = float(xp @ xp), float(xq @ xq), float(xp @ xq)
                                if not (al > 0 and be > 0):
                                    continue
                                c_ = abs(ga) / np.sqrt(al) / np.sqrt(be)
                                maxcos[b] = max(maxcos[b], c_)
                                if not c_ > np.sqrt(L) * eps:
                                    continue
                                zeta = (be - al) / (2 * ga)
                                t = np.copysign(1.0, zeta) / (abs(zeta) + np.hypot(1.0, zeta))
                                cd = 1 / np.sqrt(1 + t * t)
                                c, s_ = np.float32(cd), np.float32(cd * t)
                                for M in (Xs, Qs):
                                    u, v = M[p].copy(), M[q].copy()
                                    M[p] = c * u - s_ * v
                                    M[q] = s_ * u + c * v
                                rot = any_rot = True
                        if not rot:
                            break
                    if any_rot:
                        rows = [g for g in grow if g >= 0]
                        idx = [i for i, g in enumerate(grow) if g >= 0]
                        Xb[rows] = Xs[idx]
                        Wb[rows] = (Qs[np.ix_(idx, idx)].astype(np.float64) @ Wb[rows].astype(np.float64)).astype(W.dtype)
        for b in range(nb):
            if not conv[b]:
                nsw[b] += 1
                if maxcos[b] <= tol_stop:
                    conv[b] = True
        if all(conv):
            break
    return nsw, conv


def _sweeps(X, W, blocks, dtype, tol_stop, max_sweeps, eps):
    nb = len(blocks); conv = [False]*nb; nsw = [0]*nb
    max_rounds = max(int(r[11]) - 1 for r in blocks)
    for sw in range(max_sweeps):
        maxcos = [0.0]*nb
        for rd in range(max_rounds):
            for b, r in enumerate(blocks):
                if conv[b]: continue
                k, L, N = int(r[9]), int(r[10]), int(r[11])
                xo, wo = (int(r[13]), int(r[14])) if dtype in (np.float32, np.complex64) else (int(r[6]), int(r[7]))
                if rd >= N - 1: continue
                for pi in range(N // 2):
                    p, q = (N - 1, rd) if pi == 0 else ((rd + pi) % (N - 1), (rd - pi + N - 1) % (N - 1))
                    if p >= k or q >= k: continue
                    p, q = min(p, q), max(p, q)
                    xp = X[xo + p*L: xo + (p+1)*L]; xq = X[xo + q*L: xo + (q+1)*L]
                    wp = W[wo + p*k: wo+(p+1)*k]; wq = W[wo+q*k: wo+(q+1)*k]
                    if np.iscomplexobj(X):
                        # complex rows: align the phase of x_q (ph = ga/|ga|), then a real rotation
                        x64p, x64q = xp.astype(np.complex128), xq.astype(np.complex128)
                        al = float(np.vdot(x64p, x64p).real); be = float(np.vdot(x64q, x64q).real)
                        gac = complex(np.sum(x64p * np.conj(x64q)))
                        if not (al > 0 and be > 0): continue
                        g = abs(gac); c_ = g/np.sqrt(al)/np.sqrt(be); maxcos[b] = max(maxcos[b], c_)
                        if not c_ > np.sqrt(L)*eps: continue
                        ph = gac / g
                        zeta = (be - al)/(2*g); t = np.copysign(1.0, zeta)/(abs(zeta) + np.hypot(1.0, zeta)); cd = 1/np.sqrt(1+t*t)
                        c, s = cd, cd*t
                        for Pp, Pq in ((xp, xq), (wp, wq)):
                            u, v = Pp.copy(), ph * Pq
                            Pp[:] = c*u - s*v; Pq[:] = s*u + c*v
                        continue
                    al = float(np.dot(xp.astype(np.float64), xp)); be = float(np.dot(xq.astype(np.float64), xq)); ga = float(np.dot(xp.astype(np.float64), xq))
                    if not (al > 0 and be > 0): continue
                    c_ = abs(ga)/np.sqrt(al)/np.sqrt(be); maxcos[b] = max(maxcos[b], c_)
                    if not c_ > np.sqrt(L)*eps: continue
                    zeta = (be - al)/(2*ga); t = np.copysign(1.0, zeta)/(abs(zeta) + np.hypot(1.0, zeta)); cd = 1/np.sqrt(1+t*t)
                    c, s = dtype(cd), dtype(cd*t)
                    u, v = xp.copy(), xq.copy(); xp[:] = c*u - s*v; xq[:] = s*u + c*v
                    u, v = wp.copy(), wq.copy(); wp[:] = c*u - s*v; wq[:] = s*u + c*v
        for b in range(nb):
            if not conv[b]:
                nsw[b] += 1
                if maxcos[b] <= tol_stop: conv[b] = True
        if all(conv): break
    return nsw, conv



def eigh_adjoint_core(X, D, gD, recs, symeig, eps=1.0e-12):
    """The inner-matrix kernel of csrc/yb_adjoint.cu (eigh_adjoint_core_kernel) with numpy."""
    K = np.empty_like(X)
    for off, k, doff, _ in (tuple(int(v) for v in r) for r in recs):
        x = X[off:off + k * k].reshape(k, k)
        d = D[doff:doff + k]
        E = d[None, :] - d[:, None]
        if symeig:
            kb = x * (E / (E * E + eps))
        else:
            np.fill_diagonal(E, 1.0)
            kb = 0.5 * (x - x.conj().T) / E
        if gD is not None:
            np.fill_diagonal(kb, gD[doff:doff + k])
        elif symeig:
            np.fill_diagonal(kb, 0)
        K[off:off + k * k] = kb.ravel()
    return K


def qr_precondition(w64, w32, blocks, data, scale):
    """numpy statement of yb_svd_qr on the plan layout: Z = X_0 (A, or A^H for tall blocks),
    Householder QR of M = Z^T (LAPACK larfg conventions; M <- H^H M), R's rows, the FP32
    start X32 = scale R, W32 = I, the reflectors and tau, and Q^T formed in Z."""
    for b, r in enumerate(blocks):
        a, m, n, k, L = int(r[0]), int(r[1]), int(r[2]), int(r[9]), int(r[17])
        A = data[a:a + m * n].reshape(m, n)
        Z = (A.conj().T if m > n else A).astype(w64.dtype).copy()
        tau = np.zeros(k, dtype=w64.dtype)
        for j in range(k):
            alpha, x = Z[j, j], Z[j, j + 1:]
            xn = float(np.sum(np.abs(x) ** 2))
            if xn == 0.0 and np.imag(alpha) == 0:
                tau[j] = 0
            else:
                beta = -np.copysign(np.sqrt(abs(alpha) ** 2 + xn), np.real(alpha))
                tau[j] = (beta - alpha) / beta
                Z[j, j + 1:] = x / (alpha - beta)
                Z[j, j] = beta
            v = np.concatenate([[1.0], Z[j, j + 1:]]).astype(w64.dtype)
            t = np.conj(tau[j])
            for c in range(j + 1, k):
                w = np.sum(np.conj(v) * Z[c, j:])
                Z[c, j:] -= t * w * v
        RR = np.triu(Z[:, :k].T)  # R[i, c] = Z[c, i] for c >= i
        w64[int(r[21]):int(r[21]) + k * k] = RR.ravel()
        w32[int(r[13]):int(r[13]) + k * k] = (scale[b] * RR).ravel().astype(w32.dtype)
        w32[int(r[14]):int(r[14]) + k * k] = np.eye(k, dtype=w32.dtype).ravel()
        V = np.triu(Z, 1)
        w64[int(r[19]):int(r[19]) + k * L] = V.ravel()
        w64[int(r[20]):int(r[20]) + k] = tau
        Q = np.eye(k, L, dtype=w64.dtype)  # rows of Q^T
        for j in range(k - 1, -1, -1):
            v = np.concatenate([[1.0], V[j, j + 1:]]).astype(w64.dtype)
            for c in range(j, k):
                w = np.sum(np.conj(v) * Q[c, j:])
                Q[c, j:] -= tau[j] * w * v
        w64[int(r[18]):int(r[18]) + k * L] = Q.ravel()


def finalize_qr(w64, blocks, U, S, V):
    """numpy statement of yb_svd_finalize for QR-preconditioned blocks (no completion):
    singular values descending; wide: U columns = x_j / s_j, WS = conj(W) sorted; tall:
    Vh rows = conj(x_j) / s_j, WS = W sorted."""
    for r in blocks:
        m, n, k = int(r[1]), int(r[2]), int(r[9])
        X = w64[int(r[6]):int(r[6]) + k * k].reshape(k, k)
        W = w64[int(r[7]):int(r[7]) + k * k].reshape(k, k)
        sig = np.linalg.norm(X, axis=1)
        idx = np.argsort(-sig, kind='stable')
        S[int(r[4]):int(r[4]) + k] = sig[idx]
        Y = X[idx] / sig[idx][:, None]
        if m > n:
            V[int(r[5]):int(r[5]) + k * n] = Y.conj().ravel()
            w64[int(r[22]):int(r[22]) + k * k] = W[idx].ravel()
        else:
            U[int(r[3]):int(r[3]) + m * k] = Y.T.ravel()
            w64[int(r[22]):int(r[22]) + k * k] = W[idx].conj().ravel()


def qr_plain(work, blocks, data, Q, R):
    """numpy statement of yb_qr on the plan layout ([16] = 2): Z = the first k columns of A as
    rows (M = A), the same Householder factorisation as ``qr_precondition``, R's rows and the
    reflectors kept, Q^T formed in Z, then the finalisation: Q (m x k) and the square part of
    R with the signs that make R's diagonal positive (the right part R[:, m:] of wide blocks
    is the host's grouped GEMM)."""
    for r in blocks:
        a, m, n, k, L = int(r[0]), int(r[1]), int(r[2]), int(r[9]), int(r[17])
        A = data[a:a + m * n].reshape(m, n)
        Z = A[:, :k].T.astype(work.dtype).copy()  # k rows of length L = m
        tau = np.zeros(k, dtype=work.dtype)
        for j in range(k):
            alpha, x = Z[j, j], Z[j, j + 1:]
            xn = float(np.sum(np.abs(x) ** 2))
            if not (xn == 0.0 and np.imag(alpha) == 0):
                beta = -np.copysign(np.sqrt(abs(alpha) ** 2 + xn), np.real(alpha))
                tau[j] = (beta - alpha) / beta
                Z[j, j + 1:] = x / (alpha - beta)
                Z[j, j] = beta
            v = np.concatenate([[1.0], Z[j, j + 1:]]).astype(work.dtype)
            for c in range(j + 1, k):
                w = np.sum(np.conj(v) * Z[c, j:])
                Z[c, j:] -= np.conj(tau[j]) * w * v
        RR = np.triu(Z[:, :k].T)
        V = np.triu(Z, 1)
        Qt = np.eye(k, L, dtype=work.dtype)
        for j in range(k - 1, -1, -1):
            v = np.concatenate([[1.0], V[j, j + 1:]]).astype(work.dtype)
            for c in range(j, k):
                w = np.sum(np.conj(v) * Qt[c, j:])
                Qt[c, j:] -= tau[j] * w * v
        sg = np.where(np.real(np.diag(RR)) < 0, -1.0, 1.0)
        Q[int(r[3]):int(r[3]) + m * k] = (Qt.T * sg[None, :]).ravel()
        Rb = R[int(r[5]):int(r[5]) + k * n].reshape(k, n)
        Rb[:, :k] = sg[:, None] * RR


def split_rows(src, rec):
    """The real rows yb_ozaki_split reads for one record: element k of row i at source
    offset rec[0] + i*rec[3] + k*rec[8] (FP64 or complex elements by the mode rec[4])."""
    s0, rows, K, rs, mode = (int(x) for x in rec[:5])
    ks = int(rec[8])
    if mode == 0:
        return np.stack([src[s0 + r * rs + ks * np.arange(K)] for r in range(rows)]).reshape(rows, K)
    half = K // 2
    out = []
    for r in range(rows):
        z = src[s0 + r * rs + ks * np.arange(half)]
        out.append({1: np.concatenate([z.real, z.imag]), 2: np.concatenate([z.real, -z.imag]),
                    3: np.concatenate([z.imag, z.real])}[mode])
    return np.stack(out).reshape(rows, K)


def ozaki_digits(x, s):
    """Row exponents e (max |x| = f 2^e, f in [0.5, 1); 0 for a zero row) and the s balanced
    base-128 digits of rint(x 2^{7s-e}) (round half to even): d_0 in [-128, 128], d_t in
    [-64, 63], x 2^-e = sum_t d_t 2^{-7(t+1)} + rounding. Returns (e, digits[s, rows, K])."""
    x = np.asarray(x, dtype=np.float64)
    mx = np.abs(x).max(axis=1) if x.shape[1] else np.zeros(x.shape[0])
    e = np.where(mx > 0, np.frexp(mx)[1], 0).astype(np.int64)
    q = np.rint(np.ldexp(x, (7 * s - e)[:, None])).astype(np.int64)
    bias = 0
    for _ in range(s - 1):
        bias = (bias << 7) | 64
    u = q + bias
    d = np.empty((s,) + x.shape, dtype=np.int64)
    d[0] = u >> (7 * (s - 1))
    for t in range(1, s):
        d[t] = ((u >> (7 * (s - 1 - t))) & 127) - 64
    return e, d


def ozaki_split(recs, groups, a_src, b_src, s, sizes, n_exps):
    """yb_ozaki_split: digit planes (as integers) and row exponents of both operands in the
    records' layouts. sizes / n_exps: (A, B) lengths of the digit and exponent arrays."""
    dig = [np.zeros(sizes[0], dtype=np.int64), np.zeros(sizes[1], dtype=np.int64)]
    exps = [np.zeros(n_exps[0], dtype=np.int64), np.zeros(n_exps[1], dtype=np.int64)]
    touched = [np.zeros(sizes[0], dtype=bool), np.zeros(sizes[1], dtype=bool)]
    grouped = {}
    for ri, first in groups:
        grouped.setdefault(int(ri), []).append(int(first))
    for ri, rec in enumerate(recs):
        op, th = int(rec[9]) & 1, int(rec[9]) >> 8
        rows, K, Kp, dst, eo = int(rec[1]), int(rec[2]), int(rec[7]), int(rec[5]), int(rec[6])
        rows_p = -(-rows // th) * th if th else rows
        assert sorted(grouped.get(ri, [])) == list(range(0, rows_p, P.OZ_SPLIT_ROWS)), "groups do not cover the rows"
        x = split_rows(b_src if op else a_src, rec)
        e, d = ozaki_digits(x, s)
        exps[op][eo:eo + rows] = e
        full = np.zeros((s, rows_p, Kp), dtype=np.int64)
        full[:, :rows, :K] = d[:, :, :]
        full[:, :rows, K:] = 0
        r = np.arange(rows_p)[:, None]
        k = np.arange(Kp)[None, :]
        if th == 0:
            off = r * Kp + k
        else:
            off = (r // th) * (Kp // 16) * th * 16 + (k // 16) * th * 16 + ((r % th) // 8) * 128 + \
                ((k % 16) // 8) * 64 + (r % 8) * 8 + k % 8
        for t in range(s):
            idx = dst + t * rows_p * Kp + off
            assert not touched[op][idx].any(), "records overlap"
            touched[op][idx] = True
            dig[op][idx] = full[t]
    return dig, exps
