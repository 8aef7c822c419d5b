"""NumPy restatement of the reference backend functions on the hot path.

Test infrastructure: the oracle the CUDA backend is checked against. Each function
cites the reference file:line whose behaviour it restates. Paths are relative to the
YASTN source tree.

All ``data`` arguments are flat 1-D numpy arrays; ``meta`` arguments are the nested
tuples of Python ints that YASTN's metadata layer hands to its backend.
"""
from itertools import groupby

import numpy as np
import scipy.linalg

__all__ = [
    'transpose_and_merge', 'transpose_and_merge_backward',
    'unmerge', 'unmerge_backward',
    'dot', 'dot_backward', 'transpose_dot_sum', 'transpose_dot_sum_backward',
    'svd', 'svd_block_backward', 'svd_backward',
    'eigh', 'eigh_block_backward', 'eigh_block_backward_hermitian', 'eigh_backward', 'fix_svd_signs',
    'fix_svd_signs_backward',
    'qr', 'qr_block_backward', 'qr_backward',
    'apply_mask', 'apply_mask_backward', 'embed_mask',
    'truncation_mask', 'rand_normal',
]


def _sl(x):
    return slice(x[0], x[1])


# ---------------------------------------------------------------- family (a): merge / unmerge

def transpose_and_merge(data, order, meta_new, meta_mrg, Dsize):
    """Gather-permute-merge of source blocks into fused blocks.

    Restates ``yastn/backend/backend_np.py:653-661``. The output starts zero-filled;
    for each fused block ``(tn, Dn, sln)`` every source ``(tn, slo, Do, Dslc, Drsh)``
    with the same ``tn`` (``meta_mrg`` is grouped by ``tn`` in the order of
    ``meta_new``) is transposed by ``order``, reshaped to ``Drsh`` and written at the
    sub-slices ``Dslc`` of the row-major fused block ``Dn``.
    """
    out = np.zeros(Dsize, dtype=data.dtype)
    groups = groupby(meta_mrg, key=lambda rec: rec[0])
    for (tn, Dn, sln), (tg, recs) in zip(meta_new, groups):
        if tn != tg:
            raise AssertionError("meta_mrg is not grouped in the order of meta_new")
        fused = out[_sl(sln)].reshape(Dn)
        for _, slo, Do, Dslc, Drsh in recs:
            piece = data[_sl(slo)].reshape(Do).transpose(order).reshape(Drsh)
            fused[tuple(_sl(x) for x in Dslc)] = piece
    return out


def transpose_and_merge_backward(data_b, order, meta_new, meta_mrg, D_source):
    """Adjoint of :func:`transpose_and_merge`.

    Restates ``yastn/backend/_backend_torch_backwards.py:376-392``: each source block
    receives the inverse-permuted sub-block of the fused cotangent; source positions
    not listed in ``meta_mrg`` stay zero.
    """
    inv = tuple(int(i) for i in np.argsort(order))
    out = np.zeros(D_source, dtype=data_b.dtype)
    groups = groupby(meta_mrg, key=lambda rec: rec[0])
    for (tn, Dn, sln), (tg, recs) in zip(meta_new, groups):
        if tn != tg:
            raise AssertionError("meta_mrg is not grouped in the order of meta_new")
        fused = data_b[_sl(sln)].reshape(Dn)
        for _, slo, Do, Dslc, _ in recs:
            Dt = tuple(Do[i] for i in order)
            sub = fused[tuple(_sl(x) for x in Dslc)]
            out[_sl(slo)].reshape(Do)[...] = sub.reshape(Dt).transpose(inv)
    return out


def unmerge(data, meta):
    """Cut fused blocks back into their constituent blocks.

    Restates ``yastn/backend/backend_np.py:664-669``: for each record
    ``(sln, Dn, slo, Do, sub_slc)`` the sub-block ``sub_slc`` of the row-major fused
    block ``Do`` at ``slo`` is reshaped to ``Dn`` and written at ``sln``. Output has
    the length of the input (no zero blocks are introduced).
    """
    out = np.empty_like(data)
    for sln, Dn, slo, Do, sub_slc in meta:
        out[_sl(sln)].reshape(Dn)[...] = data[_sl(slo)].reshape(Do)[tuple(_sl(x) for x in sub_slc)]
    return out


def unmerge_backward(data_b, meta, fwd_size):
    """Adjoint of :func:`unmerge`; restates ``_backend_torch_backwards.py:417-426``."""
    out = np.empty(fwd_size, dtype=data_b.dtype)
    for sln, Dn, slo, Do, sub_slc in meta:
        out[_sl(slo)].reshape(Do)[tuple(_sl(x) for x in sub_slc)] = data_b[_sl(sln)].reshape(Dn)
    return out


# ---------------------------------------------------------------- family (b): sector GEMMs

def dot(A, B, meta_dot, Dsize):
    """Block-diagonal product ``C[slc] = A[sla] @ B[slb]`` per charge sector.

    Restates ``yastn/backend/backend_np.py:580-587`` (dtype promotion by
    ``np.promote_types``).
    """
    dtype = np.promote_types(A.dtype, B.dtype)
    out = np.empty(Dsize, dtype=dtype)
    for slc, Dc, sla, Da, slb, Db in meta_dot:
        out[_sl(slc)] = (A[_sl(sla)].reshape(Da) @ B[_sl(slb)].reshape(Db)).ravel()
    return out


def dot_backward(C_b, A, B, meta_dot):
    """Adjoint of :func:`dot`: ``A_b += C_b B^H``, ``B_b += A^H C_b``.

    Restates ``yastn/backend/_backend_torch_backwards.py:117-138``; the ``+=`` matters
    when several sectors share an operand block (``fuse_contracted`` policy).
    """
    dtype = np.promote_types(A.dtype, B.dtype)
    A_b = np.zeros(A.shape, dtype=dtype)
    B_b = np.zeros(B.shape, dtype=dtype)
    for slc, Dc, sla, Da, slb, Db in meta_dot:
        Cb = C_b[_sl(slc)].reshape(Dc)
        Ablk = A[_sl(sla)].reshape(Da)
        Bblk = B[_sl(slb)].reshape(Db)
        A_b[_sl(sla)] += (Cb @ Bblk.conj().T).ravel()
        B_b[_sl(slb)] += (Ablk.conj().T @ Cb).ravel()
    return A_b, B_b


def transpose_dot_sum(A, B, meta_dot, Areshape, Breshape, Aorder, Border, Dsize):
    """No-fusion contraction ``C_k = sum_(a,b) A_a B_b`` of permuted blocks.

    Restates ``yastn/backend/backend_np.py:590-601``.
    """
    dtype = np.promote_types(A.dtype, B.dtype)
    out = np.empty(Dsize, dtype=dtype)
    Am = [A[_sl(sl)].reshape(Di).transpose(Aorder).reshape(Dl, Dr) for sl, Di, Dl, Dr in Areshape]
    Bm = [B[_sl(sl)].reshape(Di).transpose(Border).reshape(Dl, Dr) for sl, Di, Dl, Dr in Breshape]
    for sl, Dslc, pairs in meta_dot:
        acc = np.zeros(Dslc, dtype=dtype)
        for ta, tb in pairs:
            acc += Am[ta] @ Bm[tb]
        out[_sl(sl)] = acc.ravel()
    return out


def transpose_dot_sum_backward(C_b, A, B, meta_dot, Areshape, Breshape, Aorder, Border):
    """Adjoint of :func:`transpose_dot_sum`.

    Restates ``yastn/backend/_backend_torch_backwards.py:170-226``: cotangents of the
    permuted (Dl, Dr) matrices accumulate ``C_b B^H`` / ``A^H C_b`` over the pairs, then
    are permuted back into the layout of A and B (positions of blocks not listed stay 0).
    """
    dtype = np.promote_types(A.dtype, B.dtype)
    Am = [A[_sl(sl)].reshape(Di).transpose(Aorder).reshape(Dl, Dr) for sl, Di, Dl, Dr in Areshape]
    Bm = [B[_sl(sl)].reshape(Di).transpose(Border).reshape(Dl, Dr) for sl, Di, Dl, Dr in Breshape]
    Ag = [np.zeros(x.shape, dtype=dtype) for x in Am]
    Bg = [np.zeros(x.shape, dtype=dtype) for x in Bm]
    for sl, Dslc, pairs in meta_dot:
        cb = C_b[_sl(sl)].reshape(Dslc)
        for ta, tb in pairs:
            Ag[ta] += cb @ Bm[tb].conj().T
            Bg[tb] += Am[ta].conj().T @ cb
    A_b = np.zeros(A.shape, dtype=dtype)
    B_b = np.zeros(B.shape, dtype=dtype)
    for g, (sl, Di, _, _) in zip(Ag, Areshape):
        A_b[_sl(sl)] = g.reshape(tuple(Di[o] for o in Aorder)).transpose(np.argsort(Aorder)).ravel()
    for g, (sl, Di, _, _) in zip(Bg, Breshape):
        B_b[_sl(sl)] = g.reshape(tuple(Di[o] for o in Border)).transpose(np.argsort(Border)).ravel()
    return A_b, B_b


# ---------------------------------------------------------------- family (c): SVD / eigh / truncation

def _safe_svd(a):
    """gesdd with a gesvd fallback; restates ``yastn/backend/backend_np.py:281-286``."""
    try:
        return scipy.linalg.svd(a, full_matrices=False)
    except scipy.linalg.LinAlgError:
        return scipy.linalg.svd(a, full_matrices=False, lapack_driver='gesvd')


def svd(data, meta, sizes):
    """Thin SVD of every sector block; restates ``yastn/backend/backend_np.py:330-340``.

    ``meta`` records are ``(sl, D, slU, DU, slS, slV, DV)``; singular values are
    returned in descending order per block (LAPACK convention).
    """
    real = data.real.dtype if np.iscomplexobj(data) else data.dtype
    U = np.empty(sizes[0], dtype=data.dtype)
    S = np.empty(sizes[1], dtype=real)
    V = np.empty(sizes[2], dtype=data.dtype)
    for sl, D, slU, DU, slS, slV, DV in meta:
        u, s, vh = _safe_svd(data[_sl(sl)].reshape(D))
        U[_sl(slU)] = u.ravel()
        S[_sl(slS)] = s
        V[_sl(slV)] = vh.ravel()
    return U, S, V


def fix_svd_signs(U, V, meta):
    """Gauge fix: the largest-|.| entry of each U column becomes real positive.

    Restates ``yastn/backend/backend_np.py:447-458``: the magnitude comparison is done
    on ``int64(|U| * 2**40)`` (so near-ties resolve to the first row), and the
    conjugate phase multiplies U's column while the phase multiplies V's row.
    """
    U = U.copy()
    V = V.copy()
    amp = (np.abs(U) * (2 ** 40)).astype(np.int64)
    for _, _, slU, DU, _, slV, DV in meta:
        Ub = U[_sl(slU)].reshape(DU)
        Vb = V[_sl(slV)].reshape(DV)
        rows = np.argmax(amp[_sl(slU)].reshape(DU), axis=0)
        phase = Ub[rows, np.arange(DU[1])]
        phase = phase / np.abs(phase)
        Ub *= phase.conj()[None, :]
        Vb *= phase[:, None]
    return U, V


def fix_svd_signs_backward(U, V, gU, gV, meta):
    """Adjoint of ``fix_svd_signs`` as torch's autograd differentiates the reference's
    ``backend_torch.py:353-366`` (gradients in torch's convention for complex tensors,
    grad = dL/dRe + i dL/dIm). Per column c with phase p = u/|u| of the selected entry
    u = U[r*, c] (the row choice is piecewise constant):
    gU[:, c] = gU'[:, c] p, gV[c, :] = gV'[c, :] conj(p), and, through p,
    gU[r*, c] += -i (p / |u|) Im(conj(G) p) with G = sum_i U[i, c] conj(gU'[i, c]) +
    sum_j conj(V[c, j]) gV'[c, j]; for real data the last term vanishes."""
    dU = np.zeros_like(U)
    dV = np.zeros_like(V)
    amp = (np.abs(U) * (2 ** 40)).astype(np.int64)
    for _, _, slU, DU, _, slV, DV in meta:
        Ub, Vb = U[_sl(slU)].reshape(DU), V[_sl(slV)].reshape(DV)
        gUb, gVb = gU[_sl(slU)].reshape(DU), gV[_sl(slV)].reshape(DV)
        cols = np.arange(DU[1])
        rows = np.argmax(amp[_sl(slU)].reshape(DU), axis=0)
        u = Ub[rows, cols]
        p = u / np.abs(u)
        dUb = gUb * p[None, :]
        dVb = gVb * p.conj()[:, None]
        if np.iscomplexobj(U):
            G = np.sum(Ub * gUb.conj(), axis=0) + np.sum(Vb.conj() * gVb, axis=1)
            dUb[rows, cols] += -1j * (p / np.abs(u)) * np.imag(G.conj() * p)
        dU[_sl(slU)] = dUb.ravel()
        dV[_sl(slV)] = dVb.ravel()
    return dU, dV


def eigh(data, meta, sizes):
    """Hermitian eigendecomposition per block (ascending eigenvalues).

    Restates ``yastn/backend/backend_np.py:461-474``; records are ``(sl, D, slU, DU, slS)``.
    """
    real = data.real.dtype if np.iscomplexobj(data) else data.dtype
    S = np.zeros(sizes[0], dtype=real)
    U = np.zeros(sizes[1], dtype=data.dtype)
    for sl, D, slU, DU, slS in meta:
        s, u = scipy.linalg.eigh(data[_sl(sl)].reshape(D))
        S[_sl(slS)] = s
        U[_sl(slU)] = u.ravel()
    return S, U


def _safe_inverse(x, eps=1.0e-12):
    """Lorentzian-broadened inverse x/(x^2+eps).

    Restates ``yastn/backend/linalg/torch_svd_gesdd.py:4-6``, where the ``eps_abs``
    argument is overwritten by 1e-12, so the broadening is always 1e-12.
    """
    return x / (x * x + 1.0e-12)


def svd_block_backward(u, s, vh, gu, gs, gvh):
    """Regularised SVD adjoint of one block.

    Restates ``yastn/backend/linalg/torch_svd_gesdd.py:296-428`` (real and complex):
    F_ij = 1/(s_j - s_i), G_ij = 1/(s_j + s_i) broadened by x/(x^2+1e-12), zero
    diagonal, plus the projector terms for rectangular blocks and the complex
    imaginary-diagonal term. ``gu``/``gs``/``gvh`` may be None (no cotangent).
    """
    m, k = u.shape
    n = vh.shape[1]
    if gs is not None:
        sigma_term = (u * gs[None, :]) @ vh
    else:
        sigma_term = np.zeros((m, n), dtype=u.dtype)
    if gu is None and gvh is None:
        return sigma_term
    s_inv = _safe_inverse(s)
    F = _safe_inverse(s[None, :] - s[:, None])
    np.fill_diagonal(F, 0)
    G = _safe_inverse(s[None, :] + s[:, None])
    np.fill_diagonal(G, 0)
    uh = u.conj().T
    if gu is not None:
        guh = gu.conj().T
        u_term = u @ ((F + G) * (uh @ gu - guh @ u)) * 0.5
        if m > k:
            proj = np.eye(m, dtype=u.dtype) - u @ uh
            u_term = u_term + proj @ (gu * s_inv[None, :])
        u_term = u_term @ vh
    else:
        u_term = np.zeros((m, n), dtype=u.dtype)
    v = vh.conj().T
    if gvh is not None:
        gv = gvh.conj().T
        v_term = ((F - G) * (vh @ gv - gvh @ v)) @ vh * 0.5
        if n > k:
            proj = np.eye(n, dtype=u.dtype) - v @ vh
            v_term = v_term + s_inv[:, None] * (gvh @ proj)
        v_term = u @ v_term
    else:
        v_term = np.zeros((m, n), dtype=u.dtype)
    dA = u_term + sigma_term + v_term
    if np.iscomplexobj(u) and gu is not None:
        L = np.diagonal(uh @ gu).copy()
        L = 1j * L.imag * s_inv
        dA = dA + (u * L[None, :]) @ vh
    return dA


def svd_backward(U, S, V, gU, gS, gV, meta, data_size, dtype):
    """Block-sparse SVD adjoint; restates ``_backend_torch_backwards.py:53-66``."""
    out = np.zeros(data_size, dtype=dtype)
    for sl, D, slU, DU, slS, slV, DV in meta:
        u = U[_sl(slU)].reshape(DU)
        vh = V[_sl(slV)].reshape(DV)
        s = S[_sl(slS)]
        gu = None if gU is None else gU[_sl(slU)].reshape(DU)
        gs = None if gS is None else gS[_sl(slS)]
        gvh = None if gV is None else gV[_sl(slV)].reshape(DV)
        out[_sl(sl)] = svd_block_backward(u, s, vh, gu, gs, gvh).ravel()
    return out


def eigh_block_backward(d, u, gd, gu, eps=1.0e-12):
    """Symmetric-eig adjoint ``U (diag(gD) + F o U^T gU) U^T`` with F = (d_j - d_i)
    broadened by x/(x^2+eps); restates ``yastn/backend/linalg/torch_eig_sym.py:43-54``."""
    F = d[None, :] - d[:, None]
    F = F / (F * F + eps)
    np.fill_diagonal(F, 0)
    ut = u.T
    gd = np.zeros_like(d) if gd is None else gd
    inner = np.diag(gd).astype(u.dtype)
    if gu is not None:
        inner = inner + F * (ut @ gu)
    return u @ inner @ ut


def eigh_block_backward_hermitian(d, u, gd, gu):
    """Adjoint of torch.linalg.eigh, the path of ``eigh`` without order_by_magnitude
    (backend_torch.py:376-378): U (diag(gD) + skew(U^H gU) / E) U^H with skew(X) =
    (X - X^H) / 2 and E_ij = d_j - d_i (E_ii = 1; the diagonal is gD when given)."""
    X = u.conj().T @ gu if gu is not None else np.zeros((len(d), len(d)), dtype=u.dtype)
    X = 0.5 * (X - X.conj().T)
    E = d[None, :] - d[:, None]
    np.fill_diagonal(E, 1.0)
    inner = X / E
    if gd is not None:
        np.fill_diagonal(inner, gd)
    return u @ inner @ u.conj().T


def qr(data, meta, sizes):
    """Reduced QR per block with R's diagonal made positive; restates
    ``yastn/backend/backend_np.py:511-520`` (records ``(sl, D, slQ, DQ, slR, DR)``; a zero
    diagonal entry keeps sign +1)."""
    Q = np.empty(sizes[0], dtype=data.dtype)
    R = np.empty(sizes[1], dtype=data.dtype)
    for sl, D, slQ, DQ, slR, DR in meta:
        q, r = scipy.linalg.qr(data[_sl(sl)].reshape(D), mode='economic')
        sr = np.sign(np.real(np.diag(r)))
        sr[sr == 0] = 1
        Q[_sl(slQ)] = (q * sr).ravel()
        R[_sl(slR)] = (sr.reshape(-1, 1) * r).ravel()
    return Q, R


def qr_block_backward(q, r, gq, gr, a):
    """Adjoint of one block's reduced QR, the rule torch's autograd applies to the reference's
    ``torch.linalg.qr`` + sign fix (``backend_torch.py:475-484``; R's diagonal is real): with
    U = r[:, :k], gU = gr[:, :k], gq' = gq (+ a[:, m:] gr[:, m:]^H for wide blocks),
    M = U gU^H - gq'^H q, dA[:, :k] = (gq' + q copyltu(M)) U^{-H}, copyltu(M) =
    tril(M, -1) + tril(M, -1)^H + Re diag(M), and dA[:, m:] = q gr[:, m:] for wide blocks
    (gradients in torch's convention for complex tensors)."""
    m, k = q.shape
    n = r.shape[1]
    u, gu, b = r[:, :k], gr[:, :k], gq.copy()
    if n > m:
        b = b + a[:, m:] @ gr[:, m:].conj().T
    M = u @ gu.conj().T - b.conj().T @ q
    low = np.tril(M, -1)
    b = b + q @ (low + low.conj().T + np.diag(np.real(np.diag(M))))
    da = np.zeros((m, n), dtype=q.dtype)
    da[:, :k] = scipy.linalg.solve_triangular(u, b.conj().T, lower=False).conj().T
    if n > m:
        da[:, m:] = q @ gr[:, m:]
    return da


def qr_backward(Q, R, gQ, gR, data, meta):
    """Block-sparse QR adjoint (real and complex)."""
    out = np.zeros(data.size, dtype=data.dtype)
    for sl, D, slQ, DQ, slR, DR in meta:
        q = Q[_sl(slQ)].reshape(DQ)
        r = R[_sl(slR)].reshape(DR)
        out[_sl(sl)] = qr_block_backward(q, r, gQ[_sl(slQ)].reshape(DQ), gR[_sl(slR)].reshape(DR),
                                         data[_sl(sl)].reshape(D)).ravel()
    return out


def eigh_backward(U, S, gU, gS, meta, data_size, dtype, order_by_magnitude=False, eps=1.0e-12):
    """Adjoint of ``eigh`` over all blocks: SYMEIG's broadened formula when
    ``order_by_magnitude`` (torch_eig_sym.py:43-54), torch.linalg.eigh's otherwise."""
    out = np.zeros(data_size, dtype=dtype)
    for sl, D, slU, DU, slS in meta:
        u = U[_sl(slU)].reshape(DU)
        d = S[_sl(slS)]
        gu = None if gU is None else gU[_sl(slU)].reshape(DU)
        gd = None if gS is None else gS[_sl(slS)]
        if order_by_magnitude:
            blk = eigh_block_backward(d, u, gd, gu, eps)
        else:
            blk = eigh_block_backward_hermitian(d, u, gd, gu)
        out[_sl(sl)] = blk.ravel()
    return out


# ---------------------------------------------------------------- masks

def apply_mask(A, mask, meta, Dsize, axis, ndim):
    """Keep the masked indices along ``axis`` of every block.

    Restates ``yastn/backend/backend_np.py:626-633``; ``mask`` maps a charge to an
    integer index array, records are ``(sln, Dn, sla, Da, tm)``.
    """
    out = np.empty(Dsize, dtype=A.dtype)
    for sln, Dn, sla, Da, tm in meta:
        blk = A[_sl(sla)].reshape(Da)
        out[_sl(sln)] = np.take(blk, np.asarray(mask[tm]), axis=axis).ravel()
    return out


def apply_mask_backward(C_b, mask, meta, size_A, axis, ndim):
    """Adjoint of :func:`apply_mask`; restates ``_backend_torch_backwards.py:270-279``."""
    out = np.zeros(size_A, dtype=C_b.dtype)
    for sln, Dn, sla, Da, tm in meta:
        Da = (Da,) if isinstance(Da, int) else Da  # diagonal tensors carry an int length
        blk = out[_sl(sla)].reshape(Da)
        idx = [slice(None)] * len(Da)
        idx[axis] = np.asarray(mask[tm])
        blk[tuple(idx)] = C_b[_sl(sln)].reshape(Dn)
    return out


def embed_mask(A, mask, meta, Dsize, axis, ndim):
    """Inverse of :func:`apply_mask` into zeros; restates ``backend_np.py:636-643``."""
    out = np.zeros(Dsize, dtype=A.dtype)
    for sln, Dn, sla, Da, tm in meta:
        Dn = (Dn,) if isinstance(Dn, int) else Dn
        blk = out[_sl(sln)].reshape(Dn)
        idx = [slice(None)] * len(Dn)
        idx[axis] = np.asarray(mask[tm])
        blk[tuple(idx)] = A[_sl(sla)].reshape(Da)
    return out


def truncation_mask(S, slices, charges=None, tol=0, tol_block=0, D_block=float('inf'),
                    D_total=float('inf'), truncate_multiplets=False, argsort=np.argsort):
    """Boolean keep-mask over a flat diagonal spectrum ``S`` split into blocks.

    Restates ``yastn/tensor/linalg.py:637-735`` at the level of flat arrays:

    1. per block: keep at most ``D_block`` values above ``tol_block * max(block)``,
       dropping the smallest by ``argsort`` order (:700-711);
    2. globally: ``D_total`` is capped by the count of masked values above
       ``tol * max`` (:713-716); all values outside the top ``D_total`` of
       ``S * mask`` in ``argsort`` order are dropped (:722-734), with the optional
       multiplet-gap extension (:724-732).

    ``slices`` is a sequence of ``(start, stop)``; ``charges`` (one tuple per block)
    is needed only when ``tol_block``/``D_block`` are dicts keyed by charge.
    ``argsort`` defaults to ``np.argsort`` (the NumPy backend's choice,
    ``backend_np.py:527-528``).
    """
    S = np.asarray(S)
    mask = np.ones(S.shape, dtype=bool)
    if truncate_multiplets:
        tol_block, D_block = 0, float('inf')
    tol_null = 0. if isinstance(tol_block, dict) else tol_block
    D_null = 0 if isinstance(D_block, dict) else D_block
    for i, (lo, hi) in enumerate(slices):
        t = charges[i] if charges is not None else None
        blk = S[lo:hi]
        tol_rel = tol_block[t] if (isinstance(tol_block, dict) and t in tol_block) else tol_null
        bmax = np.abs(blk).max() if blk.size > 0 else 0
        D_tol = int(np.sum(blk > tol_rel * bmax))
        D_bl = D_block[t] if (isinstance(D_block, dict) and t in D_block) else D_null
        D_bl = min(D_bl, D_tol)
        if 0 < D_bl < hi - lo:
            inds = argsort(blk)
            mask[lo:hi][inds[:-D_bl]] = False
        elif D_bl == 0:
            mask[lo:hi] = False
    temp = S * mask
    tmax = np.abs(temp).max() if temp.size > 0 else 0
    D_tol = int(np.sum(temp > tol * tmax))
    D_total = min(D_total, D_tol)
    if D_total == 0:
        mask[:] = False
        return mask
    inds = argsort(temp)
    if truncate_multiplets and D_total < len(inds):
        gap = -1
        for p in range(D_total, len(inds)):
            gap_p = abs(S[inds[-p]] - S[inds[-p - 1]])
            if gap_p > gap:
                D_total = p
                gap = gap_p
            if gap > abs(S[inds[-p]]):
                break
    mask[inds[:-D_total]] = False
    return mask


# ---------------------------------------------------------------- synthetic inputs

def rand_normal(rng, size, dtype='float64'):
    """Normal draws in YASTN's convention; restates ``backend_np.py:186-201``.

    One vector of length ``size`` from ``rng.normal``; complex draws are
    ``(N + iN)/sqrt(2)`` with the real vector drawn first.
    """
    if 'complex' in dtype:
        re = rng.normal(size=size)
        im = rng.normal(size=size)
        return ((re + 1j * im) / (2. ** 0.5)).astype(dtype)
    return rng.normal(size=size).astype(dtype)
