"""The plain FP64 path: YASTN's backend functions as one torch operation per charge block.

This is the comparison path of the measurements: the same backend interface as
``yastn_gb300.backend`` (the reference torch backend's structure,
yastn/backend/backend_torch.py), but every hot function loops over the blocks on the host
and issues one torch launch per block — a permute-copy per merged piece
(backend_torch.py:518-531), one ``matmul`` per sector GEMM (backend_torch.py:466-473),
one ``torch.linalg.svd`` per block (cuSOLVER's gesvd on the GPU, as the reference forces
in yastn/backend/linalg/torch_svd_gesdd.py:16-17; LAPACK on the host; backend_torch.py:318-319), one ``torch.linalg.qr`` per block with the sign fix
(backend_torch.py:475-484) — and autograd differentiates the torch operations themselves
(the SVD through the reference's broadened adjoint, evaluated per block).
Everything that is not on the hot path is taken from ``yastn_gb300.backend`` unchanged.
It runs on any torch device, so the same object is the plain GPU path and the host-core
path of a benchmark.
"""
import torch

from . import backend_gb300 as _fast

__all__ = ['PlainBackend']


def _sl(x):
    return slice(x[0], x[1])


def _safe_inverse(x, eps):
    return x / (x * x + eps)


def _svd_block_adjoint(u, s, vh, gu, gs, gvh, eps):
    """Adjoint of one block's thin SVD with the Lorentzian broadening x / (x^2 + eps) of
    1/(s_j - s_i) and 1/(s_j + s_i) (yastn/backend/linalg/torch_svd_gesdd.py:296-428)."""
    m, k = u.shape
    n = vh.shape[1]
    dA = (u * gs.reshape(1, -1)) @ vh
    s_inv = _safe_inverse(s, eps)
    F = _safe_inverse(s.reshape(1, -1) - s.reshape(-1, 1), eps)
    F.fill_diagonal_(0)
    G = _safe_inverse(s.reshape(1, -1) + s.reshape(-1, 1), eps)
    G.fill_diagonal_(0)
    uh = u.conj().T
    u_term = u @ ((F + G) * (uh @ gu - gu.conj().T @ u)) * 0.5
    if m > k:
        u_term = u_term + (gu * s_inv.reshape(1, -1)) - u @ (uh @ (gu * s_inv.reshape(1, -1)))
    dA = dA + u_term @ vh
    v = vh.conj().T
    v_term = ((F - G) * (vh @ gvh.conj().T - gvh @ v)) @ vh * 0.5
    if n > k:
        v_term = v_term + s_inv.reshape(-1, 1) * (gvh - (gvh @ v) @ vh)
    dA = dA + u @ v_term
    if u.is_complex():
        L = torch.diagonal(uh @ gu).imag * s_inv
        dA = dA + (u * (1j * L).reshape(1, -1)) @ vh
    return dA


class _PlainSvd(torch.autograd.Function):
    @staticmethod
    def forward(ctx, data, meta, sizes, eps):
        real = data.real.dtype if data.is_complex() else data.dtype
        U = torch.empty(sizes[0], dtype=data.dtype, device=data.device)
        S = torch.empty(sizes[1], dtype=real, device=data.device)
        V = torch.empty(sizes[2], dtype=data.dtype, device=data.device)
        for sl, D, slU, DU, slS, slV, DV in meta:
            blk = data[_sl(sl)].view(D)
            # the reference forces cuSOLVER's gesvd on CUDA (yastn/backend/linalg/torch_svd_gesdd.py:16-17)
            u, s, vh = (torch.linalg.svd(blk, full_matrices=False, driver='gesvd') if blk.is_cuda
                        else torch.linalg.svd(blk, full_matrices=False))
            U[_sl(slU)].view(DU)[...] = u
            S[_sl(slS)] = s
            V[_sl(slV)].view(DV)[...] = vh
        ctx.save_for_backward(U, S, V)
        ctx.meta, ctx.eps, ctx.size, ctx.dtype = meta, eps, data.numel(), data.dtype
        return U, S, V

    @staticmethod
    def backward(ctx, gU, gS, gV):
        U, S, V = ctx.saved_tensors
        gU = torch.zeros_like(U) if gU is None else gU
        gS = torch.zeros_like(S) if gS is None else gS
        gV = torch.zeros_like(V) if gV is None else gV
        out = torch.zeros(ctx.size, dtype=ctx.dtype, device=U.device)
        for sl, D, slU, DU, slS, slV, DV in ctx.meta:
            out[_sl(sl)] = _svd_block_adjoint(U[_sl(slU)].view(DU), S[_sl(slS)], V[_sl(slV)].view(DV),
                                              gU[_sl(slU)].view(DU), gS[_sl(slS)].to(ctx.dtype),
                                              gV[_sl(slV)].view(DV), ctx.eps).reshape(-1)
        return out, None, None, None


class PlainBackend:
    """Backend module object (attribute access like the module ``yastn_gb300.backend``)."""

    BACKEND_ID = 'plain_torch'

    def __getattr__(self, name):
        return getattr(_fast, name)

    @staticmethod
    def transpose_and_merge(data, order, meta_new, meta_mrg, Dsize):
        out = torch.zeros(Dsize, dtype=data.dtype, device=data.device)
        pos = 0
        for tn, Dn, sln in meta_new:
            fused = out[_sl(sln)].view(Dn)
            while pos < len(meta_mrg) and meta_mrg[pos][0] == tn:
                _, slo, Do, Dslc, Drsh = meta_mrg[pos]
                fused[tuple(_sl(x) for x in Dslc)] = data[_sl(slo)].view(Do).permute(order).reshape(Drsh)
                pos += 1
        return out

    @staticmethod
    def unmerge(data, meta):
        out = torch.empty_like(data)
        for sln, Dn, slo, Do, sub in meta:
            out[_sl(sln)].view(Dn)[...] = data[_sl(slo)].view(Do)[tuple(_sl(x) for x in sub)]
        return out

    @staticmethod
    def transpose(data, axes, meta_transpose):
        out = torch.empty_like(data)
        for sln, Dn, slo, Do in meta_transpose:
            out[_sl(sln)].view(Dn)[...] = data[_sl(slo)].view(Do).permute(axes)
        return out

    @staticmethod
    def dot(Adata, Bdata, meta_dot, Dsize):
        dtype = torch.promote_types(Adata.dtype, Bdata.dtype)
        A, B = Adata.to(dtype), Bdata.to(dtype)
        out = torch.empty(Dsize, dtype=dtype, device=Adata.device)
        for slc, Dc, sla, Da, slb, Db in meta_dot:
            out[_sl(slc)].view(Dc)[...] = A[_sl(sla)].view(Da) @ B[_sl(slb)].view(Db)
        return out

    @staticmethod
    def apply_mask(Adata, mask, meta, Dsize, axis, a_ndim):
        out = torch.empty(Dsize, dtype=Adata.dtype, device=Adata.device)
        for sln, Dn, sla, Da, tm in meta:
            out[_sl(sln)].view(Dn)[...] = torch.index_select(Adata[_sl(sla)].view(Da), axis, mask[tm])
        return out

    @staticmethod
    def svd(data, meta, sizes, fullrank_uv=False, ad_decomp_reg=1.0e-12, diagnostics=None, **kwargs):
        return _PlainSvd.apply(data, meta, sizes, ad_decomp_reg)

    @staticmethod
    def qr(data, meta, sizes):
        Q = torch.zeros(sizes[0], dtype=data.dtype, device=data.device)
        R = torch.zeros(sizes[1], dtype=data.dtype, device=data.device)
        for sl, D, slQ, DQ, slR, DR in meta:
            q, r = torch.linalg.qr(data[_sl(sl)].view(D))
            sr = torch.sign(torch.real(torch.diagonal(r)))
            sr = torch.where(sr == 0, torch.ones_like(sr), sr).to(data.dtype)
            Q[_sl(slQ)].view(DQ)[...] = q * sr.reshape(1, -1)
            R[_sl(slR)].view(DR)[...] = sr.reshape(-1, 1) * r
        return Q, R

    @staticmethod
    def fix_svd_signs(Udata, Vhdata, meta):
        Uo = torch.empty_like(Udata)
        Vo = torch.empty_like(Vhdata)
        for _, _, slU, DU, _, slV, DV in meta:
            u = Udata[_sl(slU)].view(DU)
            vh = Vhdata[_sl(slV)].view(DV)
            with torch.no_grad():
                amp = (u.abs() * (2 ** 40)).to(torch.int64)
                rows = amp.argmax(dim=0)
                ph = u[rows, torch.arange(DU[1], device=u.device)]
                ph = ph / ph.abs()
            Uo[_sl(slU)].view(DU)[...] = u * ph.conj().reshape(1, -1)
            Vo[_sl(slV)].view(DV)[...] = vh * ph.reshape(-1, 1)
        return Uo, Vo
