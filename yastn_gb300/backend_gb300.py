"""YASTN backend module for GB300: drop-in for ``yastn/backend/backend_torch.py``.

Select it with ``yastn.make_config(backend=yastn_gb300.backend, default_device='cuda')``
(``yastn/tensor/_initialize.py:106-115`` accepts a module object). The module exposes
every name of the reference backend's ``__all__`` (``backend_torch.py:32-49``) plus
``BACKEND_ID``/``DTYPE``.

Hot path — hand-written sm_103a kernels of ``libyastn_gb300.so`` (through :mod:`.ops`),
each behind a ``torch.autograd.Function`` with a hand-written adjoint:

* ``transpose_and_merge`` / ``unmerge`` / ``transpose`` (family (a), one launch each);
* ``dot`` / ``transpose_dot_sum`` (family (b), one grouped GEMM launch);
* ``svd`` / ``svdvals`` (family (c), batched Jacobi for all blocks);
* ``apply_mask`` / ``fix_svd_signs`` (device gather / gauge kernels).

Everything else is cold bookkeeping implemented with ordinary torch tensor calls on
the tensors' own device, as in the reference torch backend. ``BACKEND_ID`` is "torch", the
reference torch backend's: the tensors are torch tensors of the same dtypes and layout, YASTN
enables torch checkpointing for it (``yastn/tn/fpeps/envs/_env_ctm.py:579``), its
serialisation names the backend by this string (a tensor saved from this backend loads into
YASTN's torch backend), and it differs from ``'torch_cpp'`` (``yastn/tensor/_contractions.py:199``).
"""
from functools import reduce

import numpy as np
import torch
from torch.utils.checkpoint import checkpoint as _checkpoint

from . import ops

try:
    import torch.cuda.nvtx as nvtx
except Exception:  # pragma: no cover
    nvtx = None
cuda = torch.cuda

__all__ = ['DTYPE', 'get_dtype', 'get_yastn_dtype',
           'nvtx', 'cuda_is_available', 'get_device', 'move_to',
           'grad', 'requires_grad_', 'requires_grad', 'detach', 'detach_', 'clone', 'copy', 'checkpoint',
           'random_seed', 'randint',
           'to_numpy', 'get_shape', 'get_size', 'diag_create', 'diag_get', 'real', 'is_complex', 'conj',
           'imag', 'max_abs', 'maximum', 'norm_matrix', 'delete', 'insert',
           'expm', 'first_element', 'item', 'sum_elements', 'norm', 'entropy',
           'zeros', 'ones', 'rand', 'to_tensor', 'to_mask', 'square_matrix_from_dict',
           'trace', 'rsqrt', 'reciprocal', 'exp', 'sqrt', 'absolute', 'permute_dims',
           'fix_svd_signs', 'svdvals', 'svd_lowrank', 'svd', 'svd_randomized', 'svds_scipy',
           'eigh', 'qr', 'pinv', 'eig', 'eigh_lowrank', 'eigvals',
           'argsort', 'eigs_which', 'allclose',
           'add', 'sub', 'apply_mask', 'vdot', 'diag_1dto2d', 'diag_2dto1d',
           'dot', 'dot_diag', 'transpose_dot_sum',
           'merge_to_dense', 'merge_super_blocks', 'is_independent',
           'embed_mask', 'transpose', 'transpose_and_merge', 'unmerge',
           'negate_blocks', 'bitwise_not']

BACKEND_ID = "torch"
DTYPE = {'float32': torch.float32,
         'float64': torch.float64,
         'complex64': torch.complex64,
         'complex128': torch.complex128,
         'bool': torch.bool}


def _sl(x):
    return slice(x[0], x[1])


# Sector GEMMs of ``dot`` for FP64 / complex128 operands: 'fp64' runs the native grouped GEMM;
# 'emulated' runs the split-operand emulation on BF16 tensor cores (8 digit slices, results
# within a few FP64 rounding errors of the native product, normwise per row/column scale).
_GEMM_MODE = ['fp64']
_EMULATED = (torch.float64, torch.complex128)


def set_gemm_mode(mode):
    """Select 'fp64' (default) or 'emulated' sector GEMMs for float64 / complex128 ``dot``."""
    if mode not in ('fp64', 'emulated'):
        raise ValueError("gemm mode must be 'fp64' or 'emulated'")
    _GEMM_MODE[0] = mode


def get_gemm_mode():
    return _GEMM_MODE[0]


# ============================================================================ hot path

# The autograd Functions keep the forward free of ctx and store what the backward needs in
# setup_context, the form torch.func transforms (vjp, jvp, grad) require: YASTN's fixed-point
# CTMRG differentiates its CTM iteration with torch.func.vjp
# (yastn/tn/fpeps/envs/fixed_pt.py:851-853).

class _TransposeAndMerge(torch.autograd.Function):
    """transpose_and_merge (backend_torch.py:588-589); adjoint = the inverse copy."""

    @staticmethod
    def forward(data, order, meta_new, meta_mrg, Dsize):
        return ops.merge(data, order, meta_new, meta_mrg, Dsize)

    @staticmethod
    def setup_context(ctx, inputs, output):
        data, order, meta_new, meta_mrg, Dsize = inputs
        ctx.args = (order, meta_new, meta_mrg, Dsize, data.numel())

    @staticmethod
    def backward(ctx, g):
        order, meta_new, meta_mrg, Dsize, n = ctx.args
        g = _unwrap(g)
        return ops.merge_backward(g, order, meta_new, meta_mrg, Dsize, n), None, None, None, None


class _Unmerge(torch.autograd.Function):
    """unmerge (backend_torch.py:592-593); adjoint = the inverse copy."""

    @staticmethod
    def forward(data, meta):
        return ops.unmerge(data, meta)

    @staticmethod
    def setup_context(ctx, inputs, output):
        data, meta = inputs
        ctx.args = (meta, data.numel())

    @staticmethod
    def backward(ctx, g):
        meta, n = ctx.args
        g = _unwrap(g)
        return ops.unmerge_backward(g, meta, n), None


class _Transpose(torch.autograd.Function):
    """transpose of every block (backend_torch.py:584-585)."""

    @staticmethod
    def forward(data, axes, meta_transpose):
        return ops.transpose(data, axes, meta_transpose)

    @staticmethod
    def setup_context(ctx, inputs, output):
        _, axes, meta_transpose = inputs
        ctx.args = (axes, meta_transpose)

    @staticmethod
    def backward(ctx, g):
        axes, meta = ctx.args
        g = _unwrap(g)
        return ops.transpose_backward(g, axes, meta), None, None


def _unwrap(t):
    """The tensor under torch.func's wrappers (same values): inside a torch.func.vjp the
    backward receives wrapped cotangents and saved tensors, which have no storage pointer for
    the kernels."""
    if not isinstance(t, torch.Tensor):
        return t
    fx = torch._C._functorch
    while fx.is_functorch_wrapped_tensor(t):
        t = fx.get_unwrapped(t)
    return t


def _unwrap_all(*ts):
    return tuple(_unwrap(t) for t in ts)


def _grad_like(g, x):
    """Cast a cotangent to the dtype of the primal (real part for real primals)."""
    if g is None:
        return None
    if not x.is_complex() and g.is_complex():
        g = g.real
    return g.to(x.dtype)


class _Dot(torch.autograd.Function):
    """dot (backend_torch.py:549-550): one grouped GEMM; adjoints A_b += C_b B^H,
    B_b += A^H C_b as two grouped GEMMs with terms grouped by operand block."""

    @staticmethod
    def forward(A, B, meta_dot, Dsize):
        if _GEMM_MODE[0] == 'emulated' and A.dtype in _EMULATED and B.dtype in _EMULATED:
            return ops.dot_ozaki(A, B, meta_dot, Dsize)
        return ops.dot(A, B, meta_dot, Dsize)

    @staticmethod
    def setup_context(ctx, inputs, output):
        A, B, meta_dot, _ = inputs
        ctx.save_for_backward(A, B)
        ctx.meta_dot = meta_dot

    @staticmethod
    def backward(ctx, g):
        A, B, g = _unwrap_all(*ctx.saved_tensors, g)
        need_a, need_b = ctx.needs_input_grad[0], ctx.needs_input_grad[1]
        Ab, Bb = ops.dot_backward(g.contiguous(), A, B, ctx.meta_dot, need_a, need_b)
        return _grad_like(Ab, A), _grad_like(Bb, B), None, None


class _TransposeDotSum(torch.autograd.Function):
    """transpose_dot_sum (backend_torch.py:553-554)."""

    @staticmethod
    def forward(A, B, meta_dot, Areshape, Breshape, Aorder, Border, Dsize):
        return ops.transpose_dot_sum(A, B, meta_dot, Areshape, Breshape, Aorder, Border, Dsize)

    @staticmethod
    def setup_context(ctx, inputs, output):
        A, B, meta_dot, Areshape, Breshape, Aorder, Border, _ = inputs
        ctx.save_for_backward(A, B)
        ctx.args = (meta_dot, Areshape, Breshape, Aorder, Border)

    @staticmethod
    def backward(ctx, g):
        A, B, g = _unwrap_all(*ctx.saved_tensors, g)
        meta_dot, Areshape, Breshape, Aorder, Border = ctx.args
        Ab, Bb = ops.transpose_dot_sum_backward(g.contiguous(), A, B, meta_dot, Areshape, Breshape, Aorder, Border)
        return _grad_like(Ab, A), _grad_like(Bb, B), None, None, None, None, None, None


class _ApplyMask(torch.autograd.Function):
    """apply_mask (backend_torch.py:576-577); adjoint = scatter into zeros."""

    @staticmethod
    def forward(A, mask, meta, Dsize, axis, ndim):
        return ops.apply_mask(A, mask, meta, Dsize, axis, ndim)

    @staticmethod
    def setup_context(ctx, inputs, output):
        A, mask, meta, _, axis, ndim = inputs
        ctx.args = (mask, meta, axis, ndim, A.numel())

    @staticmethod
    def backward(ctx, g):
        mask, meta, axis, ndim, n = ctx.args
        g = _unwrap(g)
        return ops.apply_mask(g.contiguous(), mask, meta, None, axis, ndim, scatter_size=n), None, None, None, None, None


class _Svd(torch.autograd.Function):
    """svd (backend_torch.py:318-319): batched Jacobi forward, regularised adjoint of
    yastn/backend/linalg/torch_svd_gesdd.py:296-428 on all blocks at once."""

    @staticmethod
    def forward(data, meta, sizes, fullrank_uv, ad_decomp_reg, diagnostics):
        return ops.svd(data, meta, sizes)

    @staticmethod
    def setup_context(ctx, inputs, output):
        data, meta = inputs[0], inputs[1]
        ctx.save_for_backward(*output)
        ctx.meta, ctx.n, ctx.dtype = meta, data.numel(), data.dtype

    @staticmethod
    def backward(ctx, gU, gS, gV):
        U, S, V, gU, gS, gV = _unwrap_all(*ctx.saved_tensors, gU, gS, gV)
        dA = ops.svd_backward(U, S, V, gU, gS, gV, ctx.meta, ctx.n, ctx.dtype)
        return dA, None, None, None, None, None


class _Eigh(torch.autograd.Function):
    """eigh (backend_torch.py:369-384): batched Jacobi forward; the adjoint of SYMEIG
    (order_by_magnitude, yastn/backend/linalg/torch_eig_sym.py:43-54) or of
    torch.linalg.eigh, on all blocks at once."""

    @staticmethod
    def forward(data, meta, sizes, order_by_magnitude, ad_decomp_reg):
        return ops.eigh(data, meta, sizes, order_by_magnitude)

    @staticmethod
    def setup_context(ctx, inputs, output):
        data, meta, _, order_by_magnitude, ad_decomp_reg = inputs
        ctx.save_for_backward(*output)
        ctx.meta, ctx.n, ctx.dtype = meta, data.numel(), data.dtype
        ctx.by_mag, ctx.eps = order_by_magnitude, ad_decomp_reg

    @staticmethod
    def backward(ctx, gS, gU):
        S, U, gS, gU = _unwrap_all(*ctx.saved_tensors, gS, gU)
        dA = ops.eigh_backward(U, S, gU, gS, ctx.meta, ctx.n, ctx.dtype, ctx.by_mag, ctx.eps)
        return dA, None, None, None, None


class _FixSigns(torch.autograd.Function):
    """fix_svd_signs (backend_torch.py:353-366); the adjoint (yb_fix_signs_adjoint) follows
    torch's autograd of the reference: the cotangents times the phases and, for complex data,
    the gradient through the phase of each column's largest entry."""

    @staticmethod
    def forward(U, V, meta):
        Uo, Vo, _ = ops.fix_svd_signs(U, V, meta)
        return Uo, Vo

    @staticmethod
    def setup_context(ctx, inputs, output):
        U, V, meta = inputs
        ctx.save_for_backward(U, V)
        ctx.meta = meta

    @staticmethod
    def backward(ctx, gU, gV):
        U, V, gU, gV = _unwrap_all(*ctx.saved_tensors, gU, gV)
        gUi, gVi = ops.fix_svd_signs_backward(U, V, gU, gV, ctx.meta)
        return gUi, gVi, None


def transpose_and_merge(data, order, meta_new, meta_mrg, Dsize):
    return _TransposeAndMerge.apply(data, order, meta_new, meta_mrg, Dsize)


def unmerge(data, meta):
    return _Unmerge.apply(data, meta)


def transpose(data, axes, meta_transpose):
    return _Transpose.apply(data, axes, meta_transpose)


def dot(Adata, Bdata, meta_dot, Dsize):
    return _Dot.apply(Adata, Bdata, meta_dot, Dsize)


def transpose_dot_sum(Adata, Bdata, meta_dot, Areshape, Breshape, Aorder, Border, Dsize):
    return _TransposeDotSum.apply(Adata, Bdata, meta_dot, Areshape, Breshape, Aorder, Border, Dsize)


def apply_mask(Adata, mask, meta, Dsize, axis, a_ndim):
    return _ApplyMask.apply(Adata, mask, meta, Dsize, axis, a_ndim)


def svd(data, meta, sizes, fullrank_uv=False, ad_decomp_reg=1.0e-12, diagnostics=None, **kwargs):
    if fullrank_uv:
        raise NotImplementedError("yastn_gb300 svd computes the thin SVD (fullrank_uv=False)")
    return _Svd.apply(data, meta, sizes, fullrank_uv, ad_decomp_reg, diagnostics)


def svdvals(data, meta, sizeS, **kwargs):
    with torch.no_grad():
        nU = sum((m[3][0] * m[3][1]) for m in meta)
        nV = sum((m[6][0] * m[6][1]) for m in meta)
        _, S, _ = ops.svd(data.detach(), meta, (nU, sizeS, nV))
    return S


def fix_svd_signs(Udata, Vhdata, meta):
    return _FixSigns.apply(Udata, Vhdata, meta)


# ============================================================================ cold bookkeeping

def cuda_is_available():
    return torch.cuda.is_available()


def get_dtype(t):
    return t.dtype


def get_yastn_dtype(t):
    names = [k for k, v in DTYPE.items() if v == t.dtype]
    return names[0] if len(names) == 1 else 'unknown'


def is_complex(x):
    return x.is_complex()


def get_device(x):
    return str(x.device)


def random_seed(seed):
    torch.random.manual_seed(seed)


def grad(x):
    return x.grad


def detach(x):
    return x.detach()


def detach_(x):
    x.detach_()


def clone(x):
    return x.clone()


def copy(x):
    return x.detach().clone()


def to_numpy(x):
    if isinstance(x, (int, float, complex)):
        return x
    return x.detach().resolve_conj().cpu().numpy().copy()


def get_shape(x):
    return x.size()


def get_size(x):
    return x.numel()


def diag_create(x, p=0):
    return torch.diag(x, diagonal=p)


def diag_get(x):
    return torch.diag(x)


def real(x):
    return torch.real(x)


def imag(x):
    return torch.imag(x) if x.is_complex() else torch.zeros_like(x)


def max_abs(x):
    return x.abs().max() if x.numel() > 0 else torch.zeros((), dtype=torch.float64, device=x.device)


def maximum(a, b):
    return torch.maximum(a, b)


def norm_matrix(x):
    return torch.linalg.norm(x)


def delete(x, sl):
    return torch.cat([x[:sl[0]], x[sl[1]:]])


def insert(x, start, values):
    return torch.cat([x[:start], values, x[start:]])


def expm(x):
    return torch.matrix_exp(x)


def permute_dims(x, axes):
    return x.permute(*axes)


def first_element(x):
    return x.reshape(-1)[0]


def item(x):
    return x.item()


def sum_elements(data):
    return data.sum().reshape(1)


def norm(data, p):
    if p == "fro":
        return torch.linalg.vector_norm(data)
    return data.abs().max() if data.numel() > 0 else torch.zeros((), dtype=torch.float64, device=data.device)


def entropy(data, alpha, tol):
    total = data.sum() if data.numel() > 0 else 0.
    if total > 0:
        p = data / total
        p = p[p > tol]
        if alpha == 1:
            return -torch.sum(p * torch.log2(p))
        return torch.log2(torch.sum(p ** alpha)) / (1 - alpha)
    return torch.zeros((), dtype=torch.float64)


def zeros(D, dtype='float64', device='cpu'):
    return torch.zeros(D, dtype=DTYPE[dtype], device=device)


def ones(D, dtype='float64', device='cpu'):
    return torch.ones(D, dtype=DTYPE[dtype], device=device)


def rand(D, dtype='float64', distribution=(0, 1), device='cpu'):
    if dtype == 'bool':
        return torch.rand(D, dtype=torch.float64, device=device) > 0.5
    if distribution == 'normal':
        return torch.randn(D, dtype=DTYPE[dtype], device=device)
    out = torch.rand(D, dtype=DTYPE[dtype], device=device)
    if distribution == (0, 1):
        return out
    lo, hi = distribution
    shift = lo if ('float' in dtype) else lo * (1 + 1j)
    return (hi - lo) * out + shift


def randint(low, high):
    return torch.randint(low, high, (1,))[0]


def to_tensor(val, Ds=None, dtype='float64', device='cpu'):
    T = torch.as_tensor(val, dtype=DTYPE[dtype], device=device)
    return T if Ds is None else T.reshape(Ds).contiguous()


@torch.no_grad()
def to_mask(val):
    return torch.as_tensor(val).nonzero().reshape(-1)


def square_matrix_from_dict(H, D=None, **kwargs):
    dtype = reduce(torch.promote_types, (a.dtype for a in H.values()))
    device = next(iter(H.values())).device
    T = torch.zeros((D, D), dtype=dtype, device=device)
    for (i, j), v in H.items():
        if i < D and j < D:
            T[i, j] = v
    return T


def requires_grad_(data, requires_grad=True):
    data.requires_grad_(requires_grad)


def requires_grad(data):
    return data.requires_grad


def move_to(data, *args, **kwargs):
    dtype = kwargs.pop("dtype", None)
    if dtype is not None:
        kwargs["dtype"] = DTYPE[dtype]
    return data.to(*args, **kwargs)


def conj(data):
    return data.conj()


def trace(data, order, meta, Dsize):
    out = torch.zeros(Dsize, dtype=data.dtype, device=data.device)
    for sln, recs in meta:
        acc = out[_sl(sln)]
        for slo, Do, Drsh in recs:
            blk = data[_sl(slo)].reshape(Do).permute(order).reshape(Drsh)
            acc += torch.diagonal(blk, dim1=0, dim2=1).sum(dim=-1)
    return out


def rsqrt(data, cutoff=0):
    res = torch.zeros_like(data)
    sel = data.abs() > cutoff
    res[sel] = data[sel].rsqrt()
    return res


def reciprocal(data, cutoff=0):
    res = torch.zeros_like(data)
    sel = data.abs() > cutoff
    res[sel] = 1. / data[sel]
    return res


def exp(data, step):
    return torch.exp(step * data)


def sqrt(data):
    return torch.sqrt(data)


def absolute(data):
    return torch.abs(data)


def bitwise_not(data):
    return torch.bitwise_not(data)


def _not_hot(name):
    raise NotImplementedError(f"yastn_gb300: {name} is not provided by this backend")


def _leading_svd(data, meta, sizes):
    """The leading k singular triplets of every block (k = the block's slS length), as the
    partial-SVD policies return them: the thin SVD of all blocks on the device (this
    backend's Jacobi, with its adjoint), then the first k columns of U, values of S and
    rows of Vh gathered in one launch each. The reference computes them with SciPy's
    ARPACK / PROPACK (``svds_scipy``) or torch.svd_lowrank on the host or device; the exact
    leading triplets answer both."""
    full, offs, ks = [], [0, 0, 0], set()
    for sl, D, slU, DU, slS, slV, DV in meta:
        m, n = D
        kf, k = min(m, n), slS[1] - slS[0]
        ks.add(k)
        full.append((sl, D, (offs[0], offs[0] + m * kf), (m, kf), (offs[1], offs[1] + kf),
                     (offs[2], offs[2] + kf * n), (kf, n)))
        offs = [offs[0] + m * kf, offs[1] + kf, offs[2] + kf * n]
    Uf, Sf, Vf = svd(data, tuple(full), tuple(offs))
    mask = {k: torch.arange(k, dtype=torch.int64, device=data.device) for k in ks}
    mU, mS, mV = [], [], []
    for (sl, D, slU, DU, slS, slV, DV), f in zip(meta, full):
        k = slS[1] - slS[0]
        mU.append((slU, DU, f[2], f[3], k))
        mS.append((slS, k, f[4], f[4][1] - f[4][0], k))
        mV.append((slV, DV, f[5], f[6], k))
    U = apply_mask(Uf, mask, tuple(mU), sizes[0], 1, 2)
    S = apply_mask(Sf, mask, tuple(mS), sizes[1], 0, 1)
    V = apply_mask(Vf, mask, tuple(mV), sizes[2], 0, 2)
    return U, S, V


def svd_lowrank(data, meta, sizes, **kwargs):
    return _leading_svd(data, meta, sizes)


def svd_randomized(data, meta, sizes, q=None, niter=3, **kwargs):
    return _leading_svd(data, meta, sizes)


def svds_scipy(data, meta, sizes, thresh=0.1, solver='arpack', **kwargs):
    return _leading_svd(data, meta, sizes)


def eigh_lowrank(data, meta, sizes, thresh=None, **kwargs):
    _not_hot('eigh_lowrank')


def eig(data, meta=None, sizes=(1, 1), **kwargs):
    _not_hot('eig (non-Hermitian)')


def eigvals(data, meta, sizeS, **kwargs):
    _not_hot('eigvals (non-Hermitian)')


class _Qr(torch.autograd.Function):
    """qr (backend_torch.py:475-484): batched Householder QR, positive diagonal of R; the
    adjoint (real and complex blocks) by grouped GEMMs, a symmetrisation and a triangular
    solve."""

    @staticmethod
    def forward(data, meta, sizes):
        return ops.qr(data, meta, sizes)

    @staticmethod
    def setup_context(ctx, inputs, output):
        data, meta, _ = inputs
        ctx.save_for_backward(data, *output)
        ctx.meta = meta

    @staticmethod
    def backward(ctx, gQ, gR):
        data, Q, R, gQ, gR = _unwrap_all(*ctx.saved_tensors, gQ, gR)
        return ops.qr_backward(Q, R, gQ, gR, data, ctx.meta), None, None


def qr(data, meta, sizes):
    return _Qr.apply(data, meta, sizes)


def pinv(A, rcond=None, hermitian=False, out=None, atol=None, rtol=None):
    return torch.linalg.pinv(A, atol=atol, rtol=rtol if rtol is not None else rcond, hermitian=hermitian)


def eigh(data, meta=None, sizes=(1, 1), order_by_magnitude=False, ad_decomp_reg=1.0e-12):
    if meta is None:
        # one dense D x D matrix (YASTN's eigs diagonalises its Krylov matrix this way,
        # yastn/krylov/_krylov.py:231): the batched kernel on a single block; (S ascending, U)
        # as torch.linalg.eigh returns them (backend_torch.py:384)
        D = int(data.shape[0])
        if data.dim() != 2 or data.shape[1] != D:
            raise ValueError("eigh of a dense matrix needs a square 2-D tensor")
        meta1 = (((0, D * D), (D, D), (0, D * D), (D, D), (0, D)),)
        S, U = _Eigh.apply(data.reshape(-1), meta1, (D, D * D), order_by_magnitude, ad_decomp_reg)
        return S, U.reshape(D, D)
    return _Eigh.apply(data, meta, sizes, order_by_magnitude, ad_decomp_reg)


@torch.no_grad()
def argsort(data):
    return torch.argsort(data)


@torch.no_grad()
def eigs_which(val, which):
    if which == 'LM':
        return (-val.abs()).argsort()
    if which == 'SM':
        return val.abs().argsort()
    if which == 'LR':
        return (-torch.real(val)).argsort()
    return torch.real(val).argsort()


def allclose(Adata, Bdata, rtol, atol):
    dtype = torch.promote_types(Adata.dtype, Bdata.dtype)
    return torch.allclose(Adata.to(dtype=dtype), Bdata.to(dtype=dtype), rtol=rtol, atol=atol)


def add(datas, metas, Dsize):
    dtype = reduce(torch.promote_types, (d.dtype for d in datas))
    out = torch.zeros(Dsize, dtype=dtype, device=datas[0].device)
    for d, meta in zip(datas, metas):
        for sl_c, sl_a in meta:
            out[_sl(sl_c)] += d[_sl(sl_a)]
    return out


def sub(Adata, Bdata, metas, Dsize):
    dtype = torch.promote_types(Adata.dtype, Bdata.dtype)
    out = torch.zeros(Dsize, dtype=dtype, device=Adata.device)
    for sl_c, sl_a in metas[0]:
        out[_sl(sl_c)] += Adata[_sl(sl_a)]
    for sl_c, sl_b in metas[1]:
        out[_sl(sl_c)] -= Bdata[_sl(sl_b)]
    return out


def vdot(Adata, Bdata, meta):
    dtype = torch.promote_types(Adata.dtype, Bdata.dtype)
    Adata, Bdata = Adata.to(dtype), Bdata.to(dtype)
    if len(meta) == 0:
        return torch.zeros((), dtype=dtype, device=Adata.device)
    return torch.stack([torch.dot(Adata[_sl(a)], Bdata[_sl(b)]) for a, b in meta]).sum()


def dot_diag(Adata, Bdata, meta, Dsize, axis, a_ndim):
    shape = [1] * a_ndim
    shape[axis] = -1
    dtype = torch.promote_types(Adata.dtype, Bdata.dtype)
    out = torch.empty(Dsize, dtype=dtype, device=Adata.device)
    for sln, slb, Db, sla in meta:
        out[_sl(sln)].reshape(Db)[:] = Adata[_sl(sla)].reshape(shape) * Bdata[_sl(slb)].reshape(Db)
    return out


def negate_blocks(Adata, slices):
    sign = torch.ones(Adata.numel(), dtype=torch.float64, device=Adata.device)
    for slc in slices:
        sign[_sl(slc)] = -1.
    return Adata * sign.to(Adata.real.dtype if Adata.is_complex() else Adata.dtype)


def embed_mask(Adata, mask, meta, Dsize, axis, a_ndim):
    pre = (slice(None),) * axis
    post = (slice(None),) * (a_ndim - axis - 1)
    out = torch.zeros(Dsize, dtype=Adata.dtype, device=Adata.device)
    for sln, Dn, sla, Da, tm in meta:
        out[_sl(sln)].view(Dn)[pre + (mask[tm],) + post] = Adata[_sl(sla)].view(Da)
    return out


def merge_to_dense(data, Dtot, meta):
    out = torch.zeros(Dtot, dtype=data.dtype, device=data.device)
    for sl, Dss in meta:
        out[tuple(slice(*Ds) for Ds in Dss)] = data[sl].reshape(tuple(Ds[1] - Ds[0] for Ds in Dss))
    return out.reshape(-1)


def merge_super_blocks(pos_tens, meta_new, meta_block, Dsize):
    from itertools import groupby
    dtype = reduce(torch.promote_types, (a._data.dtype for a in pos_tens.values()))
    device = next(iter(pos_tens.values()))._data.device
    out = torch.zeros(Dsize, dtype=dtype, device=device)
    for (tn, Dn, sln), (t1, gr) in zip(meta_new, groupby(meta_block, key=lambda x: x[0])):
        assert tn == t1
        for (_, slo, Do, pos, Dslc) in gr:
            out[_sl(sln)].reshape(Dn)[tuple(slice(*x) for x in Dslc)] = pos_tens[pos]._data[_sl(slo)].reshape(Do)
    return out


def diag_1dto2d(data, meta, Dsize):
    out = torch.zeros(Dsize, dtype=data.dtype, device=data.device)
    for sln, slo in meta:
        out[_sl(sln)] = torch.diag(data[_sl(slo)]).reshape(-1)
    return out


def diag_2dto1d(data, meta, Dsize):
    out = torch.zeros(Dsize, dtype=data.dtype, device=data.device)
    for sln, slo, Do in meta:
        out[_sl(sln)] = torch.diagonal(data[_sl(slo)].reshape(Do))
    return out


def checkpoint(f, *args, **kwargs):
    return _checkpoint(f, *args,
                       use_reentrant=kwargs.pop('use_reentrant', None),
                       determinism_check=kwargs.pop('determinism_check', 'default'),
                       debug=kwargs.pop('debug', False),
                       **kwargs)


def is_independent(x, y):
    return (x is not y) and (x.numel() == 0 or x.untyped_storage().data_ptr() != y.untyped_storage().data_ptr())
