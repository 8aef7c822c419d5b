"""Device-resident Lanczos for YASTN's ``eigs`` (hermitian Krylov expansion).

YASTN's ``eigs`` (yastn/krylov/_krylov.py:177-238) expands the Krylov space with
``Tensor.expand_krylov_space`` (yastn/tensor/_krylov.py:17-46): per step one matvec, a
``vdot``, an ``add`` with the previous two vectors and a ``norm``, and a comparison of the
norm with the breakdown tolerance on the host -- one device-to-host synchronisation per
step, and one torch launch per block inside ``add``/``vdot``. Here the basis is one
(ncv + 1) x n matrix in device memory, the tridiagonal coefficients stay device scalars and
the vector work is four fused kernels of ``libyastn_gb300.so`` per step (yb_krylov_dot,
yb_krylov_update, yb_krylov_scale), so the expansion never waits for the host and can be
captured once as a CUDA graph (:class:`LanczosGraph`) and replayed. The breakdown test
(``beta_j < tol``, happy breakdown) is applied once after the expansion to the coefficients
read back together; the basis vectors after a breakdown are computed but discarded, which
leaves the Ritz values and vectors those of YASTN's loop.

:func:`eigs` has the signature and return convention of ``yastn.eigs``; for ``hermitian=True``
on this backend it runs the device Lanczos (the matvec's output must keep the input's block
structure, as the DMRG effective Hamiltonians do), otherwise it defers to YASTN's own
routine. To use it inside ``yastn.tn.mps.dmrg_``, rebind the name that module calls:
``yastn.tn.mps._dmrg.eigs = yastn_gb300.eigs``.
"""
import ctypes

import numpy as np
import torch

from . import _native as N
from . import ops
from .ops import _check, _ptr, _stream, _dtype_code

_PARTS = [None]


def _parts():
    if _PARTS[0] is None:
        _PARTS[0] = int(N.lib().yb_krylov_parts())
    return _PARTS[0]


class LanczosState:
    """Device buffers of one expansion: the basis V ((ncv + 1) x n), alphas (ncv), betas
    (ncv) and the partial-sum workspace; reused across expansions of the same size/dtype."""

    def __init__(self, n, ncv, dtype, device):
        self.n, self.ncv, self.dtype, self.device = n, ncv, dtype, device
        self.V = torch.empty((ncv + 1, n), dtype=dtype, device=device)
        self.alpha = torch.zeros(ncv, dtype=dtype, device=device)
        self.beta = torch.zeros(ncv + 1, dtype=torch.float64, device=device)  # [ncv] = |v0|
        self.parts = torch.empty(2 * _parts(), dtype=torch.float64, device=device)  # complex: pairs
        self.code = _dtype_code(dtype)


def lanczos(matvec, v0, ncv, state=None):
    """Hermitian Lanczos expansion of ``ncv`` steps from ``v0`` (1-D CUDA tensor, float64 or
    complex128), sync-free: V_0 = v0/|v0|; w = matvec(V_j); alpha_j = <V_j, w>;
    w -= alpha_j V_j + beta_{j-1} V_{j-1}; beta_j = |w|; V_{j+1} = w / beta_j.
    ``matvec`` maps a 1-D tensor to a 1-D tensor of the same length. Returns the state (V,
    alpha, beta on the device)."""
    v0 = _check(v0, 'v0')
    n = v0.numel()
    if state is None or state.n != n or state.ncv != ncv or state.dtype != v0.dtype or state.device != v0.device:
        state = LanczosState(n, ncv, v0.dtype, v0.device)
    st = _stream()
    code = state.code
    V, parts = state.V, state.parts
    nb = state.beta[ncv:ncv + 1]
    N.call('yb_krylov_norm', _ptr(v0), ctypes.c_int64(n), code, _ptr(parts), _ptr(nb), st, launches=2)
    N.call('yb_krylov_scale', _ptr(v0), _ptr(nb), ctypes.c_int64(n), code, _ptr(V[0]), st)
    for j in range(ncv):
        w = _check(matvec(V[j]), 'matvec output')
        if w.numel() != n:
            raise ValueError("matvec changed the vector length")
        if w.data_ptr() == V[j].data_ptr():
            w = w.clone()
        a = state.alpha[j:j + 1]
        N.call('yb_krylov_dot', _ptr(V[j]), _ptr(w), ctypes.c_int64(n), code, _ptr(parts), _ptr(a), st, launches=2)
        b = state.beta[j:j + 1]
        prev = V[j - 1] if j > 0 else None
        N.call('yb_krylov_update', _ptr(w), _ptr(V[j]), _ptr(prev) if prev is not None else ctypes.c_void_p(0),
               _ptr(a), _ptr(state.beta[j - 1:j]) if prev is not None else ctypes.c_void_p(0), ctypes.c_int64(n),
               code, _ptr(parts), _ptr(b), st, launches=2)
        N.call('yb_krylov_scale', _ptr(w), _ptr(b), ctypes.c_int64(n), code, _ptr(V[j + 1]), st)
    return state


def ritz(state, which='SR', tol=1e-13):
    """Krylov dimension m after the breakdown test, and the eigenvalues / eigenvectors of the
    m x m tridiagonal matrix (host, one read of the coefficients), ordered as ``which``
    ('SR', 'LR', 'LM', 'SM'; yastn/backend/backend_torch.py:eigs_which)."""
    import scipy.linalg
    al = state.alpha.cpu().numpy()
    be = state.beta[:state.ncv].cpu().numpy()
    m = state.ncv
    for j in range(state.ncv):
        if be[j] < tol:  # happy breakdown: V_{j+1} is not part of the basis
            m = j + 1
            break
    T = np.diag(al[:m]).astype(np.result_type(al, be))
    for j in range(m - 1):
        T[j + 1, j] = be[j]
        T[j, j + 1] = np.conj(be[j])
    val, vr = scipy.linalg.eigh(T)
    if which == 'LM':
        ind = np.argsort(-np.abs(val))
    elif which == 'SM':
        ind = np.argsort(np.abs(val))
    elif which == 'LR':
        ind = np.argsort(-val.real)
    else:
        ind = np.argsort(val.real)
    return m, val[ind], vr[:, ind]


def combine(state, coeffs, m):
    """sum_{i < m} coeffs_i V_i on the device (yb_krylov_combine)."""
    c = torch.as_tensor(np.ascontiguousarray(coeffs[:m]), dtype=state.dtype).to(state.device)
    y = torch.empty(state.n, dtype=state.dtype, device=state.device)
    N.call('yb_krylov_combine', _ptr(state.V), ctypes.c_int64(state.n), _ptr(c), int(m), ctypes.c_int64(state.n),
           state.code, _ptr(y), _stream())
    return y


class LanczosGraph:
    """A Lanczos expansion of ``matvec`` captured once as a CUDA graph and replayed.

    ``v0`` is the static input (copy new start vectors into ``self.v0`` before ``replay``);
    the basis and the coefficients are written into ``self.state`` by every replay. The
    matvec must be capturable (no host synchronisation, plans warmed by a first eager run,
    which the constructor performs)."""

    def __init__(self, matvec, v0, ncv, warmup=2):
        self.v0 = v0.clone()
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            st = None
            for _ in range(warmup):
                st = lanczos(matvec, self.v0, ncv, st)
        torch.cuda.current_stream().wait_stream(side)
        self.graph = torch.cuda.CUDAGraph()
        l0 = N.LAUNCHES[0]
        # the operator's constant operands (environments, their merges and digit planes) are
        # computed once per replay, by its first matvec
        with ops.hold_constant_operands(), torch.cuda.graph(self.graph):
            self.state = lanczos(matvec, self.v0, ncv, st)
        self.launches = N.LAUNCHES[0] - l0

    def replay(self):
        self.graph.replay()
        return self.state


class _StructureGrew(Exception):
    """The operator returned blocks its argument does not have."""

    def __init__(self, w):
        super().__init__("operator output has a larger block structure")
        self.w = w


def eigs(f, v0, k=1, which='SR', ncv=10, maxiter=None, tol=1e-13, hermitian=False, **kwargs):
    """``yastn.eigs`` with the hermitian Krylov expansion on the device (see the module
    docstring); returns (eigenvalues[:k], list of k Ritz-vector Tensors).

    The basis shares the start vector's block structure. When the operator returns blocks
    the start vector lacks (zero blocks are not stored, and an effective Hamiltonian can fill
    them), the start vector is extended by those blocks (zeros) and the expansion restarts;
    zero blocks change neither the Ritz values nor the vectors, and YASTN's own loop ends with
    the same union structure."""
    from . import backend_gb300
    backend = v0.config.backend
    if not hermitian or backend is not backend_gb300 or not v0._data.is_cuda:
        import yastn
        return yastn.eigs(f, v0, k=k, which=which, ncv=ncv, maxiter=maxiter, tol=tol, hermitian=hermitian, **kwargs)
    if v0.norm() == 0:
        import yastn
        raise yastn.YastnError('Initial vector v0 of eigs should be nonzero.')
    v = v0
    for _ in range(64):  # each restart adds blocks; the structure is finite
        struct, slices = v.struct, v.slices

        def matvec(x, v=v, struct=struct, slices=slices):
            w = f(v._replace(data=x))
            if w.struct != struct or w.slices != slices:
                if w.struct.t != struct.t or w.struct.D != struct.D:
                    raise _StructureGrew(w)
                w = v._replace(data=x).add(w, amplitudes=[0, 1])  # same blocks, other layout
            return w._data

        try:
            with ops.hold_constant_operands():  # the environments' merges and splits, once per expansion
                st = lanczos(matvec, v._data.detach(), ncv)
        except _StructureGrew as e:
            v = v.add(e.w, amplitudes=[1, 0])  # v's data, the union of the block structures
            continue
        m, val, vr = ritz(st, which, tol)
        vals = torch.as_tensor(val[:k], device=v.device)
        Y = [v._replace(data=combine(st, vr[:, i], m)) for i in range(k)]
        return vals, Y
    raise RuntimeError("device eigs: the block structure did not settle")
