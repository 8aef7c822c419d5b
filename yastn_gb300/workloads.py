"""Recorded backend-call traces and synthetic inputs for tests and benchmarks.

YASTN's metadata layer (``yastn/tensor/_merging.py``, ``_contractions.py``,
``linalg.py``) turns charge bookkeeping into nested tuples of ints that it hands
to the backend. The fixtures under ``tests/golden`` hold such tuples, recorded
from the reference's own calls, so the backend can be exercised exactly as YASTN
drives it without YASTN being installed.
"""
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), 'tests', 'golden')


def _decode(x, arrays):
    if isinstance(x, list):
        return tuple(_decode(y, arrays) for y in x)
    if isinstance(x, dict):
        if '__array__' in x:
            key = x['__array__']
            return arrays[key] if (arrays is not None and key in arrays) else ArraySpec(x)
        if '__mask__' in x:
            return {tuple(k): np.asarray(_decode(v, arrays)) for k, v in x['__mask__']}
        if '__dict__' in x:
            return {tuple(k): v for k, v in x['__dict__']}
        return {k: _decode(v, arrays) for k, v in x.items()}
    return x


class ArraySpec:
    """Placeholder for an array that was summarised (shape, dtype, checksum) instead of stored."""

    def __init__(self, rec):
        self.key = rec['__array__']
        self.shape = tuple(rec.get('shape', ()))
        self.dtype = rec.get('dtype')
        self.checksum = rec.get('checksum')

    def __repr__(self):
        return f"ArraySpec({self.key}, shape={self.shape}, dtype={self.dtype})"


def load_trace(name, directory=GOLDEN):
    """Load ``<name>.json`` (+ ``<name>.npz``): returns the payload with decoded calls.

    Each call is a dict ``{'fn', 'args', 'kwargs', 'out'}`` whose metadata are
    tuples again and whose arrays are numpy arrays (or :class:`ArraySpec`).
    """
    with open(os.path.join(directory, name + '.json')) as f:
        payload = json.load(f)
    npz = os.path.join(directory, name + '.npz')
    arrays = dict(np.load(npz)) if os.path.exists(npz) else {}
    if 'calls' in payload:
        for c in payload['calls']:
            for k in list(c.keys()):
                if k != 'fn':
                    c[k] = _decode(c[k], arrays)
    payload['_arrays'] = arrays
    return payload


def cfg1_inputs(trace=None):
    """Data of the U(1) D=64 rank-4 benchmark tensors A and B.

    YASTN's ``rand(..., distribution='normal')`` draws one normal vector of length
    ``size`` per tensor from ``np.random.default_rng(seed)``, A first and then B
    (``yastn/backend/backend_np.py:186-201``, ``yastn/tensor/_initialize.py:328-336``).
    """
    trace = trace or load_trace('cfg1')
    rng = np.random.default_rng(trace['seed'])
    A = rng.normal(size=trace['A_size'])
    B = rng.normal(size=trace['B_size'])
    return A, B


def cfg3_inputs(trace=None):
    """Data of the U(1)xU(1) complex128 tensors: real and imaginary parts N(0,1) from
    ``default_rng(seed)``, A's real part, A's imaginary part, then B's."""
    trace = trace or load_trace('cfg3')
    rng = np.random.default_rng(trace['seed'])
    A = rng.normal(size=trace['A_size']) + 1j * rng.normal(size=trace['A_size'])
    B = rng.normal(size=trace['B_size']) + 1j * rng.normal(size=trace['B_size'])
    return A, B


def cfg5_inputs(trace=None):
    """Data of the precision-study tensors (U(1), D=128 per leg over t=-16..16).

    Normal draws as ``cfg1_inputs`` (A then B from ``default_rng(seed)``), then every block
    multiplied by its recorded scale 10^u, u ~ U(-4, 0) (block order, A's blocks first).
    """
    trace = trace or load_trace('cfg5')
    rng = np.random.default_rng(trace['seed'])
    A = rng.normal(size=trace['A_size'])
    B = rng.normal(size=trace['B_size'])
    for X, sls, scs in ((A, trace['A_slices'], trace['A_scales']), (B, trace['B_slices'], trace['B_scales'])):
        for (lo, hi), f in zip(sls, scs):
            X[lo:hi] *= f
    return A, B


def meta_mask(struct_t, struct_D, slices, mask_D, axis, nsym=1):
    """Metadata of ``apply_mask`` for a non-diagonal tensor.

    Restates ``yastn/tensor/_merging.py:554-583`` for ``a_isdiag=False``: blocks whose
    charge on ``axis`` has a non-empty mask are kept, their ``axis`` dimension becomes
    the mask length, and the new blocks are laid out contiguously in order.
    ``mask_D`` maps a leg charge (tuple) to the number of kept indices.
    Returns ``(meta, new_t, new_D, new_slices, size)``.
    """
    keep = {t: d for t, d in mask_D.items() if d > 0}
    meta, new_t, new_D, new_sl, low = [], [], [], [], 0
    for t, D, sl in zip(struct_t, struct_D, slices):
        tm = tuple(t[axis * nsym:(axis + 1) * nsym])
        if tm not in keep:
            continue
        Dn = tuple(D[:axis]) + (keep[tm],) + tuple(D[axis + 1:])
        n = int(np.prod(Dn, dtype=np.int64))
        meta.append(((low, low + n), Dn, tuple(sl), tuple(D), tm))
        new_t.append(tuple(t)); new_D.append(Dn); new_sl.append((low, low + n))
        low += n
    return tuple(meta), tuple(new_t), tuple(new_D), tuple(new_sl), low


def meta_mask_diag(struct_t, slices, mask_D, nsym=1):
    """``_meta_mask`` for a diagonal tensor (``_merging.py:554-583``, ``a_isdiag=True``)."""
    keep = {t: d for t, d in mask_D.items() if d > 0}
    meta, low = [], 0
    new_t, new_sl = [], []
    for t, sl in zip(struct_t, slices):
        tm = tuple(t[:nsym])
        if tm not in keep:
            continue
        d = keep[tm]
        meta.append(((low, low + d), d, tuple(sl), sl[1] - sl[0], tm))
        new_t.append(tuple(t)); new_sl.append((low, low + d))
        low += d
    return tuple(meta), tuple(new_t), tuple(new_sl), low


class Heff2Workload:
    """DMRG two-site effective-Hamiltonian matvec replayed from YASTN's recorded calls.

    ``Env.Heff2`` (yastn/tn/mps/_env.py:512-518) for a spin-1/2 XXZ chain with virtual
    legs D=1024 is four tensordots under the fuse_contracted policy; YASTN turns them into
    10 backend calls (4 ``dot`` and 6 ``transpose_and_merge``) whose metadata and dataflow
    (array keys) are stored in the ``cfg2`` fixture. ``matvec(v, dot, merge, scale)``
    replays them with the given backend functions (GPU backend or CPU oracle).
    """

    def __init__(self, trace=None):
        self.tr = trace or load_trace('cfg2')
        rng = np.random.default_rng(self.tr['seed'])
        sizes = {'L': self.tr['L_size'], 'R': self.tr['R_size'], 'AA': self.tr['AA_size']}
        data = {}
        for name in self.tr['order']:  # YASTN draws L, R, AA in this order after random_seed
            data[name] = rng.normal(size=sizes[name])
        data['W1'] = np.array(self.tr['W1'])
        data['W2'] = np.array(self.tr['W2'])
        self.data = data
        self.keys = self.tr['inputs']  # tensor name -> array key of the recorded calls
        self.calls = self.tr['calls']
        self.factor = self.tr['factor']
        from . import _plans as P
        self.flops = sum(P.dot_plan(c['args'][2]).flops for c in self.calls if c['fn'] == 'dot')
        # dataflow: per call, the array keys of its inputs (None for metadata) and of its output
        self.steps = []
        for c in self.calls:
            keys = [a.key if isinstance(a, ArraySpec) else (_key_of(self.tr, a) if isinstance(a, np.ndarray) else None)
                    for a in c['args']]
            o = c['out'][0]
            self.steps.append((c['fn'], keys, c['args'], o.key if isinstance(o, ArraySpec) else _key_of(self.tr, o)))

    def matvec(self, v, env, dot, merge, scale):
        """Heff2 applied to ``v``; ``env`` maps the fixed operands' keys to backend arrays."""
        vals = dict(env)
        vals[self.keys['AA']] = v
        out = None
        for fn, keys, args, okey in self.steps:
            a = [vals[k] if k is not None else x for k, x in zip(keys, args)]
            if fn == 'dot':
                out = dot(a[0], a[1], a[2], a[3])
            elif fn == 'transpose_and_merge':
                out = merge(a[0], a[1], a[2], a[3], a[4])
            else:
                raise ValueError(fn)
            vals[okey] = out
        return scale(out, self.factor)

    def env(self, convert):
        """The fixed operands (L, R, W1, W2) converted by ``convert`` and keyed as in the calls."""
        return {self.keys[n]: convert(self.data[n]) for n in ('L', 'R', 'W1', 'W2')}


def _key_of(trace, arr):
    """Key of a small stored array (stored arrays are deduplicated by content)."""
    for k, v in trace['_arrays'].items():
        if v.shape == arr.shape and v.dtype == arr.dtype and np.array_equal(v, arr):
            return k
    raise KeyError("array not in the trace")


def lanczos(matvec, v0, ncv, vdot, norm):
    """Hermitian Krylov expansion of YASTN's ``eigs`` (yastn/krylov/_krylov.py:177-238 with
    yastn/tensor/_krylov.py:17-46): three-term Lanczos without restarts or breakdown checks
    inside the loop. Works on numpy or torch vectors (``vdot``/``norm`` return scalars of
    the same library, so a torch run stays on the device). Returns (V, alphas, betas)."""
    V = [v0 / norm(v0)]
    alphas, betas = [], []
    for j in range(ncv):
        w = matvec(V[-1])
        a = vdot(V[j], w)
        if j == 0:
            w = w - a * V[j]
        else:
            w = w - betas[-1] * V[j - 1] - a * V[j]
        b = norm(w)
        alphas.append(a)
        betas.append(b)
        V.append(w / b)
    return V, alphas, betas


def ritz_lowest(alphas, betas):
    """Lowest eigenvalue/vector of the Lanczos tridiagonal matrix (host, 'SR' ordering)."""
    import scipy.linalg
    a = np.array([float(x) for x in alphas])
    b = np.array([float(x) for x in betas[:-1]])
    w, v = scipy.linalg.eigh_tridiagonal(a, b)
    i = int(np.argmin(w))
    return float(w[i]), v[:, i]
