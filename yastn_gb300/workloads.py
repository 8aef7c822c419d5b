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
