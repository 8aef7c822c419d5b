"""Generate golden fixtures from the unmodified reference (YASTN, NumPy backend).

Run in a container that has the reference source tree:

    python tests/golden/make_golden.py [/path/to/yastn/source]

It imports YASTN from that path, wraps the hot-path functions of the NumPy backend
(``yastn/backend/backend_np.py``) with a recorder, runs scenarios modelled on the
reference's own tests (``tests/tensor/test_tensordot.py``, ``test_svd.py``,
``test_fuse_hard.py``) and the benchmark workload, and writes:

* ``<scenario>.json`` — the ordered list of backend calls with their metadata
  arguments (nested tuples of ints stored as lists) and the names of their array
  arguments / results;
* ``<scenario>.npz`` — the arrays (inputs and reference outputs).

Adjoint fixtures come from the reference's torch backend on CPU
(``yastn/backend/_backend_torch_backwards.py``). Large arrays of the benchmark
workload are not stored; the workload's data is regenerated from its seed and the
fixture keeps only checksums, the full singular-value vector and the truncation
result.

Nothing at run time (tests, bench, smoke) reads the reference tree; only this script does.
"""
import json
import os
import sys
import weakref

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF = sys.argv[1] if len(sys.argv) > 1 else '/root/reference'
sys.path.insert(0, REF)

import yastn  # noqa: E402
import yastn.backend.backend_np as bnp  # noqa: E402

HOT = ['transpose_and_merge', 'unmerge', 'dot', 'transpose_dot_sum', 'svd', 'eigh', 'qr',
       'fix_svd_signs', 'apply_mask', 'embed_mask']


class Recorder:
    """Wraps hot-path functions of a backend module and records every call."""

    def __init__(self, module, store_arrays=True, big=None):
        self.module = module
        self.calls = []
        self.arrays = {}
        self.seen = {}
        self.store_arrays = store_arrays
        self.big = big  # arrays with more elements than this are summarised
        self.orig = {nm: getattr(module, nm) for nm in HOT}
        for nm in HOT:
            setattr(module, nm, self._wrap(nm, self.orig[nm]))

    def restore(self):
        for nm, f in self.orig.items():
            setattr(self.module, nm, f)

    def _put(self, arr):
        import hashlib
        digest = hashlib.sha1(np.ascontiguousarray(arr).tobytes() + str(arr.dtype).encode()).hexdigest()
        if digest in self.seen:  # identical array already stored: reuse its key
            return dict(self.seen[digest])
        key = f"a{len(self.arrays)}"
        arr = np.array(arr, copy=True)
        self.seen[digest] = self._put_new(key, arr)
        return dict(self.seen[digest])

    def _put_new(self, key, arr):
        if self.big is not None and arr.size > self.big:
            self.arrays[key] = None
            return {'__array__': key, 'shape': list(arr.shape), 'dtype': str(arr.dtype),
                    'checksum': checksum(arr)}
        self.arrays[key] = arr
        return {'__array__': key}

    def _enc(self, x):
        if isinstance(x, np.ndarray):
            return self._put(x)
        if isinstance(x, dict):
            return {'__mask__': [[list(k), self._enc(np.asarray(v))] for k, v in x.items()]}
        if isinstance(x, (tuple, list)):
            return [self._enc(y) for y in x]
        if isinstance(x, (np.integer,)):
            return int(x)
        if isinstance(x, (np.floating,)):
            return float(x)
        return x

    def _wrap(self, nm, f):
        def wrapped(*args, **kwargs):
            enc_args = [self._enc(a) for a in args]
            out = f(*args, **kwargs)
            outs = out if isinstance(out, tuple) else (out,)
            enc_out = [self._enc(o) for o in outs]
            self.calls.append({'fn': nm, 'args': enc_args, 'kwargs': {k: self._enc(v) for k, v in kwargs.items()},
                               'out': enc_out})
            return out
        return wrapped


def checksum(arr):
    a = np.asarray(arr).ravel()
    if np.iscomplexobj(a):
        parts = [a.real, a.imag]
    else:
        parts = [a.astype(np.float64)]
    res = {'n': int(a.size)}
    for i, p in enumerate(parts):
        res[f'sum{i}'] = float(np.sum(p))
        res[f'abs{i}'] = float(np.sum(np.abs(p)))
        res[f'sq{i}'] = float(np.sum(p * p))
        res[f'head{i}'] = [float(x) for x in p[:8]]
        res[f'tail{i}'] = [float(x) for x in p[-8:]]
    return res


def save(name, rec, extra=None):
    payload = {'scenario': name, 'calls': rec.calls}
    if extra:
        payload.update(extra)
    with open(os.path.join(HERE, name + '.json'), 'w') as f:
        json.dump(payload, f, separators=(',', ':'))
    arrays = {k: v for k, v in rec.arrays.items() if v is not None}
    np.savez_compressed(os.path.join(HERE, name + '.npz'), **arrays)
    print(f"{name}: {len(rec.calls)} calls, {sum(v.size for v in arrays.values())} stored elements")


def leg_dims(ts, w, Dtot):
    """Sector dims proportional to w(t), rounded to sum to Dtot (largest-remainder repair)."""
    p = np.array([w(t) for t in ts]); p = p / p.sum()
    D = np.round(p * Dtot).astype(int)
    while D.sum() > Dtot:
        D[np.argmax(D - p * Dtot)] -= 1
    while D.sum() < Dtot:
        D[np.argmin(D - p * Dtot)] += 1
    return tuple(int(x) for x in D)


# ----------------------------------------------------------------------------- scenarios

def scen_tensordot(policy):
    cfg = yastn.make_config(sym='U1', backend='np', tensordot_policy=policy)
    cfgz = yastn.make_config(sym=yastn.sym.sym_Z2xU1, backend='np', tensordot_policy=policy)
    cfgd = yastn.make_config(sym='none', backend='np', tensordot_policy=policy)
    bnp.random_seed(11)
    a = yastn.rand(config=cfg, s=(-1, 1, 1, -1), t=((-1, 1, 2),) * 4,
                   D=((1, 2, 3), (4, 2, 3), (3, 1, 2), (5, 4, 2)))
    b = yastn.rand(config=cfg, s=(1, -1, 1), t=((-1, 1, 2), (-1, 1, 2), (-1, 0, 1)),
                   D=((1, 2, 3), (4, 2, 3), (5, 3, 4)))
    rec = Recorder(bnp)
    yastn.tensordot(a, b, axes=((0, 1), (0, 1)))
    yastn.tensordot(a, b, axes=((1, 3), (1, 2)))
    yastn.tensordot(a, b, axes=((1, 0), (1, 0)), conj=(1, 1))
    yastn.tensordot(b, a, axes=((1, 0), (1, 0)))
    t1 = [(0, -1), (0, 1), (1, -1), (1, 1)]
    t2 = [(0, 0), (0, 2), (1, 0), (1, 2)]
    for dtype in ('float64', 'complex128'):
        az = yastn.rand(config=cfgz, s=(-1, 1, 1, -1), t=(t1, t1, t1, t1),
                        D=((1, 2, 2, 4), (5, 4, 3, 2), (3, 2, 4, 1), (2, 3, 1, 2)), dtype=dtype)
        bz = yastn.rand(config=cfgz, s=(1, -1, 1), t=(t1, t1, t2),
                        D=((1, 2, 2, 4), (5, 4, 3, 2), (3, 2, 4, 1)), dtype=dtype)
        yastn.tensordot(az, bz, axes=((0, 1), (0, 1)))
        yastn.tensordot(bz, az, axes=((1, 0), (1, 0)))
    ad = yastn.rand(config=cfgd, s=(-1, 1, 1, -1), D=(2, 3, 4, 5), dtype='complex128')
    bd = yastn.rand(config=cfgd, s=(1, -1, 1), D=(2, 3, 5), dtype='complex128')
    yastn.tensordot(ad, bd, axes=((0, 3), (0, 2)))
    # hard-fused legs: merges of blocks whose legs carry a fusion history
    D1, D2 = (1, 3, 2), (3, 3, 4)
    tt1, tt2 = (-1, 0, 1), (-2, 0, 2)
    ah = yastn.rand(config=cfg, s=(-1, 1, 1, -1), t=(tt1, tt1, tt2, tt2), D=(D1, D2, D2, D1))
    bh = yastn.rand(config=cfg, s=(-1, -1, 1, 1), t=(tt1, tt2, tt1, tt2), D=(D2, D1, D1, D1))
    ahf = ah.fuse_legs(axes=(0, (1, 3), 2), mode='hard')
    bhf = bh.fuse_legs(axes=((0, 3), 1, 2), mode='hard')
    yastn.tensordot(ahf, bhf, axes=((1,), (0,)))
    rec.restore()
    save(f'tensordot_{policy}', rec)


def scen_svd():
    cfg = yastn.make_config(sym='U1', backend='np')
    bnp.random_seed(12)
    legs = [yastn.Leg(cfg, s=-1, t=(-1, 0, 1), D=(2, 3, 2)),
            yastn.Leg(cfg, s=-1, t=(-2, 0, 2), D=(3, 2, 4)),
            yastn.Leg(cfg, s=1, t=(-2, -1, 0, 1, 2), D=(3, 2, 4, 3, 2)),
            yastn.Leg(cfg, s=1, t=(0, 1), D=(2, 3))]
    rec = Recorder(bnp)
    for dtype in ('float64', 'complex128'):
        a = yastn.rand(config=cfg, n=1, legs=legs, dtype=dtype)
        yastn.linalg.svd(a, axes=((3, 1), (2, 0)), sU=-1)
        yastn.linalg.svd(a, axes=((3, 1), (2, 0)), sU=1, nU=False, fix_signs=True)
        yastn.linalg.svd_with_truncation(a, axes=((0, 1), (2, 3)), D_total=20, tol=1e-3)
    # tall, wide and square blocks in one tensor
    a = yastn.rand(config=cfg, s=(-1, 1), t=((-1, 0, 1), (-1, 0, 1)), D=((30, 7, 5), (4, 7, 40)))
    yastn.linalg.svd(a, axes=(0, 1), fix_signs=True)
    rec.restore()
    save('svd', rec)


def _tup(x):
    return tuple(_tup(y) for y in x) if isinstance(x, list) else x


def scen_qr():
    """yastn.linalg.qr (linalg.py:738-828; backend_np.py:511-520, positive diagonal of R) on
    U(1) tensors with tall, square and wide blocks, float64 and complex128, including a
    rank-deficient block; and the adjoints from the torch backend on CPU (backend_torch.py:
    475-484: torch.linalg.qr + the sign fix, differentiated by torch; complex gradients in
    torch's convention)."""
    import torch
    import yastn.backend.backend_torch as bt
    cfg = yastn.make_config(sym='U1', backend='np')
    bnp.random_seed(17)
    rec = Recorder(bnp)
    for dtype in ('float64', 'complex128'):
        a = yastn.rand(config=cfg, s=(-1, 1), t=((-1, 0, 1), (-1, 0, 1)), D=((30, 7, 5), (4, 7, 40)), dtype=dtype)
        yastn.linalg.qr(a, axes=(0, 1))
        b = yastn.rand(config=cfg, s=(-1, -1, 1), t=((0, 1), (0, 1), (0, 1, 2)), D=((3, 4), (2, 5), (6, 9, 2)),
                       dtype=dtype)
        yastn.linalg.qr(b, axes=((0, 1), 2))
    # a rank-deficient block: two equal columns
    c = yastn.rand(config=cfg, s=(-1, 1), t=((0,), (0,)), D=((9,), (6,)))
    blk = c[(0, 0)]
    blk[:, 3] = blk[:, 1]
    yastn.linalg.qr(c, axes=(0, 1))
    rec.restore()
    # adjoints through the reference's torch backend
    g = torch.Generator().manual_seed(5)
    for call in rec.calls:
        if call['fn'] != 'qr':
            continue
        data = rec.arrays[call['args'][0]['__array__']]
        meta = _tup(call['args'][1])
        sizes = tuple(call['args'][2])
        d_ = torch.from_numpy(data.copy()).requires_grad_(True)
        Q, R = bt.qr(d_, meta, sizes)
        dt = torch.complex128 if np.iscomplexobj(data) else torch.float64
        gQ = torch.randn(sizes[0], dtype=dt, generator=g)
        gR = torch.randn(sizes[1], dtype=dt, generator=g)
        (grad,) = torch.autograd.grad((Q, R), (d_,), grad_outputs=(gQ, gR))
        call['adjoint'] = {'gQ': rec._put(gQ.numpy()), 'gR': rec._put(gR.numpy()), 'grad': rec._put(grad.numpy())}
    save('qr', rec)


def scen_fix_signs():
    """test_svd.py:159-186: phases of U columns, complex blocks."""
    cfg = yastn.make_config(sym='U1', backend='np')
    U = yastn.Tensor(config=cfg, s=(-1, 1), dtype='complex128')
    S = yastn.Tensor(config=cfg, s=(-1, 1), isdiag=True)
    V = yastn.Tensor(config=cfg, s=(-1, 1), dtype='complex128')
    is2 = 0.5 ** 0.5
    U.set_block(ts=(0, 0), Ds=(3, 2), val=[[-is2, -1 / 2], [is2, -1 / 2], [0, is2 * 1j]])
    U.set_block(ts=(1, 1), Ds=(2, 2), val=[[0, 1j], [1, 0]])
    S.set_block(ts=(0, 0), Ds=(2, 2), val=[0.5, 0.2])
    S.set_block(ts=(1, 1), Ds=(2, 2), val=[0.3, 0.2])
    V.set_block(ts=(0, 0), Ds=(2, 2), val=[[0, 1], [1, 0]])
    V.set_block(ts=(1, 1), Ds=(2, 3), val=[[1, 0, 0], [0, 0.8j, 0.6]])
    USV = U @ S @ V
    rec = Recorder(bnp)
    nU, nS, nV = yastn.svd(USV, axis=(0, 1), fix_signs=True)
    rec.restore()
    extra = {'Ufixed': {'(0,0)': [[is2, 0, 0, 0.5], [-is2, 0, 0, 0.5], [0, 0, is2, 0]],
                        '(1,1)': [[0, 0, 1, 0], [1, 0, 0, 0]]}}
    save('fix_signs', rec, extra)


def scen_fix_signs_adjoint():
    """Adjoint of fix_svd_signs through the reference torch backend on CPU
    (backend_torch.py:353-366, differentiated by torch): U and Vh from the thin SVD of random
    blocks (square, tall, wide; float64 and complex128, where the phase of each column's
    largest entry carries a gradient), random cotangents of the fixed U and Vh, and the
    gradients with respect to the unfixed U and Vh (torch's convention for complex tensors)."""
    import torch
    import yastn.backend.backend_torch as bt
    g = torch.Generator().manual_seed(9)
    arrays, calls = {}, []

    def put(x):
        key = f"a{len(arrays)}"
        arrays[key] = x.detach().resolve_conj().cpu().numpy().copy()
        return key

    for dtype in (torch.float64, torch.complex128):
        shapes = [(6, 6), (9, 4), (3, 8)]
        meta, offU, offS, offV = [], 0, 0, 0
        Us, Vs = [], []
        for m, n in shapes:
            k = min(m, n)
            u, _, vh = torch.linalg.svd(torch.randn(m, n, dtype=dtype, generator=g), full_matrices=False)
            Us.append(u.reshape(-1)); Vs.append(vh.reshape(-1))
            meta.append(((0, 0), (m, n), (offU, offU + m * k), (m, k), (offS, offS + k), (offV, offV + k * n), (k, n)))
            offU += m * k; offS += k; offV += k * n
        meta = tuple(meta)
        U = torch.cat(Us).requires_grad_(True)
        V = torch.cat(Vs).requires_grad_(True)
        Uf, Vf = bt.fix_svd_signs(U, V, meta)
        gU = torch.randn(offU, dtype=dtype, generator=g)
        gV = torch.randn(offV, dtype=dtype, generator=g)
        dU, dV = torch.autograd.grad((Uf, Vf), (U, V), grad_outputs=(gU, gV))
        calls.append({'fn': 'fix_svd_signs_backward', 'meta': [list(map(list, r)) for r in meta], 'U': put(U),
                      'V': put(V), 'Uf': put(Uf), 'Vf': put(Vf), 'gU': put(gU), 'gV': put(gV), 'dU': put(dU),
                      'dV': put(dV)})
    with open(os.path.join(HERE, 'fix_signs_adjoint.json'), 'w') as f:
        json.dump({'scenario': 'fix_signs_adjoint', 'calls': calls}, f, separators=(',', ':'))
    np.savez_compressed(os.path.join(HERE, 'fix_signs_adjoint.npz'), **arrays)
    print(f"fix_signs_adjoint: {len(calls)} cases")


def scen_truncation():
    """Spectra and options of test_svd.py:189-266 and :344-388 with the reference's masks."""
    out = []
    cfg = yastn.make_config(sym='U1', backend='np')
    bnp.random_seed(0)
    legs = [yastn.Leg(cfg, s=1, t=(0, 1), D=(5, 6)),
            yastn.Leg(cfg, s=1, t=(-1, 0), D=(5, 6)),
            yastn.Leg(cfg, s=-1, t=(-1, 0, 1), D=(2, 3, 4)),
            yastn.Leg(cfg, s=-1, t=(-1, 0, 1), D=(2, 3, 4))]
    a = yastn.rand(config=cfg, n=1, legs=legs)
    U, S, V = yastn.linalg.svd(a, axes=((0, 1), (2, 3)), sU=-1)
    S.set_block(ts=(-2, -2), Ds=4, val=[2 ** (-ii - 6) for ii in range(4)])
    S.set_block(ts=(-1, -1), Ds=12, val=[2 ** (-ii - 2) for ii in range(12)])
    S.set_block(ts=(0, 0), Ds=25, val=[2 ** (-ii - 1) for ii in range(25)])
    opts_list = [{'tol': 0.01, 'D_block': 100, 'D_total': 12},
                 {'tol': 0.02, 'D_block': 5, 'D_total': 100},
                 {'tol': 0, 'tol_block': 0.2, 'D_total': 100},
                 {'D_block': {(0,): 2, (-1,): 3}, 'tol_block': {(0,): 0.6, (-1,): 0.1}},
                 {'D_total': 10, 'truncate_multiplets': True},
                 {'D_total': 0}]
    for opts in opts_list:
        m = yastn.linalg.truncation_mask(S, **opts)
        out.append(_trunc_case(S, m, opts))
    # multiplets
    bnp.random_seed(0)
    legs = [yastn.Leg(cfg, s=1, t=(-1, 0, 1), D=(2, 3, 2)),
            yastn.Leg(cfg, s=1, t=(-1, 0, 1), D=(3, 4, 3)),
            yastn.Leg(cfg, s=-1, t=(-1, 0, 1), D=(4, 5, 4)),
            yastn.Leg(cfg, s=-1, t=(-1, 0, 1), D=(5, 6, 5))]
    a = yastn.rand(config=cfg, n=0, legs=legs)
    U, S, V = yastn.linalg.svd(a, axes=((0, 1), (2, 3)))
    v00 = [1, 1, 0.1001, 0.1000, 0.1000, 0.0999, 0.001001, 0.001000] + [0] * 16
    S.set_block(ts=(0, 0), Ds=24, val=v00)
    v11 = [1, 1, 0.1001, 0.1000, 0.0999, 0.001000, 0.000999] + [0] * 10
    S.set_block(ts=(1, 1), Ds=17, val=v11)
    S.set_block(ts=(-1, -1), Ds=17, val=v11)
    v22 = [1, 1, 0.1001, 0.1000, 0.001000, 0]
    S.set_block(ts=(2, 2), Ds=6, val=v22)
    S.set_block(ts=(-2, -2), Ds=6, val=v22)
    for opts in [{'tol': 0.0001, 'D_block': 7, 'D_total': 30},
                 {'tol': 0.001, 'truncate_multiplets': True},
                 {'D_total': 17, 'truncate_multiplets': True}]:
        m = yastn.linalg.truncation_mask(S, **opts)
        out.append(_trunc_case(S, m, opts))
    # random spectra with many blocks
    rng = np.random.default_rng(5)
    for trial in range(4):
        nb = 9
        Ds = rng.integers(1, 30, size=nb)
        t = [(int(q),) for q in range(-4, 5)]
        Sx = yastn.Tensor(config=cfg, s=(-1, 1), isdiag=True)
        for tq, d in zip(t, Ds):
            vals = np.sort(np.abs(rng.normal(size=d)) * 10 ** rng.uniform(-6, 0))[::-1]
            Sx.set_block(ts=tq + tq, Ds=int(d), val=vals.tolist())
        opts = [{'tol': 1e-3, 'D_total': 40}, {'D_block': 6, 'D_total': 35},
                {'tol_block': 0.05, 'tol': 1e-4}, {'D_total': 25, 'truncate_multiplets': True}][trial]
        m = yastn.linalg.truncation_mask(Sx, **opts)
        out.append(_trunc_case(Sx, m, opts))
    with open(os.path.join(HERE, 'truncation.json'), 'w') as f:
        json.dump({'scenario': 'truncation', 'cases': out}, f, separators=(',', ':'))
    print(f"truncation: {len(out)} cases")


def _trunc_case(S, mask, opts):
    def enc(v):
        if isinstance(v, dict):
            return {'__dict__': [[list(k), vv] for k, vv in v.items()]}
        return v
    return {'S': [float(x) for x in S._data], 'slices': [list(sl.slcs[0]) for sl in S.slices],
            'charges': [list(t[:1]) for t in S.struct.t],
            'opts': {k: enc(v) for k, v in opts.items()},
            'mask': [bool(x) for x in mask._data]}


def scen_eigh():
    cfg = yastn.make_config(sym='U1', backend='np')
    bnp.random_seed(13)
    rec = Recorder(bnp)
    for dtype in ('float64', 'complex128'):
        a = yastn.rand(config=cfg, s=(1, -1), t=((-1, 0, 1), (-1, 0, 1)), D=((3, 9, 5), (3, 9, 5)), dtype=dtype)
        a = a + a.transpose(axes=(1, 0)).conj()
        yastn.linalg.eigh(a, axes=(0, 1))
    rec.restore()
    save('eigh', rec)


def scen_adjoints():
    """Reference adjoints from the torch backend on CPU (_backend_torch_backwards.py)."""
    import torch
    import yastn.backend.backend_torch as bt
    from yastn.backend._backend_torch_backwards import (kernel_svd, kernel_dot,
                                                         kernel_transpose_and_merge, kernel_unmerge,
                                                         kernel_apply_mask)
    arrays, calls = {}, []

    def put(x):
        key = f"a{len(arrays)}"
        arrays[key] = x.detach().resolve_conj().cpu().numpy().copy() if isinstance(x, torch.Tensor) else np.asarray(x)
        return key

    g = torch.Generator().manual_seed(7)
    # SVD adjoint on blocks: square, tall, wide; real and complex
    for dtype in (torch.float64, torch.complex128):
        shapes = [(6, 6), (9, 4), (3, 8)]
        meta, off, offU, offS, offV = [], 0, 0, 0, 0
        for (m, n) in shapes:
            k = min(m, n)
            meta.append(((off, off + m * n), (m, n), (offU, offU + m * k), (m, k), (offS, offS + k),
                         (offV, offV + k * n), (k, n)))
            off += m * n; offU += m * k; offS += k; offV += k * n
        data = torch.randn(off, dtype=dtype, generator=g)
        U, S, V = kernel_svd.apply(data, tuple(meta), (offU, offS, offV))
        gU = torch.randn(offU, dtype=dtype, generator=g)
        gS = torch.randn(offS, dtype=torch.float64, generator=g)
        gV = torch.randn(offV, dtype=dtype, generator=g)
        d = data.clone().requires_grad_(True)
        U2, S2, V2 = kernel_svd.apply(d, tuple(meta), (offU, offS, offV))
        # the cotangents handed to kernel_svd.backward are exactly (gU, gS, gV)
        (grad,) = torch.autograd.grad((U2, S2, V2), (d,), grad_outputs=(gU, gS, gV))
        calls.append({'fn': 'svd_backward', 'meta': meta, 'data': put(data), 'U': put(U), 'S': put(S),
                      'V': put(V), 'gU': put(gU), 'gS': put(gS), 'gV': put(gV), 'grad': put(grad)})
    # dot adjoint with shared operand blocks (fuse_contracted style)
    cfg = yastn.make_config(sym='U1', backend='np', tensordot_policy='fuse_contracted')
    bnp.random_seed(14)
    a = yastn.rand(config=cfg, s=(-1, 1, 1), t=((-1, 0, 1),) * 3, D=((2, 3, 2), (4, 5, 4), (3, 3, 2)))
    b = yastn.rand(config=cfg, s=(-1, 1, 1), t=((-1, 0, 1),) * 3, D=((3, 3, 2), (2, 6, 2), (5, 1, 4)))
    rec = Recorder(bnp)
    yastn.tensordot(a, b, axes=((2,), (0,)))
    rec.restore()
    dcall = [c for c in rec.calls if c['fn'] == 'dot'][0]
    A = torch.from_numpy(rec.arrays[dcall['args'][0]['__array__']]).requires_grad_(True)
    B = torch.from_numpy(rec.arrays[dcall['args'][1]['__array__']]).requires_grad_(True)
    meta_dot = _tup(dcall['args'][2])
    C = kernel_dot.apply(A, B, meta_dot, dcall['args'][3])
    Cb = torch.randn(C.shape, dtype=C.dtype, generator=g)
    C.backward(Cb)
    calls.append({'fn': 'dot_backward', 'meta': dcall['args'][2], 'A': put(A), 'B': put(B), 'Cb': put(Cb),
                  'Ab': put(A.grad), 'Bb': put(B.grad)})
    # merge / unmerge adjoints with a permutation
    cfg = yastn.make_config(sym='U1', backend='np', tensordot_policy='fuse_to_matrix')
    bnp.random_seed(15)
    a = yastn.rand(config=cfg, s=(-1, 1, 1, -1), t=((-1, 1, 2),) * 4, D=((1, 2, 3), (2, 3, 2), (3, 2, 1), (3, 4, 1)))
    b = yastn.rand(config=cfg, s=(1, -1, 1), t=((-1, 1, 2), (-1, 1, 2), (-1, 0, 1)), D=((1, 2, 3), (2, 3, 2), (3, 2, 4)))
    rec = Recorder(bnp)
    yastn.tensordot(a, b, axes=((1, 3), (1, 2)))
    rec.restore()
    mcall = [c for c in rec.calls if c['fn'] == 'transpose_and_merge'][0]
    data = torch.from_numpy(rec.arrays[mcall['args'][0]['__array__']]).requires_grad_(True)
    order, mnew, mmrg, Dsize = (_tup(x) for x in mcall['args'][1:])
    out = kernel_transpose_and_merge.apply(data, order, mnew, mmrg, Dsize)
    ob = torch.randn(out.shape, dtype=out.dtype, generator=g)
    out.backward(ob)
    calls.append({'fn': 'transpose_and_merge_backward', 'order': mcall['args'][1], 'meta_new': mcall['args'][2],
                  'meta_mrg': mcall['args'][3], 'Dsize': Dsize, 'data': put(data), 'out_b': put(ob),
                  'grad': put(data.grad)})
    ucall = [c for c in rec.calls if c['fn'] == 'unmerge'][0]
    data = torch.from_numpy(rec.arrays[ucall['args'][0]['__array__']]).requires_grad_(True)
    meta = _tup(ucall['args'][1])
    out = kernel_unmerge.apply(data, meta)
    ob = torch.randn(out.shape, dtype=out.dtype, generator=g)
    out.backward(ob)
    calls.append({'fn': 'unmerge_backward', 'meta': ucall['args'][1], 'data': put(data), 'out_b': put(ob),
                  'grad': put(data.grad)})
    with open(os.path.join(HERE, 'adjoints.json'), 'w') as f:
        json.dump({'scenario': 'adjoints', 'calls': calls}, f, separators=(',', ':'))
    np.savez_compressed(os.path.join(HERE, 'adjoints.npz'), **arrays)
    print(f"adjoints: {len(calls)} calls")


def scen_eigh_adjoint():
    """Reference eigh adjoints from the torch backend on CPU (backend_torch.py:369-384):
    order_by_magnitude=True goes through SYMEIG (torch_eig_sym.py:43-54, broadened F,
    ad_decomp_reg=1e-12), False through torch.linalg.eigh's own adjoint. Blocks of 5, 8, 3
    (one with a degenerate pair); real symmetric for both modes, complex Hermitian for the
    torch.linalg.eigh mode with a cotangent whose diag(U^H gU) is real (gauge invariant)."""
    import torch
    import yastn.backend.backend_torch as bt
    g = torch.Generator().manual_seed(21)
    arrays, calls = {}, []

    def put(x):
        key = f"a{len(arrays)}"
        arrays[key] = x.detach().resolve_conj().cpu().numpy().copy()
        return key

    for dtype, by_mag in ((torch.float64, True), (torch.float64, False), (torch.complex128, False)):
        sizes_ = [5, 8, 3]
        meta, off, offU, offS, parts = [], 0, 0, 0, []
        for i, d in enumerate(sizes_):
            a = torch.randn(d, d, dtype=dtype, generator=g)
            h = a + a.mH
            if i == 1:  # a degenerate pair: eigenvalues (1, 1, ...) in a random basis
                q, _ = torch.linalg.qr(torch.randn(d, d, dtype=dtype, generator=g))
                ev = torch.linspace(-3, 4, d, dtype=torch.float64)
                ev[2] = ev[3]
                h = (q * ev.to(dtype)) @ q.mH
            parts.append(h.reshape(-1))
            meta.append(((off, off + d * d), (d, d), (offU, offU + d * d), (d, d), (offS, offS + d)))
            off += d * d; offU += d * d; offS += d
        data = torch.cat(parts)
        d_ = data.clone().requires_grad_(True)
        S, U = bt.eigh(d_, tuple(meta), (offS, offU), order_by_magnitude=by_mag)
        gS = torch.randn(offS, dtype=torch.float64, generator=g)
        gU = torch.randn(offU, dtype=dtype, generator=g)
        if dtype.is_complex:  # remove the gauge-dependent part: diag(U^H gU) real
            for sl, D, slU, DU, slS in meta:
                u = U[slice(*slU)].detach().view(DU)
                gu = gU[slice(*slU)].view(DU)
                x = torch.diagonal(u.mH @ gu)
                gu -= u * (1j * x.imag)
        (grad,) = torch.autograd.grad((S, U), (d_,), grad_outputs=(gS, gU))
        calls.append({'fn': 'eigh_backward', 'order_by_magnitude': by_mag, 'meta': meta, 'data': put(data),
                      'S': put(S), 'U': put(U), 'gS': put(gS), 'gU': put(gU), 'grad': put(grad)})
    with open(os.path.join(HERE, 'eigh_adjoint.json'), 'w') as f:
        json.dump({'scenario': 'eigh_adjoint', 'calls': calls}, f, separators=(',', ':'))
    np.savez_compressed(os.path.join(HERE, 'eigh_adjoint.npz'), **arrays)
    print(f"eigh_adjoint: {len(calls)} calls")


def scen_svd_ill():
    """The ill-conditioned fixture of the reference tests (test_svd.py:335-341), where
    LAPACK gesdd can fail; records the backend calls of its truncated SVD."""
    cfg = yastn.make_config(sym='U1', backend='np')
    fname = os.path.join(REF, 'tests', 'tensor', 'inputs', 'ill_conditioned_svd.npy')
    tensor_dict = np.load(fname, allow_pickle=True).item()
    tensor = yastn.from_dict(tensor_dict, cfg)
    rec = Recorder(bnp)
    yastn.svd_with_truncation(tensor, axes=((0, 1), (2, 3)), D_total=12)
    rec.restore()
    save('svd_ill', rec)


def scen_tds_adjoint():
    """transpose_dot_sum adjoint from the reference torch backend (:170-226)."""
    import torch
    from yastn.backend._backend_torch_backwards import kernel_transpose_dot_sum
    tr_calls = []
    cfg = yastn.make_config(sym='U1', backend='np', tensordot_policy='no_fusion')
    bnp.random_seed(16)
    a = yastn.rand(config=cfg, s=(-1, 1, 1, -1), t=((-1, 1, 2),) * 4, D=((1, 2, 3), (2, 3, 2), (3, 2, 1), (3, 4, 1)))
    b = yastn.rand(config=cfg, s=(1, -1, 1), t=((-1, 1, 2), (-1, 1, 2), (-1, 0, 1)), D=((1, 2, 3), (2, 3, 2), (3, 2, 4)))
    rec = Recorder(bnp)
    yastn.tensordot(a, b, axes=((1, 3), (1, 2)))
    rec.restore()
    c = [c for c in rec.calls if c['fn'] == 'transpose_dot_sum'][0]
    A = torch.from_numpy(rec.arrays[c['args'][0]['__array__']]).requires_grad_(True)
    B = torch.from_numpy(rec.arrays[c['args'][1]['__array__']]).requires_grad_(True)
    rest = [_tup(x) for x in c['args'][2:]]
    C = kernel_transpose_dot_sum.apply(A, B, *rest)
    g = torch.Generator().manual_seed(8)
    Cb = torch.randn(C.shape, dtype=C.dtype, generator=g)
    C.backward(Cb)
    arrays = {'A': A.detach().numpy(), 'B': B.detach().numpy(), 'Cb': Cb.numpy(), 'Ab': A.grad.numpy(),
              'Bb': B.grad.numpy()}
    with open(os.path.join(HERE, 'tds_adjoint.json'), 'w') as f:
        json.dump({'scenario': 'tds_adjoint', 'args': c['args'][2:]}, f, separators=(',', ':'))
    np.savez_compressed(os.path.join(HERE, 'tds_adjoint.npz'), **arrays)
    print("tds_adjoint: 1 call")


def scen_cfg2():
    """DMRG two-site effective-Hamiltonian matvec (``Env.Heff2``, yastn/tn/mps/_env.py:512-518)
    for a spin-1/2 XXZ chain (Jz = Jxy = 1, MPO bond 5), virtual legs D=1024 over U(1)
    charges -12..12 with dims ~ exp(-t^2/18) (empty sectors dropped), L, R, AA drawn with
    rand(normal) after random_seed(0), fuse_contracted policy. Records the 10 backend calls
    of one matvec (their array keys give the dataflow), the MPO blocks, and the lowest
    Ritz value of the reference's eigs(ncv=30, which='SR', hermitian=True)."""
    import yastn.tn.mps as mps
    ops_ = yastn.operators.Spin12(sym='U1', backend='np')
    N = 4
    gen = mps.Generator(N=N, operators=ops_)
    gen.random_seed(seed=0)
    H = gen.mpo_from_latex(r"\sum_{i,j \in NN} (Jz sz_{i} sz_{j} + 0.5 Jxy (sp_{i} sm_{j} + sm_{i} sp_{j}))",
                           {"Jz": 1.0, "Jxy": 1.0, "NN": [(i, i + 1) for i in range(N - 1)]})
    psi = gen.random_mps(D_total=8)
    env = mps.Env(psi, [H, psi]).setup_(to='first').setup_(to='last')
    L0, R0 = env.F[(0, 1)], env.F[(3, 2)]
    cfg = psi.config
    cfg.backend.random_seed(0)
    ts0 = tuple(range(-12, 13))
    Ds0 = leg_dims(ts0, lambda t: np.exp(-t * t / 18), 1024)
    ts, Ds = zip(*[(t, d) for t, d in zip(ts0, Ds0) if d > 0])
    lL, lR = L0.get_legs(), R0.get_legs()
    vl = lambda sg: yastn.Leg(cfg, s=sg, t=ts, D=Ds)
    L = yastn.rand(cfg, legs=[vl(lL[0].s), lL[1], vl(lL[2].s)], distribution='normal')
    R = yastn.rand(cfg, legs=[vl(lR[0].s), lR[1], vl(lR[2].s)], distribution='normal')
    la = psi.pre_2site((1, 2)).get_legs()
    AA = yastn.rand(cfg, legs=[vl(la[0].s), la[1], la[2], vl(la[3].s)], distribution='normal')
    W1, W2 = H[1], H[2]

    def heff2(v):
        tmp = v @ R
        tmp = yastn.tensordot(W2, tmp, axes=((2, 3), (3, 2)))
        tmp = yastn.tensordot(W1, tmp, axes=((2, 3), (0, 3)))
        tmp = yastn.tensordot(L, tmp, axes=((0, 1), (3, 0)))
        return tmp * H.factor

    rec = Recorder(bnp, big=5000)
    out = heff2(AA)
    rec.restore()
    assert out.struct == AA.struct and out.slices == AA.slices
    val, _ = yastn.eigs(heff2, AA, k=1, ncv=30, which='SR', hermitian=True)
    keys = {}
    for name, t in (('L', L), ('R', R), ('AA', AA), ('W1', W1), ('W2', W2)):
        d = np.ascontiguousarray(t._data)
        import hashlib
        keys[name] = hashlib.sha1(d.tobytes() + str(d.dtype).encode()).hexdigest()
    # map tensor names to the recorder's array keys (content digests)
    name_of = {}
    for dig, ent in rec.seen.items():
        for name, k in keys.items():
            if k == dig:
                name_of[name] = ent['__array__']
    extra = {'seed': 0, 'L_size': int(L.size), 'R_size': int(R.size), 'AA_size': int(AA.size),
             'order': ['L', 'R', 'AA'], 'factor': float(H.factor), 'inputs': name_of,
             'W1': [float(x) for x in W1._data], 'W2': [float(x) for x in W2._data],
             'out_checksum': checksum(out._data), 'lanczos_ncv': 30, 'lanczos_lowest': float(val[0]),
             'leg_t': list(ts), 'leg_D': list(Ds)}
    save('cfg2', rec, extra)


def _tup(x):
    if isinstance(x, list):
        return tuple(_tup(y) for y in x)
    return x


def scen_cfg1():
    """Benchmark workload: U(1) rank-4 D=64 tensordot (2,3)x(0,1) + SVD, D_total=64.

    Sector dims follow exp(-t^2/4) over t=-3..3 rounded to 64; A then B are drawn
    with ``rand(distribution='normal')`` after ``random_seed(0)`` (one normal vector
    of length ``size`` per tensor, in block order).
    """
    cfg = yastn.make_config(sym='U1', backend='np', tensordot_policy='fuse_to_matrix')
    bnp.random_seed(0)
    ts = tuple(range(-3, 4))
    Ds = leg_dims(ts, lambda t: np.exp(-t * t / 4), 64)
    legs = [yastn.Leg(cfg, s=s, t=ts, D=Ds) for s in (1, 1, -1, -1)]
    A = yastn.rand(cfg, legs=legs, distribution='normal')
    B = yastn.rand(cfg, legs=legs, distribution='normal')
    rec = Recorder(bnp, big=5000)
    C = yastn.tensordot(A, B, axes=((2, 3), (0, 1)))
    U, S, V = yastn.svd_with_truncation(C, axes=((0, 1), (2, 3)), D_total=64)
    rec.restore()
    scall = [c for c in rec.calls if c['fn'] == 'svd'][0]
    extra = {'leg_t': list(ts), 'leg_D': list(Ds), 'signatures': [1, 1, -1, -1], 'seed': 0,
             'A_size': int(A.size), 'B_size': int(B.size),
             'A_struct': {'t': [list(t) for t in A.struct.t], 'D': [list(d) for d in A.struct.D]},
             'S_kept_t': [list(t) for t in S.struct.t], 'S_kept_D': [list(d) for d in S.struct.D],
             'S_kept': [float(x) for x in S._data], 'C_checksum': checksum(C._data)}
    # record the full spectrum from the svd call output
    srec = scall['out'][1]
    if rec.arrays.get(srec['__array__']) is not None:
        extra['S_full'] = [float(x) for x in rec.arrays[srec['__array__']]]
    save('cfg1', rec, extra)


def scen_cfg5():
    """Precision-study workload: U(1) rank-4 tensors with D=128 per leg over t=-16..16,
    sector dims ~ exp(-t^2/50) (empty sectors dropped), signatures (1,1,-1,-1), entries
    N(0,1) from rand(normal) after random_seed(0) (A then B), every block then scaled by
    10^u, u ~ U(-4, 0) drawn in block order from default_rng(1) (A's blocks, then B's).
    tensordot(A, B, ((2,3),(0,1))) under fuse_to_matrix: fused sectors up to ~946, sector
    GEMMs up to ~946 x 946 x 946. (Per-leg D=4096 over t=-16..16 would give ~1.1e13 nonzero
    elements; D=128 per leg gives the stated ~900^3 sector GEMMs.)"""
    cfg = yastn.make_config(sym='U1', backend='np', tensordot_policy='fuse_to_matrix')
    bnp.random_seed(0)
    ts0 = tuple(range(-16, 17))
    Ds0 = leg_dims(ts0, lambda t: np.exp(-t * t / 50), 128)
    ts, Ds = zip(*[(t, d) for t, d in zip(ts0, Ds0) if d > 0])
    legs = [yastn.Leg(cfg, s=sg, t=ts, D=Ds) for sg in (1, 1, -1, -1)]
    A = yastn.rand(cfg, legs=legs, distribution='normal')
    B = yastn.rand(cfg, legs=legs, distribution='normal')
    rng = np.random.default_rng(1)
    scales = {}
    for name, T in (('A', A), ('B', B)):
        sc = 10.0 ** rng.uniform(-4, 0, size=len(T.struct.t))
        for sl, f in zip(T.slices, sc):
            T._data[sl.slcs[0][0]:sl.slcs[0][1]] *= f
        scales[name] = [float(x) for x in sc]
    rec = Recorder(bnp, big=5000)
    C = yastn.tensordot(A, B, axes=((2, 3), (0, 1)))
    rec.restore()
    extra = {'leg_t': list(ts), 'leg_D': list(Ds), 'signatures': [1, 1, -1, -1], 'seed': 0, 'scale_seed': 1,
             'A_size': int(A.size), 'B_size': int(B.size),
             'A_slices': [list(x.slcs[0]) for x in A.slices], 'B_slices': [list(x.slcs[0]) for x in B.slices],
             'A_scales': scales['A'], 'B_scales': scales['B'], 'C_checksum': checksum(C._data)}
    save('cfg5', rec, extra)


def cfg3_legs():
    """Charges and sector dims of the U(1)xU(1) complex workload: the 11 (N, Sz) charges of
    smallest |N| + |Sz| (N in -6..6, Sz in -3..3; 11 charges give 595 blocks in the rank-4
    tensor), sector dims drawn from a geometric distribution (p = 0.15) clipped to 1..64
    with default_rng(0). The dims are not rescaled to a leg total of 512: with ~600 blocks
    that would need ~4e9 complex elements (68 GB) per tensor and fused SVD sectors of
    ~33000; the block count and the dim distribution are kept (leg total 116)."""
    charges = sorted(((n, sz) for n in range(-6, 7) for sz in range(-3, 4)),
                     key=lambda c: (abs(c[0]) + abs(c[1]), c))[:11]
    D = np.clip(np.random.default_rng(0).geometric(0.15, size=11), 1, 64)
    order = sorted(range(11), key=lambda i: charges[i])
    return tuple(charges[i] for i in order), tuple(int(D[i]) for i in order)


def scen_cfg3():
    """U(1)xU(1) complex128 workload with many small uneven blocks: rank-4 tensors with the
    legs of cfg3_legs (signatures (1,1,-1,-1), 595 blocks each), real and imaginary parts of
    every entry N(0,1) drawn from default_rng(0) (A: real part, imaginary part; then B);
    tensordot(A, B, ((2,3),(0,1))) under the default policy, then
    svd_with_truncation(C, axes=((0,1),(2,3)), tol=1e-8)."""
    cfg = yastn.make_config(sym='U1xU1', backend='np', default_dtype='complex128')
    ts, Ds = cfg3_legs()
    legs = [yastn.Leg(cfg, s=sg, t=ts, D=Ds) for sg in (1, 1, -1, -1)]
    A = yastn.zeros(cfg, legs=legs, dtype='complex128')
    B = yastn.zeros(cfg, legs=legs, dtype='complex128')
    rng = np.random.default_rng(0)
    for T in (A, B):
        T._data = rng.normal(size=T.size) + 1j * rng.normal(size=T.size)
    rec = Recorder(bnp, big=5000)
    C = yastn.tensordot(A, B, axes=((2, 3), (0, 1)))
    U, S, V = yastn.svd_with_truncation(C, axes=((0, 1), (2, 3)), tol=1e-8)
    rec.restore()
    scall = [c for c in rec.calls if c['fn'] == 'svd'][0]
    extra = {'leg_t': [list(t) for t in ts], 'leg_D': list(Ds), 'signatures': [1, 1, -1, -1], 'seed': 0,
             'n_blocks': len(A.struct.t), 'A_size': int(A.size), 'B_size': int(B.size),
             'C_checksum': checksum(C._data), 'S_kept_t': [list(t) for t in S.struct.t],
             'S_kept_D': [list(d) for d in S.struct.D], 'S_kept_checksum': checksum(S._data),
             'svd_S_checksum': scall['out'][1].get('checksum') if isinstance(scall['out'][1], dict) else None}
    save('cfg3', rec, extra)


class OpRecorder:
    """Records every call into a backend module and the torch operations applied to tensors
    outside those calls (a TorchFunctionMode), as the op list of yastn_gb300.replay: tensors
    become dataflow keys; tensors the sequence never produced become stored constants.
    ``checkpoint`` is transparent: the function it wraps is recorded step by step, between
    markers."""

    def __init__(self, module):
        import torch
        from torch.overrides import TorchFunctionMode
        self.torch = torch
        self.module = module
        self.ops, self.consts, self.keys = [], {}, {}
        self.count = 0
        self.depth = 0
        self.active = False
        self.orig = {}
        rec = self

        class Mode(TorchFunctionMode):
            def __torch_function__(mode, func, types, args=(), kwargs=None):
                kwargs = kwargs or {}
                out = func(*args, **kwargs)
                if rec.active and rec.depth == 0:
                    rec._torch_op(func, args, kwargs, out)
                return out
        self.mode = Mode()
        for nm in module.__all__:
            f = getattr(module, nm)
            if callable(f) and not isinstance(f, type):
                self.orig[nm] = f
                setattr(module, nm, self._wrap(nm, f))

    def restore(self):
        for nm, f in self.orig.items():
            setattr(self.module, nm, f)

    def key(self, t, name=None):
        k = self.keys.get(id(t))
        if k is None:
            self.count += 1
            k = name or f"t{self.count}"
            self.keys[id(t)] = k
            # forget the id when the tensor dies (ids are reused); holding every tensor alive
            # instead does not fit in memory at chi = 144
            weakref.finalize(t, self.keys.pop, id(t), None)
        return k

    def _enc(self, x):
        torch = self.torch
        if isinstance(x, torch.Tensor):
            if id(x) not in self.keys:  # a constant made before recording
                k = self.key(x, f"c{len(self.consts)}")
                self.consts[k] = x.detach().resolve_conj().cpu().numpy().copy()
            return {'__t__': self.keys[id(x)]}
        if isinstance(x, np.ndarray):
            k = f"c{len(self.consts)}"
            self.consts[k] = np.array(x, copy=True)
            return {'__t__': k}
        if isinstance(x, tuple) or isinstance(x, torch.Size):
            return [self._enc(y) for y in x]
        if isinstance(x, list):
            return {'__list__': [self._enc(y) for y in x]}
        if isinstance(x, dict):
            return {'__dict__': [[self._enc(k), self._enc(v)] for k, v in x.items()]}
        if isinstance(x, slice):
            return {'__slice__': [x.start, x.stop, x.step]}
        if isinstance(x, torch.dtype):
            return {'__dtype__': str(x).replace('torch.', '')}
        if isinstance(x, torch.device):
            return {'__device__': 1}
        if x is Ellipsis:
            return {'__ellipsis__': 1}
        if isinstance(x, str) and x == 'cpu':
            return {'__devstr__': 1}
        if isinstance(x, (np.integer,)):
            return int(x)
        if isinstance(x, (np.floating,)):
            return float(x)
        if isinstance(x, (np.bool_,)):
            return bool(x)
        if isinstance(x, (int, float, bool, str)) or x is None:
            return x
        raise TypeError(f"cannot record argument of type {type(x)}")

    def _outs(self, out):
        torch = self.torch
        if isinstance(out, torch.Tensor):
            return self.key(out)
        if isinstance(out, (tuple, list)) and any(isinstance(o, torch.Tensor) for o in out):
            return [self.key(o) if isinstance(o, torch.Tensor) else None for o in out]
        return None

    def _wrap(self, nm, f):
        rec = self

        def wrapped(*args, **kwargs):
            if not rec.active or rec.depth > 0:
                return f(*args, **kwargs)
            if nm == 'checkpoint':  # transparent: record the wrapped function's steps
                fn, fargs = args[0], args[1:]
                rec.ops.append({'k': 'mark', 'fn': 'checkpoint_begin'})
                out = fn(*fargs)
                rec.ops.append({'k': 'mark', 'fn': 'checkpoint_end'})
                return out
            rec.depth += 1
            try:
                a = [rec._enc(x) for x in args]
                kw = {k: rec._enc(v) for k, v in kwargs.items()}
                out = f(*args, **kwargs)
                o = rec._outs(out)
            finally:
                rec.depth -= 1
            rec.ops.append({'k': 'b', 'fn': nm, 'a': a, 'kw': kw, 'o': o})
            return out
        return wrapped

    def _torch_op(self, func, args, kwargs, out):
        torch = self.torch
        name = getattr(func, '__name__', '')
        qual = getattr(func, '__qualname__', '')
        inplace = name == '__setitem__' or (name.endswith('_') and not name.startswith('_'))
        tensor_out = isinstance(out, torch.Tensor) or (isinstance(out, (tuple, list)) and
                                                         any(isinstance(o, torch.Tensor) for o in out))
        if not (tensor_out or inplace):
            return
        self.depth += 1
        try:
            if qual.startswith('getset_descriptor') or type(func).__name__ == 'method-wrapper':
                attr = getattr(getattr(func, '__self__', None), '__name__', None)
                fn = 'a:' + str(attr)
                a = [self._enc(args[0])]
            elif qual.startswith(('TensorBase.', 'Tensor.', '_TensorBase.')):
                fn = 'm:' + name
                a = [self._enc(x) for x in args]
            else:
                fn = 'f:' + name
                a = [self._enc(x) for x in args]
            kw = {k: self._enc(v) for k, v in kwargs.items()}
            o = self._outs(out) if tensor_out else None
        finally:
            self.depth -= 1
        self.ops.append({'k': 't', 'fn': fn, 'a': a, 'kw': kw, 'o': o})

    def __enter__(self):
        self.active = True
        self.mode.__enter__()
        return self

    def __exit__(self, *exc):
        self.mode.__exit__(*exc)
        self.active = False


def scen_ctmrg(chi=24, sweeps=8, name='ctmrg_z2_d6', use_qr=False):
    """Differentiable CTMRG of an iPEPS on a 1x1 unit cell (yastn.tn.fpeps): Z2 symmetry,
    site tensor with bond D=6 (3+3 over parities) and physical d=2 (1+1), rand(normal) after
    random_seed(0); EnvCTM(init='eye'), ctmrg_ with D_total=chi for a fixed number of sweeps
    (moves 'hv', SVD projectors: use_qr=False, checkpoint_move='nonreentrant'); energy of the
    transverse-field Ising model per site E = -h <Z> - sum over the two bonds <X X> with
    h = 3, and its gradient with respect to the site tensor (backward through torch
    autograd of the reference torch backend, on CPU). Records the forward call sequence
    (OpRecorder), the site tensor, E and the gradient."""
    import time
    import torch
    import yastn.tn.fpeps as fpeps
    import yastn.backend.backend_torch as bt
    torch.set_default_dtype(torch.float64)
    cfg = yastn.make_config(sym='Z2', backend=bt, default_dtype='float64')
    cfg.backend.random_seed(0)
    vl = yastn.Leg(cfg, s=1, t=(0, 1), D=(3, 3))
    pl = yastn.Leg(cfg, s=1, t=(0, 1), D=(1, 1))
    A = yastn.rand(cfg, legs=[vl.conj(), vl, vl, vl.conj(), pl], distribution='normal')
    op = yastn.operators.Spin12(sym='Z2', backend=bt, default_dtype='float64')
    Z, X = op.z(), op.x()
    A._data.requires_grad_(True)
    rec = OpRecorder(bt)
    rec.key(A._data, 'in:A')
    t0 = time.time()
    with rec:
        psi = fpeps.Peps(fpeps.SquareLattice(dims=(1, 1), boundary='infinite'), tensors={(0, 0): A})
        env = fpeps.EnvCTM(psi, init='eye', leg=yastn.Leg(cfg, s=1, t=(0, 1), D=(1, 1)))
        for _ in env.ctmrg_(opts_svd={'D_total': chi}, max_sweeps=sweeps, iterator=True, use_qr=use_qr,
                            checkpoint_move='nonreentrant'):
            pass
        ez = env.measure_1site(Z)
        exx = env.measure_nn(X, X)
        E = -3.0 * sum(ez.values()) - sum(exx.values())
    t_fwd = time.time() - t0
    rec.restore()
    ekey = rec.key(E)
    t1 = time.time()
    E.backward()
    t_bwd = time.time() - t1
    grad = A._data.grad.detach().numpy().copy()
    arrays = dict(rec.consts)
    arrays['in:A'] = A._data.detach().numpy().copy()
    arrays['ref:grad'] = grad
    payload = {'scenario': name, 'ops': rec.ops, 'inputs': {'A': 'in:A'}, 'outputs': {'E': ekey},
               'E': float(E.detach()), 'chi': chi, 'sweeps': sweeps, 'D': 6, 'h': 3.0, 'use_qr': use_qr,
               'cpu_seconds': {'forward': t_fwd, 'backward': t_bwd}}
    with open(os.path.join(HERE, name + '.json'), 'w') as f:
        json.dump(payload, f, separators=(',', ':'))
    np.savez_compressed(os.path.join(HERE, name + '.npz'), **arrays)
    nb = sum(1 for o in rec.ops if o['k'] == 'b')
    print(f"{name}: {len(rec.ops)} ops ({nb} backend calls), E = {float(E.detach()):.12f}, "
          f"fwd {t_fwd:.1f} s, bwd {t_bwd:.1f} s")


def _arr_from(rec, x):
    return rec.arrays[x['__array__']]


def scen_ctmrg_qr():
    """The chi=24 CTMRG scenario with YASTN's default projector path use_qr=True (QR of each
    half-system, then the SVD of the product of the R factors)."""
    scen_ctmrg(name='ctmrg_z2_d6_qr', use_qr=True)


def scen_ctmrg_chi144():
    """The CTMRG scenario at the environment dimension of the benchmark configuration
    (chi = 144; blocks of 2592 x 2592 in the projector SVDs)."""
    scen_ctmrg(chi=144, name='ctmrg_z2_d6_chi144')


if __name__ == '__main__' and len(sys.argv) > 2:
    # python make_golden.py <reference tree> <scenario function> ...: only those
    for fn in sys.argv[2:]:
        globals()[fn]()
elif __name__ == '__main__':
    for pol in ('fuse_to_matrix', 'fuse_contracted', 'no_fusion'):
        scen_tensordot(pol)
    scen_svd()
    scen_fix_signs()
    scen_fix_signs_adjoint()
    scen_qr()
    scen_truncation()
    scen_eigh()
    scen_adjoints()
    scen_eigh_adjoint()
    scen_svd_ill()
    scen_tds_adjoint()
    scen_cfg1()
    scen_cfg2()
    scen_cfg3()
    scen_cfg5()
    scen_ctmrg()
    scen_ctmrg_qr()
    scen_ctmrg_chi144()
