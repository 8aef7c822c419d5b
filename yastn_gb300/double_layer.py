"""Fused double-layer PEPS contractions: ``append_vec_tl`` / ``append_vec_br`` /
``append_vec_tr`` / ``append_vec_bl``.

YASTN contracts a CTM boundary vector with both layers of a PEPS site (ket ``A`` and bra
``Ac``) without materialising the double-layer tensor (``fuse_layers``):
``yastn/tn/fpeps/envs/_env_contractions.py:211-365``, called by
``DoublePepsTensor.tensordot`` (``yastn/tn/fpeps/_doublePepsTensor.py:246-283``), by the CTM
projectors and corners (``yastn/tn/fpeps/envs/_env_ctm.py``) and by the reduced density
matrices (``yastn/tn/fpeps/envs/rdm.py``). Each call is a chain of backend calls: the vector is
fused, unfused and swap-gated (``transpose_and_merge``, ``unmerge``, ``negate_blocks``), the bra
is conjugated (``conj``), each of the two ``tensordot`` calls merges its operands into sector
matrices, runs ``dot`` and the result is re-fused, and the output is fused and unfused into its
final leg order: 7 to 8 copy passes over the environment-sized data around 2 grouped GEMMs.

Here a call runs as a compiled program of the same two GEMMs (the backend's ``dot``: grouped
FP64 / complex128 sector GEMMs, or their BF16 tensor-core emulation) and of one composed copy
(``yb_map_gather``) per GEMM operand and for the output. The program is built once per input
structure (block charges, dims, fusion trees, leg order, dtype, mode and legs):

1. record: YASTN's own function runs once on shape-only ('meta' device) copies of the inputs
   through a recording backend, so every metadata tuple comes from YASTN's unchanged metadata
   layer and nothing is computed;
2. compose: every chain of copies between a root (an input, or a GEMM result) and a sink (a
   GEMM operand, or the output) is executed once on the device on an int64 iota of the root
   (source indices + 1) with the backend's own copy kernels; the result is the chain's gather
   map (0 where the chain zero-fills, negative where it negates a block), checked to be
   injective, with its inverse for the adjoint; a chain that is the identity is dropped;
3. run: gathers and GEMMs, each a ``torch.autograd.Function`` (the gather's adjoint is the
   gather by the inverse map, the GEMMs keep the backend's adjoints), so the result is
   differentiable and re-entrant under ``torch.utils.checkpoint`` (the same program runs in
   the forward and in the recomputation).

A call whose chain holds any other backend call, whose data are not FP64 / complex128 CUDA
tensors of this backend, or whose sources exceed 2^31 - 2 elements runs YASTN's own function
unchanged on this backend. ``install()`` rebinds the four names in the YASTN modules that
imported them; ``uninstall()`` restores them.
"""
from collections import OrderedDict

import torch

from . import backend_gb300
from . import ops

__all__ = ['append_vec_tl', 'append_vec_br', 'append_vec_tr', 'append_vec_bl', 'install', 'uninstall',
           'compile_program', 'DoubleLayerProgram', 'cache_info', 'clear_cache']

_NAMES = ('append_vec_tl', 'append_vec_br', 'append_vec_tr', 'append_vec_bl')
_COPIES = frozenset(('transpose_and_merge', 'unmerge', 'transpose', 'negate_blocks', 'conj'))
_GEMMS = frozenset(('dot', 'transpose_dot_sum'))
# functions of the backend that only inspect a tensor: allowed while recording
_INSPECT = frozenset(('get_dtype', 'get_yastn_dtype', 'is_complex', 'get_device', 'get_shape', 'get_size',
                      'requires_grad', 'cuda_is_available'))
_MAX_SOURCE = 2 ** 31 - 2
_CACHE_SIZE = 256            # programs kept (least recently used dropped first) ...
_CACHE_BYTES = 32 << 30      # ... and at most this much device memory in their gather maps


class Unfusable(Exception):
    """The recorded call chain holds something a compiled program does not run."""


# ----------------------------------------------------------------------------- recording

class _Recorder:
    """A backend module stand-in for YASTN's function under recording: copies and GEMMs return
    shape-only ('meta' device) tensors and are logged with their metadata arguments; inspection
    functions and constants pass through; any other function raises Unfusable."""

    def __init__(self, backend):
        self._backend = backend
        self.ops = []     # (name, input tensor ids, other args, output id, output size)
        self.keep = []    # every tensor seen, kept alive so that ids stay unique

    def __getattr__(self, name):
        if name.startswith('__'):
            raise AttributeError(name)
        if name in _COPIES or name in _GEMMS:
            return lambda *args, **kwargs: self._record(name, args, kwargs)
        attr = getattr(self._backend, name)
        if callable(attr) and name not in _INSPECT:
            def refuse(*args, **kwargs):
                raise Unfusable(f"backend call {name} inside the contraction")
            return refuse
        return attr

    def _record(self, name, args, kwargs):
        if kwargs:
            raise Unfusable(f"keyword arguments to {name}")
        n_in = 2 if name in _GEMMS else 1
        ins, rest = args[:n_in], args[n_in:]
        for t in ins:
            if not isinstance(t, torch.Tensor):
                raise Unfusable(f"non-tensor operand of {name}")
        if name in _GEMMS:
            dtype = torch.promote_types(ins[0].dtype, ins[1].dtype)
            size = rest[-1]
        else:
            dtype = ins[0].dtype
            size = rest[-1] if name == 'transpose_and_merge' else ins[0].numel()
        out = torch.empty(int(size), dtype=dtype, device='meta')
        self.keep.extend(ins)
        self.keep.append(out)
        self.ops.append((name, tuple(id(t) for t in ins), rest, id(out), out.numel()))
        return out


# ----------------------------------------------------------------------------- programs

class _Gather(torch.autograd.Function):
    """A composed copy (``yb_map_gather``); its adjoint is the gather by the inverse map.

    Under torch.func transforms (YASTN's fixed-point CTMRG differentiates its CTM step with
    torch.func.vjp) the maps reach setup_context as wrapped tensors, which have no storage
    pointer for the kernel: they are unwrapped before use, as the cotangent is."""

    @staticmethod
    def forward(src, gmap, inv, conj):
        unwrap = backend_gb300._unwrap
        return ops.map_gather(unwrap(src), unwrap(gmap), conj)

    @staticmethod
    def setup_context(ctx, inputs, output):
        _, _, inv, conj = inputs
        ctx.inv, ctx.conj = inv, conj

    @staticmethod
    def backward(ctx, g):
        unwrap = backend_gb300._unwrap
        return ops.map_gather(unwrap(g).contiguous(), unwrap(ctx.inv), ctx.conj), None, None, None


def _native_gather(src, gmap, inv, conj):
    return _Gather.apply(src, gmap, inv, conj)


class DoubleLayerProgram:
    """A compiled contraction: ``steps`` is a list of

    * ``('gather', sink, root, chain)``: the sink's data are the root's data through the chain
      of recorded copies (name, arguments), executed as one composed copy;
    * ``('gemm', name, out, (a, b), args)``: the backend's ``dot`` / ``transpose_dot_sum``.

    Node keys are ('in', i) for the i-th input tensor's data and ('op', j) for the result of
    the j-th recorded call. ``template`` is YASTN's result with shape-only data: its structure,
    fusion trees and leg order are the output's."""

    def __init__(self, steps, output, template, sizes):
        self.steps = steps
        self.output = output
        self.template = template
        self.sizes = sizes          # node -> number of elements
        self._maps = {}             # (device, backend id) -> {sink: (gmap, inv, conj) | None}

    def n_gathers(self, device=None):
        if device is None:
            return sum(1 for s in self.steps if s[0] == 'gather')
        maps = next((m for (d, _), m in self._maps.items() if d == str(device)), {})
        return sum(1 for v in maps.values() if v is not None)

    def maps(self, backend, device):
        """The gather maps of every sink on ``device``, composed with ``backend``'s copies."""
        key = (str(device), id(backend))
        maps = self._maps.get(key)
        if maps is None:
            maps = {}
            for step in self.steps:
                if step[0] == 'gather':
                    _, sink, root, chain = step
                    maps[sink] = _compose(backend, device, self.sizes[root], chain)
            self._maps[key] = maps
        return maps

    def map_bytes(self):
        """Device bytes held by the gather maps (and inverses) of every device."""
        return sum(m[0].numel() * 4 + m[1].numel() * 4 for maps in self._maps.values()
                   for m in maps.values() if m is not None)

    def run(self, datas, backend, gather=_native_gather):
        """Execute on the inputs' data (in the recorded order); returns the output's data."""
        device = datas[0].device
        maps = self.maps(backend, device)
        env = {('in', i): d for i, d in enumerate(datas)}
        for step in self.steps:
            if step[0] == 'gather':
                _, sink, root, _ = step
                m = maps[sink]
                src = env[root]
                if src.numel() != self.sizes[root]:  # the maps index a source of the recorded size
                    raise ValueError("double-layer program: input size differs from the recorded structure")
                env[sink] = src if m is None else gather(src, *m)
            else:
                _, name, out, (a, b), args = step
                env[out] = getattr(backend, name)(env[a], env[b], *args)
        return env[self.output]


def _compose(backend, device, n_root, chain):
    """The gather map of a chain of copies (None for the identity)."""
    if not chain:
        return None
    if n_root > _MAX_SOURCE:
        raise Unfusable("source too large for an int32 gather map")
    iota = torch.arange(1, n_root + 1, dtype=torch.int64, device=device)
    x, conj = iota, False
    for name, args in chain:
        if name == 'conj':
            conj = not conj
        else:
            x = getattr(backend, name)(x, *args)
    x = x.reshape(-1)
    if x.numel() == n_root and torch.equal(x, iota):
        return None if not conj else (x.to(torch.int32), x.to(torch.int32), True)
    gmap = x.to(torch.int32)
    pos = torch.nonzero(gmap).reshape(-1)
    val = gmap[pos]
    inv = torch.zeros(n_root, dtype=torch.int32, device=device)
    inv[val.abs().long() - 1] = (torch.sign(val).long() * (pos + 1)).to(torch.int32)
    if int(torch.count_nonzero(inv)) != pos.numel():
        raise Unfusable("a copy chain maps two destinations to one source")
    return gmap, inv, conj


def compile_program(fn, tensors, kwargs):
    """Record ``fn(*tensors, **kwargs)`` (YASTN's contraction) on shape-only copies of the
    tensors and compile it; raises Unfusable when the chain cannot run as a program."""
    cfg = tensors[0].config
    rec = _Recorder(cfg.backend)
    pcfg = cfg._replace(backend=rec)
    shadows = []
    for t in tensors:
        if t is None:
            shadows.append(None)
            continue
        m = torch.empty(t._data.numel(), dtype=t._data.dtype, device='meta')
        shadows.append(t._replace(config=pcfg, data=m))
    n_pos = 3
    res = fn(*shadows[:n_pos], **dict(kwargs, op=shadows[n_pos] if len(shadows) > n_pos else None))
    ids, producer = {}, {}
    sizes = {}
    for i, sh in enumerate(shadows):
        if sh is not None:
            ids.setdefault(id(sh._data), ('in', i))
            sizes[('in', i)] = sh._data.numel()
    for j, (name, ins, rest, out, numel) in enumerate(rec.ops):
        producer[out] = j
        ids[out] = ('op', j)
        sizes[('op', j)] = numel

    def node_of(tid):
        node = ids.get(tid)
        if node is None:
            raise Unfusable("an operand that is neither an input nor a recorded result")
        return node

    def trace(tid):
        """The root of a tensor id and the chain of copies from it."""
        chain = []
        while tid in producer and rec.ops[producer[tid]][0] in _COPIES:
            name, ins, rest = rec.ops[producer[tid]][:3]
            chain.append((name, rest))
            tid = ins[0]
        return node_of(tid), chain[::-1]

    steps, sinks = [], {}
    for j, (name, ins, rest, out, _) in enumerate(rec.ops):
        if name not in _GEMMS:
            continue
        operands = []
        for tid in ins:
            root, chain = trace(tid)
            if not chain:
                operands.append(root)
                continue
            sink = sinks.get(tid)
            if sink is None:
                sink = sinks[tid] = ('sink', len(sinks))
                steps.append(('gather', sink, root, tuple(chain)))
            operands.append(sink)
        steps.append(('gemm', name, ('op', j), tuple(operands), rest))
    if not isinstance(res._data, torch.Tensor):
        raise Unfusable("the contraction returned no data")
    root, chain = trace(id(res._data))
    output = root
    if chain:
        output = ('sink', len(sinks))
        steps.append(('gather', output, root, tuple(chain)))
    template = res._replace(config=cfg)
    return DoubleLayerProgram(steps, output, template, sizes)


# ----------------------------------------------------------------------------- drop-ins

_PROGRAMS = OrderedDict()
_STATS = {'hits': 0, 'compiled': 0, 'unfused': 0, 'bytes': 0}
_ORIGINAL = {}
_SUPPORTED = (torch.float64, torch.complex128)


def _reference(name):
    """YASTN's own function (captured before install() rebinds the name)."""
    f = _ORIGINAL.get(name)
    if f is None:
        import yastn.tn.fpeps.envs._env_contractions as ec
        f = getattr(ec, name)
        if getattr(f, '_yastn_gb300_fused', False):
            raise RuntimeError(f"YASTN's {name} is not available (rebound without its original)")
        _ORIGINAL[name] = f
    return f


def _tensor_key(t):
    return (t.struct, t.slices, t.hfs, t.mfs, t.trans, t._data.dtype)


def _eligible(tensors):
    cfg = tensors[0].config
    if cfg.backend is not backend_gb300:
        return False
    for t in tensors:
        if t is None:
            continue
        d = t._data
        if not isinstance(d, torch.Tensor) or not d.is_cuda or d.dtype not in _SUPPORTED:
            return False
        if t.config.backend is not backend_gb300:
            return False
    return True


def _run(name, Ac, A, vec, op, mode, in_b, out_a):
    ref = _reference(name)
    kwargs = dict(mode=mode, in_b=tuple(in_b), out_a=tuple(out_a))
    tensors = (Ac, A, vec) + ((op,) if op is not None else ())
    if not _eligible(tensors):
        return ref(Ac, A, vec, op=op, **kwargs)
    cfg = A.config
    key = (name, mode, tuple(in_b), tuple(out_a), cfg._replace(backend=None),
           tuple(_tensor_key(t) for t in tensors))
    prog = _PROGRAMS.get(key, False)
    if prog is False:
        try:
            prog = compile_program(ref, tensors, kwargs)
            prog.maps(backend_gb300, A._data.device)
            _STATS['compiled'] += 1
        except Exception:  # noqa: BLE001 -- Unfusable, or YASTN's own error, which its function raises again
            prog = None
        _PROGRAMS[key] = prog
        _STATS['bytes'] = _STATS.get('bytes', 0) + (prog.map_bytes() if prog is not None else 0)
        while len(_PROGRAMS) > 1 and (len(_PROGRAMS) > _CACHE_SIZE or _STATS['bytes'] > _CACHE_BYTES):
            _, old = _PROGRAMS.popitem(last=False)
            _STATS['bytes'] -= old.map_bytes() if old is not None else 0
    else:
        _PROGRAMS.move_to_end(key)
        _STATS['hits'] += 1
    if prog is None:
        _STATS['unfused'] += 1
        return ref(Ac, A, vec, op=op, **kwargs)
    data = prog.run([t._data for t in tensors], backend_gb300)
    return prog.template._replace(config=cfg, data=data)


def append_vec_tl(Ac, A, vectl, op=None, mode='old', in_b=(2, 1), out_a=(2, 3)):
    """``append_vec_tl`` (``_env_contractions.py:211-246``): the top-left vector
    ``x [l l'] [t t'] y`` with the site's ket ``A`` and bra ``Ac``, as one compiled program."""
    return _run('append_vec_tl', Ac, A, vectl, op, mode, in_b, out_a)


def append_vec_br(Ac, A, vecbr, op=None, mode='old', in_b=(2, 1), out_a=(0, 1)):
    """``append_vec_br`` (``_env_contractions.py:249-284``): the bottom-right vector."""
    return _run('append_vec_br', Ac, A, vecbr, op, mode, in_b, out_a)


def append_vec_tr(Ac, A, vectr, op=None, mode='old', in_b=(1, 2), out_a=(1, 2)):
    """``append_vec_tr`` (``_env_contractions.py:287-319``): the top-right vector."""
    return _run('append_vec_tr', Ac, A, vectr, op, mode, in_b, out_a)


def append_vec_bl(Ac, A, vecbl, op=None, mode='old', in_b=(2, 1), out_a=(0, 3)):
    """``append_vec_bl`` (``_env_contractions.py:322-365``): the bottom-left vector."""
    return _run('append_vec_bl', Ac, A, vecbl, op, mode, in_b, out_a)


for _f in (append_vec_tl, append_vec_br, append_vec_tr, append_vec_bl):
    _f._yastn_gb300_fused = True


def _yastn_modules():
    import yastn.tn.fpeps._doublePepsTensor as dpt
    import yastn.tn.fpeps.envs._env_contractions as ec
    import yastn.tn.fpeps.envs._env_ctm as ctm
    import yastn.tn.fpeps.envs.rdm as rdm
    return (ec, dpt, ctm, rdm)


def install():
    """Rebind YASTN's four ``append_vec_*`` names (in ``_env_contractions`` and the modules that
    imported them: ``_doublePepsTensor``, ``_env_ctm``, ``rdm``) to the compiled versions."""
    mods = _yastn_modules()
    fused = {n: globals()[n] for n in _NAMES}
    for n in _NAMES:
        _reference(n)
    for m in mods:
        for n in _NAMES:
            if hasattr(m, n):
                setattr(m, n, fused[n])


def uninstall():
    """Restore YASTN's own functions."""
    for m in _yastn_modules():
        for n in _NAMES:
            if hasattr(m, n) and n in _ORIGINAL:
                setattr(m, n, _ORIGINAL[n])


def cache_info():
    return dict(_STATS, programs=len(_PROGRAMS))


def clear_cache():
    _PROGRAMS.clear()
    for k in _STATS:
        _STATS[k] = 0
