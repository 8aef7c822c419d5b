"""Replay of a recorded sequence of backend calls and tensor operations.

YASTN's algorithms (CTMRG, DMRG, ...) drive the backend through the functions of the backend
module plus a few torch operations on the blocks' data (scalar scalings, reshapes, in-place
block writes). A recording made with the reference backend (tests/golden/make_golden.py,
``scen_ctmrg``) stores that sequence: for every step the function name, the arguments
(metadata tuples and Python values verbatim, tensors as keys of the dataflow) and the keys of
its results. ``CallReplay.run`` executes the same sequence with another backend module —
the same names and signatures, e.g. ``yastn_gb300.backend`` — on another device, so the
whole algorithm, forward and (through the backend's autograd Functions) backward, runs on
the GPU without YASTN itself. Data-dependent decisions the algorithm took on the host
(truncated dimensions, ...) are part of the recorded metadata; the replay reproduces them
when its values agree with the recording's.
"""
import json
import os

import numpy as np
import torch
import torch.utils.checkpoint

from .workloads import GOLDEN

__all__ = ['CallReplay', 'load_replay']


def load_replay(name, directory=GOLDEN):
    with open(os.path.join(directory, name + '.json')) as f:
        payload = json.load(f)
    npz = os.path.join(directory, name + '.npz')
    arrays = dict(np.load(npz)) if os.path.exists(npz) else {}
    return CallReplay(payload, arrays)


_DTYPES = {'float64': torch.float64, 'complex128': torch.complex128, 'float32': torch.float32,
           'complex64': torch.complex64, 'bool': torch.bool, 'int64': torch.int64, 'int32': torch.int32,
           'uint8': torch.uint8}


class CallReplay:
    """A recorded call sequence (see the module docstring)."""

    def __init__(self, payload, arrays):
        self.payload = payload
        self.ops = payload['ops']
        self.arrays = arrays
        self.inputs = payload.get('inputs', {})
        self.outputs = payload.get('outputs', {})

    def backend_calls(self):
        """Names of the backend functions the sequence calls, with counts."""
        out = {}
        for op in self.ops:
            if op['k'] == 'b':
                out[op['fn']] = out.get(op['fn'], 0) + 1
        return out

    def run(self, backend, device, inputs, constants_dtype=None, checkpoint=False):
        """Execute the sequence. ``inputs`` maps recorded input names to tensors; returns the
        dict of every produced tensor by key (outputs under ``self.outputs``).

        The recorded arguments are decoded once per device (``_compiled``): metadata and other
        tensor-free arguments become the same Python objects on every run (so the backend's
        plan caches hit by identity), tensor references are resolved per run.

        ``checkpoint``: the segments the recording marks (YASTN's per-CTM-move checkpoint,
        ``checkpoint_move``) run under ``torch.utils.checkpoint`` (non-reentrant): only their
        inputs and the tensors used after them are kept for the backward, which recomputes
        each segment; tensors a segment writes in place are cloned inside it first."""
        dev = torch.device(device)
        env = {}
        for name, key in self.inputs.items():
            env[key] = inputs[name]
        consts = {}
        ops = self._compiled(dev)
        if not checkpoint:
            self._exec(ops, 0, len(ops), env, consts, backend, dev)
            return env
        i = 0
        for kind, a, b, ins, outs, inplace in self._segments(dev):
            if kind == 'plain':
                self._exec(ops, a, b, env, consts, backend, dev)
                continue

            def seg(*tensors, a=a, b=b, ins=ins, outs=outs, inplace=inplace):
                local = dict(zip(ins, tensors))
                for k in inplace:
                    local[k] = local[k].clone()
                self._exec(ops, a, b, local, consts, backend, dev)
                return tuple(local[k] for k in outs)
            res = torch.utils.checkpoint.checkpoint(seg, *[env[k] for k in ins], use_reentrant=False)
            env.update(zip(outs, res))
        return env

    def _exec(self, ops, a, b, env, consts, backend, dev):
        def tensor(k):
            t = env.get(k)
            if t is None:
                t = consts.get(k)
                if t is None:
                    t = consts[k] = torch.from_numpy(np.ascontiguousarray(self.arrays[k])).to(dev)
            return t

        def dec(x):
            if isinstance(x, list):
                return tuple(dec(y) for y in x)
            if isinstance(x, dict):
                if '__t__' in x:
                    return tensor(x['__t__'])
                if '__list__' in x:
                    return [dec(y) for y in x['__list__']]
                if '__dict__' in x:
                    return {dec(k): dec(v) for k, v in x['__dict__']}
                return _decode_leaf(x, dev)
            return x

        def arg(spec):
            kind, v = spec
            if kind == 'c':
                return v
            if kind == 'r':
                return tensor(v)
            return dec(v)

        for kind, fn, aspec, kwspec, keys in ops[a:b]:
            if kind == 'mark':
                continue
            args = tuple(arg(x) for x in aspec)
            kwargs = {k: arg(v) for k, v in kwspec.items()}
            if kind == 'b':
                out = getattr(backend, fn)(*args, **kwargs)
            else:
                out = _torch_call(fn, args, kwargs)
            if keys is None:
                continue
            if isinstance(keys, list):
                for k, v in zip(keys, out):
                    if k is not None:
                        env[k] = v
            else:
                env[keys] = out

    def _segments(self, dev):
        """[(kind, start, stop, inputs, outputs, in-place targets)] over the compiled ops:
        'plain' runs of ops and 'ckpt' segments between checkpoint markers. A segment's inputs
        are the tensors it reads that an earlier op (or the caller) produced; its outputs the
        tensors it produces (or writes in place) that a later op reads or that are results."""
        key = str(dev)
        cache = self.__dict__.setdefault('_segments_by_dev', {})
        if key in cache:
            return cache[key]
        ops = self._compiled(dev)
        reads, writes = [], []
        for kind, fn, aspec, kwspec, keys in ops:
            r = set()
            if kind != 'mark':
                for sp in list(aspec) + list(kwspec.values()):
                    _refs(sp, r)
            w = set()
            if isinstance(keys, list):
                w.update(k for k in keys if k is not None)
            elif keys is not None:
                w.add(keys)
            if kind == 't' and fn == 'm:__setitem__' and aspec[0][0] == 'r':
                w.add(aspec[0][1])
            reads.append(r)
            writes.append(w)
        later = [set() for _ in range(len(ops) + 1)]  # keys read at or after op i
        for i in range(len(ops) - 1, -1, -1):
            later[i] = later[i + 1] | reads[i]
        results = set(self.outputs.values())
        segs, i, start = [], 0, 0
        produced = set(self.inputs.values())
        while i < len(ops):
            if ops[i][0] == 'mark' and ops[i][1] == 'checkpoint_begin':
                j = i + 1
                while not (ops[j][0] == 'mark' and ops[j][1] == 'checkpoint_end'):
                    j += 1
                if start < i:
                    segs.append(('plain', start, i, (), (), ()))
                made, ins, inplace = set(), [], []
                for t in range(i + 1, j):
                    for k in sorted(reads[t]):
                        if k not in made and k in produced and k not in ins:
                            ins.append(k)
                    for k in sorted(writes[t]):
                        if k in produced and k not in made and k not in inplace:
                            inplace.append(k)
                        made.add(k)
                outs = sorted(k for k in made if k in later[j + 1] or k in results)
                for k in inplace:
                    if k not in ins:
                        ins.append(k)
                segs.append(('ckpt', i + 1, j, tuple(ins), tuple(outs), tuple(inplace)))
                produced |= made
                i = start = j + 1
                continue
            for w in writes[i]:
                produced.add(w)
            i += 1
        if start < len(ops):
            segs.append(('plain', start, len(ops), (), (), ()))
        cache[key] = segs
        return segs

    def _compiled(self, dev):
        key = str(dev)
        cache = self.__dict__.setdefault('_compiled_by_dev', {})
        if key not in cache:
            def spec(x):
                if isinstance(x, dict) and '__t__' in x:
                    return ('r', x['__t__'])
                if _has_ref(x):
                    return ('d', x)
                return ('c', _decode_const(x, dev))
            cache[key] = [(op['k'], op['fn'], None, None, None) if op['k'] == 'mark' else
                          (op['k'], op['fn'], [spec(a) for a in op['a']],
                           {k: spec(v) for k, v in op.get('kw', {}).items()}, op.get('o'))
                          for op in self.ops]
        return cache[key]


def _refs(spec, out):
    kind, v = spec
    if kind == 'r':
        out.add(v)
    elif kind == 'd':
        _collect_refs(v, out)


def _collect_refs(x, out):
    if isinstance(x, list):
        for y in x:
            _collect_refs(y, out)
    elif isinstance(x, dict):
        if '__t__' in x:
            out.add(x['__t__'])
        else:
            for v in x.values():
                _collect_refs(v, out)


def _has_ref(x):
    if isinstance(x, list):
        return any(_has_ref(y) for y in x)
    if isinstance(x, dict):
        if '__t__' in x:
            return True
        return any(_has_ref(v) for v in x.values())
    return False


def _decode_leaf(x, dev):
    if '__slice__' in x:
        return slice(*x['__slice__'])
    if '__dtype__' in x:
        return _DTYPES[x['__dtype__']]
    if '__device__' in x:
        return dev
    if '__devstr__' in x:
        return str(dev)
    if '__ellipsis__' in x:
        return Ellipsis
    raise ValueError(f"unknown encoding {list(x)}")


def _decode_const(x, dev):
    """Decodes a tensor-free argument (lists become tuples, as in the recording's metadata)."""
    if isinstance(x, list):
        return tuple(_decode_const(y, dev) for y in x)
    if isinstance(x, dict):
        if '__list__' in x:
            return [_decode_const(y, dev) for y in x['__list__']]
        if '__dict__' in x:
            return {_decode_const(k, dev): _decode_const(v, dev) for k, v in x['__dict__']}
        return _decode_leaf(x, dev)
    return x


def check_dataflow(replay):
    """Every tensor argument is an input, a stored constant or the result of an earlier step;
    returns (number of steps, set of keys used)."""
    have = set(replay.inputs.values()) | set(replay.arrays)
    used = set()

    def walk(x):
        if isinstance(x, list):
            for y in x:
                walk(y)
        elif isinstance(x, dict):
            if '__t__' in x:
                k = x['__t__']
                if k not in have:
                    raise KeyError(f"tensor {k} used before it is produced")
                used.add(k)
            else:
                for v in x.values():
                    walk(v)
    n = 0
    for op in replay.ops:
        if op['k'] == 'mark':
            continue
        walk(op['a'])
        walk(list(op.get('kw', {}).values()))
        o = op.get('o')
        if isinstance(o, list):
            have.update(k for k in o if k is not None)
        elif o is not None:
            have.add(o)
        n += 1
    return n, used


def _torch_call(name, args, kwargs):
    kind, _, fn = name.partition(':')
    if kind == 'm':  # a Tensor method
        if fn == '__setitem__':
            args[0][args[1]] = args[2]
            return None
        return getattr(args[0], fn)(*args[1:], **kwargs)
    if kind == 'a':  # a Tensor attribute
        return getattr(args[0], fn)
    return getattr(torch, fn)(*args, **kwargs)
