"""Device operations of the hot path: torch tensors in, C ABI calls, torch tensors out.

Every function here launches the hand-written sm_103a kernels of
``libyastn_gb300.so`` on torch's current CUDA stream. Inputs must be contiguous 1-D
CUDA tensors of dtype float64 or complex128; anything else raises (there is no
fallback path).
"""
import ctypes
import weakref

import numpy as np
import torch

from . import _native as N
from . import _plans as P

_SUPPORTED = (torch.float64, torch.complex128)
MAX_SWEEPS = 64


def _vp(x):
    return ctypes.c_void_p(x)


def _ptr(t):
    if t.is_conj() or t.is_neg():  # a lazy view: its memory is not what the kernels would read
        raise ValueError("yastn_gb300: a conjugate/negative view reached a kernel unresolved")
    return ctypes.c_void_p(t.data_ptr())


def _plain(t):
    """t with torch's lazy conjugate / negative flags resolved, contiguous."""
    if t.is_conj():
        t = t.resolve_conj()
    if t.is_neg():
        t = t.resolve_neg()
    return t.contiguous()


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _dtype_code(dtype):
    if dtype == torch.float64:
        return N.YB_F64
    if dtype == torch.complex128:
        return N.YB_C128
    raise NotImplementedError(f"yastn_gb300 kernels support float64 and complex128, got {dtype}")


_COPY_UNITS = (1, 2, 4, 8, 16)  # element sizes the block copy and mask kernels move as raw units
_NARROW = {torch.float32: torch.float64, torch.complex64: torch.complex128}


def _check(t, name='data', any_dtype=False):
    """A CUDA tensor, flat, contiguous, with lazy conjugate / negative views resolved. The
    arithmetic kernels take float64 and complex128; the copies (``any_dtype``) any element of
    1, 2, 4, 8 or 16 bytes (bool masks, float32, complex64, ...)."""
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise TypeError(f"{name} must be a CUDA tensor (yastn_gb300 has no CPU path)")
    if any_dtype:
        if t.element_size() not in _COPY_UNITS:
            raise NotImplementedError(f"yastn_gb300 copies move 1-16 byte elements, got {t.dtype}")
    elif t.dtype not in _SUPPORTED:
        raise NotImplementedError(f"yastn_gb300 kernels support float64 and complex128, got {t.dtype}")
    # torch's lazy conjugate / negative views (conj(), neg() of a conjugate) keep the memory
    # unchanged and only set a flag that the kernels, reading raw memory, would not see
    if t.is_conj():
        t = t.resolve_conj()
    if t.is_neg():
        t = t.resolve_neg()
    if t.dim() != 1 or not t.is_contiguous():
        t = t.reshape(-1).contiguous()
    return t


def _dev(plan, key, arrays, device):
    """Device copies of a plan's packed arrays, cached on the plan per device."""
    k = (key, str(device))
    d = plan._dev.get(k)
    if d is None:
        d = tuple(torch.from_numpy(np.ascontiguousarray(a)).to(device) for a in arrays)
        plan._dev[k] = d
    return d


# ----------------------------------------------------------------------------- family (a)

def run_copy(plan, src, dst):
    """Run a CopyPlan from ``src`` into ``dst`` (both 1-D, same dtype)."""
    vec_ok = src.dtype == torch.float64 and src.data_ptr() % 16 == 0 and dst.data_ptr() % 16 == 0
    tasks, items = plan.packed(vec_ok)
    if len(items) == 0:
        return dst
    dt, di = _dev(plan, ('copy', vec_ok), (tasks, items), src.device)
    N.call('yb_block_copy', _ptr(src), _ptr(dst), src.element_size(), _ptr(dt), len(tasks), _ptr(di), len(items),
           _stream())
    return dst


def map_gather(src, gmap, conj=False):
    """One composed copy: ``out[i] = conj?(sign * src[|gmap[i]| - 1])`` (0 where gmap[i] == 0),
    ``gmap`` an int32 CUDA tensor of source indices + 1 with the sign of a block negation
    (``yb_map_gather``)."""
    src = _check(src, 'src')
    if gmap.dtype != torch.int32 or not gmap.is_cuda or gmap.dim() != 1 or not gmap.is_contiguous():
        raise TypeError("gmap must be a contiguous 1-D int32 CUDA tensor")
    if src.numel() == 0:  # nothing to gather: every entry of a valid map is 0 (zero fill)
        return torch.zeros(gmap.numel(), dtype=src.dtype, device=src.device)
    out = torch.empty(gmap.numel(), dtype=src.dtype, device=src.device)
    if out.numel():
        N.call('yb_map_gather', _ptr(src), _ptr(out), _dtype_code(src.dtype), _ptr(gmap), gmap.numel(),
               int(bool(conj) and src.is_complex()), _stream())
    return out


# ----------------------------------------------------------------------------- constant operands

_HOLD = {'depth': 0, 'capturing': None, 'merge': {}, 'split': {}}


class hold_constant_operands:
    """Scope in which the merges and digit splits of unchanged operands are computed once.

    An iterative solver applies one operator many times: in YASTN's ``eigs`` the effective
    Hamiltonian's environment tensors, and their merged sector matrices, are the same tensor
    objects in every call. Inside this scope a merge of the same source tensor object (its
    version counter unchanged) by the same plan returns its earlier output while that output
    is unmodified (its version counter unchanged), and an emulated dot reuses the BF16 digit
    planes of an operand object it split before; tensors that require grad are never held.
    Entries refer to their sources weakly (an entry ends with its source, so the temporaries
    of each operator application are not kept), end with the outermost scope, and are
    dropped when the stream capture state changes: entries made during a CUDA-graph capture
    are used within that capture only, whose replays recompute them in order."""

    def __enter__(self):
        _HOLD['depth'] += 1
        return self

    def __exit__(self, *exc):
        _HOLD['depth'] -= 1
        if _HOLD['depth'] == 0:
            _HOLD['merge'].clear()
            _HOLD['split'].clear()
        return False


def _held(kind, key, src):
    """(cache, key) for ``src`` in the current scope, or None (no scope, or src requires grad)."""
    if _HOLD['depth'] == 0 or src.requires_grad:
        return None
    cap = torch.cuda.is_current_stream_capturing()
    if _HOLD['capturing'] != cap:
        _HOLD['merge'].clear()
        _HOLD['split'].clear()
        _HOLD['capturing'] = cap
    return _HOLD[kind], key + (id(src),)


def _hit(held, src):
    """The held payload of src, if its entry is current."""
    if held is None:
        return None
    cache, key = held
    e = cache.get(key)
    if e is None or e[0]() is not src or e[1] != src._version:
        return None
    payload, out_version = e[2], e[3]
    if out_version is not None and payload._version != out_version:
        return None
    return payload


def _store(held, src, payload, track_output=False):
    cache, key = held

    def drop(ref, cache=cache, key=key):
        e = cache.get(key)
        if e is not None and e[0] is ref:
            del cache[key]
    cache[key] = (weakref.ref(src, drop), src._version, payload, payload._version if track_output else None)


def merge(data, order, meta_new, meta_mrg, Dsize):
    """transpose_and_merge: fused blocks, zero where no source block lands (inside
    ``hold_constant_operands``, the earlier output for an unchanged source)."""
    data = _check(data, any_dtype=True)
    plan = P.merge_plan(order, meta_new, meta_mrg, Dsize)
    held = _held('merge', (id(plan),), data)
    out = _hit(held, data)
    if out is not None:
        return out
    out = (torch.empty if plan.full else torch.zeros)(Dsize, dtype=data.dtype, device=data.device)
    run_copy(plan, data, out)
    if held is not None:
        _store(held, data, out, track_output=True)
    return out


def merge_backward(data_b, order, meta_new, meta_mrg, Dsize, D_source):
    data_b = _check(data_b, any_dtype=True)
    plan = P.merge_plan(order, meta_new, meta_mrg, Dsize)
    inv = P.CACHE.get((order, meta_new, meta_mrg), ('merge_bwd', Dsize, D_source), lambda: plan.swapped(D_source))
    out = (torch.empty if inv.full else torch.zeros)(D_source, dtype=data_b.dtype, device=data_b.device)
    return run_copy(inv, data_b, out)


def unmerge(data, meta):
    data = _check(data, any_dtype=True)
    plan = P.unmerge_plan(meta, data.numel())
    out = (torch.empty if plan.full else torch.zeros)(data.numel(), dtype=data.dtype, device=data.device)
    return run_copy(plan, data, out)


def unmerge_backward(data_b, meta, fwd_size):
    data_b = _check(data_b, any_dtype=True)
    plan = P.unmerge_plan(meta, fwd_size)
    inv = P.CACHE.get((meta,), ('unmerge_bwd', fwd_size), lambda: plan.swapped(fwd_size))
    out = (torch.empty if inv.full else torch.zeros)(fwd_size, dtype=data_b.dtype, device=data_b.device)
    return run_copy(inv, data_b, out)


def transpose(data, axes, meta_transpose):
    data = _check(data, any_dtype=True)
    plan = P.transpose_plan(axes, meta_transpose, data.numel())
    out = (torch.empty if plan.full else torch.zeros)(data.numel(), dtype=data.dtype, device=data.device)
    return run_copy(plan, data, out)


def transpose_backward(data_b, axes, meta_transpose):
    data_b = _check(data_b, any_dtype=True)
    plan = P.transpose_plan(axes, meta_transpose, data_b.numel())
    inv = P.CACHE.get((axes, meta_transpose), ('transpose_bwd', data_b.numel()), lambda: plan.swapped(data_b.numel()))
    out = (torch.empty if inv.full else torch.zeros)(data_b.numel(), dtype=data_b.dtype, device=data_b.device)
    return run_copy(inv, data_b, out)


# ----------------------------------------------------------------------------- family (b)

def run_gemm(plan, a, b, c, alpha=1.0, beta=0.0):
    code = _dtype_code(c.dtype)
    if len(plan.tiles):
        do, dtm, dti = _dev(plan, 'gemm', (plan.outs, plan.terms, plan.tiles), a.device)
        N.call('yb_grouped_gemm_short' if plan.all_short else 'yb_grouped_gemm', _ptr(a), _ptr(b), _ptr(c), code,
               _ptr(do), _ptr(dtm), _ptr(dti), len(plan.tiles), float(alpha), float(beta), _stream())
    sp = plan.split
    if sp is not None:
        # split-K: chunk products into a workspace, then the ordered sum into C
        ws = torch.empty(sp.ws, dtype=c.dtype, device=c.device)
        do, dtm, dti, dred, dtask = _dev(plan, 'gemm_split', (sp.outs, sp.terms, sp.tiles, sp.red, sp.tasks),
                                         a.device)
        N.call('yb_grouped_gemm', _ptr(a), _ptr(b), _ptr(ws), code, _ptr(do), _ptr(dtm), _ptr(dti),
               len(sp.tiles), 1.0, 0.0, _stream())
        N.call('yb_gemm_reduce', _ptr(c), _ptr(ws), code, _ptr(dred), _ptr(dtask), len(sp.tasks), float(alpha),
               float(beta), _stream())
    return c


def promote(A, B):
    dtype = torch.promote_types(A.dtype, B.dtype)
    return (A if A.dtype == dtype else A.to(dtype)), (B if B.dtype == dtype else B.to(dtype))


def _narrow_inputs(*ts):
    """True when a float32 / complex64 operand is present: the product then runs in float64 /
    complex128 on the same kernels and the result is rounded to the promoted input dtype (at
    least the accuracy of a single-precision product)."""
    return any(isinstance(t, torch.Tensor) and t.dtype in _NARROW for t in ts)


def _wide(t):
    return t.to(_NARROW[t.dtype]) if t.dtype in _NARROW else t


def dot(A, B, meta_dot, Dsize):
    if _narrow_inputs(A, B):
        return dot(_wide(A), _wide(B), meta_dot, Dsize).to(torch.promote_types(A.dtype, B.dtype))
    A, B = promote(_check(A, 'A'), _check(B, 'B'))
    plan = P.dot_plan(meta_dot)
    # every element is written by one sector when the sectors tile the output
    out = (torch.empty if plan.covered == Dsize else torch.zeros)(Dsize, dtype=A.dtype, device=A.device)
    return run_gemm(plan, A, B, out)


OZAKI_SLICES = 8  # 57 bits per operand: FP64-grade products


OZAKI_TC = [None]  # emulated GEMM kernel: None = autotuned per dot; False = mma.sync; 64 (or True) / 32 =
                  # tcgen05/TMEM with 128 x 64 / 128 x 32 output tiles
OZAKI_AUTOTUNE = [True]  # False: choose by the tile-padding estimate without timing


def dot_ozaki(A, B, meta_dot, Dsize, slices=OZAKI_SLICES):
    """``dot`` with the FP64 sector GEMMs emulated on BF16 tensor cores (split operands).

    float64 or complex128 operands (a complex product is two real products with doubled
    K). Each A row / B column is split into ``slices`` BF16 digit
    planes (scratch of 2 * slices bytes per operand element); all slice-pair products
    with digit-weight sum below ``slices`` are accumulated exactly in FP32 per K-chunk and
    combined in FP64. ``slices=8`` reproduces the FP64 product to its rounding level.
    """
    if _narrow_inputs(A, B):
        return dot_ozaki(_wide(A), _wide(B), meta_dot, Dsize, slices).to(torch.promote_types(A.dtype, B.dtype))
    A, B = promote(_check(A, 'A'), _check(B, 'B'))
    plan = P.ozaki_dot_plan(meta_dot, slices, A.is_complex())
    out = (torch.empty if plan.covered == Dsize else torch.zeros)(Dsize, dtype=A.dtype, device=A.device)
    if len(plan.tiles) == 0:
        return run_gemm(plan.native, A, B, out)  # short (K < 16) and skinny sectors: native FP64
    if OZAKI_TC[0] is not None:
        tc = OZAKI_TC[0]
    else:
        if getattr(plan, 'tuned_tc', None) is None:
            plan.tuned_tc = _autotune_ozaki(plan, A, B, out, slices)
        tc = plan.tuned_tc
    # the native sectors (disjoint outputs) run on a second stream beside the split and the
    # emulated GEMM, and the current stream waits for them (a fork and join inside a CUDA graph)
    fork = len(plan.native.tiles) > 0 or plan.native.split is not None
    if fork:
        main, side = torch.cuda.current_stream(A.device), _side_stream(A.device)
        side.wait_stream(main)
        with torch.cuda.stream(side):
            run_gemm(plan.native, A, B, out)
    _ozaki_run(plan, A, B, out, slices, tc)
    if fork:
        main.wait_stream(side)
    return out


_SIDE = {}


def _side_stream(device):
    """The second stream of a device (created once; independent work of one call runs on it)."""
    s = _SIDE.get(device.index)
    if s is None:
        s = _SIDE[device.index] = torch.cuda.Stream(device=device)
    return s


def _autotune_ozaki(plan, A, B, out, slices):
    """Kernel choice for one dot metadata: the mma.sync kernel and the tcgen05 kernel with
    128 x 64 or 128 x 32 tiles produce the same bits, so the first call times the three (CUDA
    events; skipped during stream capture, where the tile-padding estimate decides) and the
    plan keeps the fastest."""
    if not OZAKI_AUTOTUNE[0] or torch.cuda.is_current_stream_capturing():
        return plan.prefer_tc
    times = {}
    for tc in (False, 64, 32, False, 64, 32):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda._sleep(2_000_000)  # hold the stream while the host enqueues: time the GPU, not the host
        e0.record()
        _ozaki_run(plan, A, B, out, slices, tc)
        e1.record()
        e1.synchronize()
        times[tc] = e0.elapsed_time(e1)  # the second (warm) measurement of each kernel is kept
    return min(times, key=times.get)


def _ozaki_run(plan, A, B, out, slices, tc):
    """Both operands split by one yb_ozaki_split launch (B's blocks read by columns in
    place), then the emulated GEMM: tcgen05 (tile layout) or mma.sync (digit planes). Inside
    ``hold_constant_operands`` an operand split before, unchanged, keeps its digit planes and
    only the other operand is split (or neither)."""
    dev = A.device
    st = _stream()
    tile_n = 0 if not tc else (32 if tc == 32 else 64)
    if tile_n:
        # tiles grouped by CTA (one CTA per SM) with balanced work
        sfx = '_tc' if tile_n == 64 else '_tc32'
        tiles, offs = P.ozaki_tc_schedule(plan, _sm_count(dev), tile_n)
        key, arrs = 'ozaki' + sfx, (getattr(plan, 'split_recs' + sfx), getattr(plan, 'split_groups' + sfx),
                                    getattr(plan, 'outs' + sfx), tiles, offs)
        asz, bsz = getattr(plan, 'a_size' + sfx), getattr(plan, 'b_size' + sfx)
        by_op = getattr(plan, 'split_groups' + sfx + '_ab')
    else:
        key, arrs = 'ozaki', (plan.split_recs, plan.split_groups, plan.outs, plan.tiles)
        asz, bsz = plan.a_size, plan.b_size
        by_op = plan.split_groups_ab
    # the per-operand group lists travel with the plan's arrays (no upload during a capture)
    darr = _dev(plan, key, arrs + tuple(by_op), dev)
    drec, dgrp, dout, dtl = darr[:4]
    held_a = _held('split', (id(plan), 0, tile_n, slices), A)
    held_b = _held('split', (id(plan), 1, tile_n, slices), B)
    hit_a, hit_b = _hit(held_a, A), _hit(held_b, B)
    a_sl, a_ex = hit_a if hit_a else (torch.empty(max(asz, 1), dtype=torch.bfloat16, device=dev),
                                      torch.empty(max(plan.a_exps, 1), dtype=torch.int32, device=dev))
    b_sl, b_ex = hit_b if hit_b else (torch.empty(max(bsz, 1), dtype=torch.bfloat16, device=dev),
                                      torch.empty(max(plan.b_exps, 1), dtype=torch.int32, device=dev))
    if not hit_a and not hit_b:
        groups, n_groups = dgrp, len(arrs[1])
    elif hit_a != hit_b:
        side = 1 if hit_a else 0  # split only the operand that is not held
        groups, n_groups = darr[len(arrs) + side], len(by_op[side])
    else:
        groups, n_groups = None, 0
    if n_groups:
        N.call('yb_ozaki_split', _ptr(A), _ptr(B), _ptr(a_sl), _ptr(b_sl), _ptr(a_ex), _ptr(b_ex), _ptr(drec),
               _ptr(groups), n_groups, slices, st)
    if held_a is not None and not hit_a:
        _store(held_a, A, (a_sl, a_ex))
    if held_b is not None and not hit_b:
        _store(held_b, B, (b_sl, b_ex))
    if tile_n:
        N.call('yb_ozaki_gemm_tc', _ptr(a_sl), _ptr(a_ex), _ptr(b_sl), _ptr(b_ex), _ptr(out), _ptr(dout), _ptr(dtl),
               len(arrs[3]), _ptr(darr[4]), len(arrs[4]) - 1, tile_n, slices, st)
    else:
        N.call('yb_ozaki_gemm', _ptr(a_sl), _ptr(a_ex), _ptr(b_sl), _ptr(b_ex), _ptr(out), _ptr(dout), _ptr(dtl),
               len(arrs[3]), slices, st)


_SMS = {}


def _sm_count(device):
    n = _SMS.get(device.index)
    if n is None:
        n = _SMS[device.index] = torch.cuda.get_device_properties(device).multi_processor_count
    return n


def ozaki_device_error(reset=True):
    """Status word of the tcgen05 emulated GEMM (synchronises the current stream)."""
    import ctypes
    v = ctypes.c_int(0)
    N.call('yb_ozaki_device_error', ctypes.addressof(v), int(bool(reset)), _stream(), launches=0)
    return v.value


def dot_backward(C_b, A, B, meta_dot, need_a=True, need_b=True):
    if _narrow_inputs(C_b, A, B):
        A_b, B_b = dot_backward(_wide(C_b), _wide(A), _wide(B), meta_dot, need_a, need_b)
        return (None if A_b is None else A_b.to(A.dtype)), (None if B_b is None else B_b.to(B.dtype))
    A, B = promote(_check(A, 'A'), _check(B, 'B'))
    C_b = _check(C_b, 'C_b')
    if C_b.dtype != A.dtype:
        C_b = C_b.to(A.dtype)
    pa, pb = P.dot_backward_plans(meta_dot)
    A_b = B_b = None
    if need_a:
        A_b = run_gemm(pa, C_b, B, torch.zeros(A.numel(), dtype=A.dtype, device=A.device))
    if need_b:
        B_b = run_gemm(pb, A, C_b, torch.zeros(B.numel(), dtype=A.dtype, device=A.device))
    return A_b, B_b


def permute_blocks(data, reshape, order):
    """Blocks (sl, Di, Dl, Dr) of ``data`` permuted by ``order`` into consecutive (Dl, Dr)
    matrices; returns (buffer, offsets, plan)."""
    def build():
        tasks, offs, low = [], [], 0
        for sl, Di, Dl, Dr in reshape:
            sst = P.row_major_strides(Di)
            Dt = [Di[o] for o in order]
            tasks.append((sl[0], low, Dt, [sst[o] for o in order], P.row_major_strides(Dt)))
            offs.append(low)
            low += Dl * Dr
        return P.CopyPlan(tasks, low, low), tuple(offs)
    plan, offs = P.CACHE.get((reshape, order), ('permute_blocks',), build)
    buf = torch.empty(plan.size_dst, dtype=data.dtype, device=data.device)
    return run_copy(plan, data, buf), offs, plan


def transpose_dot_sum(A, B, meta_dot, Areshape, Breshape, Aorder, Border, Dsize):
    if _narrow_inputs(A, B):
        return transpose_dot_sum(_wide(A), _wide(B), meta_dot, Areshape, Breshape, Aorder, Border,
                                 Dsize).to(torch.promote_types(A.dtype, B.dtype))
    A, B = promote(_check(A, 'A'), _check(B, 'B'))
    Ap, Aoffs, _ = permute_blocks(A, Areshape, Aorder)
    Bp, Boffs, _ = permute_blocks(B, Breshape, Border)
    plan = P.tds_plan(meta_dot, Areshape, Breshape, Aoffs, Boffs)
    out = torch.zeros(Dsize, dtype=A.dtype, device=A.device)
    return run_gemm(plan, Ap, Bp, out)


def transpose_dot_sum_backward(C_b, A, B, meta_dot, Areshape, Breshape, Aorder, Border):
    if _narrow_inputs(C_b, A, B):
        A_b, B_b = transpose_dot_sum_backward(_wide(C_b), _wide(A), _wide(B), meta_dot, Areshape, Breshape, Aorder,
                                              Border)
        return A_b.to(A.dtype), B_b.to(B.dtype)
    A, B = promote(_check(A, 'A'), _check(B, 'B'))
    C_b = _check(C_b, 'C_b').to(A.dtype)
    Ap, Aoffs, pa_perm = permute_blocks(A, Areshape, Aorder)
    Bp, Boffs, pb_perm = permute_blocks(B, Breshape, Border)
    pa, pb = P.tds_backward_plans(meta_dot, Areshape, Breshape, Aoffs, Boffs)
    At_b = run_gemm(pa, C_b, Bp, torch.zeros(Ap.numel(), dtype=A.dtype, device=A.device))
    Bt_b = run_gemm(pb, Ap, C_b, torch.zeros(Bp.numel(), dtype=A.dtype, device=A.device))
    inv_a = P.CACHE.get((Areshape, Aorder), ('permute_blocks_bwd', A.numel()), lambda: pa_perm.swapped(A.numel()))
    inv_b = P.CACHE.get((Breshape, Border), ('permute_blocks_bwd', B.numel()), lambda: pb_perm.swapped(B.numel()))
    A_b = run_copy(inv_a, At_b, (torch.empty if inv_a.full else torch.zeros)(A.numel(), dtype=A.dtype, device=A.device))
    B_b = run_copy(inv_b, Bt_b, (torch.empty if inv_b.full else torch.zeros)(B.numel(), dtype=A.dtype, device=A.device))
    return A_b, B_b


# ----------------------------------------------------------------------------- family (c)

MAX_SWEEPS32 = 40
TOL_STOP32 = 1.0e-4   # FP32 phase ends after a sweep whose largest rotation |cos| is below this
TOL_STOP64 = 1.0e-8   # FP64 phase: idem; Jacobi converges quadratically (a sweep that starts at
                      # max |cos| c leaves ~c^2), so the residual after such a sweep is ~1e-16
TOL_STOP64_QR = 1.0e-7  # the same for the QR-preconditioned SVD (separated, graded rows: ~1e-14 left)
TOL_STOP64_EIGH = 1.0e-11  # eigh: the shifted block A + shift I (shift = ||A||_F + 1) has its singular
                           # values clustered around the shift, so a sweep that starts at |cos| c leaves
                           # ~c^2 shift / gap rather than c^2: 1e-8 left 1e-9 relative reconstruction
                           # errors on rank-deficient blocks, 1e-11 reaches the rounding level
INNER_SWEEPS32 = 1    # blocked FP32 phase: Jacobi sweeps among the rows of a super pair per visit
BLOCKED_FP32 = [True]  # FP32 phase on super-vectors in shared memory (False: one pair per warp)
BLOCKED_FP64 = [True]  # FP64 phase likewise, on 4-row super-vectors (False: one pair per warp)
ROWS_PER_SUPER = [None]  # super-vector height (None: largest of 16, 8, 4 that fits)
NS_STEPS = 2          # Newton-Schulz steps: non-orthogonality ~1e-6 -> 1e-12 -> ~eps
SVD_QR = [True]       # svd: Jacobi on the rows of R of a Householder QR (few FP64 sweeps on graded spectra)


SVD_STATE_REC = 6     # int64 words of per-block Jacobi state (yb_svd.cu)


def _svd_state_check(state, nb, phase, require_converged):
    st = state.cpu().numpy()
    R = SVD_STATE_REC
    if st[R * nb + 2] != 0:
        raise RuntimeError(f"yastn_gb300 svd: grid barrier timed out in the {phase} phase")
    conv = st[1:R * nb:R]
    if require_converged and not conv.all():
        raise torch.linalg.LinAlgError(f"yastn_gb300 svd: Jacobi did not converge ({phase} phase)")
    return st[2:R * nb:R]


def _jacobi(data, plan, U, S, V, mode, max_sweeps=MAX_SWEEPS):
    """Mixed-precision batched Jacobi of ``plan`` on ``data``; writes U, S (and Vh for mode 0)."""
    nb = len(plan.blocks)
    dev = data.device
    code = _dtype_code(data.dtype)
    cplx = code == N.YB_C128
    dblocks, dpairs = _dev(plan, 'svd', (plan.blocks, plan.pair_items), dev)
    w64 = torch.empty(plan.n64, dtype=torch.complex128 if cplx else torch.float64, device=dev)
    w32 = torch.empty(plan.n32, dtype=torch.complex64 if cplx else torch.float32, device=dev)
    state = torch.zeros(SVD_STATE_REC * nb + 4, dtype=torch.int64, device=dev)
    aux = torch.empty(2 * nb, dtype=torch.float64, device=dev)  # [scale | shift]
    shift = aux[nb:] if mode != 0 else None
    sp = _vp(shift.data_ptr() if shift is not None else 0)
    st = _stream()
    qctrl = None
    if plan.qr:
        qctrl = torch.zeros(nb + 4 * min(nb, 4096), dtype=torch.int64, device=dev)
        N.call('yb_svd_qr', _ptr(data), _ptr(w64), _ptr(w32), _ptr(dblocks), nb, code, _ptr(state), _ptr(aux[:nb]),
               _ptr(qctrl), qctrl.numel(), st, launches=4)
    else:
        N.call('yb_svd_init', _ptr(data), _ptr(w32), _ptr(dblocks), nb, code, _ptr(state), sp, _ptr(aux[:nb]), st,
               launches=2)
    if plan.rows_per_super and BLOCKED_FP32[0]:
        (dsup,) = _dev(plan, 'svd_super', (plan.super_items,), dev)
        N.call('yb_svd_block_sweeps', _ptr(w32), _ptr(dblocks), nb, _ptr(dsup), len(plan.super_items),
               plan.super_rounds, plan.rows_per_super, 32, code, MAX_SWEEPS32, INNER_SWEEPS32, TOL_STOP32,
               plan.lmax, _ptr(state), st)
    else:
        N.call('yb_svd_sweeps', _ptr(w32), _ptr(dblocks), nb, _ptr(dpairs), len(plan.pair_items), plan.max_rounds,
               32, code, MAX_SWEEPS32, TOL_STOP32, _ptr(state), st)
    _svd_state_check(state, nb, 'FP32', False)
    if qctrl is not None and bool(qctrl[nb + 2::4].any()):
        raise RuntimeError("yastn_gb300 svd: QR group barrier timed out")
    N.call('yb_svd_widen', _ptr(w32), _ptr(w64), _ptr(dblocks), nb, code, _ptr(state), st)
    w0, t0, n0, ws = plan.w_range
    W, Wn = w64[w0:w0 + ws], w64[n0:n0 + ws]
    for _ in range(NS_STEPS):
        Wn.copy_(W)
        run_gemm(plan.gram, w64, w64, w64)
        run_gemm(plan.ns, w64, w64, w64, alpha=-0.5, beta=1.5)
        W.copy_(Wn)
    if plan.qr:
        run_gemm(plan.xform, w64, w64, w64)  # X = W R
    elif shift is not None:
        N.call('yb_svd_shift_prefill', _ptr(w64), _ptr(dblocks), nb, code, _ptr(shift), st)
        run_gemm(plan.xform, w64, data, w64, beta=1.0)
    else:
        run_gemm(plan.xform, w64, data, w64)
    tol64 = TOL_STOP64_QR if plan.qr else (TOL_STOP64 if mode == 0 else TOL_STOP64_EIGH)
    if plan.rows_per_super64 and BLOCKED_FP64[0]:
        (dsup64,) = _dev(plan, 'svd_super64', (plan.super_items64,), dev)
        N.call('yb_svd_block_sweeps', _ptr(w64), _ptr(dblocks), nb, _ptr(dsup64), len(plan.super_items64),
               plan.super_rounds64, plan.rows_per_super64, 64, code, max_sweeps, 1, tol64, plan.lmax,
               _ptr(state), st)
    else:
        N.call('yb_svd_sweeps', _ptr(w64), _ptr(dblocks), nb, _ptr(dpairs), len(plan.pair_items), plan.max_rounds,
               64, code, max_sweeps, tol64, _ptr(state), st)
    _svd_state_check(state, nb, 'FP64', True)
    n_small = torch.zeros(nb, dtype=torch.int64, device=dev) if mode == 0 else None
    N.call('yb_svd_finalize', _ptr(w64), _ptr(U), _ptr(S), _vp(V.data_ptr() if V is not None else 0), _ptr(dblocks),
           nb, code, plan.max_k, mode, sp, _ptr(state), _vp(n_small.data_ptr() if n_small is not None else 0), st)
    if n_small is not None:
        nz = n_small.cpu().numpy()
        if nz.any():
            _complete(plan, U, V, nz, cplx)
    if plan.qr:  # the factor that comes from Q: Vh = conj(W) Q^T (wide), U = conj(Q) W^T (tall)
        run_gemm(plan.qfin_v, w64, w64, V)
        run_gemm(plan.qfin_u, w64, w64, U)


def _complete(plan, U, V, nz, cplx):
    """Blocked completion of the vectors of small singular values (blocks left by
    yb_svd_finalize): per block, nz candidate vectors with entries uniform in [-1, 1)
    (yb_fill_candidates), projected twice off the k - nz earlier vectors by grouped GEMMs
    (C = V_g^H G, G -= V_g C), orthonormalised by the batched Householder QR, and copied into
    the factor's last nz vectors (U columns or Vh rows, whichever the rows of X built)."""
    key = tuple(int(x) for x in nz)
    cache = plan.__dict__.setdefault('_completion', {})
    if key not in cache:
        cache[key] = P.completion_plans(plan.blocks, nz, cplx)
    dev = U.device
    for cp in cache[key]:
        F = U if cp.to_u else V
        G = torch.empty(max(cp.G, 1), dtype=F.dtype, device=dev)
        C = torch.empty(max(cp.C, 1), dtype=F.dtype, device=dev)
        (dfill,) = _dev(cp, 'fill', (cp.fill,), dev)
        N.call('yb_fill_candidates', _ptr(G), _ptr(dfill), len(cp.fill), _dtype_code(F.dtype), _stream())
        for _ in range(2):
            run_gemm(cp.g1, F, G, C)
            run_gemm(cp.g2, F, C, G, alpha=-1.0, beta=1.0)
        Qc, _ = qr(G, cp.meta, (max(cp.Q, 1), max(cp.R, 1)))
        run_copy(cp.copy, Qc, F)


def svd(data, meta, sizes, max_sweeps=MAX_SWEEPS):
    """Thin SVD of every block (one-sided Jacobi); returns (U, S, Vh) flat tensors."""
    data = _check(data)
    dev = data.device
    U = torch.empty(sizes[0], dtype=data.dtype, device=dev)
    S = torch.empty(sizes[1], dtype=torch.float64, device=dev)
    V = torch.empty(sizes[2], dtype=data.dtype, device=dev)
    plan = P.svd_plan(meta, ROWS_PER_SUPER[0], data.is_complex(), qr=SVD_QR[0])
    if len(plan.blocks) == 0:
        return U, S, V
    _jacobi(data, plan, U, S, V, 0, max_sweeps)
    return U, S, V


def qr(data, meta, sizes):
    """Reduced QR of every block with R's diagonal made positive (backend_np.py:511-520):
    the batched Householder factorisation of yb_svd_qr, then R[:, m:] = Q^H A[:, m:] for
    wide blocks by a grouped GEMM. Returns (Q, R) flat tensors."""
    data = _check(data)
    dev = data.device
    Q = torch.zeros(sizes[0], dtype=data.dtype, device=dev)
    R = torch.zeros(sizes[1], dtype=data.dtype, device=dev)
    plan = P.qr_plan(meta, data.is_complex())
    nb = len(plan.blocks)
    if nb == 0:
        return Q, R
    (dblocks,) = _dev(plan, 'qr', (plan.blocks,), dev)
    work = torch.empty(plan.n64, dtype=data.dtype, device=dev)
    qctrl = torch.zeros(nb + 4 * min(nb, 4096), dtype=torch.int64, device=dev)
    N.call('yb_qr', _ptr(data), _ptr(Q), _ptr(R), _ptr(work), _ptr(dblocks), nb, _dtype_code(data.dtype),
           _ptr(qctrl), qctrl.numel(), _stream(), launches=4)
    run_gemm(plan.right, Q, data, R)
    if bool(qctrl[nb + 2::4].any()):
        raise RuntimeError("yastn_gb300 qr: QR group barrier timed out")
    return Q, R


def qr_backward(Q, R, gQ, gR, data, meta):
    """Adjoint of ``qr`` for float64 and complex128 blocks (the reduced-QR rule that torch's
    autograd applies to the reference's torch.linalg.qr + sign fix, backend_torch.py:475-484):
    dA = (gQ' + Q copyltu(M)) U^{-H}, M = U gU^H - gQ'^H Q, with U = R[:, :k], gU = gR[:, :k],
    gQ' = gQ + A[:, m:] gR[:, m:]^H and dA[:, m:] = Q gR[:, m:] for wide blocks;
    copyltu(M) = tril(M, -1) + tril(M, -1)^H + Re diag(M) (gradients in torch's convention
    for complex tensors)."""
    plan = P.qr_plan(meta, Q.is_complex())
    dev = Q.device
    dA = torch.zeros(data.numel(), dtype=data.dtype, device=dev)
    if len(plan.blocks) == 0:
        return dA
    Bw = torch.zeros_like(Q) if gQ is None else _plain(gQ).to(Q.dtype).clone()
    gR = torch.zeros_like(R) if gR is None else _plain(gR).to(R.dtype)
    M = torch.empty(plan.m_size, dtype=Q.dtype, device=dev)
    run_gemm(plan.w1, data, gR, Bw, beta=1.0)
    run_gemm(plan.m1, R, gR, M)
    run_gemm(plan.m2, Bw, Q, M, alpha=-1.0, beta=1.0)
    (drecs,) = _dev(plan, 'qradj', (plan.adj,), dev)
    code = _dtype_code(Q.dtype)
    N.call('yb_qr_adjoint_sym', _ptr(M), _ptr(drecs), len(plan.adj), code, _stream())
    run_gemm(plan.s1, Q, M, Bw, beta=1.0)
    N.call('yb_trsm_rt', _ptr(Bw), _ptr(R), _ptr(drecs), len(plan.adj), code, _stream())
    if not hasattr(plan, 'copy_plan'):
        plan.copy_plan = P.CopyPlan(plan.copies, sum(int(np.prod(c[2])) for c in plan.copies), data.numel())
    run_copy(plan.copy_plan, Bw, dA)
    run_gemm(plan.y1, Q, gR, dA)
    return dA


def svd_backward(U, S, V, gU, gS, gV, meta, data_size, dtype):
    """Regularised SVD adjoint of every block (torch_svd_gesdd.py:296-428) in 7 launches."""
    plan = P.svd_adjoint_plan(meta)
    dev = U.device
    dA = torch.zeros(data_size, dtype=dtype, device=dev)
    if len(plan.recs) == 0:
        return dA
    code = _dtype_code(U.dtype)
    gU = torch.zeros_like(U) if gU is None else _plain(gU).to(U.dtype)
    gV = torch.zeros_like(V) if gV is None else _plain(gV).to(V.dtype)
    gS = None if gS is None else _plain(gS).to(torch.float64)
    Pm = torch.empty(plan.kk, dtype=U.dtype, device=dev)
    Qm = torch.empty(plan.kk, dtype=U.dtype, device=dev)
    Km = torch.empty(plan.kk, dtype=U.dtype, device=dev)
    TR = torch.empty(max(plan.tr, 1), dtype=U.dtype, device=dev)
    run_gemm(plan.gP, U, gU, Pm)
    run_gemm(plan.gQ, V, gV, Qm)
    (drecs,) = _dev(plan, 'adj', (plan.recs,), dev)
    N.call('yb_svd_adjoint_core', _ptr(Pm), _ptr(Qm), _ptr(S), _vp(gS.data_ptr() if gS is not None else 0), _ptr(Km),
           _ptr(gU), _ptr(gV), _ptr(TR), _ptr(drecs), len(plan.recs), code, _stream())
    run_gemm(plan.gT, Km, V, TR, beta=1.0)
    run_gemm(plan.gR, U, Km, TR, beta=1.0)
    run_gemm(plan.gA1, U, TR, dA)
    run_gemm(plan.gA2, TR, V, dA)
    if not (dtype.is_complex if hasattr(dtype, 'is_complex') else False) and dA.is_complex():
        dA = dA.real.contiguous()
    return dA


def eigh(data, meta, sizes, order_by_magnitude=False, max_sweeps=MAX_SWEEPS):
    """Hermitian eigendecomposition of every block (records (sl, D, slU, DU, slS) of
    yastn/backend/backend_np.py:461-474): eigenvalues ascending, or by descending
    magnitude when ``order_by_magnitude`` (yastn/backend/linalg/torch_eig_sym.py:25-32)."""
    data = _check(data)
    dev = data.device
    S = torch.zeros(sizes[0], dtype=torch.float64, device=dev)
    U = torch.zeros(sizes[1], dtype=data.dtype, device=dev)
    svd_meta = tuple((sl, D, slU, DU, slS, (0, 0), (DU[1], D[1])) for sl, D, slU, DU, slS in meta)
    plan = P.svd_plan(svd_meta, ROWS_PER_SUPER[0], data.is_complex())
    if len(plan.blocks) == 0:
        return S, U
    _jacobi(data, plan, U, S, None, 2 if order_by_magnitude else 1, max_sweeps)
    return S, U


def eigh_backward(U, S, gU, gS, meta, data_size, dtype, order_by_magnitude=False, eps=1.0e-12):
    """Adjoint of ``eigh`` on every block in 4 launches: X = op(U)^T gU, the inner matrix K
    (csrc/yb_adjoint.cu), T = U K, dA = T op(U)^T. order_by_magnitude follows SYMEIG
    (yastn/backend/linalg/torch_eig_sym.py:43-54), otherwise torch.linalg.eigh's adjoint."""
    cplx = U.is_complex()
    plan = P.eigh_adjoint_plan(meta, bool(order_by_magnitude), cplx)
    dev = U.device
    dA = torch.zeros(data_size, dtype=dtype, device=dev)
    if len(plan.recs) == 0:
        return dA
    gU = torch.zeros_like(U) if gU is None else _plain(gU).to(U.dtype)
    gS = None if gS is None else _plain(gS).to(torch.float64)
    X = torch.empty(plan.kk, dtype=U.dtype, device=dev)
    K = torch.empty(plan.kk, dtype=U.dtype, device=dev)
    run_gemm(plan.gX, U, gU, X)
    (drecs,) = _dev(plan, 'eigh_adj', (plan.recs,), dev)
    N.call('yb_eigh_adjoint_core', _ptr(X), _ptr(S), _vp(gS.data_ptr() if gS is not None else 0), _ptr(K),
           _ptr(drecs), len(plan.recs), _dtype_code(U.dtype), int(bool(order_by_magnitude)), float(eps), _stream())
    run_gemm(plan.gT, U, K, X)
    run_gemm(plan.gA, X, U, dA)
    return dA


def fix_svd_signs(U, V, meta):
    """Gauge fix of every block; returns (U', Vh', phases)."""
    U, V = _check(U, 'U'), _check(V, 'V')
    plan = P.fix_signs_plan(meta)
    nb = len(plan.blocks)
    Uo, Vo = torch.empty_like(U), torch.empty_like(V)
    S_size = max((int(r[4] + r[9]) for r in plan.blocks), default=0)
    phases = torch.zeros(S_size, dtype=U.dtype, device=U.device)
    if nb == 0:
        return U.clone(), V.clone(), phases
    (dblocks,) = _dev(plan, 'svd_blocks', (plan.blocks,), U.device)
    N.call('yb_fix_signs', _ptr(U), _ptr(V), _ptr(Uo), _ptr(Vo), _ptr(phases), _ptr(dblocks), nb, plan.max_k,
           _dtype_code(U.dtype), 0, _stream())
    return Uo, Vo, phases


def fix_svd_signs_backward(U, V, gU, gV, meta):
    """Adjoint of the gauge fix (real and complex; yb_fix_signs_adjoint) given the forward's
    inputs U, V and the cotangents of its outputs."""
    plan = P.fix_signs_plan(meta)
    nb = len(plan.blocks)
    need_u, need_v = gU is not None, gV is not None
    gU = torch.zeros_like(U) if gU is None else _plain(gU).to(U.dtype)
    gV = torch.zeros_like(V) if gV is None else _plain(gV).to(V.dtype)
    dU, dV = torch.zeros_like(U), torch.zeros_like(V)  # the kernel writes every position of the records
    if nb:
        (dblocks,) = _dev(plan, 'svd_blocks', (plan.blocks,), U.device)
        N.call('yb_fix_signs_adjoint', _ptr(U), _ptr(V), _ptr(gU), _ptr(gV), _ptr(dU), _ptr(dV), _ptr(dblocks), nb,
               plan.max_k, _dtype_code(U.dtype), _stream())
    return (dU if need_u else None), (dV if need_v else None)


# ----------------------------------------------------------------------------- masks / truncation

def _idx_buffer(mask, meta, device, axis=0):
    """The masks' kept indices concatenated in one device buffer, and per mask (per mask and
    axis length for slice masks, which YASTN passes for whole-axis copies) its offset and
    count."""
    order, lengths, off = [], {}, 0
    for rec in meta:
        tm = rec[4]
        v = mask[tm]
        if isinstance(v, slice):
            Da = (rec[3],) if isinstance(rec[3], int) else rec[3]
            key = (tm, Da[axis])
            if key in lengths:
                continue
            ind = torch.arange(*v.indices(Da[axis]), dtype=torch.int64, device=device)
        else:
            key = tm
            if key in lengths:
                continue
            ind = torch.as_tensor(v, device=device).reshape(-1).to(torch.int64)
        lengths[key] = (off, int(ind.numel()))
        order.append(ind)
        off += int(ind.numel())
    idx = torch.cat(order) if order else torch.zeros(1, dtype=torch.int64, device=device)
    return idx, lengths


def apply_mask(A, mask, meta, Dsize, axis, ndim, scatter_size=None):
    """Gather kept indices along ``axis`` (scatter_size given: the adjoint scatter)."""
    A = _check(A, any_dtype=True)
    idx, lengths = _idx_buffer(mask, meta, A.device, axis)
    recs, items, _ = P.mask_plan(meta, axis, lengths)
    if scatter_size is None:
        out = torch.empty(Dsize, dtype=A.dtype, device=A.device)
    else:
        out = torch.zeros(scatter_size, dtype=A.dtype, device=A.device)
    if len(items) == 0:
        return out
    drecs = torch.from_numpy(recs).to(A.device)
    ditems = torch.from_numpy(items).to(A.device)
    N.call('yb_mask_gather', _ptr(A), _ptr(out), A.element_size(), _ptr(drecs), _ptr(ditems), len(items), _ptr(idx),
           int(scatter_size is not None), _stream())
    return out


def truncation_mask_data(S, slices, charges=None, tol=0, tol_block=0, D_block=float('inf'), D_total=float('inf'),
                         truncate_multiplets=False):
    """The truncation rule of yastn/tensor/linalg.py:637-735 in one device launch.

    ``S`` is the flat float64 spectrum on the device, ``slices`` the (start, stop) of
    each block, ``charges`` the block charges (needed when tol_block/D_block are dicts).
    Returns (mask: bool CUDA tensor, kept: list of kept counts per block).
    """
    S = _check(S, 'S')
    if S.dtype != torch.float64:
        raise TypeError("truncation requires a real float64 spectrum")
    n = S.numel()
    nb = len(slices)
    # the kernel locates blocks by binary search over ascending starts: order them here and
    # return the kept counts in the caller's order
    order = sorted(range(nb), key=lambda i: slices[i][0])
    if order != list(range(nb)):
        slices = [slices[i] for i in order]
        charges = None if charges is None else [charges[i] for i in order]
        mask, kept_sorted = truncation_mask_data(S, slices, charges, tol, tol_block, D_block, D_total,
                                                 truncate_multiplets)
        kept = [0] * nb
        for j, i in enumerate(order):
            kept[i] = kept_sorted[j]
        return mask, kept
    if truncate_multiplets:
        tol_block, D_block = 0, float('inf')
    blk = np.zeros((max(nb, 1), 4), dtype=np.int64)
    tb = np.zeros(max(nb, 1), dtype=np.float64)
    tol_null = 0. if isinstance(tol_block, dict) else tol_block
    D_null = 0 if isinstance(D_block, dict) else D_block
    for i, (lo, hi) in enumerate(slices):
        t = tuple(charges[i]) if charges is not None else None
        tb[i] = tol_block[t] if (isinstance(tol_block, dict) and t in tol_block) else tol_null
        d = D_block[t] if (isinstance(D_block, dict) and t in D_block) else D_null
        blk[i] = (lo, hi, -1 if d == float('inf') else int(d), 0)
    dt = -1 if D_total == float('inf') else int(D_total)
    mask = torch.empty(n, dtype=torch.uint8, device=S.device)
    kept = torch.empty(max(nb, 1), dtype=torch.int64, device=S.device)
    if nb == 0 or n == 0:
        return mask.bool(), [0] * nb
    dblk = torch.from_numpy(blk).to(S.device)
    dtb = torch.from_numpy(tb).to(S.device)
    N.call('yb_truncation_mask', _ptr(S), n, _ptr(dblk), _ptr(dtb), nb, float(tol), dt, int(bool(truncate_multiplets)),
           _ptr(mask), _ptr(kept), _stream())
    return mask.view(torch.bool), kept[:nb].tolist()
