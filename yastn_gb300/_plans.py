"""Plan compiler: YASTN metadata tuples -> packed int64 device records.

YASTN's metadata layer hands the backend nested tuples (``meta_new``/``meta_mrg`` of
``transpose_and_merge``, unmerge records, ``meta_dot``, svd records). Each plan below
turns one such tuple into the flat records of the C ABI (``include/yastn_gb300.h``).
Plans depend only on the metadata, so they are cached by the identity of the tuple
(YASTN memoises its metadata with ``lru_cache``, so the same tuple object comes back)
and, failing that, by value.
"""
import pickle
from collections import OrderedDict

import numpy as np

# record layout constants (must match include/yastn_gb300.h)
COPY_REC, CP_SRC, CP_DST, CP_NDIM, CP_COUNT, CP_VEC = 48, 0, 1, 2, 3, 4
CP_MAXD, CP_SIZE, CP_SSTR, CP_DSTR, CP_MAGIC, CP_SHIFT = 8, 8, 16, 24, 32, 40
CP_KIND, CP_NX, CP_NY = 5, 6, 7
COPY_ITEM_UNITS, COPY_TILE, COPY_ITEM_TILES = 2048, 32, 2
GEMM_OUT_REC, GEMM_TERM_REC, GEMM_TILE = 8, 8, 64
SVD_REC = 24
MASK_REC = 8


class PlanError(ValueError):
    """The metadata cannot be expressed as a plan of the C ABI."""


# ----------------------------------------------------------------------------- caching

class PlanCache:
    """LRU cache keyed by metadata identity with a by-value fallback."""

    def __init__(self, maxsize=32768):
        self.by_id = OrderedDict()
        self.by_val = OrderedDict()
        self.maxsize = maxsize
        self.hits = 0
        self.misses = 0

    def get(self, key_objs, extra, build):
        kid = (tuple(id(o) for o in key_objs), extra)
        ent = self.by_id.get(kid)
        if ent is not None and all(a is b for a, b in zip(ent[0], key_objs)):
            self.by_id.move_to_end(kid)
            self.hits += 1
            return ent[1]
        kval = (tuple(key_objs), extra)
        try:
            plan = self.by_val.get(kval)
        except TypeError:  # unhashable metadata (e.g. masks): no by-value cache
            kval, plan = None, None
        if plan is None:
            self.misses += 1
            plan = build()
            if kval is not None:
                self.by_val[kval] = plan
                if len(self.by_val) > self.maxsize:
                    self.by_val.popitem(last=False)
        else:
            self.hits += 1
        self.by_id[kid] = (tuple(key_objs), plan)
        if len(self.by_id) > self.maxsize:
            self.by_id.popitem(last=False)
        return plan


CACHE = PlanCache()


def cache_info():
    return {'hits': CACHE.hits, 'misses': CACHE.misses, 'size': len(CACHE.by_id)}


# ----------------------------------------------------------------------------- serialization

PLAN_FILE_VERSION = 1
_DEVICE_ONLY = ('_dev', 'tuned_tc')  # per-process state: device copies, autotuned kernel choices


class _PlanPickler(pickle.Pickler):
    """Pickles plans without their device state (torch tensors are written as None)."""

    def reducer_override(self, obj):
        import torch
        if isinstance(obj, torch.Tensor):
            return type(None), ()
        return NotImplemented


def _reset_device_state(obj, seen):
    """Drop the per-process state of every plan reachable from obj (after unpickling)."""
    if id(obj) in seen:
        return
    seen.add(id(obj))
    if isinstance(obj, (list, tuple)):
        for x in obj:
            _reset_device_state(x, seen)
        return
    if isinstance(obj, dict):
        for x in obj.values():
            _reset_device_state(x, seen)
        return
    d = getattr(obj, '__dict__', None)
    if d is None or type(obj).__module__ != __name__:
        return
    for k in _DEVICE_ONLY:
        if k == '_dev':
            if k in d:
                d[k] = {}
        else:
            d.pop(k, None)
    for v in list(d.values()):
        _reset_device_state(v, seen)


def save_cache(path):
    """Write every plan of the cache (keyed by its metadata by value) to ``path``, without
    device state, so that a later process (``load_cache``) skips building them: a long CTMRG
    or DMRG run restarts with the plans of its metadata ready. The file is a pickle: load only
    files this library wrote."""
    entries = [(k, v) for k, v in CACHE.by_val.items()]
    with open(path, 'wb') as f:
        _PlanPickler(f, protocol=pickle.HIGHEST_PROTOCOL).dump({'version': PLAN_FILE_VERSION, 'entries': entries})
    return len(entries)


def load_cache(path):
    """Add the plans saved by ``save_cache`` to the cache (by value: the first lookup of a
    metadata tuple finds its plan without building it). Returns the number of plans loaded."""
    with open(path, 'rb') as f:
        payload = pickle.load(f)
    if payload.get('version') != PLAN_FILE_VERSION:
        raise PlanError(f"plan file version {payload.get('version')} (this library reads {PLAN_FILE_VERSION})")
    n = 0
    for key, plan in payload['entries']:
        _reset_device_state(plan, set())
        CACHE.by_val[key] = plan
        n += 1
    while len(CACHE.by_val) > CACHE.maxsize:
        CACHE.by_val.popitem(last=False)
    return n


# ----------------------------------------------------------------------------- helpers

def fast_div_consts(d):
    """(magic, shift) with n // d == (umulhi(n, magic) + n) >> shift for 0 <= n < 2^31."""
    if d < 1 or d >= 2 ** 31:
        raise PlanError(f"extent {d} out of range for 32-bit fast division")
    shift = 0
    while (1 << shift) < d:
        shift += 1
    magic = ((1 << 32) * ((1 << shift) - d)) // d + 1
    return magic & 0xFFFFFFFF, shift


def row_major_strides(D):
    st = [1] * len(D)
    for i in range(len(D) - 2, -1, -1):
        st[i] = st[i + 1] * D[i + 1]
    return st


def group_dims(dims, targets):
    """Assign consecutive ``dims`` to groups whose products equal ``targets``.

    Returns a list with the group index of every dim. Dims of extent 1 may sit in
    any group; they are attached to the current group.
    """
    G = len(targets)
    out = []
    g, prod = 0, 1
    for d in dims:
        while g < G - 1 and prod == targets[g] and d != 1:
            g, prod = g + 1, 1
        prod *= d
        out.append(g)
    # trailing groups of product 1 are legal
    prods = [1] * G
    for d, gi in zip(dims, out):
        prods[gi] *= d
    if tuple(prods) != tuple(targets):
        raise PlanError(f"cannot split dims {dims} into consecutive groups {targets}")
    return out


def _collapse(sizes, ss, ds):
    """Drop extent-1 dims and merge neighbours contiguous in both source and destination."""
    dims = [(n, a, b) for n, a, b in zip(sizes, ss, ds) if n != 1]
    if not dims:
        return [1], [1], [1]
    out = [list(dims[0])]
    for n, a, b in dims[1:]:
        pn, pa, pb = out[-1]
        if pa == a * n and pb == b * n:
            out[-1] = [pn * n, a, b]
        else:
            out.append([n, a, b])
    return [x[0] for x in out], [x[1] for x in out], [x[2] for x in out]


def _transpose_task(so, do, sizes, ss, ds):
    """Tiled-transpose record (kind 1) for a collapsed task whose destination is contiguous
    along the innermost dim x and whose source is contiguous along another dim y; None if
    the task is not such a transpose (or too narrow to profit)."""
    last = len(sizes) - 1
    if last < 1 or ds[last] != 1 or ss[last] == 1 or sizes[last] < 4:
        return None
    ys = [j for j in range(last) if ss[j] == 1 and sizes[j] >= 4]
    if not ys:
        return None
    y = ys[-1]
    outer = [j for j in range(last) if j != y]
    T = COPY_TILE
    ty, tx = -(-sizes[y] // T), -(-sizes[last] // T)
    dims = [(sizes[j], ss[j], ds[j]) for j in outer] + [(ty, T, T * ds[y]), (tx, T * ss[last], T)]
    count = int(np.prod([d[0] for d in dims], dtype=np.int64))
    if count >= 2 ** 31:
        raise PlanError("copy task larger than 2^31 tiles")
    rec = np.zeros(COPY_REC, dtype=np.int64)
    rec[CP_SRC], rec[CP_DST], rec[CP_NDIM], rec[CP_COUNT], rec[CP_VEC] = so, do, len(dims), count, 0
    rec[CP_KIND], rec[CP_NX], rec[CP_NY] = 1, sizes[last], sizes[y]
    for i, (n, a, b) in enumerate(dims):
        m, sh = fast_div_consts(n)
        rec[CP_SIZE + i], rec[CP_SSTR + i], rec[CP_DSTR + i] = n, a, b
        rec[CP_MAGIC + i], rec[CP_SHIFT + i] = m, sh
    return rec


class CopyPlan:
    """Host copy of a family-(a) plan: tasks, items, element coverage."""

    def __init__(self, tasks, covered, size_dst):
        self.tasks_list = tasks  # list of (src_off, dst_off, sizes, sstr, dstr) in elements
        self.covered = covered
        self.size_dst = size_dst
        self.full = covered == size_dst
        self._packed = {}
        self._dev = {}

    def swapped(self, size_src):
        """The inverse copy (adjoint): source and destination exchanged."""
        t = [(d, s, sz, dd, sd) for (s, d, sz, sd, dd) in self.tasks_list]
        return CopyPlan(t, self.covered, size_src)

    def packed(self, vec_ok):
        """(tasks int64 [n, COPY_REC], items int64 [m, 2]) with 16-byte units where allowed."""
        if vec_ok in self._packed:
            return self._packed[vec_ok]
        recs, items = [], []
        expanded = []
        for (so, do, sizes, ss, ds) in self.tasks_list:
            sizes, ss, ds = _collapse(sizes, ss, ds)
            if len(sizes) <= CP_MAXD:
                expanded.append((so, do, sizes, ss, ds))
                continue
            # more dims than a record holds (tensors of a dozen legs): one record per index of
            # the leading dims, each with the trailing CP_MAXD dims
            lead = len(sizes) - CP_MAXD
            for idx in np.ndindex(*sizes[:lead]):
                o_s = so + sum(int(i) * int(x) for i, x in zip(idx, ss[:lead]))
                o_d = do + sum(int(i) * int(x) for i, x in zip(idx, ds[:lead]))
                expanded.append((o_s, o_d, sizes[lead:], ss[lead:], ds[lead:]))
        for (so, do, sizes, ss, ds) in expanded:
            ti = len(recs)
            tr = _transpose_task(so, do, sizes, ss, ds)
            if tr is not None:
                recs.append(tr)
                items.extend((ti, f) for f in range(0, int(tr[CP_COUNT]), COPY_ITEM_TILES))
                continue
            vec = 0
            if vec_ok and ss[-1] == 1 and ds[-1] == 1 and sizes[-1] % 2 == 0 and so % 2 == 0 and do % 2 == 0 \
                    and all(x % 2 == 0 for x in ss[:-1]) and all(x % 2 == 0 for x in ds[:-1]):
                vec = 1
                sizes = sizes[:-1] + [sizes[-1] // 2]
                ss = [x // 2 for x in ss[:-1]] + [1]
                ds = [x // 2 for x in ds[:-1]] + [1]
                so, do = so // 2, do // 2
            count = int(np.prod(sizes, dtype=np.int64))
            if count >= 2 ** 31:
                raise PlanError("copy task larger than 2^31 units")
            rec = np.zeros(COPY_REC, dtype=np.int64)
            rec[CP_SRC], rec[CP_DST], rec[CP_NDIM], rec[CP_COUNT], rec[CP_VEC] = so, do, len(sizes), count, vec
            for i, (n, a, b) in enumerate(zip(sizes, ss, ds)):
                m, sh = fast_div_consts(n)
                rec[CP_SIZE + i], rec[CP_SSTR + i], rec[CP_DSTR + i] = n, a, b
                rec[CP_MAGIC + i], rec[CP_SHIFT + i] = m, sh
            recs.append(rec)
            items.extend((ti, f) for f in range(0, count, COPY_ITEM_UNITS))
        tasks = np.stack(recs) if recs else np.zeros((0, COPY_REC), dtype=np.int64)
        items = np.array(items, dtype=np.int64).reshape(-1, 2)
        self._packed[vec_ok] = (tasks, items)
        return self._packed[vec_ok]


# ----------------------------------------------------------------------------- merge / unmerge

def merge_plan(order, meta_new, meta_mrg, Dsize):
    """Plan of transpose_and_merge (restating yastn/backend/backend_np.py:653-661)."""
    def build():
        order_ = tuple(order)
        tasks, covered = [], 0
        it = iter(meta_new)
        cur = None
        for tn, slo, Do, Dslc, Drsh in meta_mrg:
            if cur is None or cur[0] != tn:
                cur = next(it)
                while cur[0] != tn:
                    cur = next(it)
            _, Dn, sln = cur
            ndim = len(Do)
            sst = row_major_strides(Do)
            Dt = [Do[o] for o in order_]
            tss = [sst[o] for o in order_]
            groups = group_dims(Dt, Drsh)
            dn_str = row_major_strides(Dn)
            dst = [0] * ndim
            for gi in range(len(Drsh)):
                members = [i for i in range(ndim) if groups[i] == gi]
                w = 1
                for i in reversed(members):
                    dst[i] = w * dn_str[gi]
                    w *= Dt[i]
            doff = sln[0] + sum(s[0] * st for s, st in zip(Dslc, dn_str))
            n = int(np.prod(Do, dtype=np.int64))
            if n == 0:
                continue
            tasks.append((slo[0], doff, Dt, tss, dst))
            covered += n
        return CopyPlan(tasks, covered, Dsize)
    return CACHE.get((order, meta_new, meta_mrg), ('merge', Dsize), build)


def unmerge_plan(meta, size):
    """Plan of unmerge (restating yastn/backend/backend_np.py:664-669)."""
    def build():
        tasks, covered = [], 0
        for sln, Dn, slo, Do, sub_slc in meta:
            n = int(np.prod(Dn, dtype=np.int64))
            if n == 0:
                continue
            widths = [b - a for a, b in sub_slc]
            groups = group_dims(list(Dn), widths)
            do_str = row_major_strides(Do)
            ss = [0] * len(Dn)
            for gi in range(len(widths)):
                members = [i for i in range(len(Dn)) if groups[i] == gi]
                w = 1
                for i in reversed(members):
                    ss[i] = w * do_str[gi]
                    w *= Dn[i]
            soff = slo[0] + sum(a * st for (a, _), st in zip(sub_slc, do_str))
            tasks.append((soff, sln[0], list(Dn), ss, row_major_strides(Dn)))
            covered += n
        return CopyPlan(tasks, covered, size)
    return CACHE.get((meta,), ('unmerge', size), build)


def transpose_plan(axes, meta_transpose, size):
    """Plan of transpose (yastn/backend/backend_np.py:646-650): blocks permuted in place."""
    def build():
        tasks, covered = [], 0
        for sln, Dn, slo, Do in meta_transpose:
            n = int(np.prod(Do, dtype=np.int64))
            if n == 0:
                continue
            sst = row_major_strides(Do)
            tasks.append((slo[0], sln[0], [Do[a] for a in axes], [sst[a] for a in axes], row_major_strides(Dn)))
            covered += n
        return CopyPlan(tasks, covered, size)
    return CACHE.get((axes, meta_transpose), ('transpose', size), build)


# ----------------------------------------------------------------------------- grouped GEMM

class GemmPlan:
    """Grouped GEMM records: the outputs computed directly (outs, terms, tiles) and, when
    some outputs' K range is split, their partial products and reduction (``split``)."""

    def __init__(self, outs, terms, tiles, flops, split=None):
        self.outs = outs
        self.terms = terms
        self.tiles = tiles
        self.flops = flops  # real multiply-adds x 2 (complex counted by the caller)
        self.split = split
        # every tile a short skinny one: the plan runs on the kernel of those alone
        self.all_short = bool(len(tiles)) and bool((tiles[:, 3] == 2).all())
        self._dev = {}


class SplitK:
    """Partial products of split outputs into a workspace (outs/terms/tiles addressed in it),
    and the reduction records (c offset, m, n, ldc, p offset, chunks) with their tasks."""

    def __init__(self, outs, terms, tiles, red, tasks, ws):
        self.outs, self.terms, self.tiles = outs, terms, tiles
        self.red, self.tasks, self.ws = red, tasks, ws


SKINNY_ROWS, SKINNY_COLS = 8, 1024  # skinny tiles: up to 8 rows (the kernel takes 16), 1024 columns
                                    # (256 above 8 rows)
SKINNY_WIDE_ROWS, SKINNY_WIDE_N = 16, 4096  # outputs of 9..16 rows take skinny tiles when this wide
SHORT_K, SHORT_COLS = 8, 512  # short skinny tiles (kind 2): one term with K <= 8, 512 columns
TALL_COLS, TALL_ROWS = 16, 256  # tall skinny tiles (kind 3): all n <= 16 columns x 256 rows


def skinny_cols(rows):
    return SKINNY_COLS if rows <= 8 else SKINNY_COLS // 4


def tile_kind(m, n, ks=None):
    """0: 64x64 tiles; 1: skinny tiles over the m <= 16 rows (m <= 8 and n > 64, or
    m <= 16 and n >= SKINNY_WIDE_N); 2: short skinny tiles (m <= 8 rows and a single term whose
    K <= SHORT_K, any n; ``ks`` = the output's term lengths); 3: tall skinny tiles over the
    n <= 16 columns (m > 64)."""
    if m <= SKINNY_ROWS and ks is not None and len(ks) == 1 and ks[0] <= SHORT_K:
        return 2
    if m <= SKINNY_ROWS and n > GEMM_TILE:
        return 1
    if m <= SKINNY_WIDE_ROWS and n >= SKINNY_WIDE_N:
        return 1
    if n <= TALL_COLS and m > GEMM_TILE:
        return 3
    return 0


def _tile_cols(kind, m):
    return SHORT_COLS if kind == 2 else skinny_cols(m)
GEMM_RED_REC, GEMM_RED_ITEM = 8, 1024
SPLITK_MAX_TILES = 304   # plans with this many tiles (2 per SM) are not split
SPLITK_UNITS = 608       # tiles x chunks aimed at after splitting (4 per SM)
SPLITK_MIN_K = 128       # shortest K chunk


def _tiles_for(outs, terms):
    """Tiles (output, tile row, tile col, kind): kind 0 = 64x64, kind 1 = skinny (all m <= 16
    rows x 1024 columns, 256 above 8 rows), kind 3 = tall skinny (256 rows x all n <= 16
    columns; tile row = the 256-row block), kind 2 = short skinny (all m <= 8 rows x 512
    columns; its tile row holds the output's single term index, so the kernel loads the output
    and term records at once), ordered by descending work so long tiles start first."""
    tiles = []
    for oi, o in enumerate(outs):
        m, n = int(o[1]), int(o[2])
        if m == 0 or n == 0:
            continue
        ks = [int(terms[t][2]) for t in range(o[4], o[5])]
        kk = sum(ks)
        kind = tile_kind(m, n, ks)
        if kind == 3:
            for tr in range((m + TALL_ROWS - 1) // TALL_ROWS):
                tiles.append((kk * n * TALL_ROWS // GEMM_TILE, oi, tr, 0, 3))
            continue
        if kind:
            w = _tile_cols(kind, m)
            tr = int(o[4]) if kind == 2 else 0
            for tc in range((n + w - 1) // w):
                tiles.append((kk * m * 16, oi, tr, tc, kind))
            continue
        for tr in range((m + GEMM_TILE - 1) // GEMM_TILE):
            for tc in range((n + GEMM_TILE - 1) // GEMM_TILE):
                tiles.append((kk * GEMM_TILE, oi, tr, tc, 0))
    tiles.sort(key=lambda x: -x[0])
    arr = np.array([(oi, tr, tc, kind) for _, oi, tr, tc, kind in tiles], dtype=np.int32).reshape(-1, 4)
    return arr


def _n_tiles(m, n, ks=None):
    if m == 0 or n == 0:
        return 0
    kind = tile_kind(m, n, ks)
    if kind == 3:
        return (m + TALL_ROWS - 1) // TALL_ROWS
    if kind:
        return (n + _tile_cols(kind, m) - 1) // _tile_cols(kind, m)
    return ((m + GEMM_TILE - 1) // GEMM_TILE) * ((n + GEMM_TILE - 1) // GEMM_TILE)


def _split_chunk_k(out_list):
    """K per chunk when the plan has too few tiles to fill the GPU and some output's K is
    long (None: no split). Work is counted as tiles x K."""
    tiles = sum(_n_tiles(m, n, [t[2] for t in tl]) for _, m, n, _, tl in out_list)
    if tiles == 0 or tiles >= SPLITK_MAX_TILES:
        return None
    work = sum(_n_tiles(m, n, [t[2] for t in tl]) * sum(t[2] for t in tl) for _, m, n, _, tl in out_list)
    ck = max(SPLITK_MIN_K, -(-work // SPLITK_UNITS))
    ck = -(-ck // 16) * 16
    if not any(sum(t[2] for t in tl) >= 2 * ck for _, m, n, _, tl in out_list if m and n):
        return None
    return ck


def _chunks(tl, ck):
    """Cut a term list into chunks of at most ``ck`` contracted indices (terms longer than
    ``ck`` are cut into pieces; consecutive short ones share a chunk)."""
    chunks, cur, cur_k = [], [], 0
    for t in tl:
        a_off, b_off, k, ars, acs, brs, bcs, fl = t
        for k0 in range(0, k, ck):
            kp = min(ck, k - k0)
            if cur and cur_k + kp > ck:
                chunks.append(cur)
                cur, cur_k = [], 0
            cur.append((a_off + k0 * acs, b_off + k0 * brs, kp, ars, acs, brs, bcs, fl))
            cur_k += kp
    if cur:
        chunks.append(cur)
    return chunks


def _records(out_list):
    outs, terms, flops = [], [], 0
    for c_off, m, n, ldc, tl in out_list:
        t0 = len(terms)
        for t in tl:
            terms.append(t)
            flops += 2 * m * n * t[2]
        outs.append((c_off, m, n, ldc, t0, len(terms), 0, 0))
    outs = np.array(outs, dtype=np.int64).reshape(-1, GEMM_OUT_REC)
    terms = np.array(terms, dtype=np.int64).reshape(-1, GEMM_TERM_REC)
    return outs, terms, flops


def _pack_gemm(out_list, allow_split=True):
    """out_list: [(c_off, m, n, ldc, [term tuples])] -> GemmPlan. When the outputs make
    too few tiles for the GPU, outputs with a long K are split into K chunks computed into
    a workspace and summed by a reduction pass (split-K; not with ``allow_split=False``)."""
    ck = _split_chunk_k(out_list) if allow_split else None
    split = None
    if ck is not None:
        direct, parts, red, tasks, ws = [], [], [], [], 0
        for c_off, m, n, ldc, tl in out_list:
            if m == 0 or n == 0 or sum(t[2] for t in tl) < 2 * ck:
                direct.append((c_off, m, n, ldc, tl))
                continue
            kk = sum(t[2] for t in tl)
            nch = -(-kk // ck)
            ch = _chunks(tl, -(-(-(-kk // nch)) // 16) * 16)  # nch near-equal chunks, multiples of 16
            for ci, cl in enumerate(ch):
                parts.append((ws + ci * m * n, m, n, n, cl))
            ri = len(red)
            red.append((c_off, m, n, ldc, ws, len(ch), 0, 0))
            tasks.extend((ri, it) for it in range((m * n + GEMM_RED_ITEM - 1) // GEMM_RED_ITEM))
            ws += len(ch) * m * n
        po, pt, _ = _records(parts)
        split = SplitK(po, pt, _tiles_for(po, pt), np.array(red, dtype=np.int64).reshape(-1, GEMM_RED_REC),
                       np.array(tasks, dtype=np.int32).reshape(-1, 2), ws)
        out_list = direct
    outs, terms, _ = _records(out_list)
    flops = sum(2 * m * n * t[2] for _, m, n, _, tl in out_list for t in tl)
    if split is not None:
        flops += sum(2 * int(o[1]) * int(o[2]) * int(t[2]) for o in split.outs
                     for t in split.terms[int(o[4]):int(o[5])])
    return GemmPlan(outs, terms, _tiles_for(outs, terms), flops, split)


def dot_coverage(meta_dot):
    """Number of output elements that the sectors of ``meta_dot`` write, when their output
    slices are disjoint (0 otherwise): equal to Dsize, the output needs no zero fill."""
    spans = sorted((slc[0], slc[1]) for slc, *_ in meta_dot)
    end = 0
    for a, b in spans:
        if a < end:
            return 0
        end = b
    return sum(b - a for a, b in spans)


def dot_plan(meta_dot):
    """C[slc] = A[sla] @ B[slb] (yastn/backend/backend_np.py:580-587)."""
    def build():
        out_list = []
        for slc, Dc, sla, Da, slb, Db in meta_dot:
            out_list.append((slc[0], Dc[0], Dc[1], Dc[1], [(sla[0], slb[0], Da[1], Da[1], 1, Db[1], 1, 0)]))
        plan = _pack_gemm(out_list)
        plan.covered = dot_coverage(meta_dot)
        return plan
    return CACHE.get((meta_dot,), ('dot',), build)


def dot_backward_plans(meta_dot):
    """A_b[sla] += C_b[slc] B[slb]^H and B_b[slb] += A[sla]^H C_b[slc], grouped by operand block
    (restating yastn/backend/_backend_torch_backwards.py:117-138)."""
    def build():
        ga, gb = OrderedDict(), OrderedDict()
        for slc, Dc, sla, Da, slb, Db in meta_dot:
            # A_b block: (Da0 x Da1) = (Dc0 x Dc1) @ (Db1 x Db0)^H ; terms use a:=C_b, b:=B
            ga.setdefault((sla[0], Da[0], Da[1]), []).append((slc[0], slb[0], Dc[1], Dc[1], 1, 1, Db[1], 2))
            # B_b block: (Db0 x Db1) = (Da1 x Da0) @ (Dc0 x Dc1) ; terms use a:=A, b:=C_b
            gb.setdefault((slb[0], Db[0], Db[1]), []).append((sla[0], slc[0], Da[0], 1, Da[1], Dc[1], 1, 1))
        pa = _pack_gemm([(off, m, n, n, tl) for (off, m, n), tl in ga.items()])
        pb = _pack_gemm([(off, m, n, n, tl) for (off, m, n), tl in gb.items()])
        return pa, pb
    return CACHE.get((meta_dot,), ('dot_bwd',), build)


def tds_plan(meta_dot, Areshape, Breshape, Aoffs, Boffs):
    """transpose_dot_sum after the operands were permuted into (Dl, Dr) matrices stored at
    ``Aoffs``/``Boffs`` (restating yastn/backend/backend_np.py:590-601)."""
    def build():
        out_list = []
        for sl, Dslc, pairs in meta_dot:
            tl = []
            for ta, tb in pairs:
                _, _, Dla, Dra = Areshape[ta]
                _, _, Dlb, Drb = Breshape[tb]
                tl.append((Aoffs[ta], Boffs[tb], Dra, Dra, 1, Drb, 1, 0))
            out_list.append((sl[0], Dslc[0], Dslc[1], Dslc[1], tl))
        return _pack_gemm(out_list)
    return CACHE.get((meta_dot, Areshape, Breshape), ('tds',), build)


class OzakiPlan:
    """Split records and GEMM tiles of the split-operand (Ozaki) emulated FP64 dot."""

    def __init__(self, outs, tiles, flops, s):
        self.outs, self.tiles = outs, tiles
        self.flops = flops
        self.slices = s
        self._dev = {}


OZAKI_TC_M, OZAKI_TC_N = 128, 64  # output tile of the tcgen05 emulated GEMM (also 128 x 32)
OZAKI_MIN_DIM = 16  # sector GEMMs contracting fewer indices than this stay on the native FP64 kernel
OZAKI_SKINNY_ROWS = 8  # sector GEMMs with at most this many rows (and more than 64 columns) too
OZ_SPLIT_REC = 10  # YB_OZ_SPLIT_REC
OZ_SPLIT_ROWS = 8  # rows per split CTA


def _split_layout(blocks, s, th_a, th_b):
    """Split records (YB_OZ_SPLIT_REC int64) and 8-row groups for the operand blocks
    ``blocks`` = [(operand, src offset, rows, Kr, row stride, k stride, mode, Kp)], with the
    digit planes of operand A in tile rows ``th_a`` and of B in ``th_b`` (0: planes
    [slice][row][Kp]). Returns (records, groups, A size, B size, A exps, B exps) and the
    slice-0 offset and exponent offset of every block."""
    recs, groups, where = [], [], []
    size, nex = [0, 0], [0, 0]
    for op, src, rows, Kr, rs, ks, mode, Kp in blocks:
        th = th_b if op else th_a
        rows_p = -(-rows // th) * th if th else rows
        where.append((size[op], nex[op]))
        ri = len(recs)
        recs.append((src, rows, Kr, rs, mode, size[op], nex[op], Kp, ks, op | (th << 8)))
        groups.extend((ri, g) for g in range(0, rows_p, OZ_SPLIT_ROWS))
        size[op] += s * rows_p * Kp
        nex[op] += rows
    recs = np.array(recs, dtype=np.int64).reshape(-1, OZ_SPLIT_REC)
    groups = np.array(groups, dtype=np.int32).reshape(-1, 2)
    return recs, groups, size[0], size[1], nex[0], nex[1], where


def _groups_by_operand(recs, groups):
    """The split groups of operand A and of operand B (a split launch of one operand)."""
    op = (recs[groups[:, 0], 9] & 0xff) if len(groups) else np.zeros(0, dtype=np.int64)
    return (np.ascontiguousarray(groups[op == 0]).reshape(-1, 2),
            np.ascontiguousarray(groups[op == 1]).reshape(-1, 2))


OZ_TC_FOLD_STEPS = 6  # fold + write of a full 128 x 64 tile, in K-step units of the tcgen05 kernel


def ozaki_tc_schedule(plan, n_ctas, tile_n=64):
    """Tiles of the tcgen05 kernel (128 x ``tile_n``) grouped by CTA (longest processing time
    first: each tile, by decreasing cost, to the least loaded CTA; cost = K steps + the fold of
    its valid elements). Returns (tiles reordered, int32 offsets of the n_ctas + 1 CTA ranges)."""
    key = ('tc_sched', n_ctas, tile_n)
    got = plan._dev.get(key)
    if got is not None:
        return got
    import heapq
    sfx = '_tc' if tile_n == 64 else '_tc32'
    tiles, outs = getattr(plan, 'tiles' + sfx), getattr(plan, 'outs' + sfx)
    n_ctas = max(1, min(n_ctas, len(tiles)))
    cost = []
    for i, (oi, tr, tc, _) in enumerate(tiles):
        o = outs[oi]
        m, n, Kp = int(o[1]), int(o[2]), int(o[9])
        steps = Kp // 16
        chunks = -(-steps // 25)
        valid = min(OZAKI_TC_M, m - OZAKI_TC_M * int(tr)) * min(tile_n, n - tile_n * int(tc))
        cost.append((steps + OZ_TC_FOLD_STEPS * chunks * valid / (OZAKI_TC_M * 64), i))
    cost.sort(reverse=True)
    heap = [(0.0, b) for b in range(n_ctas)]
    lists = [[] for _ in range(n_ctas)]
    for c, i in cost:
        load, b = heapq.heappop(heap)
        lists[b].append(i)
        heapq.heappush(heap, (load + c, b))
    order = [i for lst in lists for i in lst]
    offs = np.cumsum([0] + [len(lst) for lst in lists]).astype(np.int32)
    got = (np.ascontiguousarray(tiles[order]), offs)
    plan._dev[key] = got
    return got


def ozaki_dot_plan(meta_dot, s, cplx=False):
    """C[slc] = A[sla] @ B[slb] with A rows / B columns split into ``s`` BF16 digit slices.

    Both operands are split by one launch of yb_ozaki_split: A blocks by rows, B blocks by
    columns read in place (k stride n). Complex blocks (``cplx``) become two real products
    with doubled K, C_r = [A_r, A_i][B_r; -B_i] and C_i = [A_r, A_i][B_i; B_r]: A is split
    once in mode 1 ([re | im] rows), each B block twice (modes 2 and 3), and the two outputs
    of a sector write the real and imaginary parts of the complex result (column stride 2 in
    FP64 units). The records exist twice: digit planes for the mma.sync kernel (64 x 64
    tiles) and the tile layout of the tcgen05 kernel (128 x 64 tiles).
    """
    def build():
        a_map, b_map, blocks = {}, {}, []
        outs_ref, flops, small = [], 0, []
        f = 2 if cplx else 1  # FP64 words per element
        for slc, Dc, sla, Da, slb, Db in meta_dot:
            m, K = Da
            n = Db[1]
            if K < OZAKI_MIN_DIM or (m <= OZAKI_SKINNY_ROWS and n > GEMM_TILE):
                # short contractions and skinny outputs stay on the native FP64 kernel
                small.append((slc[0], m, n, n, [(sla[0], slb[0], K, K, 1, n, 1, 0)]))
                continue
            Kr = f * K  # length of the real rows that are split
            Kp = (Kr + 15) // 16 * 16
            if sla[0] not in a_map:
                a_map[sla[0]] = len(blocks)
                blocks.append((0, sla[0], m, Kr, K, 1, int(cplx), Kp))
            if slb[0] not in b_map:
                b_map[slb[0]] = []
                for mode in ((2, 3) if cplx else (0,)):
                    b_map[slb[0]].append(len(blocks))
                    blocks.append((1, slb[0], n, Kr, 1, n, mode, Kp))
            for part, bi in enumerate(b_map[slb[0]]):
                # complex: part 0 = real part (even FP64 words), part 1 = imaginary part
                outs_ref.append((f * slc[0] + part, m, n, f * n, a_map[sla[0]], bi, Kr, Kp, f))
            flops += (8 if cplx else 2) * m * n * K

        def outs_for(where):
            return np.array([(c, m, n, ld, where[ai][0], where[ai][1], where[bi][0], where[bi][1], Kr, Kp, cs,
                              0, 0, 0, 0, 0) for c, m, n, ld, ai, bi, Kr, Kp, cs in outs_ref],
                            dtype=np.int64).reshape(-1, 16)

        sr, sg, asz, bsz, aex, bex, where = _split_layout(blocks, s, 0, 0)
        outs = outs_for(where)
        tiles = []
        for oi, o in enumerate(outs):
            m, n, K = int(o[1]), int(o[2]), int(o[8])
            if m == 0 or n == 0:
                continue
            for tr in range((m + 63) // 64):
                for tc in range((n + 63) // 64):
                    tiles.append((K, oi, tr, tc))
        tiles.sort(key=lambda x: -x[0])
        tiles = np.array([(oi, tr, tc, 0) for _, oi, tr, tc in tiles], dtype=np.int32).reshape(-1, 4)
        plan = OzakiPlan(outs, tiles, flops, s)
        plan.split_recs, plan.split_groups = sr, sg
        plan.split_groups_ab = _groups_by_operand(sr, sg)
        plan.a_size, plan.b_size, plan.a_exps, plan.b_exps = asz, bsz, aex, bex
        plan.native = _pack_gemm(small)
        plan.native_direct = _pack_gemm(small, allow_split=False)  # no chunk workspace
        plan.covered = dot_coverage(meta_dot)
        # tiles of the tcgen05 kernel, 128 x 64 and 128 x 32 (longest K first), and the digit
        # planes in its tile layout (rows padded to 128 for A, to the tile width for B)
        for tn, sfx in ((64, '_tc'), (32, '_tc32')):
            sr, sg, asz, bsz, _, _, where = _split_layout(blocks, s, OZAKI_TC_M, tn)
            outs_t = outs_for(where)
            tiles_t = []
            for oi, o in enumerate(outs_t):
                m, n, K = int(o[1]), int(o[2]), int(o[8])
                for tr in range(-(-m // OZAKI_TC_M)):
                    for tc in range(-(-n // tn)):
                        tiles_t.append((K, oi, tr, tc))
            tiles_t.sort(key=lambda x: -x[0])
            setattr(plan, 'split_recs' + sfx, sr)
            setattr(plan, 'split_groups' + sfx, sg)
            setattr(plan, 'split_groups' + sfx + '_ab', _groups_by_operand(sr, sg))
            setattr(plan, 'a_size' + sfx, asz)
            setattr(plan, 'b_size' + sfx, bsz)
            setattr(plan, 'outs' + sfx, outs_t)
            setattr(plan, 'tiles' + sfx, np.array([(oi, tr, tc, 0) for _, oi, tr, tc in tiles_t],
                                                  dtype=np.int32).reshape(-1, 4))
        # padded MMA work of the tilings: a tcgen05 tiling (the narrower one unless it pads more)
        # unless its padding costs over 1.6 times the 64 x 64 tiles of the mma.sync kernel (the
        # tcgen05 kernel measured faster on the DMRG workload's sectors at 1.3 times the padded work)
        def padded(tm, tn):
            return sum(-(-int(o[1]) // tm) * tm * -(-int(o[2]) // tn) * tn * int(o[9]) for o in outs)
        w64, w128, w32 = padded(64, 64), padded(OZAKI_TC_M, 64), padded(OZAKI_TC_M, 32)
        best_tc = 32 if w32 <= w128 else 64
        plan.prefer_tc = (best_tc if min(w32, w128) <= 1.6 * w64 else False) if len(outs) else False
        return plan
    return CACHE.get((meta_dot,), ('ozaki_dot', s, bool(cplx)), build)


# ----------------------------------------------------------------------------- SVD

class SvdPlan:
    """Mixed-precision Jacobi plan: block records, pair items, workspace layout and the
    grouped-GEMM plans of the Newton-Schulz orthonormalisation and of X = W X_0."""

    def __init__(self, blocks, pair_items, max_rounds, max_k, nominal_flops, n64, n32, w_range, gram, ns, xform,
                 rows_per_super=0, super_items=None, super_rounds=0, lmax=0, qr=False, qfin_u=None, qfin_v=None,
                 rows_per_super64=0, super_items64=None, super_rounds64=0):
        self.blocks = blocks
        self.rows_per_super64 = rows_per_super64  # blocked FP64 phase (0: one pair per warp)
        self.super_items64, self.super_rounds64 = super_items64, super_rounds64
        self.qr = qr            # QR-preconditioned: Jacobi on R's rows, then U or Vh by qfin_u / qfin_v
        self.qfin_u, self.qfin_v = qfin_u, qfin_v
        self.pair_items = pair_items
        self.rows_per_super = rows_per_super  # 0: the FP32 phase uses the one-pair-per-warp kernel
        self.super_items = super_items        # (block, super pair) items of the blocked FP32 phase
        self.super_rounds = super_rounds
        self.lmax = lmax
        self.max_rounds = max_rounds
        self.max_k = max_k
        self.nominal_flops = nominal_flops
        self.n64 = n64          # FP64 workspace elements: [X | W | T | Wn]
        self.n32 = n32          # FP32 workspace elements: [X32 | W32]
        self.w_range = w_range  # (W start, T start, Wn start, total W size) in the FP64 workspace
        self.gram, self.ns, self.xform = gram, ns, xform
        self._dev = {}


SVD_SMEM_BYTES = 220 * 1024  # shared memory a blocked-Jacobi CTA may take (GB300: 227 KB per CTA)
SVD_ROWS_PER_SUPER64 = 4     # super-vector height of the blocked FP64 phase


def svd_rows_per_super(lmax, choices=(16, 8, 4), elem_bytes=4):
    """Rows per super-vector of the blocked FP32 Jacobi: the largest choice whose CTA
    (2 * rows * lmax + 4 * rows^2 elements of shared memory, 8-byte elements for complex64)
    fits; 0 if none does."""
    for br in choices:
        if (2 * br * lmax + 4 * br * br) * elem_bytes <= SVD_SMEM_BYTES:
            return br
    return 0


def svd_plan(meta, rows_per_super=None, cplx=False, qr=False):
    """Jacobi plan for svd records (sl, D, slU, DU, slS, slV, DV) of yastn/tensor/linalg.py:323-380.
    ``rows_per_super`` fixes the super-vector height of the blocked FP32 phase (default: the
    largest of 16, 8, 4 whose rows fit in shared memory). ``cplx``: complex128 blocks (the
    Gram product of Newton-Schulz is W^H W and tall blocks start from X_0 = A^H). ``qr``:
    every block starts from the rows of R of a Householder QR (yb_svd_qr), the sweeps run on
    k x k rows, and the factor not built from X's rows follows from Q by a grouped GEMM.

    FP64 workspace: [X | W | T | Wn] and, with ``qr``, [Z | Householder vectors | tau | R]."""
    def build():
        sel = []
        for sl, D, slU, DU, slS, slV, DV in meta:
            m, n = D
            k = min(m, n)
            if k == 0:
                continue
            if DU != (m, k) or DV != (k, n) or slS[1] - slS[0] != k:
                raise PlanError("svd record is not a thin full-rank SVD")
            sel.append((sl, m, n, slU, slS, slV, k, max(m, n)))
        lj = (lambda k, L: k) if qr else (lambda k, L: L)  # row length of the Jacobi vectors
        xs = sum(k * lj(k, L) for *_, k, L in sel)
        ws = sum(k * k for *_, k, L in sel)
        w0, t0, n0 = xs, xs + ws, xs + 2 * ws
        zs = sum(k * L for *_, k, L in sel) if qr else 0
        q0 = xs + 3 * ws                       # Z, then the Householder vectors, tau, R
        v0, tau0, r0 = q0 + zs, q0 + 2 * zs, q0 + 2 * zs + sum(k for *_, k, L in sel)
        recs, pairs, gram, ns, xf, qfu, qfv = [], [], [], [], [], [], []
        ox = ow = ox32 = oz = otau = 0
        max_rounds = max_k = fl = 0
        for bi, (sl, m, n, slU, slS, slV, k, L) in enumerate(sel):
            N = k + (k % 2)
            Lx = lj(k, L)
            rec = np.zeros(SVD_REC, dtype=np.int64)
            rec[:15] = (sl[0], m, n, slU[0], slS[0], slV[0], ox, w0 + ow, len(pairs), k, Lx, N, int(m > n),
                        ox32, xs + ow)
            recs.append(rec)
            pairs.extend((bi, p) for p in range(N // 2))
            # T = W^T W ; Wn = 1.5 Wn - 0.5 W T (Wn holds a copy of W) ; X = W X_0 (QR: X = W R)
            gram.append((t0 + ow, k, k, k, [(w0 + ow, w0 + ow, k, 1, k, k, 1, int(cplx))]))
            ns.append((n0 + ow, k, k, k, [(w0 + ow, t0 + ow, k, k, 1, k, 1, 0)]))
            if qr:
                rec[16:23] = (1, L, q0 + oz, v0 + oz, tau0 + otau, r0 + ow, t0 + ow)
                xf.append((ox, k, k, k, [(w0 + ow, r0 + ow, k, k, 1, k, 1, 0)]))
                if m > n:   # U (m x k) = conj(Q) W_sorted^T: A_t[l, c] = conj(Z[c L + l]), B_t[c, j] = WS[j k + c]
                    qfu.append((slU[0], m, k, k, [(q0 + oz, t0 + ow, k, 1, L, 1, k, int(cplx))]))
                else:       # Vh (k x n) = conj(W_sorted) Q^T (the conjugate is in WS)
                    qfv.append((slV[0], k, n, n, [(t0 + ow, q0 + oz, k, k, 1, L, 1, 0)]))
                oz += k * L
                otau += k
            elif m > n:
                xf.append((ox, k, L, L, [(w0 + ow, sl[0], k, k, 1, 1, n, 2 * int(cplx))]))
            else:
                xf.append((ox, k, L, L, [(w0 + ow, sl[0], k, k, 1, n, 1, 0)]))
            ox += k * Lx
            ox32 += k * Lx
            ow += k * k
            max_rounds = max(max_rounds, N - 1)
            max_k = max(max_k, k)
            fl += 14 * L * k * k + 8 * k ** 3  # nominal Golub-Reinsch count
        lmax = max((lj(k, L) for *_, k, L in sel), default=0)
        n64 = xs + 3 * ws + (2 * zs + sum(k for *_, k, L in sel) + ws if qr else 0)
        br = svd_rows_per_super(lmax, elem_bytes=8 if cplx else 4) if rows_per_super is None else rows_per_super
        # FP64 phase: 4-row super-vectors (8 rows per CTA) keep every SM busy on few blocks
        br64 = svd_rows_per_super(lmax, choices=(SVD_ROWS_PER_SUPER64,), elem_bytes=16 if cplx else 8)
        supers, super_rounds, supers64, super_rounds64 = [], 0, [], 0
        for bi, (*_, k, L) in enumerate(sel):
            if br:
                ns_ = -(-k // br)
                ns_ += ns_ % 2
                recs[bi][15] = ns_
                supers.extend((bi, p) for p in range(ns_ // 2))
                super_rounds = max(super_rounds, ns_ - 1)
            if br64:
                ns_ = -(-k // br64)
                ns_ += ns_ % 2
                recs[bi][23] = ns_
                supers64.extend((bi, p) for p in range(ns_ // 2))
                super_rounds64 = max(super_rounds64, ns_ - 1)
        blocks = np.stack(recs) if recs else np.zeros((0, SVD_REC), dtype=np.int64)
        items = np.array(pairs, dtype=np.int32).reshape(-1, 2)
        return SvdPlan(blocks, items, max_rounds, max_k, fl, n64, xs + ws, (w0, t0, n0, ws),
                       _pack_gemm(gram), _pack_gemm(ns), _pack_gemm(xf),
                       br, np.array(supers, dtype=np.int32).reshape(-1, 2), super_rounds, lmax,
                       qr, _pack_gemm(qfu) if qr else None, _pack_gemm(qfv) if qr else None,
                       br64, np.array(supers64, dtype=np.int32).reshape(-1, 2), super_rounds64)
    return CACHE.get((meta,), ('svd', rows_per_super, cplx, qr), build)


class FixSignsPlan:
    """Records of the gauge fix (YB_SVD_REC int64 each, the fields yb_fix_signs reads):
    [1] m [2] n [3] U offset [4] S offset [5] Vh offset [9] k, for blocks U (m x k),
    Vh (k x n) of any k (thin or truncated SVDs)."""

    def __init__(self, blocks, max_k):
        self.blocks, self.max_k = blocks, max_k
        self._dev = {}


def fix_signs_plan(meta):
    def build():
        recs, max_k, s_off = [], 0, 0
        for sl, D, slU, DU, slS, slV, DV in meta:
            m, k = DU
            n = DV[1]
            if k == 0 or m == 0:
                continue
            if DV[0] != k or (slS is not None and slS[1] - slS[0] != k):
                raise PlanError("fix_svd_signs record: U, S and Vh disagree on the number of vectors")
            # the phases are indexed like S; YASTN's partial SVDs pass no S slice (then: in order)
            s0 = slS[0] if slS is not None else s_off
            s_off = s0 + k
            r = np.zeros(SVD_REC, dtype=np.int64)
            r[1], r[2], r[3], r[4], r[5], r[9] = m, n, slU[0], s0, slV[0], k
            recs.append(r)
            max_k = max(max_k, k)
        blocks = np.stack(recs) if recs else np.zeros((0, SVD_REC), dtype=np.int64)
        return FixSignsPlan(blocks, max_k)
    return CACHE.get((meta,), ('fix_signs',), build)


class QrPlan:
    """Plan of ``qr`` (records of yb_qr, the FP64 workspace, the GEMM of R's right part for
    wide blocks) and of its adjoint (grouped GEMMs, copyltu/TRSM records, the copy of the
    solved rows into dA)."""

    def __init__(self, **kw):
        self.__dict__.update(kw)
        self._dev = {}


QRADJ_REC = 8


def qr_plan(meta, cplx=False):
    """Reduced QR records (sl, D, slQ, DQ, slR, DR) of yastn/tensor/linalg.py:795-828, as
    computed by backend_np.py:511-520 (positive diagonal of R)."""
    def build():
        recs, right, adj = [], [], []
        w1, m1, m2, s1, y1, copies = [], [], [], [], [], []
        off = mo = 0
        max_k = 0
        for sl, D, slQ, DQ, slR, DR in meta:
            m, n = D
            k = min(m, n)
            if k == 0:
                continue
            if DQ != (m, k) or DR != (k, n):
                raise PlanError("qr record is not a reduced QR")
            rec = np.zeros(SVD_REC, dtype=np.int64)
            rec[[0, 1, 2, 3, 5, 9, 10]] = (sl[0], m, n, slQ[0], slR[0], k, k)
            z, v, tau, rr = off, off + k * m, off + 2 * k * m, off + 2 * k * m + k
            rec[16:22] = (2, m, z, v, tau, rr)
            off = rr + k * k
            recs.append(rec)
            max_k = max(max_k, k)
            q0, r0, a0 = slQ[0], slR[0], sl[0]
            cj = int(cplx)  # conjugation flags of the complex adjoint (bit 0: A, bit 1: B)
            if n > m:   # R[:, m:] = Q^H A[:, m:]
                right.append((r0 + m, k, n - m, n, [(q0, a0 + m, m, 1, k, n, 1, cj)]))
                w1.append((q0, m, m, k, [(a0 + m, r0 + m, n - m, n, 1, 1, n, 2 * cj)]))  # gQ' += A[:, m:] gV^H
                y1.append((a0 + m, m, n - m, n, [(q0, r0 + m, m, k, 1, n, 1, 0)]))      # dA[:, m:] = Q gV
            m1.append((mo, k, k, k, [(r0, r0, k, n, 1, 1, n, 2 * cj)]))                  # M = U gU^H
            m2.append((mo, k, k, k, [(q0, q0, m, 1, k, k, 1, cj)]))                      # M -= gQ'^H Q
            s1.append((q0, m, k, k, [(q0, mo, k, k, 1, k, 1, 0)]))                       # gQ' += Q copyltu(M)
            adj.append((mo, k, q0, m, k, r0, n, 0))
            copies.append((q0, a0, [m, k], [k, 1], [n, 1]))
            mo += k * k
        blocks = np.stack(recs) if recs else np.zeros((0, SVD_REC), dtype=np.int64)
        return QrPlan(blocks=blocks, n64=max(off, 1), max_k=max_k, right=_pack_gemm(right),
                      adj=np.array(adj, dtype=np.int64).reshape(-1, QRADJ_REC), m_size=max(mo, 1),
                      w1=_pack_gemm(w1), m1=_pack_gemm(m1), m2=_pack_gemm(m2), s1=_pack_gemm(s1),
                      y1=_pack_gemm(y1), copies=copies)
    return CACHE.get((meta,), ('qr', cplx), build)


class CompletionPlan:
    """Blocked completion of the vectors of small singular values for one factor (U columns
    when ``to_u``, else Vh rows): candidate fill records (offset, count), the grouped-GEMM
    projections C = V_g^H G (g1) and G -= V_g C (g2), the QR records of the candidates, and
    the copy of the orthonormalised candidates into the factor."""

    def __init__(self, to_u, g1, g2, meta, fill, copy, sizes):
        self.to_u, self.g1, self.g2, self.meta, self.fill, self.copy = to_u, g1, g2, meta, fill, copy
        self.G, self.C, self.Q, self.R = sizes
        self._dev = {}


def completion_plans(blocks, nz, cplx=False):
    """Completion plans of svd records ``blocks`` (SVD_REC) for the per-block counts ``nz`` of
    vectors to complete (the last nz of each block's k). The vectors built from X's rows are
    U's columns for tall blocks started from A's rows and for wide blocks started from R's,
    else Vh's rows; V_g are the k - nz vectors before them."""
    by_target = {}
    for b, r in enumerate(blocks):
        z = int(nz[b])
        if z == 0:
            continue
        m, n, k, tall, from_r = int(r[1]), int(r[2]), int(r[9]), bool(r[12]), bool(r[16])
        to_u = tall != from_r
        if to_u:
            f0, sv, sj, Lv = int(r[3]), k, 1, m
        else:
            f0, sv, sj, Lv = int(r[5]), 1, n, n
        j0 = k - z
        t = by_target.setdefault(to_u, {'g1': [], 'g2': [], 'meta': [], 'fill': [], 'copies': [],
                                        'G': 0, 'C': 0, 'Q': 0, 'R': 0})
        g, c_, q_, r_ = t['G'], t['C'], t['Q'], t['R']
        if j0 > 0:
            t['g1'].append((c_, j0, z, z, [(f0, g, Lv, sj, sv, z, 1, int(cplx))]))
            t['g2'].append((g, Lv, z, z, [(f0, c_, j0, sv, sj, z, 1, 0)]))
        t['meta'].append(((g, g + Lv * z), (Lv, z), (q_, q_ + Lv * z), (Lv, z), (r_, r_ + z * z), (z, z)))
        t['fill'].append((g, Lv * z))
        t['copies'].append((q_, f0 + j0 * sj, [Lv, z], [z, 1], [sv, sj]))
        t['G'] += Lv * z
        t['C'] += j0 * z
        t['Q'] += Lv * z
        t['R'] += z * z
    out = []
    for to_u, t in by_target.items():
        out.append(CompletionPlan(to_u, _pack_gemm(t['g1']), _pack_gemm(t['g2']), tuple(t['meta']),
                                  np.array(t['fill'], dtype=np.int64).reshape(-1, 2),
                                  CopyPlan(t['copies'], sum(int(np.prod(c[2])) for c in t['copies']), 0),
                                  (t['G'], t['C'], t['Q'], t['R'])))
    return out


class SvdAdjointPlan:
    def __init__(self, recs, kk, tr, gP, gQ, gT, gR, gA1, gA2):
        self.recs, self.kk, self.tr = recs, kk, tr
        self.gP, self.gQ, self.gT, self.gR, self.gA1, self.gA2 = gP, gQ, gT, gR, gA1, gA2
        self._dev = {}


def svd_adjoint_plan(meta):
    """Grouped-GEMM plans of the SVD adjoint (torch_svd_gesdd.py:296-428), all blocks at once.

    P = U^H gU, Q = Vh gVh^H (k x k); square/wide blocks: TR += K Vh, dA = U TR;
    tall blocks: TR += U K, dA = TR Vh (see csrc/yb_adjoint.cu for K and TR).
    """
    def build():
        recs, lP, lQ, lT, lR, lA1, lA2 = [], [], [], [], [], [], []
        kk = tr = 0
        for sl, D, slU, DU, slS, slV, DV in meta:
            m, n = D
            k = min(m, n)
            if k == 0:
                continue
            kind = 0 if m == n else (1 if n > m else 2)
            rec = np.zeros(16, dtype=np.int64)
            rec[:10] = (sl[0], m, n, slU[0], slS[0], slV[0], kk, tr, k, kind)
            recs.append(rec)
            lP.append((kk, k, k, k, [(slU[0], slU[0], m, 1, k, k, 1, 1)]))
            lQ.append((kk, k, k, k, [(slV[0], slV[0], n, n, 1, 1, n, 2)]))
            if kind != 2:
                lT.append((tr, k, n, n, [(kk, slV[0], k, k, 1, n, 1, 0)]))
                lA1.append((sl[0], m, n, n, [(slU[0], tr, k, k, 1, n, 1, 0)]))
                tr += k * n
            else:
                lR.append((tr, m, k, k, [(slU[0], kk, k, k, 1, k, 1, 0)]))
                lA2.append((sl[0], m, n, n, [(tr, slV[0], k, k, 1, n, 1, 0)]))
                tr += m * k
            kk += k * k
        recs = np.stack(recs) if recs else np.zeros((0, 16), dtype=np.int64)
        return SvdAdjointPlan(recs, kk, tr, *(_pack_gemm(x) for x in (lP, lQ, lT, lR, lA1, lA2)))
    return CACHE.get((meta,), ('svd_adjoint',), build)


class EighAdjointPlan:
    def __init__(self, recs, kk, gX, gT, gA):
        self.recs, self.kk, self.gX, self.gT, self.gA = recs, kk, gX, gT, gA
        self._dev = {}


def eigh_adjoint_plan(meta, symeig, cplx):
    """Grouped-GEMM plans of the eigh adjoint dA = U K op(U)^T on all blocks (records
    (sl, D, slU, DU, slS) of yastn/backend/backend_np.py:461-474): X = op(U)^T gU, then
    T = U K, dA = T op(U)^T; op(U) = U for SYMEIG (torch_eig_sym.py:43-54), conj(U) for
    torch.linalg.eigh's adjoint (complex data)."""
    def build():
        conj = int(cplx and not symeig)
        recs, lX, lT, lA = [], [], [], []
        kk = 0
        for sl, D, slU, DU, slS in meta:
            k = DU[1]
            if k == 0:
                continue
            m = DU[0]
            recs.append((kk, k, slS[0], 0))
            lX.append((kk, k, k, k, [(slU[0], slU[0], m, 1, k, k, 1, conj)]))   # X = op(U)^T gU
            lT.append((kk, m, k, k, [(slU[0], kk, k, k, 1, k, 1, 0)]))          # T = U K (into the X buffer)
            lA.append((sl[0], m, m, m, [(kk, slU[0], k, k, 1, 1, k, 2 * conj)]))  # dA = T op(U)^T
            kk += k * k
        recs = np.array(recs, dtype=np.int64).reshape(-1, 4)
        return EighAdjointPlan(recs, kk, _pack_gemm(lX), _pack_gemm(lT), _pack_gemm(lA))
    return CACHE.get((meta,), ('eigh_adjoint', bool(symeig), bool(cplx)), build)


def tds_backward_plans(meta_dot, Areshape, Breshape, Aoffs, Boffs):
    """Adjoint of transpose_dot_sum on the permuted (Dl, Dr) operand matrices:
    At_b[a] = sum C_b[sl] Bt[b]^H, Bt_b[b] = sum At[a]^H C_b[sl] (grouped by operand)."""
    def build():
        ga, gb = OrderedDict(), OrderedDict()
        for sl, Dslc, pairs in meta_dot:
            mc, nc = Dslc
            for ta, tb in pairs:
                _, _, Dla, Dra = Areshape[ta]
                _, _, Dlb, Drb = Breshape[tb]
                ga.setdefault(ta, []).append((sl[0], Boffs[tb], nc, nc, 1, 1, Drb, 2))
                gb.setdefault(tb, []).append((Aoffs[ta], sl[0], Dla, 1, Dra, nc, 1, 1))
        pa = _pack_gemm([(Aoffs[ta], Areshape[ta][2], Areshape[ta][3], Areshape[ta][3], tl) for ta, tl in ga.items()])
        pb = _pack_gemm([(Boffs[tb], Breshape[tb][2], Breshape[tb][3], Breshape[tb][3], tl) for tb, tl in gb.items()])
        return pa, pb
    return CACHE.get((meta_dot, Areshape, Breshape), ('tds_bwd',), build)


# ----------------------------------------------------------------------------- masks

def mask_plan(meta, axis, lengths):
    """apply_mask records (yastn/backend/backend_np.py:626-633); ``lengths`` maps a mask charge
    (or, for a slice mask, the pair (charge, length of the masked axis)) to (offset in the
    concatenated index buffer, number of kept indices)."""
    recs, items, total = [], [], 0
    for sln, Dn, sla, Da, tm in meta:
        if isinstance(Da, int):  # diagonal tensors carry their block length as an int
            Da = (Da,)
        ioff, cnt = lengths[(tm, Da[axis])] if (tm, Da[axis]) in lengths else lengths[tm]  # slice masks by length
        pre = int(np.prod(Da[:axis], dtype=np.int64))
        post = int(np.prod(Da[axis + 1:], dtype=np.int64))
        nout = pre * cnt * post
        if nout == 0:
            continue
        ri = len(recs)
        recs.append((sln[0], sla[0], pre, Da[axis], cnt, post, ioff, 0))
        items.extend((ri, f) for f in range(0, nout, COPY_ITEM_UNITS))
        total += nout
    recs = np.array(recs, dtype=np.int64).reshape(-1, MASK_REC)
    items = np.array(items, dtype=np.int64).reshape(-1, 2)
    return recs, items, total
