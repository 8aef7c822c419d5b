"""Charge-sector sharding across ranks (one process per GPU) and the global truncation
exchange.

YASTN's hot path decomposes into independent charge-sector units: the sector GEMMs of a
``dot`` (``meta_dot`` records, yastn/tensor/_contractions.py:281-346), the block SVDs
(``_meta_svd`` records, yastn/tensor/linalg.py:323-380) and the merge destination blocks.
A rank takes a longest-processing-time share of the units (cost 2 m n k for a GEMM,
m n min(m, n) for an SVD block), computes them on its GPU with the same single-GPU entry
points, and needs no collective for them. The one exchange is the global truncation of
``truncation_mask`` (yastn/tensor/linalg.py:637-735), which ranks singular values across
all blocks: every rank all-gathers, for each block it owns, the values that can survive
(after the per-block ``tol_block``/``D_block`` cut, at most ``D_total`` per block, all of
them under ``truncate_multiplets``) with their global positions, and applies the same
rule to the gathered candidates, so all ranks agree on the kept dimensions.

Ties in the global ranking are broken by global position (a stable ascending sort keeps
the later of two equal values), the rule of ``np.argsort(kind='stable')``.
"""
import numpy as np

__all__ = ['lpt_assign', 'shard_dot', 'shard_svd', 'block_candidates', 'global_truncation',
           'gather_truncation']


def lpt_assign(costs, world):
    """Longest-processing-time assignment: units in order of decreasing cost (ties by
    index) go to the least-loaded rank (ties by rank). Returns owner[i] for every unit."""
    owner = [0] * len(costs)
    load = [0.0] * world
    for i in sorted(range(len(costs)), key=lambda i: (-costs[i], i)):
        r = min(range(world), key=lambda r: (load[r], r))
        owner[i] = r
        load[r] += costs[i]
    return owner


def shard_dot(meta_dot, rank, world):
    """The ``meta_dot`` records (slc, Dc, sla, Da, slb, Db) that ``rank`` computes, and their
    indices in ``meta_dot``. Outputs are disjoint, so the shards need no reduction."""
    costs = [2.0 * Da[0] * Da[1] * Db[1] for _, _, _, Da, _, Db in meta_dot]
    owner = lpt_assign(costs, world)
    idx = [i for i, o in enumerate(owner) if o == rank]
    return tuple(meta_dot[i] for i in idx), idx


def shard_svd(meta, rank, world):
    """The svd records (sl, D, slU, DU, slS, slV, DV) that ``rank`` decomposes, and their
    indices."""
    costs = [float(D[0]) * D[1] * min(D) for _, D, *_ in meta]
    owner = lpt_assign(costs, world)
    idx = [i for i, o in enumerate(owner) if o == rank]
    return tuple(meta[i] for i in idx), idx


def _block_cut(blk, tol_block, D_block):
    """Per-block cut (linalg.py:700-711): indices (within the block) that survive it."""
    n = len(blk)
    bmax = np.abs(blk).max() if n else 0.0
    D_tol = int(np.sum(blk > tol_block * bmax))
    D_bl = min(D_block, D_tol)
    if D_bl <= 0:
        return np.zeros(0, dtype=np.int64)
    if D_bl >= n:
        return np.arange(n, dtype=np.int64)
    order = np.argsort(blk, kind='stable')
    return np.sort(order[-int(D_bl):])


def block_candidates(S_blocks, starts, tol_block=0, D_block=float('inf'), D_total=float('inf'),
                     truncate_multiplets=False):
    """Candidates of this rank's blocks for the global cut: (values, global positions).

    ``S_blocks``: the spectra of the blocks this rank owns; ``starts``: their offsets in
    the global flat spectrum. A block contributes the values that survive its own cut, and
    of those at most ``D_total`` (the largest; ties to the later position), unless
    ``truncate_multiplets`` (the gap search may look past ``D_total``)."""
    if truncate_multiplets:
        tol_block, D_block = 0, float('inf')
    vals, pos = [], []
    for blk, lo in zip(S_blocks, starts):
        blk = np.asarray(blk, dtype=np.float64)
        keep = _block_cut(blk, tol_block, D_block)
        if not truncate_multiplets and D_total != float('inf') and len(keep) > D_total:
            order = np.argsort(blk[keep], kind='stable')
            keep = np.sort(keep[order[-int(D_total):]])
        vals.append(blk[keep])
        pos.append(keep + int(lo))
    if not vals:
        return np.zeros(0), np.zeros(0, dtype=np.int64)
    return np.concatenate(vals), np.concatenate(pos)


def global_truncation(vals, pos, tol=0, D_total=float('inf'), truncate_multiplets=False):
    """The global cut (linalg.py:713-734) on the gathered candidates: the set of global
    positions kept. Identical on every rank (pure function of the gathered arrays)."""
    vals = np.asarray(vals, dtype=np.float64)
    pos = np.asarray(pos, dtype=np.int64)
    if vals.size == 0:
        return set()
    tmax = np.abs(vals).max()
    D_tol = int(np.sum(vals > tol * tmax))
    D = min(D_total, D_tol)
    if D == 0:
        return set()
    # ascending by value, ties ascending by position (stable argsort of the flat spectrum)
    order = np.lexsort((pos, vals))
    if truncate_multiplets and D < len(order):
        gap = -1
        for p in range(int(D), len(order)):
            gap_p = abs(vals[order[-p]] - vals[order[-p - 1]])
            if gap_p > gap:
                D = p
                gap = gap_p
            if gap > abs(vals[order[-p]]):
                break
    return set(int(x) for x in pos[order[-int(D):]])


def gather_truncation(S_blocks, starts, tol=0, tol_block=0, D_block=float('inf'), D_total=float('inf'),
                      truncate_multiplets=False, group=None):
    """All-gather this rank's candidates (torch.distributed, any backend) and apply the
    global cut. Returns the kept positions within each of this rank's blocks."""
    import torch.distributed as dist
    vals, pos = block_candidates(S_blocks, starts, tol_block, D_block, D_total, truncate_multiplets)
    world = dist.get_world_size(group)
    gathered = [None] * world
    dist.all_gather_object(gathered, (vals.tolist(), pos.tolist()), group=group)
    all_vals = np.concatenate([np.asarray(v, dtype=np.float64) for v, _ in gathered])
    all_pos = np.concatenate([np.asarray(p, dtype=np.int64) for _, p in gathered])
    kept = global_truncation(all_vals, all_pos, tol, D_total, truncate_multiplets)
    out = []
    for blk, lo in zip(S_blocks, starts):
        out.append(np.array(sorted(p - lo for p in kept if lo <= p < lo + len(blk)), dtype=np.int64))
    return out
