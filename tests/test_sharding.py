"""Sector sharding and the global-truncation exchange on CPU ranks (gloo, world size 2).

Each rank computes its longest-processing-time share of the units with the oracle; the
union of the shards reproduces the single-process result, and the all-gathered truncation
keeps exactly what the single-process rule (the oracle, stable argsort) keeps, including
ties, per-block cuts and the multiplet extension.
"""
import os
import socket

import numpy as np
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

import oracle
from yastn_gb300 import sharding

CASES = [dict(D_total=40), dict(tol=0.2), dict(D_total=25, tol_block=0.05, D_block=9),
         dict(D_total=30, truncate_multiplets=True), dict(D_total=1000)]


def _spectrum():
    rng = np.random.default_rng(5)
    sizes = [12, 7, 30, 1, 18, 25, 9, 14, 3]
    blocks = [np.sort(rng.exponential(size=n))[::-1] for n in sizes]
    blocks[2][5] = blocks[5][3]          # an exact tie across blocks
    blocks[4][:4] = blocks[4][0]         # a multiplet
    blocks[7][-3:] = 0.0                 # zero singular values
    starts = np.cumsum([0] + sizes[:-1]).tolist()
    return blocks, starts


def _free_port():
    with socket.socket() as s:
        s.bind(('127.0.0.1', 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out_dir):
    os.environ['MASTER_ADDR'] = '127.0.0.1'
    os.environ['MASTER_PORT'] = str(port)
    dist.init_process_group('gloo', rank=rank, world_size=world)
    try:
        blocks, starts = _spectrum()
        costs = [len(b) ** 3 for b in blocks]
        owner = sharding.lpt_assign(costs, world)
        mine = [i for i, o in enumerate(owner) if o == rank]
        res = {}
        for ci, case in enumerate(CASES):
            kept = sharding.gather_truncation([blocks[i] for i in mine], [starts[i] for i in mine], **case)
            res[ci] = {i: k.tolist() for i, k in zip(mine, kept)}
        # sharded sector GEMMs: each rank fills its outputs, an all-reduce sums the shards
        rng = np.random.default_rng(11)
        shapes = [(40, 70, 30), (16, 16, 16), (3, 200, 5), (64, 20, 33), (9, 9, 9)]
        meta, oa, ob, oc = [], 0, 0, 0
        for m, k, n in shapes:
            meta.append(((oc, oc + m * n), (m, n), (oa, oa + m * k), (m, k), (ob, ob + k * n), (k, n)))
            oa += m * k; ob += k * n; oc += m * n
        meta = tuple(meta)
        A, B = rng.normal(size=oa), rng.normal(size=ob)
        sub, _ = sharding.shard_dot(meta, rank, world)
        part = oracle.dot(A, B, sub, oc)
        C = torch.zeros(oc, dtype=torch.float64)
        for slc, *_ in sub:  # this rank's outputs only (the rest of the buffer is not written)
            C[slc[0]:slc[1]] = torch.from_numpy(part[slc[0]:slc[1]])
        dist.all_reduce(C)
        np.save(os.path.join(out_dir, f'C{rank}.npy'), C.numpy())
        np.save(os.path.join(out_dir, f'kept{rank}.npy'), np.array([res], dtype=object), allow_pickle=True)
    finally:
        dist.destroy_process_group()


def test_lpt_assign_covers_and_balances():
    rng = np.random.default_rng(1)
    costs = rng.integers(1, 10 ** 6, size=57).astype(float).tolist()
    for world in (1, 2, 3, 8):
        owner = sharding.lpt_assign(costs, world)
        assert sorted(set(owner)) == list(range(min(world, len(costs))))
        load = np.zeros(world)
        for c, o in zip(costs, owner):
            load[o] += c
        assert load.max() <= sum(costs) / world + max(costs)


def test_candidates_and_global_cut_match_single_process_rule():
    blocks, starts = _spectrum()
    S = np.concatenate(blocks)
    slices = [(lo, lo + len(b)) for lo, b in zip(starts, blocks)]
    for case in CASES:
        ref = oracle.truncation_mask(S, slices, argsort=lambda x: np.argsort(x, kind='stable'), **case)
        vals, pos = sharding.block_candidates(blocks, starts, case.get('tol_block', 0),
                                              case.get('D_block', float('inf')), case.get('D_total', float('inf')),
                                              case.get('truncate_multiplets', False))
        kept = sharding.global_truncation(vals, pos, case.get('tol', 0), case.get('D_total', float('inf')),
                                          case.get('truncate_multiplets', False))
        assert kept == set(np.nonzero(ref)[0].tolist()), case


def test_two_ranks_gloo(tmp_path):
    port = _free_port()
    mp.spawn(_worker, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    blocks, starts = _spectrum()
    S = np.concatenate(blocks)
    slices = [(lo, lo + len(b)) for lo, b in zip(starts, blocks)]
    per_rank = [np.load(tmp_path / f'kept{r}.npy', allow_pickle=True)[0] for r in range(2)]
    for ci, case in enumerate(CASES):
        ref = oracle.truncation_mask(S, slices, argsort=lambda x: np.argsort(x, kind='stable'), **case)
        got = np.zeros(S.shape, dtype=bool)
        owned = {}
        for r in range(2):
            for i, k in per_rank[r][ci].items():
                assert i not in owned  # every block owned by one rank
                owned[i] = r
                got[starts[i] + np.asarray(k, dtype=np.int64)] = True
        assert sorted(owned) == list(range(len(blocks)))
        np.testing.assert_array_equal(got, ref)
    C0, C1 = np.load(tmp_path / 'C0.npy'), np.load(tmp_path / 'C1.npy')
    np.testing.assert_array_equal(C0, C1)
    rng = np.random.default_rng(11)
    shapes = [(40, 70, 30), (16, 16, 16), (3, 200, 5), (64, 20, 33), (9, 9, 9)]
    meta, oa, ob, oc = [], 0, 0, 0
    for m, k, n in shapes:
        meta.append(((oc, oc + m * n), (m, n), (oa, oa + m * k), (m, k), (ob, ob + k * n), (k, n)))
        oa += m * k; ob += k * n; oc += m * n
    A, B = rng.normal(size=oa), rng.normal(size=ob)
    np.testing.assert_allclose(C0, oracle.dot(A, B, tuple(meta), oc), rtol=0, atol=1e-12)
