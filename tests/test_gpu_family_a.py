"""Family (a) on the GPU: merge / unmerge / transpose and their adjoints vs the oracle.

Data movement must be bit-exact. Inputs are the reference's recorded calls plus the
full-size benchmark tensors regenerated from their seed.
"""
import numpy as np
import pytest
import torch

import oracle
from yastn_gb300 import ops
from yastn_gb300.workloads import load_trace, cfg1_inputs

pytestmark = pytest.mark.gpu

TRACES = ['tensordot_fuse_to_matrix', 'tensordot_fuse_contracted', 'tensordot_no_fusion', 'svd', 'svd_ill']


def dev(x):
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


def host(t):
    return t.detach().cpu().numpy()


@pytest.mark.parametrize('name', TRACES)
def test_merge_unmerge_bit_exact_on_reference_calls(name, cuda_device):
    tr = load_trace(name)
    n = 0
    for c in tr['calls']:
        if c['fn'] == 'transpose_and_merge':
            data, order, mn, mm, Dsize = c['args']
            got = host(ops.merge(dev(data), order, mn, mm, Dsize))
            np.testing.assert_array_equal(got, c['out'][0])
            n += 1
        elif c['fn'] == 'unmerge':
            data, meta = c['args']
            np.testing.assert_array_equal(host(ops.unmerge(dev(data), meta)), c['out'][0])
            n += 1
    assert n > 0


@pytest.mark.parametrize('name', ['tensordot_fuse_to_matrix', 'svd'])
def test_merge_with_misaligned_buffers(name, cuda_device):
    """A source view 8 bytes off a 16-byte boundary takes the 8-byte unit path."""
    tr = load_trace(name)
    for c in tr['calls']:
        if c['fn'] == 'transpose_and_merge' and c['args'][0].dtype == np.float64:
            data, order, mn, mm, Dsize = c['args']
            big = torch.zeros(data.size + 1, dtype=torch.float64, device='cuda')
            big[1:] = dev(data)
            view = big[1:]
            assert view.data_ptr() % 16 == 8
            np.testing.assert_array_equal(host(ops.merge(view, order, mn, mm, Dsize)), c['out'][0])


@pytest.mark.parametrize('name', TRACES)
def test_merge_unmerge_adjoints_match_oracle(name, cuda_device):
    tr = load_trace(name)
    rng = np.random.default_rng(0)
    for c in tr['calls']:
        if c['fn'] == 'transpose_and_merge':
            data, order, mn, mm, Dsize = c['args']
            g = rng.normal(size=Dsize).astype(data.dtype)
            got = host(ops.merge_backward(dev(g), order, mn, mm, Dsize, data.size))
            np.testing.assert_array_equal(got, oracle.transpose_and_merge_backward(g, order, mn, mm, data.size))
        elif c['fn'] == 'unmerge':
            data, meta = c['args']
            g = rng.normal(size=data.size).astype(data.dtype)
            got = host(ops.unmerge_backward(dev(g), meta, data.size))
            np.testing.assert_array_equal(got, oracle.unmerge_backward(g, meta, data.size))


def test_merge_golden_adjoint(cuda_device):
    tr = load_trace('adjoints')
    A = tr['_arrays']
    for c in tr['calls']:
        if c['fn'] == 'transpose_and_merge_backward':
            got = host(ops.merge_backward(dev(A[c['out_b']]), c['order'], c['meta_new'], c['meta_mrg'], c['Dsize'],
                                          A[c['data']].size))
            np.testing.assert_array_equal(got, A[c['grad']])
        elif c['fn'] == 'unmerge_backward':
            got = host(ops.unmerge_backward(dev(A[c['out_b']]), c['meta'], A[c['data']].size))
            np.testing.assert_array_equal(got, A[c['grad']])


def test_transpose_blocks(cuda_device):
    """transpose (backend_np.py:646-650) of random blocks, forward and adjoint."""
    rng = np.random.default_rng(1)
    shapes = [(2, 3, 4), (1, 5, 2), (3, 1, 3), (4, 4, 4)]
    axes = (2, 0, 1)
    meta, off = [], 0
    for D in shapes:
        n = int(np.prod(D))
        Dn = tuple(D[a] for a in axes)
        meta.append(((off, off + n), Dn, (off, off + n), D))
        off += n
    meta = tuple(meta)
    data = rng.normal(size=off)
    ref = np.empty_like(data)
    for sln, Dn, slo, Do in meta:
        ref[sln[0]:sln[1]] = data[slo[0]:slo[1]].reshape(Do).transpose(axes).ravel()
    got = host(ops.transpose(dev(data), axes, meta))
    np.testing.assert_array_equal(got, ref)
    back = host(ops.transpose_backward(dev(ref), axes, meta))
    np.testing.assert_array_equal(back, data)


def test_cfg1_full_size_merges(cuda_device):
    """U(1) D=64 rank-4 tensors (2.41M FP64 each): both merges and the unmerge, bit-exact."""
    tr = load_trace('cfg1')
    A, B = cfg1_inputs(tr)
    for c, data in zip(tr['calls'][:2], (A, B)):
        _, order, mn, mm, Dsize = c['args']
        got = host(ops.merge(dev(data), order, mn, mm, Dsize))
        np.testing.assert_array_equal(got, oracle.transpose_and_merge(data, order, mn, mm, Dsize))
    _, meta = tr['calls'][3]['args']
    C = np.random.default_rng(2).normal(size=A.size)
    np.testing.assert_array_equal(host(ops.unmerge(dev(C), meta)), oracle.unmerge(C, meta))
