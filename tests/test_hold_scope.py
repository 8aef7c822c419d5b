"""CPU tests of the bookkeeping of ops.hold_constant_operands (the scope in which an iterative
solver's unchanged operands keep their merges and digit planes): which tensors are held, when
an entry stops being current, and when entries end. The device side (merges and splits that
reuse the held results, bit for bit) is tested on the GPU in tests/test_gpu_family_b.py."""
import gc

import pytest
import torch

from yastn_gb300 import ops


@pytest.fixture
def capture_state(monkeypatch):
    """The stream-capture query, controlled by the test (no GPU here)."""
    state = [False]
    monkeypatch.setattr(ops.torch.cuda, 'is_current_stream_capturing', lambda: state[0])
    return state


def test_nothing_is_held_outside_the_scope(capture_state):
    src = torch.ones(4, dtype=torch.float64)
    assert ops._held('merge', ('plan',), src) is None


def test_entries_follow_version_counters(capture_state):
    src = torch.ones(4, dtype=torch.float64)
    out = torch.zeros(4, dtype=torch.float64)
    with ops.hold_constant_operands():
        held = ops._held('merge', ('plan',), src)
        assert ops._hit(held, src) is None
        ops._store(held, src, out, track_output=True)
        assert ops._hit(ops._held('merge', ('plan',), src), src) is out
        out.mul_(2.0)  # the held output modified in place: no longer current
        assert ops._hit(ops._held('merge', ('plan',), src), src) is None
        ops._store(ops._held('merge', ('plan',), src), src, out, track_output=True)
        src.add_(1.0)  # the source modified in place: no longer current
        assert ops._hit(ops._held('merge', ('plan',), src), src) is None
        other = torch.ones(4, dtype=torch.float64)  # same values, another tensor object: not the same operand
        assert ops._hit(ops._held('merge', ('plan',), other), other) is None
        # digit planes (untracked payload): current while the source is unchanged
        planes = (torch.zeros(8, dtype=torch.bfloat16), torch.zeros(2, dtype=torch.int32))
        ops._store(ops._held('split', ('p', 0), src), src, planes)
        assert ops._hit(ops._held('split', ('p', 0), src), src) is planes
        assert ops._hit(ops._held('split', ('p', 1), src), src) is None  # the other operand's key


def test_grad_tensors_are_never_held(capture_state):
    src = torch.ones(4, dtype=torch.float64, requires_grad=True)
    with ops.hold_constant_operands():
        assert ops._held('merge', ('plan',), src) is None


def test_entries_end_with_their_source_and_with_the_scope(capture_state):
    with ops.hold_constant_operands():
        src = torch.ones(4, dtype=torch.float64)
        ops._store(ops._held('merge', ('plan',), src), src, torch.zeros(4), track_output=True)
        assert len(ops._HOLD['merge']) == 1
        del src
        gc.collect()
        assert len(ops._HOLD['merge']) == 0  # the temporaries of one application are not kept
        keep = torch.ones(4, dtype=torch.float64)
        with ops.hold_constant_operands():  # nested scopes share the entries
            ops._store(ops._held('merge', ('plan',), keep), keep, torch.zeros(4), track_output=True)
        assert len(ops._HOLD['merge']) == 1
    assert not ops._HOLD['merge'] and not ops._HOLD['split']


def test_a_change_of_capture_state_drops_the_entries(capture_state):
    keep = torch.ones(4, dtype=torch.float64)
    with ops.hold_constant_operands():
        ops._store(ops._held('merge', ('plan',), keep), keep, torch.zeros(4), track_output=True)
        capture_state[0] = True  # a CUDA-graph capture begins: earlier entries are not used in it
        assert ops._hit(ops._held('merge', ('plan',), keep), keep) is None
        assert not ops._HOLD['merge']
