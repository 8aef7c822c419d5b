"""Differentiable CTMRG on the GPU: the reference's own call sequence (iPEPS on a 1x1 unit
cell, Z2, D=6, 8 CTM sweeps with truncated block-SVD projectors, transverse-field Ising
energy; recorded from YASTN with its torch backend, tests/golden/make_golden.py scen_ctmrg)
replayed through this backend. The energy must match the reference's, the gradient
(backward through the hand-written adjoints of merges, dots, masks, the SVD with Lorentzian
broadening 1e-12 and the gauge fix) the reference's torch-autograd gradient, and central
finite differences (step 1e-6) along random directions."""
import numpy as np
import pytest
import torch

from yastn_gb300 import backend as BK
from yastn_gb300.replay import load_replay

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def replay():
    return load_replay('ctmrg_z2_d6')


def _energy(replay, A):
    env = replay.run(BK, 'cuda', {'A': A})
    return env[replay.outputs['E']]


def test_ctmrg_energy_and_gradient_match_reference(replay, cuda_device):
    A = torch.from_numpy(replay.arrays['in:A']).cuda().requires_grad_(True)
    E = _energy(replay, A)
    E_ref = replay.payload['E']
    assert abs(float(E.detach()) - E_ref) <= 1e-10 * abs(E_ref)
    E.backward()
    g, ref = A.grad.cpu().numpy(), replay.arrays['ref:grad']
    assert np.abs(g - ref).max() <= 1e-8 * np.abs(ref).max()


def test_ctmrg_gradient_finite_differences(replay, cuda_device):
    A0 = torch.from_numpy(replay.arrays['in:A']).cuda()
    A = A0.clone().requires_grad_(True)
    E = _energy(replay, A)
    E.backward()
    g = A.grad.detach()
    rng = np.random.default_rng(3)
    h = 1e-6
    with torch.no_grad():
        for _ in range(2):
            d = torch.from_numpy(rng.normal(size=A0.numel())).cuda()
            d /= d.norm()
            fd = (float(_energy(replay, A0 + h * d)) - float(_energy(replay, A0 - h * d))) / (2 * h)
            an = float((g * d).sum())
            # the central difference carries O(h^2) truncation and the SVD adjoint the 1e-12
            # broadening: agreement to 1e-7 of the gradient norm (d is a unit vector)
            assert abs(fd - an) <= 1e-7 * float(g.norm()), (fd, an)


def test_ctmrg_checkpointed_moves_match_reference(replay, cuda_device):
    """The same run with every CTM move under non-reentrant checkpointing (the recorded
    checkpoint_move markers): identical energy, and the gradient through the recomputed
    moves matches the reference's."""
    A = torch.from_numpy(replay.arrays['in:A']).cuda().requires_grad_(True)
    env = replay.run(BK, 'cuda', {'A': A}, checkpoint=True)
    E = env[replay.outputs['E']]
    assert abs(float(E.detach()) - replay.payload['E']) <= 1e-10 * abs(replay.payload['E'])
    E.backward()
    g, ref = A.grad.cpu().numpy(), replay.arrays['ref:grad']
    assert np.abs(g - ref).max() <= 1e-8 * np.abs(ref).max()
