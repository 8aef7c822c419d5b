"""Device-resident Lanczos (yastn_gb300.krylov; fused kernels yb_krylov_*) against the
host restatement of YASTN's hermitian Krylov expansion (yastn/tensor/_krylov.py:17-46,
yastn/krylov/_krylov.py:177-238) on the same operator and start vector: tridiagonal
coefficients within 1e-12, the happy-breakdown rule, complex Hermitian operators, and the
CUDA-graph replay against the eager expansion."""
import numpy as np
import pytest
import torch

from yastn_gb300 import krylov as K
from yastn_gb300.workloads import lanczos as host_lanczos, ritz_lowest

pytestmark = pytest.mark.gpu


def _hermitian(n, rng, cplx=False, spectrum=None):
    X = rng.normal(size=(n, n)) + (1j * rng.normal(size=(n, n)) if cplx else 0)
    Q, _ = np.linalg.qr(X)
    d = rng.normal(size=n) if spectrum is None else np.asarray(spectrum, dtype=float)
    return (Q * d) @ Q.conj().T


@pytest.mark.parametrize('cplx', [False, True])
def test_lanczos_coefficients_match_host_restatement(cplx, cuda_device):
    rng = np.random.default_rng(3)
    n, ncv = 300, 25
    H = _hermitian(n, rng, cplx)
    v0 = rng.normal(size=n) + (1j * rng.normal(size=n) if cplx else 0)
    Hd = torch.from_numpy(H).cuda()
    st = K.lanczos(lambda x: Hd @ x, torch.from_numpy(v0).cuda(), ncv)
    _, al, be = host_lanczos(lambda x: H @ x, v0, ncv, np.vdot, np.linalg.norm)
    al_d, be_d = st.alpha.cpu().numpy(), st.beta[:ncv].cpu().numpy()
    assert np.abs(al_d - np.array(al)).max() <= 1e-12 * np.abs(H).max() * n ** 0.5
    assert np.abs(be_d - np.array(be)).max() <= 1e-12 * np.abs(H).max() * n ** 0.5
    m, val, vr = K.ritz(st, 'SR')
    assert m == ncv
    lam, _ = ritz_lowest(np.real(al), be)
    assert abs(val[0] - lam) <= 1e-12 * abs(lam)
    # the Ritz vector: residual of the lowest eigenpair of the Krylov projection
    y = K.combine(st, vr[:, 0], m).cpu().numpy()
    assert abs(np.linalg.norm(y) - 1) <= 1e-10


def test_happy_breakdown_truncates_the_basis(cuda_device):
    """An operator with 4 distinct eigenvalues: the expansion breaks down after 4 steps and
    the Ritz values are exactly those eigenvalues (as YASTN's loop, which stops there)."""
    rng = np.random.default_rng(5)
    n = 64
    spec = np.repeat([-2.0, -0.5, 1.0, 3.0], n // 4)
    H = _hermitian(n, rng, False, spec)
    Hd = torch.from_numpy(H).cuda()
    st = K.lanczos(lambda x: Hd @ x, torch.from_numpy(rng.normal(size=n)).cuda(), 10)
    m, val, _ = K.ritz(st, 'SR', tol=1e-10)
    assert m == 4
    assert np.allclose(np.sort(val), [-2.0, -0.5, 1.0, 3.0], atol=1e-10)


def test_graph_replay_equals_eager_expansion(cuda_device):
    rng = np.random.default_rng(9)
    n, ncv = 500, 20
    H = _hermitian(n, rng)
    Hd = torch.from_numpy(H).cuda()
    mv = lambda x: Hd @ x
    v0 = torch.from_numpy(rng.normal(size=n)).cuda()
    eager = K.lanczos(mv, v0, ncv)
    al, be = eager.alpha.clone(), eager.beta.clone()
    g = K.LanczosGraph(mv, v0, ncv)
    for _ in range(3):
        st = g.replay()
        torch.cuda.synchronize()
        assert torch.equal(st.alpha, al) and torch.equal(st.beta, be)
    v1 = torch.from_numpy(rng.normal(size=n)).cuda()
    g.v0.copy_(v1)
    st = g.replay()
    ref = K.lanczos(mv, v1, ncv)
    torch.cuda.synchronize()
    assert torch.equal(st.alpha, ref.alpha) and torch.equal(st.beta, ref.beta)
