"""YASTN itself running on this backend: ``yastn.make_config(backend=yastn_gb300.backend,
default_device='cuda')``, with YASTN's own Tensor layer, metadata logic, linear algebra,
Krylov solver and PEPS environment driving the backend live (no recorded call sequences).

The reference package is imported from the ``baseline/_ref`` install (the unmodified YASTN
package; ``baseline/install_reference.py``); these tests skip where it is absent. Inputs are
built with YASTN's NumPy backend (the oracle) from seeded draws and moved to the GPU
configuration with their data bit for bit, so both sides see the same numbers. Checks:

- structure (charges, block shapes, kept sector dims after truncation) identical to the
  NumPy backend's;
- values within 1e-12 relative (tensordot), singular values within 1e-12;
- the benchmark's U(1) D=64 tensordot + ``svd_with_truncation(D_total=64)``, with YASTN's
  truncation and with ``mask_f=yastn_gb300.truncation_mask``;
- the DMRG two-site Heff2 of the D=1024 XXZ workload inside ``yastn.eigs(ncv=30)``: the
  lowest Ritz value against the reference's recorded one;
- the differentiable CTMRG (Z2, D=6, chi=24, 8 sweeps, checkpointed moves) through
  ``EnvCTM.ctmrg_`` (SVD projectors, and YASTN's default QR projectors): energy and
  gradient against the reference's recorded torch-autograd values.
"""
import json
import os
import sys

import numpy as np
import pytest
import torch

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.path.join(ROOT, 'baseline', '_ref')
if os.path.isdir(REF) and REF not in sys.path:
    sys.path.append(REF)
yastn = pytest.importorskip('yastn', reason='the reference package is not installed under baseline/_ref')

import yastn_gb300  # noqa: E402
from yastn_gb300 import backend as gb  # noqa: E402

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(ROOT, 'tests', 'golden')


def _cfg(sym, **kw):
    return yastn.make_config(sym=sym, backend=gb, default_device='cuda', default_dtype='float64', **kw)


def _to_gpu(t, cfg):
    """The same tensor (structure and data bits) under the GPU configuration."""
    d = torch.from_numpy(np.ascontiguousarray(t._data)).to('cuda')
    return t._replace(config=cfg, data=d)


def _host(t):
    return t._data.detach().cpu().numpy()


def _rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def _leg_dims(ts, w, Dtot):
    p = np.array([w(t) for t in ts]); p = p / p.sum()
    D = np.round(p * Dtot).astype(int)
    while D.sum() > Dtot:
        D[np.argmax(D - p * Dtot)] -= 1
    while D.sum() < Dtot:
        D[np.argmin(D - p * Dtot)] += 1
    return tuple(int(x) for x in D)


@pytest.mark.parametrize('policy', ['fuse_to_matrix', 'fuse_contracted', 'no_fusion'])
def test_tensordot_policies_and_hard_fusion(policy, cuda_device):
    """U(1), Z2xU(1) and dense tensors, permuted and conjugated contractions, hard-fused legs,
    under each tensordot policy: structure identical to the NumPy backend's, values within
    1e-12, and the dense contraction of the dense tensors agrees."""
    cfn = yastn.make_config(sym='U1', backend='np', tensordot_policy=policy)
    cfz = yastn.make_config(sym=yastn.sym.sym_Z2xU1, backend='np', tensordot_policy=policy)
    cfn.backend.random_seed(5)
    l1, l2, l3, l4 = (yastn.Leg(cfn, s=1, t=(-1, 1, 2), D=D) for D in ((1, 2, 3), (4, 2, 3), (3, 1, 2), (5, 4, 2)))
    l5 = yastn.Leg(cfn, s=1, t=(-1, 0, 1), D=(2, 3, 4))
    a = yastn.rand(cfn, legs=[l1.conj(), l2, l3, l4.conj()])
    b = yastn.rand(cfn, legs=[l1, l2.conj(), l5])
    c = yastn.rand(cfn, legs=[l3, l4.conj(), l5])
    d = yastn.rand(cfn, legs=[l3.conj(), l5])
    z = yastn.rand(config=cfz, s=(-1, 1, 1, -1), t=[[(0, 0), (1, 1), (0, 2)]] * 4, D=[[2, 3, 4]] * 4)
    w = yastn.rand(config=cfz, s=(1, -1, 1), t=[[(0, 0), (1, 1), (0, 2)]] * 3, D=[[2, 3, 4]] * 3)
    cases = [
        (a, b, ((0, 1), (0, 1)), False),
        (a, c, ((2, 3), (0, 1)), True),
        (a.fuse_legs(axes=((0, 1), 2, 3), mode='hard'), b.fuse_legs(axes=((0, 1), 2), mode='hard'),
         ((0,), (0,)), False),
        (z, w, ((0, 2), (0, 1)), False),
        (z, z, ((0, 1, 2), (0, 1, 2)), True),
    ]
    cg = {c_: _cfg(c_.sym, tensordot_policy=policy) for c_ in (cfn, cfz)}
    for x, y, axes, conj in cases:
        ref = yastn.tensordot(x, y, axes=axes, conj=(0, 1) if conj else (0, 0))
        xg, yg = _to_gpu(x, cg[x.config]), _to_gpu(y, cg[y.config])
        got = yastn.tensordot(xg, yg, axes=axes, conj=(0, 1) if conj else (0, 0))
        assert got.struct == ref.struct and got.slices == ref.slices
        assert _rel(_host(got), ref._data) <= 1e-12
        assert _rel(got.to_numpy(), ref.to_numpy()) <= 1e-12
    # unfusing a hard-fused result restores the unfused contraction
    f = yastn.tensordot(_to_gpu(a, cg[cfn]).fuse_legs(axes=((0, 1), 2, 3), mode='hard'),
                        _to_gpu(d, cg[cfn]), axes=((1,), (0,)))
    ref = yastn.tensordot(a, d, axes=((2,), (0,))).fuse_legs(axes=((0, 1), 2, 3), mode='hard')
    assert f.struct == ref.struct
    assert _rel(_host(f.unfuse_legs(axes=0)), ref.unfuse_legs(axes=0)._data) <= 1e-12


def test_svd_reconstruction_and_truncation(cuda_device):
    """svd / svd_with_truncation of U(1) tensors on YASTN's Tensor layer: reconstruction,
    orthogonality and singular values against the NumPy backend; truncation by tol, D_block
    and D_total keeps exactly the NumPy backend's sectors and dims."""
    cfn = yastn.make_config(sym='U1', backend='np')
    cfn.backend.random_seed(3)
    legs = [yastn.Leg(cfn, s=1, t=(-1, 0, 1), D=(3, 5, 2)), yastn.Leg(cfn, s=1, t=(-1, 0, 1), D=(4, 6, 3)),
            yastn.Leg(cfn, s=-1, t=(-1, 0, 1), D=(2, 7, 3)), yastn.Leg(cfn, s=-1, t=(-1, 0, 1), D=(5, 4, 2))]
    a = yastn.rand(cfn, legs=legs, n=0)
    ag = _to_gpu(a, _cfg('U1'))
    U, S, V = yastn.svd(ag, axes=((0, 1), (2, 3)))
    Ur, Sr, Vr = yastn.svd(a, axes=((0, 1), (2, 3)))
    assert S.struct == Sr.struct
    assert _rel(_host(S), Sr._data) <= 1e-12
    USV = yastn.ncon([U, S, V], [(-1, -2, 1), (1, 2), (2, -3, -4)])
    assert (USV - ag).norm() <= 1e-12 * ag.norm()
    UU = yastn.tensordot(U, U, axes=((0, 1), (0, 1)), conj=(1, 0))
    assert (UU - yastn.eye(UU.config, legs=UU.get_legs(), isdiag=False)).norm() <= 1e-12 * UU.norm()
    for opts in ({'D_total': 12}, {'tol': 0.3}, {'D_block': 3, 'D_total': 8}, {'tol_block': 0.5, 'D_total': 20}):
        Ug, Sg, Vg = yastn.svd_with_truncation(ag, axes=((0, 1), (2, 3)), **opts)
        Un, Sn, Vn = yastn.svd_with_truncation(a, axes=((0, 1), (2, 3)), **opts)
        assert Sg.struct == Sn.struct, opts
        assert Ug.struct == Un.struct and Vg.struct == Vn.struct, opts
        assert _rel(_host(Sg), Sn._data) <= 1e-12
        # the truncated product agrees with the NumPy backend's (gauge-invariant)
        pg = yastn.ncon([Ug, Sg, Vg], [(-1, -2, 1), (1, 2), (2, -3, -4)])
        pn = yastn.ncon([Un, Sn, Vn], [(-1, -2, 1), (1, 2), (2, -3, -4)])
        assert _rel(pg.to_numpy(), pn.to_numpy()) <= 1e-10


@pytest.mark.parametrize('mask', ['yastn', 'device'])
def test_benchmark_tensordot_and_truncated_svd(mask, cuda_device):
    """The U(1) rank-4 D=64 workload: tensordot (2,3)x(0,1) and svd_with_truncation(D_total=64)
    through YASTN, with YASTN's truncation rule or with the one-launch device mask as mask_f.
    C within 1e-12 of the NumPy backend's, S's kept sectors (11, 41, 12) as recorded."""
    with open(os.path.join(GOLDEN, 'cfg1.json')) as f:
        rec = json.load(f)
    cfn = yastn.make_config(sym='U1', backend='np', tensordot_policy='fuse_to_matrix')
    cfn.backend.random_seed(0)
    ts = tuple(range(-3, 4))
    Ds = _leg_dims(ts, lambda t: np.exp(-t * t / 4), 64)
    assert list(Ds) == rec['leg_D']
    legs = [yastn.Leg(cfn, s=s, t=ts, D=Ds) for s in (1, 1, -1, -1)]
    A = yastn.rand(cfn, legs=legs, distribution='normal')
    B = yastn.rand(cfn, legs=legs, distribution='normal')
    Cn = yastn.tensordot(A, B, axes=((2, 3), (0, 1)))
    cg = _cfg('U1', tensordot_policy='fuse_to_matrix')
    Cg = yastn.tensordot(_to_gpu(A, cg), _to_gpu(B, cg), axes=((2, 3), (0, 1)))
    assert Cg.struct == Cn.struct
    assert _rel(_host(Cg), Cn._data) <= 1e-12
    kw = {'D_total': 64}
    if mask == 'device':
        kw['mask_f'] = lambda S: yastn_gb300.truncation_mask(S, D_total=64)
    U, S, V = yastn.svd_with_truncation(Cg, axes=((0, 1), (2, 3)), **kw)
    assert [list(t) for t in S.struct.t] == rec['S_kept_t']
    assert [list(d) for d in S.struct.D] == rec['S_kept_D']
    assert _rel(_host(S), np.array(rec['S_kept'])) <= 1e-12


def test_dmrg_heff2_inside_yastn_eigs(cuda_device):
    """The DMRG two-site effective Hamiltonian of the XXZ chain (MPO bond 5) on D=1024 U(1)
    virtual legs, applied by YASTN's tensordot inside yastn.eigs(ncv=30, which='SR'): the
    lowest Ritz value against the reference's recorded one (1e-10), in native FP64 and with
    the emulated sector GEMMs."""
    import yastn.tn.mps as mps
    with open(os.path.join(GOLDEN, 'cfg2.json')) as f:
        rec = json.load(f)
    ops_ = yastn.operators.Spin12(sym='U1', backend='np')
    N = 4
    gen = mps.Generator(N=N, operators=ops_)
    gen.random_seed(seed=0)
    H = gen.mpo_from_latex(r"\sum_{i,j \in NN} (Jz sz_{i} sz_{j} + 0.5 Jxy (sp_{i} sm_{j} + sm_{i} sp_{j}))",
                           {"Jz": 1.0, "Jxy": 1.0, "NN": [(i, i + 1) for i in range(N - 1)]})
    psi = gen.random_mps(D_total=8)
    env = mps.Env(psi, [H, psi]).setup_(to='first').setup_(to='last')
    L0, R0 = env.F[(0, 1)], env.F[(3, 2)]
    cfn = psi.config
    cfn.backend.random_seed(0)
    ts0 = tuple(range(-12, 13))
    Ds0 = _leg_dims(ts0, lambda t: np.exp(-t * t / 18), 1024)
    ts, Ds = zip(*[(t, d) for t, d in zip(ts0, Ds0) if d > 0])
    lL, lR = L0.get_legs(), R0.get_legs()
    vl = lambda sg: yastn.Leg(cfn, s=sg, t=ts, D=Ds)
    L = yastn.rand(cfn, legs=[vl(lL[0].s), lL[1], vl(lL[2].s)], distribution='normal')
    R = yastn.rand(cfn, legs=[vl(lR[0].s), lR[1], vl(lR[2].s)], distribution='normal')
    la = psi.pre_2site((1, 2)).get_legs()
    AA = yastn.rand(cfn, legs=[vl(la[0].s), la[1], la[2], vl(la[3].s)], distribution='normal')
    cg = _cfg('U1')
    Lg, Rg, AAg, W1, W2 = (_to_gpu(t, cg) for t in (L, R, AA, H[1], H[2]))
    factor = H.factor

    def heff2(v):
        tmp = v @ Rg
        tmp = yastn.tensordot(W2, tmp, axes=((2, 3), (3, 2)))
        tmp = yastn.tensordot(W1, tmp, axes=((2, 3), (0, 3)))
        tmp = yastn.tensordot(Lg, tmp, axes=((0, 1), (3, 0)))
        return tmp * factor

    saved = gb.get_gemm_mode()
    try:
        for mode in ('fp64', 'emulated'):
            gb.set_gemm_mode(mode)
            out = heff2(AAg)
            assert out.struct == AAg.struct
            Ys = []
            for solver in (yastn.eigs, yastn_gb300.eigs):  # YASTN's loop, then the device-resident one
                val, Y = solver(heff2, AAg, k=1, ncv=30, which='SR', hermitian=True)
                got = float(val[0].real)
                assert abs(got - rec['lanczos_lowest']) <= 1e-10 * abs(rec['lanczos_lowest']), (mode, solver, got)
                assert Y[0].struct == AAg.struct
                Ys.append(Y[0])
            # the same Ritz vector (Lanczos without reorthogonalisation: neither has unit norm)
            ov = abs(float(yastn.vdot(Ys[0], Ys[1]).real)) / float(Ys[0].norm() * Ys[1].norm())
            assert ov >= 1 - 1e-8, ov
    finally:
        gb.set_gemm_mode(saved)


def test_dmrg_with_device_eigs(cuda_device):
    """yastn.tn.mps.dmrg_ (two-site, XXZ chain of 8 sites, D=16) on this backend with its
    eigensolver rebound to the device-resident Lanczos: the energy agrees with the NumPy
    backend's run from the same initial state within 1e-10."""
    import yastn.tn.mps as mps
    import yastn.tn.mps._dmrg as dmrg_mod
    N = 8
    H_latex = r"\sum_{i,j \in NN} (Jz sz_{i} sz_{j} + 0.5 Jxy (sp_{i} sm_{j} + sm_{i} sp_{j}))"
    params = {"Jz": 1.0, "Jxy": 1.0, "NN": [(i, i + 1) for i in range(N - 1)]}
    energies = {}
    for name in ('np', 'gb'):
        ops_ = yastn.operators.Spin12(sym='U1', backend='np')
        gen = mps.Generator(N=N, operators=ops_)
        gen.random_seed(seed=1)
        H = gen.mpo_from_latex(H_latex, params)
        psi = gen.random_mps(D_total=16, n=0)
        if name == 'gb':
            cg = _cfg('U1')
            H = H.shallow_copy()
            psi = psi.shallow_copy()
            for k in range(N):
                H[k] = _to_gpu(H[k], cg)
                psi[k] = _to_gpu(psi[k], cg)
        saved = dmrg_mod.eigs
        if name == 'gb':
            dmrg_mod.eigs = yastn_gb300.eigs
        try:
            out = mps.dmrg_(psi, H, method='2site', max_sweeps=4, opts_svd={'D_total': 16},
                            opts_eigs={'hermitian': True, 'ncv': 5, 'which': 'SR'})
        finally:
            dmrg_mod.eigs = saved
        energies[name] = float(mps.measure_mpo(psi, H, psi).real)
    assert abs(energies['gb'] - energies['np']) <= 1e-10 * abs(energies['np'])


@pytest.mark.parametrize('name', ['ctmrg_z2_d6', 'ctmrg_z2_d6_qr'])
def test_ctmrg_live_energy_and_gradient(name, cuda_device):
    """EnvCTM.ctmrg_ of an iPEPS (1x1 cell, Z2, D=6, d=2, chi=24, 8 sweeps, moves checkpointed
    'nonreentrant') run live by YASTN on this backend, SVD projectors (use_qr=False) and
    YASTN's default QR projectors; transverse-field Ising energy (h=3) and its gradient by
    backward through the backend's adjoints, against the reference's recorded torch-autograd
    values (energy 1e-10; gradient 1e-8, or 1e-5 with QR projectors, whose rank-deficient
    half-systems amplify rounding differences in the QR adjoint)."""
    import yastn.tn.fpeps as fpeps
    with open(os.path.join(GOLDEN, name + '.json')) as f:
        rec = json.load(f)
    arrs = np.load(os.path.join(GOLDEN, name + '.npz'))
    cfn = yastn.make_config(sym='Z2', backend='np', default_dtype='float64')
    vl = yastn.Leg(cfn, s=1, t=(0, 1), D=(3, 3))
    pl = yastn.Leg(cfn, s=1, t=(0, 1), D=(1, 1))
    A0 = yastn.rand(cfn, legs=[vl.conj(), vl, vl, vl.conj(), pl], distribution='normal')
    assert A0.size == arrs['in:A'].size
    cg = _cfg('Z2')
    data = torch.from_numpy(arrs['in:A'].copy()).to('cuda').requires_grad_(True)
    A = A0._replace(config=cg, data=data)
    op = yastn.operators.Spin12(sym='Z2', backend=gb, default_dtype='float64', default_device='cuda')
    Z, X = op.z(), op.x()
    psi = fpeps.Peps(fpeps.SquareLattice(dims=(1, 1), boundary='infinite'), tensors={(0, 0): A})
    env = fpeps.EnvCTM(psi, init='eye', leg=yastn.Leg(cg, s=1, t=(0, 1), D=(1, 1)))
    for _ in env.ctmrg_(opts_svd={'D_total': rec['chi']}, max_sweeps=rec['sweeps'], iterator=True,
                        use_qr=rec.get('use_qr', False), checkpoint_move='nonreentrant'):
        pass
    ez = env.measure_1site(Z)
    exx = env.measure_nn(X, X)
    E = -rec['h'] * sum(ez.values()) - sum(exx.values())
    E.backward()
    assert abs(float(E.detach()) - rec['E']) <= 1e-10 * abs(rec['E'])
    g, gr = data.grad.detach().cpu().numpy(), arrs['ref:grad']
    tol = 1e-5 if rec.get('use_qr', False) else 1e-8
    assert np.abs(g - gr).max() <= tol * np.abs(gr).max()
