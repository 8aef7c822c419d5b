"""GPU tests of the fused double-layer PEPS contractions (yastn_gb300.double_layer) and of the
composed-copy kernel behind them (yb_map_gather).

- yb_map_gather against torch indexing, bit for bit (zeros, negated entries, conjugation);
- append_vec_tl / br / tr / bl (yastn/tn/fpeps/envs/_env_contractions.py:211-365) as compiled
  programs on this backend against YASTN's own composition on this backend (bit for bit: the
  same GEMMs on the same operand bits) and against YASTN on its NumPy backend (1e-12), with
  gradients against YASTN's autograd through its composition;
- a live differentiable CTMRG (Z2, D=6, chi=24, moves checkpointed) with the compiled
  contractions installed: energy and gradient against the reference's recorded values.
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
    sys.path.insert(0, REF)
yastn = pytest.importorskip('yastn', reason='the reference package is not installed under baseline/_ref')

import yastn.tn.fpeps as fpeps  # noqa: E402
import yastn.tn.fpeps.envs._env_contractions as ec  # noqa: E402

from yastn_gb300 import backend as gb  # noqa: E402
from yastn_gb300 import double_layer as dl  # noqa: E402
from yastn_gb300 import ops  # noqa: E402

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(ROOT, 'tests', 'golden')

FUNCS = [('append_vec_tl', (1, 0), (2, 1), {'old': (2, 3), 'self-b': (2, 3), 'b-self': (3, 2)}),
         ('append_vec_br', (3, 2), (2, 1), {'old': (0, 1), 'self-b': (0, 1), 'b-self': (1, 0)}),
         ('append_vec_tr', (0, 3), (1, 2), {'old': (1, 2), 'self-b': (1, 2), 'b-self': (2, 1)}),
         ('append_vec_bl', (2, 1), (2, 1), {'old': (0, 3), 'self-b': (0, 3), 'b-self': (3, 0)})]


@pytest.mark.parametrize('dtype', [torch.float64, torch.complex128])
@pytest.mark.parametrize('conj', [False, True])
def test_map_gather_matches_indexing(dtype, conj, cuda_device):
    g = torch.Generator().manual_seed(11)
    n_src, n = 100_003, 250_017
    src = torch.randn(n_src, dtype=dtype, generator=g)
    idx = torch.randint(1, n_src + 1, (n,), generator=g)
    idx[torch.rand(n, generator=g) < 0.1] = 0
    sign = torch.where(torch.rand(n, generator=g) < 0.3, -1, 1)
    gmap = (idx * sign).to(torch.int32)
    want = torch.zeros(n, dtype=dtype)
    nz = gmap != 0
    v = src[gmap[nz].abs().long() - 1]
    v = torch.where(gmap[nz] < 0, -v, v)
    want[nz] = v.conj() if conj else v
    got = ops.map_gather(src.to(cuda_device), gmap.to(cuda_device), conj=conj).cpu()
    assert torch.equal(torch.view_as_real(got) if got.is_complex() else got,
                       torch.view_as_real(want) if want.is_complex() else want)
    # sign bits: -0.0 where a zero is negated, as torch's negation gives
    zsrc = torch.zeros(4, dtype=dtype, device=cuda_device)
    out = ops.map_gather(zsrc, torch.tensor([-1, 2, 0, -4], dtype=torch.int32, device=cuda_device))
    re = out.real if out.is_complex() else out
    assert torch.equal(torch.signbit(re.cpu()), torch.tensor([True, False, False, True]))


def _site(sym, fermionic, dtype, device, seed=0, D=(2, 3), chi=(4, 3)):
    cfg = yastn.make_config(sym=sym, backend=gb, default_dtype=dtype, fermionic=fermionic, default_device=device)
    cfn = yastn.make_config(sym=sym, backend='np', default_dtype=dtype, fermionic=fermionic)
    cfn.backend.random_seed(seed)
    vl = yastn.Leg(cfn, s=1, t=(0, 1), D=D)
    pl = yastn.Leg(cfn, s=1, t=(0, 1), D=(1, 1))
    el = yastn.Leg(cfn, s=1, t=(0, 1), D=chi)
    ket = yastn.rand(cfn, legs=[vl.conj(), vl, vl, vl.conj(), pl])
    bra = yastn.rand(cfn, legs=[vl.conj(), vl, vl, vl.conj(), pl])
    return cfg, cfn, ket, bra, el


def _vector(cfn, ket, bra, el, legs):
    la, lb = fpeps.DoublePepsTensor(bra=bra, ket=ket).get_legs(legs)
    return yastn.rand(cfn, legs=[el, la.conj(), lb.conj(), el.conj()])


def _gpu(t, cfg, device, grad=False):
    d = torch.from_numpy(np.ascontiguousarray(t._data)).to(device)
    return t._replace(config=cfg, data=d.requires_grad_(grad))


@pytest.mark.parametrize('fermionic,dtype', [(False, 'float64'), (True, 'complex128')])
@pytest.mark.parametrize('fn_name,legs,in_b,out_as', FUNCS)
def test_fused_matches_yastn_composition(fermionic, dtype, fn_name, legs, in_b, out_as, cuda_device):
    cfg, cfn, ket, bra, el = _site('Z2', fermionic, dtype, cuda_device)
    vec = _vector(cfn, ket, bra, el, legs)
    ref_fn = getattr(ec, fn_name)
    fused_fn = getattr(dl, fn_name)
    dl.clear_cache()
    for mode in ('old', 'self-b', 'b-self'):
        kw = dict(mode=mode, in_b=in_b, out_a=out_as[mode])
        want_np = ref_fn(bra, ket, vec, **kw)
        ts = [_gpu(t, cfg, cuda_device) for t in (bra, ket, vec)]
        want = ref_fn(*ts, **kw)
        got = fused_fn(*ts, **kw)
        assert got.struct == want.struct and got.hfs == want.hfs and got.trans == want.trans
        assert torch.equal(got._data, want._data)
        h = got._data.cpu().numpy()
        assert np.abs(h - want_np._data).max() <= 1e-12 * np.abs(want_np._data).max()
        got2 = fused_fn(*ts, **kw)  # the cached program
        assert torch.equal(got2._data, want._data)
    info = dl.cache_info()
    assert info['compiled'] == 3 and info['hits'] == 3 and info['unfused'] == 0


@pytest.mark.parametrize('fn_name,legs,in_b,out_as', FUNCS)
def test_fused_gradients(fn_name, legs, in_b, out_as, cuda_device):
    cfg, cfn, ket, bra, el = _site('Z2', True, 'complex128', cuda_device, seed=4)
    vec = _vector(cfn, ket, bra, el, legs)
    kw = dict(mode='b-self', in_b=in_b, out_a=out_as['b-self'])
    grads = []
    for fn in (getattr(ec, fn_name), getattr(dl, fn_name)):
        ts = [_gpu(t, cfg, cuda_device, grad=True) for t in (bra, ket, vec)]
        out = fn(*ts, **kw)
        w = torch.linspace(-1, 1, out._data.numel(), dtype=torch.float64, device=cuda_device)
        (out._data * w).real.sum().backward()
        grads.append([t._data.grad for t in ts])
    for g0, g1 in zip(*grads):
        assert torch.allclose(g0, g1, rtol=0, atol=1e-13 * float(g0.abs().max()))


def test_ctmrg_live_with_fused_contractions(cuda_device):
    """EnvCTM.ctmrg_ (Z2, D=6, chi=24, 8 sweeps, SVD projectors, moves checkpointed) with the
    compiled double-layer contractions installed: energy within 1e-10 and gradient within 1e-8
    of the reference's recorded torch-autograd values; every contraction ran compiled."""
    with open(os.path.join(GOLDEN, 'ctmrg_z2_d6.json')) as f:
        rec = json.load(f)
    arrs = np.load(os.path.join(GOLDEN, 'ctmrg_z2_d6.npz'))
    cfn = yastn.make_config(sym='Z2', backend='np', default_dtype='float64')
    vl = yastn.Leg(cfn, s=1, t=(0, 1), D=(3, 3))
    pl = yastn.Leg(cfn, s=1, t=(0, 1), D=(1, 1))
    A0 = yastn.rand(cfn, legs=[vl.conj(), vl, vl, vl.conj(), pl], distribution='normal')
    cg = yastn.make_config(sym='Z2', backend=gb, default_device='cuda', default_dtype='float64')
    data = torch.from_numpy(arrs['in:A'].copy()).to('cuda').requires_grad_(True)
    A = A0._replace(config=cg, data=data)
    op = yastn.operators.Spin12(sym='Z2', backend=gb, default_dtype='float64', default_device='cuda')
    Z, X = op.z(), op.x()
    dl.clear_cache()
    dl.install()
    try:
        psi = fpeps.Peps(fpeps.SquareLattice(dims=(1, 1), boundary='infinite'), tensors={(0, 0): A})
        env = fpeps.EnvCTM(psi, init='eye', leg=yastn.Leg(cg, s=1, t=(0, 1), D=(1, 1)))
        for _ in env.ctmrg_(opts_svd={'D_total': rec['chi']}, max_sweeps=rec['sweeps'], iterator=True,
                            use_qr=False, checkpoint_move='nonreentrant'):
            pass
        ez = env.measure_1site(Z)
        exx = env.measure_nn(X, X)
        E = -rec['h'] * sum(ez.values()) - sum(exx.values())
        E.backward()
    finally:
        dl.uninstall()
    info = dl.cache_info()
    assert info['compiled'] > 0 and info['hits'] > 0 and info['unfused'] == 0, info
    assert abs(float(E.detach()) - rec['E']) <= 1e-10 * abs(rec['E'])
    g, gr = data.grad.detach().cpu().numpy(), arrs['ref:grad']
    assert np.abs(g - gr).max() <= 1e-8 * np.abs(gr).max()
