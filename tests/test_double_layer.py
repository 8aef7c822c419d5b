"""CPU tests of the double-layer contraction compiler (yastn_gb300.double_layer).

The programs are recorded from YASTN's own append_vec_tl / br / tr / bl
(yastn/tn/fpeps/envs/_env_contractions.py:211-365) and their gather maps composed with
YASTN's torch backend on the host; the composed copies then run through a test-only torch
indexing gather (the native gather, yb_map_gather, is exercised in
tests/test_gpu_double_layer.py). Outputs and gradients must equal YASTN's own composition bit
for bit: the program runs the same GEMMs on the same operand bits.
"""
import os
import sys

import pytest
import torch

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.path.join(ROOT, 'baseline', '_ref')
if os.path.isdir(REF) and REF not in sys.path:
    sys.path.insert(0, REF)
yastn = pytest.importorskip('yastn', reason='the reference package is not installed under baseline/_ref')

import yastn.backend.backend_torch as bt  # noqa: E402
import yastn.tn.fpeps as fpeps  # noqa: E402
import yastn.tn.fpeps.envs._env_contractions as ec  # noqa: E402

from yastn_gb300 import double_layer as dl  # noqa: E402


def torch_gather(src, gmap, inv, conj):
    """out[i] = conj?(sign * src[|gmap[i]| - 1]), 0 where gmap[i] == 0 (test executor)."""
    m = gmap.long()
    out = torch.zeros(m.numel(), dtype=src.dtype)
    nz = m != 0
    v = src[m[nz].abs() - 1]
    v = torch.where(m[nz] < 0, -v, v)
    if conj:
        v = v.conj()
    out[nz] = v
    return out


CASES = [('Z2', False, 'float64'), ('Z2', True, 'complex128'), ('U1', False, 'float64'), ('U1', True, 'float64')]
# (function, the vector's two contracted double-layer legs in its order x [.] [.] y, in_b, out_a per mode)
FUNCS = [('append_vec_tl', (1, 0), (2, 1), {'old': (2, 3), 'self-b': (2, 3), 'b-self': (3, 2)}),
         ('append_vec_br', (3, 2), (2, 1), {'old': (0, 1), 'self-b': (0, 1), 'b-self': (1, 0)}),
         ('append_vec_tr', (0, 3), (1, 2), {'old': (1, 2), 'self-b': (1, 2), 'b-self': (2, 1)}),
         ('append_vec_bl', (2, 1), (2, 1), {'old': (0, 3), 'self-b': (0, 3), 'b-self': (3, 0)})]


def _site(sym, fermionic, dtype, seed=0):
    cfg = yastn.make_config(sym=sym, backend=bt, default_dtype=dtype, fermionic=fermionic)
    cfg.backend.random_seed(seed)
    if sym == 'Z2':
        vl = yastn.Leg(cfg, s=1, t=(0, 1), D=(2, 3))
        pl = yastn.Leg(cfg, s=1, t=(0, 1), D=(1, 1))
        el = yastn.Leg(cfg, s=1, t=(0, 1), D=(4, 3))
    else:
        vl = yastn.Leg(cfg, s=1, t=(-1, 0, 1), D=(1, 2, 1))
        pl = yastn.Leg(cfg, s=1, t=(-1, 1), D=(1, 1))
        el = yastn.Leg(cfg, s=1, t=(-1, 0, 1), D=(2, 3, 2))
    ket = yastn.rand(cfg, legs=[vl.conj(), vl, vl, vl.conj(), pl])
    bra = yastn.rand(cfg, legs=[vl.conj(), vl, vl, vl.conj(), pl])
    return cfg, ket, bra, el, pl


def _vector(cfg, ket, bra, el, dl_legs):
    """x [a a'] [b b'] y contracting the double-layer legs dl_legs (t=0, l=1, b=2, r=3)."""
    dpt = fpeps.DoublePepsTensor(bra=bra, ket=ket)
    la, lb = dpt.get_legs(dl_legs)
    return yastn.rand(cfg, legs=[el, la.conj(), lb.conj(), el.conj()])


def _op(cfg, pl, charged):
    n = (1,) if charged else cfg.sym.zero()
    return yastn.rand(cfg, legs=[pl, pl.conj()], n=n)


def _run_both(fn_name, bra, ket, vec, op, mode, in_b, out_a):
    ref_fn = getattr(ec, fn_name)
    ref = ref_fn(bra, ket, vec, op=op, mode=mode, in_b=in_b, out_a=out_a)
    tensors = (bra, ket, vec) + ((op,) if op is not None else ())
    prog = dl.compile_program(ref_fn, tensors, dict(mode=mode, in_b=in_b, out_a=out_a))
    data = prog.run([t._data for t in tensors], bt, gather=torch_gather)
    return ref, prog.template._replace(config=ket.config, data=data), prog


@pytest.mark.parametrize('sym,fermionic,dtype', CASES)
@pytest.mark.parametrize('fn_name,legs,in_b,out_as', FUNCS)
@pytest.mark.parametrize('mode', ['old', 'self-b', 'b-self'])
def test_program_matches_yastn(sym, fermionic, dtype, fn_name, legs, in_b, out_as, mode):
    cfg, ket, bra, el, pl = _site(sym, fermionic, dtype)
    vec = _vector(cfg, ket, bra, el, legs)
    ref, out, prog = _run_both(fn_name, bra, ket, vec, None, mode, in_b, out_as[mode])
    assert out.struct == ref.struct and out.slices == ref.slices and out.hfs == ref.hfs and out.mfs == ref.mfs
    assert out.trans == ref.trans
    assert torch.equal(out._data, ref._data)
    kinds = [s[0] for s in prog.steps]
    assert kinds.count('gemm') == 2 and kinds.count('gather') <= 5


@pytest.mark.parametrize('fn_name,legs,in_b,out_as', FUNCS)
@pytest.mark.parametrize('charged', [False, True])
def test_program_with_operator(fn_name, legs, in_b, out_as, charged):
    """An operator on the ket's physical leg (DoublePepsTensor.set_operator_): a third GEMM;
    a charged operator also enters the vector's swap gates (fermionic Z2)."""
    cfg, ket, bra, el, pl = _site('Z2', True, 'complex128', seed=3)
    vec = _vector(cfg, ket, bra, el, legs)
    op = _op(cfg, pl, charged)
    for mode in ('old', 'b-self'):
        ref, out, prog = _run_both(fn_name, bra, ket, vec, op, mode, in_b, out_as[mode])
        assert out.struct == ref.struct and torch.equal(out._data, ref._data)
        assert [s[0] for s in prog.steps].count('gemm') == 3


@pytest.mark.parametrize('sym,fermionic,dtype', [CASES[0], CASES[1]])
@pytest.mark.parametrize('fn_name,legs,in_b,out_as', FUNCS)
def test_program_gradients(sym, fermionic, dtype, fn_name, legs, in_b, out_as):
    """Backward through the program (the gather's adjoint is the gather by the inverse map)
    equals YASTN's autograd through its own composition."""
    cfg, ket, bra, el, pl = _site(sym, fermionic, dtype, seed=5)
    vec = _vector(cfg, ket, bra, el, legs)
    grads = []
    for fused in (False, True):
        ts = [t._replace(data=t._data.clone().requires_grad_(True)) for t in (bra, ket, vec)]
        if fused:
            _, out, _ = _run_both(fn_name, *ts, None, 'b-self', in_b, out_as['b-self'])
        else:
            out = getattr(ec, fn_name)(*ts, mode='b-self', in_b=in_b, out_a=out_as['b-self'])
        w = torch.linspace(-1, 1, out._data.numel(), dtype=torch.float64)
        loss = (out._data * w).real.sum() if out._data.is_complex() else (out._data * w).sum()
        loss.backward()
        grads.append([t._data.grad for t in ts])
    for g0, g1 in zip(*grads):
        assert torch.allclose(g0, g1, rtol=0, atol=1e-13 * float(g0.abs().max()))


def test_gather_maps_are_injective_with_inverse():
    cfg, ket, bra, el, pl = _site('U1', True, 'float64', seed=7)
    vec = _vector(cfg, ket, bra, el, (1, 0))
    _, _, prog = _run_both('append_vec_tl', bra, ket, vec, None, 'old', (2, 1), (2, 3))
    maps = prog.maps(bt, torch.device('cpu'))
    seen_negative = False
    for sink, m in maps.items():
        if m is None:
            continue
        gmap, inv, _ = m
        g = gmap.long()
        nz = torch.nonzero(g).reshape(-1)
        assert torch.unique(g[nz].abs()).numel() == nz.numel()
        # the inverse map sends every mapped source back to its destination, with the same sign
        back = inv.long()[g[nz].abs() - 1]
        assert torch.equal(back.abs() - 1, nz) and torch.equal(torch.sign(back), torch.sign(g[nz]))
        seen_negative |= bool((g < 0).any())
    assert seen_negative  # the fermionic swap gates negate blocks through the map


def test_unfusable_chain_is_reported():
    """A backend call outside copies and GEMMs makes the chain unfusable (the drop-in then runs
    YASTN's own function)."""
    cfg, ket, bra, el, pl = _site('Z2', False, 'float64')

    def with_norm(Ac, A, vec, op=None, mode='old', in_b=(2, 1), out_a=(2, 3)):
        return ec.append_vec_tl(Ac, A, vec / vec.norm(), op=op, mode=mode, in_b=in_b, out_a=out_a)
    vec = _vector(cfg, ket, bra, el, (1, 0))
    with pytest.raises(dl.Unfusable):
        dl.compile_program(with_norm, (bra, ket, vec), dict(mode='old', in_b=(2, 1), out_a=(2, 3)))


def test_install_rebinds_and_delegates_for_other_backends():
    """install() rebinds the names where YASTN imported them; tensors of another backend run
    YASTN's own function (the compiled path is for this backend's CUDA tensors)."""
    import yastn.tn.fpeps._doublePepsTensor as dpt_mod
    import yastn.tn.fpeps.envs._env_ctm as ctm_mod
    original = ec.append_vec_tl
    dl.install()
    try:
        assert dpt_mod.append_vec_tl is dl.append_vec_tl and ctm_mod.append_vec_tl is dl.append_vec_tl
        assert ec.append_vec_br is dl.append_vec_br
        cfg, ket, bra, el, pl = _site('Z2', False, 'float64')
        vec = _vector(cfg, ket, bra, el, (1, 0))
        dpt = fpeps.DoublePepsTensor(bra=bra, ket=ket)
        got = dpt.tensordot(vec, axes=((2, 1), (0, 1)), reverse=True)
        want = original(bra, ket, vec, mode='b-self', in_b=(2, 1), out_a=(2, 3))
        assert torch.equal(got._data, want._data)
    finally:
        dl.uninstall()
    assert ec.append_vec_tl is original and dpt_mod.append_vec_tl is original


def test_program_of_a_vector_without_blocks():
    """A boundary vector whose charges meet none of the site's (no blocks): the program's
    output has YASTN's structure (no blocks) and no data."""
    cfg, ket, bra, el, pl = _site('U1', False, 'float64', seed=2)
    la, lb = fpeps.DoublePepsTensor(bra=bra, ket=ket).get_legs((1, 0))
    far = yastn.Leg(cfg, s=1, t=(5,), D=(2,))
    vec = yastn.zeros(cfg, legs=[far, la.conj(), lb.conj(), far.conj()], n=7)
    assert vec.size == 0
    ref, out, prog = _run_both('append_vec_tl', bra, ket, vec, None, 'old', (2, 1), (2, 3))
    assert out.struct == ref.struct and out.size == 0 and torch.equal(out._data, ref._data)
