"""The oracle (NumPy restatement) against golden vectors recorded from the reference.

Every hot-path backend call recorded from YASTN's NumPy backend is replayed through
``oracle`` on the recorded inputs; outputs must match (bit-exact for pure data
movement, 1e-12 relative for arithmetic, gauge-invariant checks for SVD/eigh).
"""
import json
import os

import numpy as np
import pytest

import oracle
from yastn_gb300.workloads import load_trace, GOLDEN

TRACES = ['tensordot_fuse_to_matrix', 'tensordot_fuse_contracted', 'tensordot_no_fusion', 'svd', 'eigh',
          'fix_signs']
MOVES = ('transpose_and_merge', 'unmerge', 'apply_mask', 'embed_mask')


def _rel(a, b):
    den = max(np.abs(b).max(), 1e-300) if b.size else 1.0
    return float(np.abs(a - b).max() / den) if b.size else 0.0


@pytest.mark.parametrize('name', TRACES)
def test_oracle_replays_reference_calls(name):
    tr = load_trace(name)
    n_checked = 0
    for c in tr['calls']:
        fn, args, out = c['fn'], c['args'], c['out']
        if fn in MOVES:
            res = getattr(oracle, fn)(*args)
            assert res.dtype == out[0].dtype
            np.testing.assert_array_equal(res, out[0])
        elif fn in ('dot', 'transpose_dot_sum'):
            res = getattr(oracle, fn)(*args)
            assert res.dtype == out[0].dtype
            assert _rel(res, out[0]) < 1e-12
        elif fn == 'svd':
            data, meta, sizes = args[:3]
            U, S, V = oracle.svd(data, meta, sizes)
            assert _rel(S, out[1]) < 1e-12
            for sl, D, slU, DU, slS, slV, DV in meta:
                a = data[sl[0]:sl[1]].reshape(D)
                rec = (U[slU[0]:slU[1]].reshape(DU) * S[slS[0]:slS[1]]) @ V[slV[0]:slV[1]].reshape(DV)
                assert _rel(rec, a) < 1e-12
        elif fn == 'fix_svd_signs':
            Ui, Vi, meta = args
            Uo, Vo = oracle.fix_svd_signs(Ui, Vi, meta)
            assert _rel(Uo, out[0]) < 1e-12 and _rel(Vo, out[1]) < 1e-12
        elif fn == 'eigh':
            data, meta, sizes = args
            S, U = oracle.eigh(data, meta, sizes)
            assert _rel(S, out[0]) < 1e-12
            for sl, D, slU, DU, slS in meta:
                a = data[sl[0]:sl[1]].reshape(D)
                u = U[slU[0]:slU[1]].reshape(DU)
                s = S[slS[0]:slS[1]]
                assert _rel((u * s) @ u.conj().T, a) < 1e-12
        else:
            continue
        n_checked += 1
    assert n_checked > 0


def test_oracle_fix_signs_golden_matrix():
    """test_svd.py:159-186: the gauge-fixed U of the reference test."""
    tr = load_trace('fix_signs')
    svd_call = [c for c in tr['calls'] if c['fn'] == 'svd'][0]
    fix_call = [c for c in tr['calls'] if c['fn'] == 'fix_svd_signs'][0]
    data, meta, sizes = svd_call['args'][:3]
    U, S, V = oracle.svd(data, meta, sizes)
    Uf, Vf = oracle.fix_svd_signs(U, V, meta)
    assert _rel(Uf, fix_call['out'][0]) < 1e-12
    # the golden matrix of the reference test, columns (re, im) pairs
    gold = {k: np.array(v)[:, 0::2] + 1j * np.array(v)[:, 1::2] for k, v in tr['Ufixed'].items()}
    blocks = [Uf[m[2][0]:m[2][1]].reshape(m[3]) for m in meta]
    assert any(b.shape == (3, 2) and np.abs(b - gold['(0,0)']).max() < 1e-12 for b in blocks)
    assert any(b.shape == (2, 2) and np.abs(b - gold['(1,1)']).max() < 1e-12 for b in blocks)


def test_oracle_fix_signs_adjoint_matches_reference_autograd():
    """The adjoint of fix_svd_signs (real, and complex with the gradient through each column's
    phase) against torch's autograd of the reference's backend_torch.fix_svd_signs."""
    import json, os
    from yastn_gb300.workloads import GOLDEN, _decode
    with open(os.path.join(GOLDEN, 'fix_signs_adjoint.json')) as f:
        calls = json.load(f)['calls']
    z = np.load(os.path.join(GOLDEN, 'fix_signs_adjoint.npz'))
    kinds = set()
    for c in calls:
        meta = _decode(c['meta'], None)
        U, V, gU, gV = (z[c[k]] for k in ('U', 'V', 'gU', 'gV'))
        Uf, Vf = oracle.fix_svd_signs(U, V, meta)
        assert _rel(Uf, z[c['Uf']]) < 1e-14 and _rel(Vf, z[c['Vf']]) < 1e-14
        dU, dV = oracle.fix_svd_signs_backward(U, V, gU, gV, meta)
        assert _rel(dU, z[c['dU']]) < 1e-12 and _rel(dV, z[c['dV']]) < 1e-12
        kinds.add(np.iscomplexobj(U))
    assert kinds == {False, True}


def _decode_opts(opts):
    out = {}
    for k, v in opts.items():
        if isinstance(v, dict) and '__dict__' in v:
            v = {tuple(kk): vv for kk, vv in v['__dict__']}
        out[k] = v
    return out


def test_oracle_truncation_matches_reference_masks():
    with open(os.path.join(GOLDEN, 'truncation.json')) as f:
        cases = json.load(f)['cases']
    assert len(cases) >= 13
    for case in cases:
        S = np.array(case['S'])
        charges = [tuple(c) for c in case['charges']]
        mask = oracle.truncation_mask(S, case['slices'], charges, **_decode_opts(case['opts']))
        np.testing.assert_array_equal(mask, np.array(case['mask'], dtype=bool))


def test_oracle_truncation_reference_shapes():
    """Exact kept counts asserted by the reference tests (test_svd.py:189-266, :344-388)."""
    with open(os.path.join(GOLDEN, 'truncation.json')) as f:
        cases = json.load(f)['cases']
    kept = [int(np.sum(c['mask'])) for c in cases]
    assert kept[:6] == [12, 11, 9, 4, 12, 0]
    assert kept[6:9] == [30, 32, 24]


def test_oracle_adjoints_match_reference_autograd():
    tr = load_trace('adjoints')
    A = tr['_arrays']
    for c in tr['calls']:
        if c['fn'] == 'svd_backward':
            meta = c['meta']
            U, S, V = A[c['U']], A[c['S']], A[c['V']]
            # the golden cotangents are stored as d(loss)/d(conj x); pass them as-is
            grad = oracle.svd_backward(U, S, V, A[c['gU']], A[c['gS']], A[c['gV']], meta,
                                       A[c['data']].size, A[c['data']].dtype)
            assert _rel(grad, A[c['grad']]) < 1e-10
        elif c['fn'] == 'dot_backward':
            Ab, Bb = oracle.dot_backward(A[c['Cb']], A[c['A']], A[c['B']], c['meta'])
            assert _rel(Ab, A[c['Ab']]) < 1e-12 and _rel(Bb, A[c['Bb']]) < 1e-12
        elif c['fn'] == 'transpose_and_merge_backward':
            g = oracle.transpose_and_merge_backward(A[c['out_b']], c['order'], c['meta_new'], c['meta_mrg'],
                                                    A[c['data']].size)
            np.testing.assert_array_equal(g, A[c['grad']])
        elif c['fn'] == 'unmerge_backward':
            g = oracle.unmerge_backward(A[c['out_b']], c['meta'], A[c['data']].size)
            np.testing.assert_array_equal(g, A[c['grad']])


def test_cfg1_fixture_consistent_with_regenerated_inputs():
    """The benchmark inputs regenerate from the seed; the first merge's input checksum matches."""
    from yastn_gb300.workloads import cfg1_inputs
    tr = load_trace('cfg1')
    A, B = cfg1_inputs(tr)
    first = tr['calls'][0]['args'][0]
    assert first.shape == A.shape
    assert abs(first.checksum['sum0'] - float(A.sum())) < 1e-9 * first.checksum['abs0']
    assert first.checksum['head0'] == [float(x) for x in A[:8]]
    second = tr['calls'][1]['args'][0]
    assert second.checksum['head0'] == [float(x) for x in B[:8]]


def test_cfg3_replay_matches_reference_checksum():
    """The U(1)xU(1) complex workload regenerates from its seed and the oracle's tensordot
    (two merges and 595 complex sector GEMMs) reproduces the reference's checksum of C."""
    from yastn_gb300.workloads import cfg3_inputs
    tr = load_trace('cfg3')
    A, B = cfg3_inputs(tr)
    c0, c1, c2 = tr['calls'][:3]
    assert c0['args'][0].checksum['head0'] == [float(x) for x in A.real[:8]]
    assert c1['args'][0].checksum['head1'] == [float(x) for x in B.imag[:8]]
    Am = oracle.transpose_and_merge(A, *c0['args'][1:])
    Bm = oracle.transpose_and_merge(B, *c1['args'][1:])
    C = oracle.dot(Am, Bm, *c2['args'][2:])
    chk = tr['C_checksum']
    assert C.size == chk['n']
    for i, part in enumerate((C.real, C.imag)):
        assert abs(float(part.sum()) - chk[f'sum{i}']) <= 1e-10 * chk[f'abs{i}']
        assert abs(float((part * part).sum()) - chk[f'sq{i}']) <= 1e-10 * chk[f'sq{i}']


def test_cfg5_replay_matches_reference_checksum():
    """The precision-study workload (per-block scales over four decades) regenerates from
    its seeds, and the oracle's tensordot reproduces the reference's result checksum."""
    from yastn_gb300.workloads import cfg5_inputs
    tr = load_trace('cfg5')
    A, B = cfg5_inputs(tr)
    c0, c1, c2, c3 = tr['calls']
    assert c0['args'][0].checksum['head0'] == [float(x) for x in A[:8]]
    assert abs(c1['args'][0].checksum['sum0'] - float(B.sum())) <= 1e-9 * c1['args'][0].checksum['abs0']
    Am = oracle.transpose_and_merge(A, *c0['args'][1:])
    Bm = oracle.transpose_and_merge(B, *c1['args'][1:])
    Cm = oracle.dot(Am, Bm, *c2['args'][2:])
    C = oracle.unmerge(Cm, c3['args'][1])
    chk = tr['C_checksum']
    assert C.size == chk['n']
    assert abs(float(C.sum()) - chk['sum0']) <= 1e-10 * chk['abs0']
    assert abs(float((C * C).sum()) - chk['sq0']) <= 1e-10 * chk['sq0']


def test_oracle_eigh_adjoint_matches_reference_autograd():
    """Both eigh adjoints (SYMEIG with order_by_magnitude, torch.linalg.eigh otherwise; real
    and complex Hermitian, a degenerate pair included) against the reference's autograd."""
    import numpy as np
    from yastn_gb300.workloads import GOLDEN, _decode
    with open(os.path.join(GOLDEN, 'eigh_adjoint.json')) as f:
        calls = json.load(f)['calls']
    z = np.load(os.path.join(GOLDEN, 'eigh_adjoint.npz'))
    for c in calls:
        meta = _decode(c['meta'], None)
        g = oracle.eigh_backward(z[c['U']], z[c['S']], z[c['gU']], z[c['gS']], meta, z[c['data']].size,
                                 z[c['data']].dtype, c['order_by_magnitude'])
        assert _rel(g, z[c['grad']]) < 1e-10, c['order_by_magnitude']


def test_oracle_tds_adjoint_matches_reference_autograd():
    import numpy as np
    from yastn_gb300.workloads import GOLDEN
    with open(os.path.join(GOLDEN, 'tds_adjoint.json')) as f:
        args = json.load(f)['args']
    from yastn_gb300.workloads import _decode
    meta, Ar, Br, Ao, Bo, _ = (_decode(a, None) for a in args)
    z = np.load(os.path.join(GOLDEN, 'tds_adjoint.npz'))
    Ab, Bb = oracle.transpose_dot_sum_backward(z['Cb'], z['A'], z['B'], meta, Ar, Br, Ao, Bo)
    assert _rel(Ab, z['Ab']) < 1e-12 and _rel(Bb, z['Bb']) < 1e-12


def test_oracle_ill_conditioned_svd():
    tr = load_trace('svd_ill')
    c = [c for c in tr['calls'] if c['fn'] == 'svd'][0]
    data, meta, sizes = c['args'][:3]
    U, S, V = oracle.svd(data, meta, sizes)
    assert _rel(S, c['out'][1]) < 1e-12


def test_heff2_replay_and_lanczos_match_reference():
    """The DMRG workload replayed through the oracle reproduces the reference's matvec
    checksum and its 30-step Lanczos lowest Ritz value."""
    from yastn_gb300.workloads import Heff2Workload, lanczos, ritz_lowest
    wl = Heff2Workload()
    env = wl.env(lambda x: x)
    mv = lambda v: wl.matvec(v, env, oracle.dot, oracle.transpose_and_merge, lambda x, f: x * f)
    out = mv(wl.data['AA'])
    chk = wl.tr['out_checksum']
    assert abs(float(out.sum()) - chk['sum0']) <= 1e-10 * chk['abs0']
    assert out[:8].tolist() == pytest.approx(chk['head0'], rel=1e-12, abs=1e-12 * chk['abs0'] / out.size)
    V, al, be = lanczos(mv, wl.data['AA'], wl.tr['lanczos_ncv'], np.dot, np.linalg.norm)
    lam, _ = ritz_lowest(al, be)
    assert abs(lam - wl.tr['lanczos_lowest']) <= 1e-10 * abs(wl.tr['lanczos_lowest'])
    assert wl.flops == 630254080 or abs(wl.flops - 6.303e8) < 1e6


def test_oracle_qr_and_adjoint_match_reference():
    """qr (positive diagonal of R) against the reference's NumPy backend on tall, square,
    wide, complex and rank-deficient blocks; the adjoint (real and complex) against the
    reference torch backend's autograd gradient."""
    tr = load_trace('qr')
    n_adj = 0
    for c in tr['calls']:
        if c['fn'] != 'qr':
            continue
        data, meta, sizes = c['args']
        Q, R = oracle.qr(data, meta, sizes)
        Qr, Rr = c['out']
        for sl, D, slQ, DQ, slR, DR in meta:
            a = data[sl[0]:sl[1]].reshape(D)
            q, r = Q[slQ[0]:slQ[1]].reshape(DQ), R[slR[0]:slR[1]].reshape(DR)
            assert _rel(q @ r, a) < 1e-13
            assert np.abs(q.conj().T @ q - np.eye(DQ[1])).max() < 1e-13
            assert (np.real(np.diag(r)) >= 0).all()
            if np.linalg.matrix_rank(a) == min(D):  # unique factorisation
                assert _rel(q, Qr[slQ[0]:slQ[1]].reshape(DQ)) < 1e-11
                assert _rel(r, Rr[slR[0]:slR[1]].reshape(DR)) < 1e-11
        full = all(np.linalg.matrix_rank(data[sl[0]:sl[1]].reshape(D)) == min(D) for sl, D, *_ in meta)
        if 'adjoint' in c and full:  # (the adjoint of a rank-deficient block is not defined)
            adj = c['adjoint']
            g = oracle.qr_backward(Qr, Rr, adj['gQ'], adj['gR'], data, meta)
            assert _rel(g, adj['grad']) < 1e-10
            n_adj += 1
    assert n_adj == 4


def test_ctmrg_checkpointed_replay_on_host_reproduces_reference():
    """The chi=24 CTMRG sequence replayed on the host with the plain per-block torch backend
    and each CTM move checkpointed: the reference's energy bit for bit and its gradient (the
    recomputed moves feed the backward)."""
    import torch
    from yastn_gb300.plain import PlainBackend
    from yastn_gb300.replay import load_replay
    r = load_replay('ctmrg_z2_d6')
    A = torch.from_numpy(r.arrays['in:A'].copy()).requires_grad_(True)
    env = r.run(PlainBackend(), 'cpu', {'A': A}, checkpoint=True)
    E = env[r.outputs['E']]
    assert float(E.detach()) == r.payload['E']
    E.backward()
    g, ref = A.grad.numpy(), r.arrays['ref:grad']
    assert np.abs(g - ref).max() <= 1e-10 * np.abs(ref).max()


def test_ctmrg_use_qr_replay_on_host_reproduces_reference():
    """YASTN's default projector path (use_qr=True: a QR of each half-system, then the SVD of
    the product of the R factors) replayed on the host with the plain per-block backend and
    checkpointed moves: the reference's energy and gradient."""
    import torch
    from yastn_gb300.plain import PlainBackend
    from yastn_gb300.replay import load_replay
    r = load_replay('ctmrg_z2_d6_qr')
    assert r.backend_calls()['qr'] > 0
    A = torch.from_numpy(r.arrays['in:A'].copy()).requires_grad_(True)
    env = r.run(PlainBackend(), 'cpu', {'A': A}, checkpoint=True)
    E = env[r.outputs['E']]
    assert abs(float(E.detach()) - r.payload['E']) <= 1e-12 * abs(r.payload['E'])
    E.backward()
    g, ref = A.grad.numpy(), r.arrays['ref:grad']
    # the half-systems are rank-deficient: the QR adjoint's R^-T amplifies the rounding
    # differences between two evaluations of the same sequence (1.6e-6 measured here; the
    # reference's own gradient tests hold CTM gradients to 1e-3, tests/peps/test_ad.py:286)
    assert np.abs(g - ref).max() <= 1e-5 * np.abs(ref).max()


def test_ctmrg_checkpoint_segments():
    """The checkpoint segments of the CTMRG recording: 16 CTM moves, each with its inputs
    produced before it and its outputs read after it (or results)."""
    import torch
    from yastn_gb300.replay import load_replay
    r = load_replay('ctmrg_z2_d6')
    segs = r._segments(torch.device('cpu'))
    ck = [s for s in segs if s[0] == 'ckpt']
    assert len(ck) == 16
    assert all(len(ins) > 0 and len(outs) > 0 for _, _, _, ins, outs, _ in ck)
    # the segments and plain runs tile the op list in order
    pos = 0
    for kind, a, b, *_ in segs:
        assert 0 <= a - pos <= 2 and b >= a  # markers between runs are skipped
        pos = b


@pytest.mark.parametrize('name', ['ctmrg_z2_d6', 'ctmrg_z2_d6_chi144', 'ctmrg_z2_d6_qr'])
def test_ctmrg_recording_dataflow_is_closed(name):
    """The recorded CTMRG sequences (chi = 24 and 144) only use tensors they produced, their
    input or their stored constants, and their output (the energy) is produced by them."""
    from yastn_gb300.replay import load_replay, check_dataflow
    r = load_replay(name)
    n, used = check_dataflow(r)
    produced = set()
    for op in r.ops:
        o = op.get('o')
        produced.update(o if isinstance(o, list) else [o])
    assert r.outputs['E'] in produced and 'in:A' in used
    calls = r.backend_calls()
    assert calls['svd'] == 32 and calls['dot'] == 697
    assert calls['transpose_and_merge'] == (1109 if name.endswith('_qr') else 1045)
    assert calls.get('qr', 0) == (64 if name.endswith('_qr') else 0)
