#!/usr/bin/env python
"""Benchmark of the yastn_gb300 hot path on one or more GB300 GPUs (replicas).

Workloads. ``--workload cfg2`` (default): YASTN's DMRG two-site effective-Hamiltonian
matvec (Env.Heff2: four tensordots under the fuse_contracted policy, 10 backend calls and
772 charge-sector GEMMs per matvec, virtual D=1024) inside ``eigs`` with 30 Lanczos
steps; the 30 steps are captured once as a CUDA graph and replayed; the lowest Ritz value
is checked against the reference's own eigs result (fixture) every run.
``--workload cfg1``: YASTN ``tensordot`` of two U(1) rank-4 FP64
tensors, every leg D=64 over charges -3..3 (sector dims 2,7,14,18,14,7,2), contracting
A's legs (2,3) with B's legs (0,1) under the fuse-to-matrix policy: merge A, merge B,
one grouped GEMM over the 13 charge sectors (3.248 GFLOP), unmerge C. It is driven
through the backend module with the metadata YASTN itself produced (recorded fixture)
and data regenerated from YASTN's seeded normal draws. The headline runs the backend's
'emulated' GEMM mode (FP64 products from BF16 split operands; its error against the
native FP64 result is measured every run and must stay below 1e-10); the native FP64
path and the workload's truncated block SVD (svd_with_truncation, D_total=64) are
reported as extra fields.

``--workload cfg5``: the precision study, the same tensordot on U(1) tensors with D=128
per leg over charges -16..16 and every block scaled by 10^U(-4,0) (sector GEMMs up to
946^3), reporting emulated and native FP64 TFLOP/s and the largest relative error per
sector result of both against the FP64 oracle.

``--workload dlayer``: one double-layer PEPS contraction (append_vec_tl, the CTMRG corner
step: the boundary vector x [l l'] [t t'] y with the ket and bra site tensors; Z2, D=6, d=2,
chi=144) as a compiled program (``yastn_gb300.double_layer``: composed copies + grouped GEMMs)
against YASTN's own composition on this backend and on the reference's torch backend on the
same GPU; the composed-copy kernel's bandwidth against the measured HBM peak.

``--workload cfg4``: differentiable iPEPS CTMRG (1x1 cell, Z2, D=6, d=2, 8 CTM iterations with
truncated block-SVD projectors, transverse-field Ising energy at h=3 and its gradient) at
environment dimension chi=24: the reference's own call sequence, recorded from YASTN, replayed
through the backend, forward and backward, every step. Reported in ms per forward+backward
(lower is better), with the energy and gradient checked against the reference's every run,
next to the plain FP64 path (one torch launch per block, torch's SVD; ``yastn_gb300.plain``)
on the same GPU and on the host cores.

One JSON line is printed by rank 0. ``--impl reference`` times the CPU restatement of
the reference NumPy backend on the host cores for the same workload instead.
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "tensordot TFLOP/s (block-sparse FP64, U(1) rank-4 D=64, <=1e-10 rel)"
METRIC2 = "tensordot TFLOP/s (DMRG Heff2 x 30 Lanczos, FP64, <=1e-10 rel)"
UNIT = "TFLOP/s"
L2_FLUSH_BYTES = 256 << 20


def parse():
    p = argparse.ArgumentParser()
    p.add_argument('--gpus', type=int, default=1)
    p.add_argument('--steps', type=int, default=20)
    p.add_argument('--warmup', type=int, default=5)
    p.add_argument('--impl', default='gb300', choices=['gb300', 'reference'])
    p.add_argument('--workload', default='cfg2', choices=['cfg1', 'cfg2', 'cfg3', 'cfg4', 'cfg5', 'svd144', 'dlayer'])
    p.add_argument('--gemm', default='emulated', choices=['emulated', 'fp64'],
                   help='sector-GEMM mode of the headline (cfg2)')
    p.add_argument('--no-svd', action='store_true', help='skip the extra svd_with_truncation timing')
    p.add_argument('--chi', type=int, default=24, choices=[24, 144],
                   help='cfg4: environment dimension of the recorded CTMRG run (144 = the configuration as written)')
    p.add_argument('--use-qr', action='store_true',
                   help="cfg4 (chi=24): YASTN's default projector path use_qr=True (QR of each half-system)")
    p.add_argument('--no-plain', action='store_true', help='cfg4: skip the plain per-block GPU path and the host run')
    p.add_argument('--no-checkpoint', action='store_true',
                   help='cfg4: keep every CTM move for the backward instead of recomputing it (checkpoint_move)')
    p.add_argument('--no-extras', action='store_true',
                   help='cfg2: skip the plain per-block comparisons and the CTMRG fields of the headline line')
    p.add_argument('--headline-only', action='store_true',
                   help='cfg2: run only the headline GEMM mode (for kernel launch lists); the emulated kernel of '
                        'each dot is chosen by its padded tile work rather than by timing, so that a profiler '
                        'slowing the kernels unequally does not change the choice')
    p.add_argument('--ozaki-kernel', default='auto', choices=['auto', 'tcgen05', 'tcgen05-32', 'mma'],
                   help='emulated sector GEMM kernel: chosen per dot (auto), or forced (for kernel profiles)')
    return p.parse_args()


# ----------------------------------------------------------------------------- workload (host side)

class Cfg1:
    name = "U(1) rank-4 D=64 tensordot A(2,3)xB(0,1), fuse_to_matrix, 13 sectors, FP64"
    metric = METRIC
    has_svd = True
    complex_gemm = False
    trunc = {'D_total': 64}
    ozaki_traffic = None

    def __init__(self):
        from yastn_gb300.workloads import load_trace, cfg1_inputs
        from yastn_gb300 import _plans as P
        self.tr = load_trace('cfg1')
        self.A, self.B = cfg1_inputs(self.tr)
        c = self.tr['calls']
        self.mA = c[0]['args'][1:]
        self.mB = c[1]['args'][1:]
        self.mdot = c[2]['args'][2:]
        self.mun = c[3]['args'][1]
        self.mC = c[4]['args'][1:]
        self.msvd = c[5]['args'][1:3]
        self.mU = c[6]['args'][1]
        self.mV = c[7]['args'][1]
        self.mask_calls = [x['args'] for x in c[8:11]]
        self.flops = P.dot_plan(self.mdot[0]).flops
        self.bytes_merge = 16 * self.A.size  # read + write FP64 per merged element

    # the reference NumPy path, restated by the oracle (CPU)
    def cpu_step(self):
        import oracle
        Am = oracle.transpose_and_merge(self.A, *self.mA)
        Bm = oracle.transpose_and_merge(self.B, *self.mB)
        Cm = oracle.dot(Am, Bm, *self.mdot)
        return oracle.unmerge(Cm, self.mun)


class Cfg3(Cfg1):
    name = ("U(1)xU(1) (N,Sz) complex128 rank-4, 11 charges per leg with geometric(0.15) dims on 1..64 "
            "(leg total 116, 595 blocks per tensor), tensordot A(2,3)xB(0,1), fuse_contracted, 595 complex "
            "sector GEMMs")
    metric = "tensordot TFLOP/s (block-sparse complex128, U(1)xU(1) 595 blocks, <=1e-10 rel)"
    has_svd = True
    ozaki_traffic = None
    complex_gemm = True

    def __init__(self):
        from yastn_gb300.workloads import load_trace, cfg3_inputs
        from yastn_gb300 import _plans as P
        self.tr = load_trace('cfg3')
        self.A, self.B = cfg3_inputs(self.tr)
        c = self.tr['calls']
        self.mA = c[0]['args'][1:]
        self.mB = c[1]['args'][1:]
        self.mdot = c[2]['args'][2:]
        self.mun = None
        self.mC = c[3]['args'][1:]
        self.msvd = c[4]['args'][1:3]
        self.mU = c[5]['args'][1]
        self.mV = c[6]['args'][1]
        self.mask_calls = [x['args'] for x in c[7:10]]
        self.trunc = {'tol': 1e-8}
        # complex multiply-add = 8 real flops
        self.flops = 4 * P.dot_plan(self.mdot[0]).flops
        self.bytes_merge = 32 * self.A.size

    def cpu_step(self):
        import oracle
        Am = oracle.transpose_and_merge(self.A, *self.mA)
        Bm = oracle.transpose_and_merge(self.B, *self.mB)
        return oracle.dot(Am, Bm, *self.mdot)


class Cfg5(Cfg1):
    name = ("precision study: U(1) rank-4 D=128 per leg over t=-16..16, blocks scaled by 10^U(-4,0), "
            "tensordot A(2,3)xB(0,1), fuse_to_matrix, sector GEMMs up to 946^3, FP64")
    metric = "tensordot TFLOP/s (precision study U(1) D=128/leg, per-block scales 1e-4..1, FP64, <=1e-10 rel)"
    has_svd = False
    ozaki_traffic = None

    def __init__(self):
        from yastn_gb300.workloads import load_trace, cfg5_inputs
        from yastn_gb300 import _plans as P
        self.tr = load_trace('cfg5')
        self.A, self.B = cfg5_inputs(self.tr)
        c = self.tr['calls']
        self.mA = c[0]['args'][1:]
        self.mB = c[1]['args'][1:]
        self.mdot = c[2]['args'][2:]
        self.mun = c[3]['args'][1]
        self.flops = P.dot_plan(self.mdot[0]).flops
        self.bytes_merge = 16 * self.A.size


class Cfg4:
    """Differentiable CTMRG (forward + backward) from the recorded call sequence."""

    def __init__(self, chi=24, use_qr=False):
        from yastn_gb300.replay import load_replay
        if use_qr and chi != 24:
            raise ValueError("the use_qr=True run is recorded at chi=24")
        blocks = {24: "28 block SVDs of 2x432^2", 144: "24 block SVDs of 2x2592^2"}[chi]
        qr = ", use_qr=True: 64 block QRs of the half-systems" if use_qr else ""
        self.name = (f"differentiable iPEPS CTMRG, 1x1 cell, Z2, D=6, d=2, chi={chi}, 8 CTM iterations, TFIM h=3 "
                     f"energy + gradient (recorded YASTN call sequence replayed: {blocks} among 32 SVD calls, "
                     f"697 dots per forward{qr}), FP64")
        self.metric = f"CTMRG fwd+bwd ms (iPEPS Z2 D=6 chi={chi}, 8 CTM iterations, FP64, <=1e-10 rel)"
        name = 'ctmrg_z2_d6' + ('_qr' if use_qr else '') + ('' if chi == 24 else f'_chi{chi}')
        self.r = load_replay(name)
        # with use_qr the QR adjoint of rank-deficient half-systems amplifies rounding (two host
        # evaluations of the same sequence differ by 1.6e-6), so its gradient is held to 1e-5
        self.grad_tol = 1e-5 if use_qr else 1e-8
        self.cpu_recorded = self.r.payload.get('cpu_seconds')
        self.A = self.r.arrays['in:A']
        self.E_ref = self.r.payload['E']
        self.grad_ref = self.r.arrays['ref:grad']

    def flops(self):
        """Algorithmic work of one step counted at the backend boundary from the recorded
        metadata: forward sector-GEMM FLOP, nominal SVD FLOP (14 L k^2 + 8 k^3 per block),
        and backward GEMM FLOP (two adjoint products per dot, the SVD adjoint's products)."""
        import torch
        from yastn_gb300 import _plans as P
        from yastn_gb300.replay import _decode_const
        fg = fs = bg = 0
        for op in self.r.ops:
            if op['k'] != 'b' or op['fn'] not in ('dot', 'svd'):
                continue
            meta = _decode_const(op['a'][2] if op['fn'] == 'dot' else op['a'][1], torch.device('cpu'))
            if op['fn'] == 'dot':
                fg += P.dot_plan(meta).flops
                pa, pb = P.dot_backward_plans(meta)
                bg += pa.flops + pb.flops
            else:
                fs += P.svd_plan(meta).nominal_flops
                ap = P.svd_adjoint_plan(meta)
                bg += sum(g.flops for g in (ap.gP, ap.gQ, ap.gT, ap.gR, ap.gA1, ap.gA2))
        return fg, fs, bg

    checkpoint = True

    def step(self, torch, backend, device, A_host=None, pinned=None):
        """One forward + backward (each CTM move under non-reentrant checkpointing, as the
        recorded run's checkpoint_move, unless ``checkpoint`` is off); returns (E, grad)."""
        if pinned is not None:
            A = pinned.to(device, non_blocking=True)
        else:
            A = torch.from_numpy(self.A).to(device)
        A.requires_grad_(True)
        env = self.r.run(backend, device, {'A': A}, checkpoint=self.checkpoint)
        E = env[self.r.outputs['E']]
        E.backward()
        return E.detach(), A.grad


class Cfg2:
    """DMRG two-site Heff2 matvec inside 30 Lanczos steps (YASTN eigs, ncv=30, 'SR')."""
    name = ("DMRG two-site Heff2 x 30 Lanczos steps: U(1) spin-1/2 XXZ (Jz=Jxy=1, MPO bond 5), virtual D=1024 "
            "over t=-12..12, fuse_contracted (4 dots, 772 sector GEMMs per matvec), FP64")
    ncv = 30

    def __init__(self):
        from yastn_gb300.workloads import Heff2Workload
        self.wl = Heff2Workload()
        self.flops = self.ncv * self.wl.flops

    def cpu_step(self, ncv=None):
        import oracle
        from yastn_gb300.workloads import lanczos, ritz_lowest
        env = self.wl.env(lambda x: x)
        mv = lambda v: self.wl.matvec(v, env, oracle.dot, oracle.transpose_and_merge, lambda x, f: x * f)
        V, al, be = lanczos(mv, self.wl.data['AA'], ncv or self.ncv, np.dot, np.linalg.norm)
        return ritz_lowest(al, be)

    _yastn_setup = None

    def yastn_step(self):
        """The workload through the unmodified reference itself (its NumPy backend): YASTN's
        Heff2 contractions inside yastn.eigs(ncv=30, 'SR') on the same seeded tensors; None
        when the reference package is not installed under baseline/_ref."""
        if self._yastn_setup is None:
            self._yastn_setup = yastn_heff2_setup()
        if not self._yastn_setup:
            return None
        yastn, heff2, AA = self._yastn_setup
        val, _ = yastn.eigs(heff2, AA, k=1, ncv=self.ncv, which='SR', hermitian=True)
        return float(np.real(val[0]))


def yastn_heff2_setup():
    """(yastn, heff2, AA) of the DMRG workload built by the reference package from
    baseline/_ref with its NumPy backend (XXZ MPO of 4 sites, D=1024 virtual legs over
    t=-12..12, L, R, AA drawn after random_seed(0) in that order), or () if it is absent."""
    ref = os.path.join(ROOT, 'baseline', '_ref')
    if not os.path.isdir(ref):
        return ()
    if ref not in sys.path:
        sys.path.append(ref)
    try:
        import yastn
        import yastn.tn.mps as mps
    except ImportError:
        return ()
    ops_ = yastn.operators.Spin12(sym='U1', backend='np')
    gen = mps.Generator(N=4, operators=ops_)
    gen.random_seed(seed=0)
    H = gen.mpo_from_latex(r"\sum_{i,j \in NN} (Jz sz_{i} sz_{j} + 0.5 Jxy (sp_{i} sm_{j} + sm_{i} sp_{j}))",
                           {"Jz": 1.0, "Jxy": 1.0, "NN": [(i, i + 1) for i in range(3)]})
    psi = gen.random_mps(D_total=8)
    env = mps.Env(psi, [H, psi]).setup_(to='first').setup_(to='last')
    L0, R0 = env.F[(0, 1)], env.F[(3, 2)]
    cfg = psi.config
    cfg.backend.random_seed(0)
    ts0 = tuple(range(-12, 13))
    p = np.exp(-np.array(ts0, dtype=float) ** 2 / 18)
    p = p / p.sum()
    D = np.round(p * 1024).astype(int)
    while D.sum() > 1024:
        D[np.argmax(D - p * 1024)] -= 1
    while D.sum() < 1024:
        D[np.argmin(D - p * 1024)] += 1
    ts, Ds = zip(*[(t, int(d)) for t, d in zip(ts0, D) if d > 0])
    lL, lR = L0.get_legs(), R0.get_legs()
    vl = lambda sg: yastn.Leg(cfg, s=sg, t=ts, D=Ds)
    L = yastn.rand(cfg, legs=[vl(lL[0].s), lL[1], vl(lL[2].s)], distribution='normal')
    R = yastn.rand(cfg, legs=[vl(lR[0].s), lR[1], vl(lR[2].s)], distribution='normal')
    la = psi.pre_2site((1, 2)).get_legs()
    AA = yastn.rand(cfg, legs=[vl(la[0].s), la[1], la[2], vl(la[3].s)], distribution='normal')
    W1, W2, factor = H[1], H[2], H.factor

    def heff2(v):
        tmp = v @ R
        tmp = yastn.tensordot(W2, tmp, axes=((2, 3), (3, 2)))
        tmp = yastn.tensordot(W1, tmp, axes=((2, 3), (0, 3)))
        tmp = yastn.tensordot(L, tmp, axes=((0, 1), (3, 0)))
        return tmp * factor
    return yastn, heff2, AA


def time_cpu(fn, budget_s, min_reps=3):
    fn()
    ts = []
    t_end = time.perf_counter() + budget_s
    while len(ts) < min_reps or time.perf_counter() < t_end:
        t0 = time.perf_counter()
        fn()
        ts.append(time.perf_counter() - t0)
    return float(np.median(ts)), len(ts)


def cpu_cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:  # pragma: no cover
        return os.cpu_count()


def run_reference(args, wl):
    """--impl reference: the reference's NumPy path (oracle restatement) on host cores."""
    rank = int(os.environ.get('RANK', '0'))
    if rank != 0:
        return
    if isinstance(wl, Cfg2):
        return run_reference_cfg2(args, wl)
    if isinstance(wl, Cfg4):
        return run_reference_cfg4(args, wl)
    for _ in range(args.warmup):
        wl.cpu_step()
    ts = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        wl.cpu_step()
        ts.append(time.perf_counter() - t0)
    t = float(np.mean(ts))
    value = wl.flops / t / 1e12
    line = {"impl": "reference", "metric": wl.metric, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c128" if wl.complex_gemm else "f64",
            "data": "synthetic (seeded yastn normal draws)",
            "config": {"workload": wl.name},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cpu_cores(), "kind": "port",
                             "sample": f"{args.steps} tensordot steps (numpy BLAS, all host threads)"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_reference_cfg2(args, wl):
    """Reference arm for the Lanczos workload: every step is the whole workload, the 30
    Lanczos steps of the Heff2 matvec, run by the unmodified reference package itself
    (YASTN's tensordot and eigs on its NumPy backend, from baseline/_ref) on the host cores
    with all BLAS threads; where the package is absent, the oracle's restatement of the
    same calls."""
    use_yastn = wl.yastn_step() is not None
    step = wl.yastn_step if use_yastn else wl.cpu_step
    lam = None
    for _ in range(args.warmup):
        lam = step()
    ts = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        lam = step()
        ts.append(time.perf_counter() - t0)
    t = float(np.mean(ts))
    value = wl.flops / t / 1e12
    lam = lam if use_yastn else lam[0]
    ref_lam = wl.wl.tr['lanczos_lowest']
    kind = "reference" if use_yastn else "port"
    sample = (f"{args.steps} runs of all {wl.ncv} Lanczos steps: YASTN tensordot + eigs, NumPy backend"
              if use_yastn else f"{args.steps} runs of all {wl.ncv} Lanczos steps (oracle restatement, numpy BLAS)")
    line = {"impl": "reference", "metric": METRIC2, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded yastn normal draws)",
            "config": {"workload": wl.name, "lowest_ritz_rel_err_vs_recorded": abs(lam - ref_lam) / abs(ref_lam)},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cpu_cores(), "kind": kind, "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_reference_cfg4(args, wl):
    """Reference arm for CTMRG: the recorded sequence on the host cores with one torch
    operation per block (the reference torch backend's structure, LAPACK SVD, all threads).
    One forward+backward takes ~10 s, so at most 3 timed steps and 1 warm-up are run."""
    import torch
    from yastn_gb300.plain import PlainBackend
    steps, warm = min(args.steps, 3), min(args.warmup, 1)
    for _ in range(warm):
        wl.step(torch, PlainBackend(), 'cpu')
    ts = []
    for _ in range(steps):
        t0 = time.perf_counter()
        E, g = wl.step(torch, PlainBackend(), 'cpu')
        ts.append(time.perf_counter() - t0)
    t = float(np.mean(ts)) * 1e3
    err = abs(float(E) - wl.E_ref) / abs(wl.E_ref)
    line = {"impl": "reference", "metric": wl.metric, "value": t, "unit": "ms", "n_gpus": args.gpus,
            "steps": steps, "warmup": warm, "ms_per_step": t, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded N(0,1) site tensor, recorded call sequence)",
            "config": {"workload": wl.name, "energy_rel_err_vs_reference": err},
            "cpu_baseline": {"value": t, "unit": "ms", "cores": torch.get_num_threads(), "kind": "port",
                             "sample": f"{steps} full forward+backward steps, one torch CPU op per block (LAPACK SVD)"},
            "e2e": {"value": t, "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


# ----------------------------------------------------------------------------- GPU side

class Clocks:
    """nvidia-smi clock/throttle samples taken while the timed region runs."""

    def __init__(self, index):
        self.f = tempfile.NamedTemporaryFile(mode='w+', suffix='.csv', delete=False)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.p = subprocess.Popen(['nvidia-smi', f'--id={index}', f'--query-gpu={q}', '--format=csv,noheader,nounits',
                                       '-lms', '200'], stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:  # pragma: no cover
            self.p.kill()
        self.f.flush()
        self.f.seek(0)
        rows = [r.split(',') for r in self.f.read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, smax, reasons = [], [], set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        for r in rows:
            try:
                sm.append(float(r[1]))
                smax.append(float(r[2]))
            except (ValueError, IndexError):
                continue
            for nm, v in zip(names, r[5:9]):
                if v.strip().lower() == 'active':
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def fp64_peak_tflops(torch, dev):
    """cuBLAS DGEMM throughput on this GPU (4096^3, best of 5) as the FP64 roofline."""
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device=dev)
    b = torch.randn(n, n, dtype=torch.float64, device=dev)
    for _ in range(2):
        a @ b
    best = 0.0
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        a @ b
        e1.record()
        e1.synchronize()
        best = max(best, 2 * n ** 3 / (e0.elapsed_time(e1) * 1e-3) / 1e12)
    return best


def _tflops_of(ev, flops):
    t = sum(a.elapsed_time(b) for a, b in ev) / len(ev) * 1e-3
    return t, flops / t / 1e12


def run_gpu(args, wl):
    import torch
    import torch.distributed as dist
    from yastn_gb300 import backend as BK
    from yastn_gb300 import ops, _native, _plans

    world = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    torch.cuda.set_device(local)
    dev = torch.device('cuda', local)
    if world > 1:
        dist.init_process_group('nccl')
    _native.lib()

    dA = torch.from_numpy(wl.A).to(dev)
    dB = torch.from_numpy(wl.B).to(dev)
    hA = torch.from_numpy(wl.A).pin_memory()
    hB = torch.from_numpy(wl.B).pin_memory()

    flush = torch.empty(L2_FLUSH_BYTES // 8, dtype=torch.float64, device=dev)
    kern_ev = []

    def tensordot(a, b, record=False):
        """yastn tensordot's backend calls: merge A, merge B, dot (sector GEMMs), unmerge C."""
        Am = BK.transpose_and_merge(a, *wl.mA)
        Bm = BK.transpose_and_merge(b, *wl.mB)
        if record:
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
        Cm = BK.dot(Am, Bm, *wl.mdot)
        if record:
            e1.record()
            kern_ev.append((e0, e1))
        return Cm if wl.mun is None else BK.unmerge(Cm, wl.mun)

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    def timed(fn, steps):
        ev = []
        for _ in range(steps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            ev.append((e0, e1))
        barrier()
        return ev

    chk = wl.tr['C_checksum']
    # native FP64 path: parity guard against the reference checksum, then timing
    BK.set_gemm_mode('fp64')
    Cn = tensordot(dA, dB)
    assert abs(float(Cn.real.sum()) - chk['sum0']) <= 1e-9 * chk['abs0'], "tensordot result differs from the reference"
    hC = torch.empty(Cn.numel(), dtype=Cn.dtype).pin_memory()
    sector_err = per_sector_errors(torch, BK, wl, dA, dB)
    plain_ms = plain_per_block_ms(torch, BK, wl, dA, dB, flush)
    for _ in range(args.warmup):
        tensordot(dA, dB)
    barrier()
    kern_ev.clear()
    native_ev = timed(lambda: tensordot(dA, dB, record=True), args.steps)
    t_native, native_tflops = _tflops_of(native_ev, wl.flops)
    t_native_gemm, native_gemm_tflops = _tflops_of(kern_ev, wl.flops)

    # headline: the same tensordot with the FP64 sector GEMMs emulated on BF16 tensor cores
    BK.set_gemm_mode('emulated')
    Co = tensordot(dA, dB)
    emu_err = float((Co - Cn).abs().max() / Cn.abs().max())
    assert emu_err <= 1e-10, f"emulated tensordot error {emu_err} above 1e-10"
    for _ in range(args.warmup):
        tensordot(dA, dB)
    barrier()
    clocks = Clocks(local)
    kern_ev.clear()
    launches0 = _native.LAUNCHES[0]
    barrier()
    ev = timed(lambda: tensordot(dA, dB, record=True), args.steps)
    launches = _native.LAUNCHES[0] - launches0
    t_step, _ = _tflops_of(ev, wl.flops)
    t_dot, _ = _tflops_of(kern_ev, wl.flops)

    # end to end through the backend with host buffers (pinned H2D of A, B; D2H of C)
    for _ in range(2):
        tensordot(hA.to(dev, non_blocking=True), hB.to(dev, non_blocking=True))
    barrier()

    def e2e_step():
        c = tensordot(hA.to(dev, non_blocking=True), hB.to(dev, non_blocking=True))
        hC.copy_(c, non_blocking=True)
    e2e_ev = timed(e2e_step, args.steps)
    clk = clocks.stop()
    t_e2e, _ = _tflops_of(e2e_ev, wl.flops)

    # the dominant kernel alone (split-operand GEMM; the native grouped GEMM for complex
    # data), for the roofline
    from yastn_gb300._plans import ozaki_dot_plan
    top_kernel = 'yb_ozaki_gemm'  # either emulated GEMM kernel (tcgen05 or mma.sync)
    Am = BK.transpose_and_merge(dA, *wl.mA)
    Bm = BK.transpose_and_merge(dB, *wl.mB)
    orig = _native.call
    gemm_ev = []

    def spy(name, *a, **k):
        if name.startswith(top_kernel):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            r = orig(name, *a, **k)
            e1.record()
            gemm_ev.append((e0, e1))
            return r
        return orig(name, *a, **k)
    _native.call = spy
    try:
        for _ in range(args.steps):
            flush.zero_()
            ops.dot_ozaki(Am, Bm, *wl.mdot)
        barrier()
    finally:
        _native.call = orig
    t_gemm = sum(a.elapsed_time(b) for a, b in gemm_ev) / len(gemm_ev) * 1e-3
    oz = ozaki_dot_plan(wl.mdot[0], ops.OZAKI_SLICES, wl.complex_gemm)
    tensor_flops = oz.flops * ops.OZAKI_SLICES * (ops.OZAKI_SLICES + 1) // 2
    use_tc = getattr(oz, 'tuned_tc', oz.prefer_tc) if ops.OZAKI_TC[0] is None else ops.OZAKI_TC[0]
    top_name = (f'tcgen05 (TMEM accumulators, 128x{32 if use_tc == 32 else 64} tiles)' if use_tc else 'mma.sync')

    BK.set_gemm_mode('fp64')

    # the workload's truncated block SVD (extra field)
    svd_ms = None
    if wl.has_svd and not args.no_svd:
        C = tensordot(dA, dB)

        def svd_trunc():
            M = BK.transpose_and_merge(C, *wl.mC)
            U, S, V = BK.svd(M, *wl.msvd)
            Uu = BK.unmerge(U, wl.mU)
            Vu = BK.unmerge(V, wl.mV)
            slices = sorted(tuple(m[4]) for m in wl.msvd[0])
            mask, kept = ops.truncation_mask_data(S, slices, None, **wl.trunc)
            out = []
            for (Ain, mask_r, meta, Dsize, axis, ndim), data in zip(wl.mask_calls, (Uu, S, Vu)):
                dmask = {k: torch.as_tensor(np.asarray(v, dtype=np.int64), device=dev) for k, v in mask_r.items()}
                out.append(BK.apply_mask(data, dmask, meta, Dsize, axis, ndim))
            return out, kept
        svd_trunc()
        torch.cuda.synchronize()
        ts = []
        for _ in range(3):
            t0 = time.perf_counter()
            _, kept = svd_trunc()
            torch.cuda.synchronize()
            ts.append(time.perf_counter() - t0)
        assert sorted(k for k in kept if k) == sorted(d[0] for d in wl.tr['S_kept_D'])
        svd_ms = float(np.median(ts)) * 1e3

    # max over ranks
    t_max = t_step
    if world > 1:
        tt = torch.tensor([t_step, t_e2e], dtype=torch.float64, device=dev)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_max, t_e2e = float(tt[0]), float(tt[1])
    if rank != 0:
        if world > 1:
            dist.destroy_process_group()
        return
    fp64_peak = fp64_peak_tflops(torch, dev)
    bf16_peak, peak_src = bf16_peak_tflops()
    cpu_t, reps = time_cpu(wl.cpu_step, budget_s=8.0)
    achieved = tensor_flops / t_gemm / 1e12
    cplx_note = ', 2 real products per complex sector' if wl.complex_gemm else ''
    roof = {"bound": "tensor",
            "kernel": f"yb ozaki GEMM on {top_name}, bf16 digit products (36 slice pairs{cplx_note})",
            "achieved": achieved, "peak": bf16_peak, "unit": "TFLOP/s", "frac": achieved / bf16_peak,
            "peak_source": peak_src, "traffic": wl.ozaki_traffic,
            "traffic_note": "dram bytes read+written by one launch, ncu capture on this workload"}
    line = {
        "metric": wl.metric, "value": world * wl.flops / t_max / 1e12, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_max * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": ("c128 (sector GEMMs emulated: 2 real products of 8 bf16 digit slices)" if wl.complex_gemm else
                  "f64 (sector GEMMs emulated: 8 bf16 digit slices, fp32/fp64 accumulation)"),
        "data": "synthetic (seeded normal draws as yastn.rand, metadata recorded from yastn)",
        "config": {"workload": wl.name, "flop_per_step": wl.flops, "parallelism": f"replicas{world}",
                   "gemm_mode": "emulated",
                   "l2": "flushed between timed steps (256 MB write)",
                   "max_rel_err_vs_fp64": emu_err,
                   "max_rel_err_per_sector_vs_oracle": sector_err},
        "roofline": roof,
        "cpu_baseline": {"value": wl.flops / cpu_t / 1e12, "unit": UNIT, "cores": cpu_cores(), "kind": "port",
                         "sample": f"{reps} tensordot steps of the same workload (numpy BLAS, median)"},
        "e2e": {"value": world * wl.flops / t_e2e / 1e12, "unit": UNIT,
                "h2d_bytes_per_step": int(wl.A.nbytes + wl.B.nbytes),
                "d2h_bytes_per_step": int(hC.numel() * hC.element_size())},
        "gpu_launches": launches,
        "clocks": clk,
        "extra": {"dot_ms": t_dot * 1e3, "top_kernel_ms": t_gemm * 1e3,
                  "plain_per_block_dot_ms": plain_ms,
                  "plain_per_block_dot": "the same sector GEMMs as one torch.matmul (cuBLAS) launch per block "
                                         "from a host loop, FP64 (the reference torch backend's kernel_dot pattern)",
                  "grouped_vs_plain_per_block_dot": plain_ms / (t_native_gemm * 1e3),
                  "native_fp64_tflops": native_tflops, "native_fp64_ms_per_step": t_native * 1e3,
                  "native_fp64_gemm_tflops": native_gemm_tflops,
                  "native_fp64_gemm_frac_of_cublas_dgemm": native_gemm_tflops / fp64_peak,
                  "fp64_peak_cublas_dgemm_tflops": fp64_peak,
                  "svd_with_truncation_ms": svd_ms,
                  "svd_with_truncation": f"merge C, {len(wl.msvd[0]) if wl.has_svd else 0}-block mixed-precision "
                                         f"Jacobi SVD, unmerge U/V, device truncation {wl.trunc}, 3 masks"},
    }
    print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()


def plain_per_block_ms(torch, BK, wl, dA, dB, flush, reps=5):
    """The sector GEMMs of the same dot as one cuBLAS launch per block from a host loop (the
    pattern of the reference torch backend's kernel_dot): device time per dot, FP64."""
    Am = BK.transpose_and_merge(dA, *wl.mA)
    Bm = BK.transpose_and_merge(dB, *wl.mB)
    meta, Dsize = wl.mdot
    C = torch.zeros(Dsize, dtype=Am.dtype, device=Am.device)
    views = [(C[slc[0]:slc[1]].view(Dc), Am[sla[0]:sla[1]].view(Da), Bm[slb[0]:slb[1]].view(Db))
             for slc, Dc, sla, Da, slb, Db in meta]

    def once():
        for c, a, b in views:
            torch.matmul(a, b, out=c)
    once()
    torch.cuda.synchronize()
    ts = []
    for _ in range(reps):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        once()
        e1.record()
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1))
    return float(np.median(ts))


def per_sector_errors(torch, BK, wl, dA, dB):
    """Max relative error per sector result (max |C_s - C_s^ref| / max |C_s^ref| over the
    sector) of the native and the emulated GEMM modes against the FP64 oracle (NumPy)."""
    import oracle
    Am = oracle.transpose_and_merge(wl.A, *wl.mA)
    Bm = oracle.transpose_and_merge(wl.B, *wl.mB)
    ref = oracle.dot(Am, Bm, *wl.mdot)
    dAm = BK.transpose_and_merge(dA, *wl.mA)
    dBm = BK.transpose_and_merge(dB, *wl.mB)
    out = {}
    mode0 = BK.get_gemm_mode()
    for mode in ('fp64', 'emulated'):
        BK.set_gemm_mode(mode)
        got = BK.dot(dAm, dBm, *wl.mdot).cpu().numpy()
        worst = 0.0
        for slc, *_ in wl.mdot[0]:
            r, g = ref[slc[0]:slc[1]], got[slc[0]:slc[1]]
            mx = np.abs(r).max() if r.size else 0.0
            if mx > 0:
                worst = max(worst, float(np.abs(g - r).max() / mx))
        out[mode] = worst
    BK.set_gemm_mode(mode0)
    assert out['fp64'] <= 1e-12 and out.get('emulated', 0.0) <= 1e-10, out
    return out


def bf16_peak_tflops():
    """Dense BF16 tensor peak measured on the GB300s (cuBLAS, burst), else the fallback."""
    path = os.path.join(ROOT, 'MEASURED_PEAKS.json')
    try:
        with open(path) as f:
            return float(json.load(f)['bf16_tflops']), "measured (cuBLAS bf16 burst)"
    except (OSError, KeyError, ValueError):
        return 1900.0, "fallback (1.9 PFLOP/s bf16 burst)"


def run_gpu_cfg2(args, wl):
    """30 Lanczos steps of the Heff2 matvec, captured once as a CUDA graph and replayed."""
    import torch
    import torch.distributed as dist
    from yastn_gb300 import backend as BK
    from yastn_gb300 import _native
    from yastn_gb300 import krylov as K

    world = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    torch.cuda.set_device(local)
    dev = torch.device('cuda', local)
    if world > 1:
        dist.init_process_group('nccl')
    _native.lib()
    w = wl.wl
    env = w.env(lambda x: torch.from_numpy(x).to(dev))
    mv = lambda v: w.matvec(v, env, BK.dot, BK.transpose_and_merge, lambda x, f: x * f if f != 1.0 else x)
    h_v0 = torch.from_numpy(w.data['AA']).pin_memory()
    ref_lam = w.tr['lanczos_lowest']
    flush = torch.empty(L2_FLUSH_BYTES // 8, dtype=torch.float64, device=dev)

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    results = {}
    modes = ['fp64', 'emulated'] if args.gemm == 'emulated' else ['fp64']
    if args.headline_only:
        modes = [args.gemm]
        from yastn_gb300 import ops
        ops.OZAKI_AUTOTUNE[0] = False
    if args.ozaki_kernel != 'auto':
        from yastn_gb300 import ops
        ops.OZAKI_TC[0] = {'tcgen05': 64, 'tcgen05-32': 32, 'mma': False}[args.ozaki_kernel]
    for mode in modes:
        BK.set_gemm_mode(mode)
        v0 = h_v0.to(dev)
        # eager run: parity with the reference's eigs, and plan/device caches warmed
        st = K.lanczos(mv, v0, wl.ncv)
        _, val, _ = K.ritz(st, 'SR')
        lam = float(val[0])
        err = abs(lam - ref_lam) / abs(ref_lam)
        assert err <= 1e-10, f"{mode}: lowest Ritz value {lam} vs reference {ref_lam}"
        # the 30 Lanczos steps (matvecs and the fused Krylov vector kernels) captured once
        lg = K.LanczosGraph(mv, v0, wl.ncv)
        launches = lg.launches
        hy = torch.empty(v0.numel(), dtype=torch.float64).pin_memory()

        def step(e2e=False):
            if e2e:
                lg.v0.copy_(h_v0, non_blocking=True)
            st = lg.replay()
            m, val, vr = K.ritz(st, 'SR')  # reads the tridiagonal coefficients back (one sync)
            y = K.combine(st, vr[:, 0], m)  # the lowest Ritz vector
            if e2e:
                hy.copy_(y, non_blocking=True)
            return float(val[0])

        for _ in range(args.warmup):
            step()
        barrier()
        clocks = Clocks(local) if mode == args.gemm else None
        ts, lams = [], []
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            lams.append(step())
            torch.cuda.synchronize()
            ts.append(time.perf_counter() - t0)
        barrier()
        te = []
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            lams.append(step(e2e=True))
            torch.cuda.synchronize()
            te.append(time.perf_counter() - t0)
        clk = clocks.stop() if clocks else None
        # every timed replay's lowest Ritz value against the reference's eigs
        replay_err = max(abs(x - ref_lam) / abs(ref_lam) for x in lams)
        assert replay_err <= 1e-10, f"{mode}: a timed replay's lowest Ritz value is off by {replay_err}"
        results[mode] = dict(t=float(np.mean(ts)), te=float(np.mean(te)), err=err, replay_err=replay_err,
                             launches=launches, clocks=clk)
        del lg
    # per-entry-point device time of one eager matvec in the headline mode: the dominant kernel
    BK.set_gemm_mode(args.gemm)
    roof = kernel_roofline(torch, dev, lambda: mv(v0), w, args.gemm)
    BK.set_gemm_mode('fp64')
    emu_sector_err, emu_sectors = emulated_dot_errors(torch, BK, mv, v0)
    assert emu_sector_err <= 1e-10, f"emulated sector GEMM error {emu_sector_err} above 1e-10"
    extras = {}
    if not args.no_extras:
        extras = plain_and_ctmrg_extras(args, torch, dev, wl, w, env, h_v0, flush, results[args.gemm]['t'])
        if world == 1:
            extras["other_configs"] = other_config_lines()
    head = results[args.gemm]
    t_max, t_e2e = head['t'], head['te']
    if world > 1:
        tt = torch.tensor([t_max, t_e2e], dtype=torch.float64, device=dev)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_max, t_e2e = float(tt[0]), float(tt[1])
    if rank != 0:
        if world > 1:
            dist.destroy_process_group()
        return
    use_yastn = wl.yastn_step() is not None  # the reference package itself, when installed
    cpu_t, reps = time_cpu(wl.yastn_step if use_yastn else wl.cpu_step, budget_s=8.0, min_reps=2)
    cpu_value = wl.flops / cpu_t / 1e12
    line = {
        "metric": METRIC2, "value": world * wl.flops / t_max / 1e12, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_max * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if args.gemm == 'fp64' else "f64 (sector GEMMs emulated: 8 bf16 digit slices)",
        "data": "synthetic (seeded normal draws as yastn.rand, metadata recorded from yastn)",
        "config": {"workload": wl.name, "flop_per_step": wl.flops, "parallelism": f"replicas{world}",
                   "gemm_mode": args.gemm,
                   "cuda_graph": "30 Lanczos steps (Heff2 matvecs + fused Krylov vector kernels) captured once, "
                                 "replayed per step; tridiagonal solve and Ritz vector per step",
                   "l2": "flushed between timed steps (256 MB write)",
                   "lowest_ritz_rel_err_vs_reference": head['err'],
                   "lowest_ritz_rel_err_max_over_timed_replays": head['replay_err'],
                   "emulated_dot_max_sector_rel_err_vs_fp64": emu_sector_err,
                   "emulated_dot_sectors_checked": emu_sectors},
        "roofline": roof,
        "cpu_baseline": {"value": cpu_value, "unit": UNIT, "cores": cpu_cores(),
                         "kind": "reference" if use_yastn else "port",
                         "sample": f"{reps} runs of all {wl.ncv} Lanczos steps ("
                                   + ("YASTN tensordot + eigs on its NumPy backend" if use_yastn
                                      else "oracle restatement, numpy BLAS") + ", median)"},
        "e2e": {"value": world * wl.flops / t_e2e / 1e12, "unit": UNIT,
                "h2d_bytes_per_step": int(h_v0.numel() * 8), "d2h_bytes_per_step": int(h_v0.numel() * 8 + 8 * 60)},
        "gpu_launches": head['launches'],
        "clocks": head['clocks'],
        "extra": dict({m: {"tflops": wl.flops / r['t'] / 1e12, "ms_per_step": r['t'] * 1e3,
                           "lowest_ritz_rel_err": r['err']} for m, r in results.items()}, **extras),
    }
    print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()


_CHILD_ENV_DROP = ('RANK', 'WORLD_SIZE', 'LOCAL_RANK', 'LOCAL_WORLD_SIZE', 'GROUP_RANK', 'ROLE_RANK', 'MASTER_ADDR',
                   'MASTER_PORT', 'TORCHELASTIC_RUN_ID', 'GROUP_WORLD_SIZE', 'ROLE_WORLD_SIZE')


def other_config_lines(workloads=('cfg1', 'cfg3', 'cfg5'), extra_args=(), timeout=150, total=360):
    """The tensordot workloads of the other configurations (U(1) D=64, U(1)xU(1) complex128,
    the precision study), each run by this script in a child process (5 timed steps after 3
    warm-up steps, the truncated SVD left out) and summarised for the headline line: value,
    e2e, the emulated GEMM's roofline fraction, errors, the CPU baseline. A child that fails
    is recorded as such."""
    out = {}
    env = {k: v for k, v in os.environ.items() if k not in _CHILD_ENV_DROP}
    t_end = time.perf_counter() + total
    for name in workloads:
        left = t_end - time.perf_counter()
        if left <= 10:
            out[name] = {"skipped": f"the summaries' time budget ({total} s) is spent"}
            continue
        cmd = [sys.executable, os.path.join(ROOT, 'bench.py'), '--workload', name, '--steps', '5', '--warmup', '3',
               '--no-svd'] + list(extra_args)
        try:
            res = subprocess.run(cmd, capture_output=True, text=True, timeout=min(timeout, left), env=env, cwd=ROOT)
            lines = [ln for ln in res.stdout.splitlines() if ln.startswith('{')]
            if res.returncode != 0 or not lines:
                out[name] = {"failed": f"exit {res.returncode}: {res.stderr[-300:]}"}
                continue
            d = json.loads(lines[-1])
            roof = d.get('roofline') or {}
            out[name] = {"metric": d.get('metric'), "value": d.get('value'), "unit": d.get('unit'),
                         "ms_per_step": d.get('ms_per_step'), "dtype": d.get('dtype'),
                         "e2e": (d.get('e2e') or {}).get('value'), "roofline_kernel": roof.get('kernel'),
                         "roofline_frac": roof.get('frac'), "cpu_baseline": (d.get('cpu_baseline') or {}).get('value'),
                         "config": d.get('config'), "extra": d.get('extra')}
        except Exception as e:  # noqa: BLE001 -- a side measurement
            out[name] = {"failed": f"{type(e).__name__}: {e}"[:300]}
    return out


def emulated_dot_errors(torch, BK, mv, v0):
    """The emulated sector GEMMs of one matvec against the native FP64 ones on the same
    operands: the largest per-sector relative error max|C_emu - C_fp64| / max|C_fp64| over
    every sector of every dot (and the number of sectors compared)."""
    from yastn_gb300 import ops
    calls, orig = [], BK.dot

    def spy(A, B, meta, Dsize):
        calls.append((A, B, meta, Dsize))
        return orig(A, B, meta, Dsize)
    BK.dot = spy
    try:
        mv(v0)
    finally:
        BK.dot = orig
    worst, count = 0.0, 0
    for A, B, meta, Dsize in calls:
        ref = ops.dot(A, B, meta, Dsize).cpu().numpy()
        emu = ops.dot_ozaki(A, B, meta, Dsize).cpu().numpy()
        for slc, *_ in meta:
            r = ref[slc[0]:slc[1]]
            if r.size == 0:
                continue
            mx = np.abs(r).max()
            if mx > 0:
                worst = max(worst, float(np.abs(emu[slc[0]:slc[1]] - r).max() / mx))
            count += 1
    return worst, count


def plain_and_ctmrg_extras(args, torch, dev, wl, w, env, h_v0, flush, t_fused_cfg2):
    """Comparison fields of the headline line.

    - The DMRG workload on the plain per-block FP64 path on this GPU (``yastn_gb300.plain``:
      one torch launch per block piece, one cuBLAS matmul per sector GEMM, the reference
      torch backend's structure), the 30 Lanczos steps issued eagerly from the host, and
      its time over the fused path's.
    - The differentiable CTMRG step (Z2, D=6, chi=24, 8 CTM iterations, TFIM energy and
      gradient, each CTM move checkpointed) through this backend and through the plain
      per-block path (cuSOLVER gesvd per block, as the reference forces on CUDA), with the
      energy and gradient errors against the reference's recorded torch-autograd values.
    """
    from yastn_gb300 import backend as BK
    from yastn_gb300.plain import PlainBackend
    from yastn_gb300.workloads import lanczos, ritz_lowest
    plain = PlainBackend()
    mvp = lambda v: w.matvec(v, env, plain.dot, plain.transpose_and_merge, lambda x, f: x * f if f != 1.0 else x)
    v0 = h_v0.to(dev)
    ref_lam = w.tr['lanczos_lowest']
    _, al, be = lanczos(mvp, v0, wl.ncv, torch.dot, torch.linalg.vector_norm)  # warm-up
    tp = []
    for _ in range(2):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        _, al, be = lanczos(mvp, v0, wl.ncv, torch.dot, torch.linalg.vector_norm)
        lam, _ = ritz_lowest(al, be)
        torch.cuda.synchronize()
        tp.append(time.perf_counter() - t0)
    t_plain = float(np.mean(tp))
    out = {"dmrg_plain_per_block_gpu": {
        "ms_per_step": t_plain * 1e3, "tflops": wl.flops / t_plain / 1e12,
        "lowest_ritz_rel_err": abs(lam - ref_lam) / abs(ref_lam),
        "plain_over_fused": t_plain / t_fused_cfg2,
        "path": "one torch launch per block piece, one cuBLAS matmul per sector GEMM, host-issued (no graph)"}}

    c4 = Cfg4(24)
    c4.checkpoint = True

    def errs(E, g):
        gh = g.cpu().numpy()
        return (abs(float(E) - c4.E_ref) / abs(c4.E_ref),
                float(np.abs(gh - c4.grad_ref).max() / np.abs(c4.grad_ref).max()))

    def timed_ctm(backend, steps):
        ts = []
        for _ in range(steps):
            flush.zero_()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            E, g = c4.step(torch, backend, dev)
            torch.cuda.synchronize()
            ts.append((time.perf_counter() - t0) * 1e3)
        return float(np.mean(ts)), errs(E, g)
    c4.step(torch, BK, dev)
    t_fast, (ef, gf) = timed_ctm(BK, 2)
    assert ef <= 1e-10 and gf <= c4.grad_tol, (ef, gf)
    # warm cuSOLVER/cuBLAS for the plain path on one small block, then one timed step
    blk = torch.randn(64, 64, dtype=torch.float64, device=dev)
    torch.linalg.svd(blk, full_matrices=False, driver='gesvd')
    torch.linalg.qr(blk)
    t_plain4, (ep, gp) = timed_ctm(plain, 1)
    try:
        d = dlayer_line(args)
        out["double_layer_chi144"] = {
            "ms_per_call": d["ms_per_step"], "tflops": d["value"], "workload": d["config"]["workload"],
            "yastn_composition_gb300_ms": d["extra"]["yastn_composition_gb300_ms"],
            "reference_torch_cuda_ms": d["extra"]["reference_torch_cuda_ms"],
            "reference_over_fused": d["extra"]["reference_over_fused"],
            "rel_err_vs_reference_torch": d["extra"]["rel_err_vs_reference_torch"],
            "composed_copy_frac_of_hbm": d["roofline"]["frac"]}
    except ImportError as e:
        out["double_layer_chi144"] = {"unavailable": f"the reference package is not installed ({e})"}
    except Exception as e:  # noqa: BLE001 -- a side measurement: the headline line is printed regardless
        out["double_layer_chi144"] = {"failed": f"{type(e).__name__}: {e}"[:300]}
    out["ctmrg_chi24_fwd_bwd"] = {
        "ms_per_step": t_fast, "energy_rel_err_vs_reference": ef, "grad_rel_err_vs_reference": gf,
        "plain_per_block_gpu_ms": t_plain4, "plain_energy_rel_err": ep, "plain_grad_rel_err": gp,
        "plain_over_fused": t_plain4 / t_fast,
        "workload": c4.name + "; each CTM move checkpointed (non-reentrant)",
        "plain_path": "one torch launch per block, cuSOLVER gesvd per SVD block, torch autograd + the reference's "
                      "broadened SVD adjoint"}
    return out


def run_gpu_cfg4(args, wl):
    """CTMRG forward+backward through the backend, timed per step (CUDA events bracket the
    whole step, which includes the host's replay of the call sequence and YASTN's host-side
    decisions); the plain per-block FP64 path on the same GPU and on the host cores beside it."""
    import torch
    import torch.distributed as dist
    from yastn_gb300 import backend as BK
    from yastn_gb300 import _native, ops
    from yastn_gb300.plain import PlainBackend

    world = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    torch.cuda.set_device(local)
    dev = torch.device('cuda', local)
    if world > 1:
        dist.init_process_group('nccl')
    _native.lib()
    flush = torch.empty(L2_FLUSH_BYTES // 8, dtype=torch.float64, device=dev)
    pinned = torch.from_numpy(wl.A).pin_memory()

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    def check(E, g):
        e = abs(float(E) - wl.E_ref) / abs(wl.E_ref)
        gh = g.cpu().numpy()
        ge = float(np.abs(gh - wl.grad_ref).max() / np.abs(wl.grad_ref).max())
        return e, ge

    for _ in range(args.warmup):
        E, g = wl.step(torch, BK, dev)
    e_err, g_err = check(E, g)
    assert e_err <= 1e-10 and g_err <= wl.grad_tol, (e_err, g_err)
    barrier()
    clocks = Clocks(local)
    l0 = _native.LAUNCHES[0]
    ts = []
    with SvdSpy(torch) as spy:
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            E, g = wl.step(torch, BK, dev)
            e1.record()
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
    launches = (_native.LAUNCHES[0] - l0) // max(args.steps, 1)
    barrier()
    # end to end: the site tensor from pinned host memory, energy and gradient back to the host
    te = []
    gh = torch.empty(pinned.shape, dtype=torch.float64).pin_memory()
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        E, g = wl.step(torch, BK, dev, pinned=pinned)
        gh.copy_(g)
        Eh = float(E)
        te.append((time.perf_counter() - t0) * 1e3)
    clk = clocks.stop()
    e_err, g_err = check(E, g)
    # the same sequence on the plain per-block FP64 path (torch ops, cuSOLVER SVD) on this GPU
    plain = PlainBackend()
    tp, ep_err, gp_err = [float('nan')], None, None
    if not args.no_plain:
        wl.step(torch, plain, dev)
        tp = []
        for _ in range(min(args.steps, 2)):
            flush.zero_()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            Ep, gp = wl.step(torch, plain, dev)
            torch.cuda.synchronize()
            tp.append((time.perf_counter() - t0) * 1e3)
        ep_err, gp_err = check(Ep, gp)
    roof = spy.roofline(dev, args.steps)
    t_max, t_e2e = float(np.mean(ts)), float(np.mean(te))
    if world > 1:
        tt = torch.tensor([t_max, t_e2e], dtype=torch.float64, device=dev)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_max, t_e2e = float(tt[0]), float(tt[1])
    if rank != 0:
        if world > 1:
            dist.destroy_process_group()
        return
    if args.no_plain:  # the reference's own run, recorded on the host that made the fixture
        rec = wl.cpu_recorded or {}
        cpu_ms, cpu_kind = (rec.get('forward', float('nan')) + rec.get('backward', float('nan'))) * 1e3, \
            "reference (recorded run of YASTN's torch backend on 8 x86 threads, not this host)"
    else:
        t0 = time.perf_counter()
        wl.step(torch, plain, 'cpu')
        cpu_ms = (time.perf_counter() - t0) * 1e3
        cpu_kind = "one full forward+backward, one torch CPU op per block (LAPACK SVD)"
    fg, fs, bg = wl.flops()
    line = {
        "metric": wl.metric, "value": t_max, "unit": "ms", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_max, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded N(0,1) site tensor; call sequence recorded from YASTN)",
        "config": {"workload": wl.name, "parallelism": f"replicas{world}",
                   "l2": "flushed between timed steps (256 MB write)",
                   "checkpoint_move": "each CTM move recomputed in the backward (non-reentrant checkpoint)"
                   if wl.checkpoint else "off: every move's intermediates kept for the backward",
                   "energy_rel_err_vs_reference": e_err, "grad_rel_err_vs_reference": g_err,
                   "plain_per_block_gpu_ms": float(np.mean(tp)),
                   "plain_per_block_gpu": "the same sequence with one torch launch per block, torch.linalg.svd "
                                          "(cuSOLVER), torch autograd + the reference's broadened SVD adjoint",
                   "plain_over_fused": float(np.mean(tp)) / t_max if not args.no_plain else None,
                   "plain_energy_rel_err": ep_err, "plain_grad_rel_err": gp_err,
                   "flop_per_step": {"forward_gemm": fg, "forward_svd_nominal": fs, "backward_gemm": bg},
                   "effective_tflops": (fg + fs + bg) / (t_max * 1e-3) / 1e12},
        "roofline": roof,
        "cpu_baseline": {"value": cpu_ms, "unit": "ms", "cores": torch.get_num_threads() if not args.no_plain else 8,
                         "kind": "port" if not args.no_plain else "reference", "sample": cpu_kind},
        "e2e": {"value": t_e2e, "unit": "ms", "h2d_bytes_per_step": int(pinned.numel() * 8),
                "d2h_bytes_per_step": int(pinned.numel() * 8 + 8)},
        "gpu_launches": launches,
        "clocks": clk,
    }
    print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()


class SvdSpy:
    """Installed around the timed steps: CUDA events around every library call (per entry
    point) and, for the roofline of the FP64 Jacobi sweeps (the FP64 kernel of the block
    SVDs), their algorithmic work per launch = sum over blocks of sweeps x k(k-1)/2 pairs x
    (12 L + 6 k) real FLOP (three length-L dot products and the rotation of two X rows and two
    W rows; x4 for complex), against the FP64 rate of this GPU (cuBLAS DGEMM, measured live)."""

    def __init__(self, torch):
        from yastn_gb300 import _native, ops
        self.torch, self.N, self.ops = torch, _native, ops
        self.ev, self.work, self.cur = {}, [], {}

    def __enter__(self):
        N, ops, torch = self.N, self.ops, self.torch
        self.orig = (N.call, ops._svd_state_check, ops._jacobi)
        orig_call, orig_check, orig_jac = self.orig

        def spy(name, *a, **k):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            r = orig_call(name, *a, **k)
            e1.record()
            fp64 = (name == 'yb_svd_sweeps' and a[6] == 64) or (name == 'yb_svd_block_sweeps' and a[7] == 64)
            self.ev.setdefault('fp64_sweeps' if fp64 else name, []).append((e0, e1))
            return r

        def jac(data, plan, *a, **k):
            self.cur['kL'] = [(int(r[9]), int(r[10])) for r in plan.blocks]
            self.cur['cplx'] = data.is_complex()
            return orig_jac(data, plan, *a, **k)

        def check(state, nb, phase, req):
            sw = orig_check(state, nb, phase, req)
            if phase == 'FP64':
                f = sum(int(x) * k * (k - 1) // 2 * (12 * L + 6 * k) for x, (k, L) in zip(sw, self.cur['kL']))
                self.work.append(f * (4 if self.cur['cplx'] else 1))
            return sw
        N.call, ops._svd_state_check, ops._jacobi = spy, check, jac
        return self

    def __exit__(self, *exc):
        self.N.call, self.ops._svd_state_check, self.ops._jacobi = self.orig
        return False

    def roofline(self, dev, steps):
        torch = self.torch
        torch.cuda.synchronize()
        tot = {k: sum(a.elapsed_time(b) for a, b in v) * 1e-3 / steps for k, v in self.ev.items()}
        t64 = tot.get('fp64_sweeps', 0.0)
        n64 = len(self.ev.get('fp64_sweeps', [])) // steps
        work = sum(self.work) / steps
        peak = fp64_peak_tflops(torch, dev)
        achieved = work / t64 / 1e12 if t64 > 0 else 0.0
        return {"bound": "fp64", "kernel": "Jacobi FP64 phase (yb_svd_block_sweeps / yb_svd_sweeps)",
                "achieved": achieved, "peak": peak,
                "unit": "TFLOP/s", "frac": achieved / peak, "peak_source": "measured live: cuBLAS DGEMM 4096^3",
                "traffic": None, "launches": n64, "ms_per_launch": t64 / max(n64, 1) * 1e3,
                "measured": "CUDA events around every library call over the timed steps",
                "device_ms_per_step": {k: v * 1e3 for k, v in sorted(tot.items(), key=lambda x: -x[1])[:8]}}


def kernel_roofline(torch, dev, run_once, w, gemm_mode, reps=5):
    """Device time per entry point over ``reps`` eager matvecs (CUDA events on the launching
    stream; the stream is first held by a spin kernel long enough for the host to enqueue
    the whole matvec, so the events time back-to-back kernels, not host launch gaps); the
    roofline of the entry point that takes the most time, with its algorithmic work: BF16
    tensor FLOP of the split-operand GEMM, FP64 FLOP of the native GEMM, or 16 bytes per
    FP64 element moved by the block copies."""
    from yastn_gb300 import _native, _plans as P, ops
    orig = _native.call
    ev = {}

    def spy(name, *a, **k):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        r = orig(name, *a, **k)
        e1.record()
        ev.setdefault(name, []).append((e0, e1))
        return r
    run_once()
    torch.cuda.synchronize()
    _native.call = spy
    try:
        for _ in range(reps):
            torch.cuda._sleep(50_000_000)
            run_once()
        torch.cuda.synchronize()
    finally:
        _native.call = orig
    tot = {k: sum(a.elapsed_time(b) for a, b in v) * 1e-3 / reps for k, v in ev.items()}
    # the two emulated-GEMM kernels (tcgen05, mma.sync; the autotuner picks one per dot) count as one
    gemm_keys = [k for k in tot if k in ('yb_ozaki_gemm', 'yb_ozaki_gemm_tc')]
    if len(gemm_keys) > 1:
        tot['yb_ozaki_gemm'] = sum(tot.pop(k) for k in gemm_keys)
    top = max(tot, key=tot.get)
    dots = [st for st in w.steps if st[0] == 'dot']
    merges = [st for st in w.steps if st[0] == 'transpose_and_merge']
    peaks = {}
    try:
        with open(os.path.join(ROOT, 'MEASURED_PEAKS.json')) as f:
            peaks = json.load(f)
    except (OSError, ValueError):
        pass
    if top.startswith('yb_ozaki_gemm'):
        s = ops.OZAKI_SLICES
        work = sum(P.ozaki_dot_plan(st[2][2], s).flops for st in dots) * s * (s + 1) // 2
        peak, unit, bound, src = peaks.get('bf16_tflops', 1900.0), "TFLOP/s", "tensor", "bf16 (cuBLAS burst)"
        achieved = work / tot[top] / 1e12
    elif top == 'yb_grouped_gemm':
        work = sum((P.ozaki_dot_plan(st[2][2], ops.OZAKI_SLICES).native.flops if gemm_mode == 'emulated'
                    else P.dot_plan(st[2][2]).flops) for st in dots)
        peak, unit, bound, src = fp64_peak_tflops(torch, dev), "TFLOP/s", "tensor", "fp64 (cuBLAS DGEMM, measured live)"
        achieved = work / tot[top] / 1e12
    else:
        work = sum(16 * st[2][4] for st in merges)
        peak, unit, bound, src = peaks.get('hbm_gbs', 6800.0), "GB/s", "hbm", "hbm copy"
        achieved = work / tot[top] / 1e9
    out = {"bound": bound, "kernel": top, "achieved": achieved, "peak": peak, "unit": unit,
           "frac": achieved / peak, "peak_source": "measured: " + src, "traffic": None,
           "device_ms_per_matvec": {k: v * 1e3 for k, v in tot.items()}}
    if top == 'yb_ozaki_gemm_tc':
        # DRAM bytes (read + write) of the two tcgen05 GEMM launches of one matvec, from the ncu
        # capture in profiles/ozaki_gemm_tcgen05_dmrg_heff2.md; the digit planes they read
        # (algorithmic bytes, tile layout) are computed here
        def tc_digits(plan):
            tn = getattr(plan, 'tuned_tc', plan.prefer_tc)
            sfx = '_tc32' if tn == 32 else '_tc'
            return 2 * (getattr(plan, 'a_size' + sfx) + getattr(plan, 'b_size' + sfx))
        digits = sum(tc_digits(P.ozaki_dot_plan(st[2][2], ops.OZAKI_SLICES)) for st in dots)
        out.update(traffic=TC_GEMM_DRAM_BYTES_PER_MATVEC, traffic_unit="bytes per matvec (2 launches)",
                   traffic_source="ncu dram__bytes_read.sum + dram__bytes_write.sum, "
                                  "profiles/ozaki_gemm_tcgen05_dmrg_heff2.md",
                   algorithmic_bytes_per_matvec=digits)
    return out


TC_GEMM_DRAM_BYTES_PER_MATVEC = 21.497344e6 + 45.472512e6 + 256 + 25856  # ncu capture, DMRG Heff2 matvec


def svd144_blocks(torch, dev):
    """The first projector SVD call of the chi=144 CTMRG run (two Z2 blocks of ~2592^2): the
    recorded call sequence is replayed through the backend until that call, whose input is
    returned as (data, meta, sizes)."""
    from yastn_gb300 import backend as BK
    from yastn_gb300.replay import load_replay
    r = load_replay('ctmrg_z2_d6_chi144')
    found = []

    class Found(Exception):
        pass

    class Intercept:
        def __getattr__(self, name):
            return getattr(BK, name)

        def svd(self, data, meta, sizes, *a, **k):
            if max(max(m[1]) for m in meta) >= 2000:
                found.append((data.detach().clone(), meta, sizes))
                raise Found
            return BK.svd(data, meta, sizes, *a, **k)
    A = torch.from_numpy(r.arrays['in:A']).to(dev)
    try:
        with torch.no_grad():
            r.run(Intercept(), dev, {'A': A})
    except Found:
        pass
    return found[0]


def run_svd144(args):
    """Block SVD of the chi=144 projector call: this backend (ops.svd) against cuSOLVER's gesvd
    per block (the driver the reference forces on CUDA, yastn/backend/linalg/
    torch_svd_gesdd.py:16-17) on the same device tensors; ms per call (both blocks), best
    of the timed calls after a warm-up, with the singular values compared."""
    import torch
    from yastn_gb300 import ops
    dev = torch.device('cuda', 0)
    torch.cuda.set_device(dev)
    data, meta, sizes = svd144_blocks(torch, dev)

    def ours():
        return ops.svd(data, meta, sizes)[1]

    def gesvd():
        return torch.cat([torch.linalg.svd(data[sl[0]:sl[1]].view(D), full_matrices=False, driver='gesvd')[1]
                          for sl, D, *_ in meta])

    def timed(fn, reps):
        fn()
        torch.cuda.synchronize()
        ts = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            out = fn()
            e1.record()
            e1.synchronize()
            ts.append(e0.elapsed_time(e1))
        return min(ts), out
    reps = max(1, min(args.steps, 3))
    t_ours, S0 = timed(ours, reps)
    t_lib, S1 = timed(gesvd, reps)
    S0 = torch.sort(S0.cpu(), descending=True).values
    S1 = torch.sort(S1.cpu(), descending=True).values
    err = float((S0 - S1).abs().max() / S1.max())
    line = {"metric": "block SVD ms per call (CTMRG chi=144 projectors, 2 Z2 blocks of 2592^2, FP64)",
            "value": t_ours, "unit": "ms", "n_gpus": 1, "steps": reps, "warmup": 1, "ms_per_step": t_ours,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "projector blocks of the recorded CTMRG run (seeded N(0,1) site tensor)",
            "config": {"workload": "first projector SVD of the chi=144 CTMRG step",
                       "blocks": [list(m[1]) for m in meta]},
            "extra": {"cusolver_gesvd_ms": t_lib, "gesvd_over_ours": t_lib / t_ours,
                      "max_abs_dS_over_max_S": err}}
    print(json.dumps(line))


DLAYER_METRIC = "double-layer contraction TFLOP/s (append_vec_tl, Z2 D=6 chi=144, FP64)"
DLAYER_WORKLOAD = "append_vec_tl mode b-self, vector x [l l'] [t t'] y, chi=144, D=6, d=2, Z2"
DLAYER_KW = dict(mode='b-self', in_b=(2, 1), out_a=(3, 2))


def _yastn_ref():
    ref = os.path.join(ROOT, 'baseline', '_ref')
    if ref not in sys.path:
        sys.path.insert(0, ref)
    import yastn
    return yastn


def dlayer_inputs(chi=144):
    """The site tensor (bra = ket) and the boundary vector x [l l'] [t t'] y of the chi=144
    CTMRG corner step, as YASTN tensors on its NumPy backend (seeded normal draws)."""
    yastn = _yastn_ref()
    import yastn.tn.fpeps as fpeps
    cfn = yastn.make_config(sym='Z2', backend='np', default_dtype='float64')
    cfn.backend.random_seed(0)
    vl = yastn.Leg(cfn, s=1, t=(0, 1), D=(3, 3))
    pl = yastn.Leg(cfn, s=1, t=(0, 1), D=(1, 1))
    el = yastn.Leg(cfn, s=1, t=(0, 1), D=(chi // 2, chi // 2))
    ket = yastn.rand(cfn, legs=[vl.conj(), vl, vl, vl.conj(), pl])
    la, lb = fpeps.DoublePepsTensor(bra=ket, ket=ket).get_legs((1, 0))
    vec = yastn.rand(cfn, legs=[el, la.conj(), lb.conj(), el.conj()])
    return ket, ket, vec


def dlayer_flops(bra, ket, vec):
    """FP64 FLOP of the sector GEMMs of one append_vec_tl call (2 m n k per sector), counted
    by running YASTN's function once with its NumPy backend's dot observed."""
    import yastn.backend.backend_np as bnp
    import yastn.tn.fpeps.envs._env_contractions as ec
    count = [0]
    dot = bnp.dot

    def counting_dot(A, B, meta_dot, Dsize):
        count[0] += sum(2 * Da[0] * Da[1] * Db[1] for _, _, _, Da, _, Db in meta_dot)
        return dot(A, B, meta_dot, Dsize)
    bnp.dot = counting_dot
    try:
        ec.append_vec_tl(bra, ket, vec, **DLAYER_KW)
    finally:
        bnp.dot = dot
    return count[0]


def run_reference_dlayer(args):
    """Reference arm of the double-layer workload: YASTN's own append_vec_tl on its NumPy
    backend (the reference's CPU path) on all host cores, each step one call."""
    try:
        _yastn_ref()
        import yastn.tn.fpeps.envs._env_contractions as ec
    except ImportError as e:
        print(json.dumps({"impl": "reference", "unavailable": f"the reference package is not installed under "
                                                              f"baseline/_ref ({e})"}))
        return
    bra, ket, vec = dlayer_inputs()
    flops = dlayer_flops(bra, ket, vec)
    for _ in range(args.warmup):
        ec.append_vec_tl(bra, ket, vec, **DLAYER_KW)
    ts = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        ec.append_vec_tl(bra, ket, vec, **DLAYER_KW)
        ts.append(time.perf_counter() - t0)
    t = float(np.mean(ts))
    value = flops / t / 1e12
    line = {"impl": "reference", "metric": DLAYER_METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded yastn normal draws)",
            "config": {"workload": DLAYER_WORKLOAD, "gemm_flop_per_call": flops},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cpu_cores(), "kind": "reference",
                             "sample": f"{args.steps} calls of YASTN's append_vec_tl on its NumPy backend"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def dlayer_e2e(reps):
    """One call through the public API with host data: the three tensors' data copied from
    pinned host memory to the device, the compiled contraction, the result read back; mean
    seconds per call and the bytes copied each way."""
    import torch
    yastn = _yastn_ref()
    from yastn_gb300 import backend as BK
    from yastn_gb300 import double_layer as dl
    bra, ket, vec = dlayer_inputs()
    cfg = yastn.make_config(sym='Z2', backend=BK, default_dtype='float64', default_device='cuda')
    host = [torch.from_numpy(np.ascontiguousarray(t._data)).pin_memory() for t in (bra, ket, vec)]
    saved_mode = BK.get_gemm_mode()
    BK.set_gemm_mode('fp64')
    try:
        def step():
            ts = [t._replace(config=cfg, data=h.to('cuda', non_blocking=True)) for t, h in zip((bra, ket, vec), host)]
            return dl.append_vec_tl(*ts, **DLAYER_KW)._data.to('cpu')
        out = step()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            out = step()
        torch.cuda.synchronize()
        t = (time.perf_counter() - t0) / reps
    finally:
        BK.set_gemm_mode(saved_mode)
    return t, int(sum(h.numel() * h.element_size() for h in host)), int(out.numel() * out.element_size())


def run_dlayer(args):
    line = dlayer_line(args)
    flops = line['config']['gemm_flop_per_call']
    t_e2e, bi, bo = dlayer_e2e(max(3, args.steps))
    line['e2e'] = {"value": flops / t_e2e / 1e12, "unit": UNIT, "h2d_bytes_per_step": bi, "d2h_bytes_per_step": bo}
    # the reference's CPU path on the host cores: YASTN's own function on its NumPy backend
    import yastn.tn.fpeps.envs._env_contractions as ec
    bra, ket, vec = dlayer_inputs()
    t_cpu, reps = time_cpu(lambda: ec.append_vec_tl(bra, ket, vec, **DLAYER_KW), budget_s=10.0, min_reps=2)
    line['cpu_baseline'] = {"value": flops / t_cpu / 1e12, "unit": UNIT, "cores": cpu_cores(), "kind": "reference",
                            "sample": f"{reps} calls of YASTN's append_vec_tl on its NumPy backend (median)"}
    print(json.dumps(line))


def dlayer_line(args):
    """Double-layer contraction (append_vec_tl, mode 'b-self' as the CTM corners call it) at the
    chi=144 CTMRG shape: the compiled program against YASTN's composition on this backend and
    on the reference's torch backend (default_device='cuda'); FP64 GEMM FLOP of the program's
    sector GEMMs per call; every output compared with the reference torch backend's."""
    import torch
    ref = os.path.join(ROOT, 'baseline', '_ref')
    if ref not in sys.path:
        sys.path.insert(0, ref)
    import yastn
    import yastn.tn.fpeps as fpeps
    import yastn.tn.fpeps.envs._env_contractions as ec
    from yastn_gb300 import backend as BK
    from yastn_gb300 import double_layer as dl
    from yastn_gb300 import ops
    dev = torch.device('cuda', 0)
    torch.cuda.set_device(dev)
    chi = 144
    cfn = yastn.make_config(sym='Z2', backend='np', default_dtype='float64')
    cfn.backend.random_seed(0)
    vl = yastn.Leg(cfn, s=1, t=(0, 1), D=(3, 3))
    pl = yastn.Leg(cfn, s=1, t=(0, 1), D=(1, 1))
    el = yastn.Leg(cfn, s=1, t=(0, 1), D=(chi // 2, chi // 2))
    ket = yastn.rand(cfn, legs=[vl.conj(), vl, vl, vl.conj(), pl])
    bra = ket
    la, lb = fpeps.DoublePepsTensor(bra=bra, ket=ket).get_legs((1, 0))
    vec = yastn.rand(cfn, legs=[el, la.conj(), lb.conj(), el.conj()])
    kw = dict(mode='b-self', in_b=(2, 1), out_a=(3, 2))
    arms = {}
    for name, backend in (('gb300', BK), ('reference_torch_cuda', 'torch')):
        cfg = yastn.make_config(sym='Z2', backend=backend, default_dtype='float64', default_device='cuda')
        arms[name] = [t._replace(config=cfg, data=torch.from_numpy(np.ascontiguousarray(t._data)).to(dev))
                      for t in (bra, ket, vec)]
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)

    def timed(fn, ts, reps):
        out = fn(*ts, **kw)
        torch.cuda.synchronize()
        ms = []
        for _ in range(reps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            out = fn(*ts, **kw)
            e1.record()
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
        return float(np.median(ms)), out
    reps = max(3, args.steps)
    dl.clear_cache()
    saved_mode = BK.get_gemm_mode()
    try:
        BK.set_gemm_mode('fp64')
        t_fused, out_f = timed(dl.append_vec_tl, arms['gb300'], reps)
        t_comp, out_c = timed(ec.append_vec_tl, arms['gb300'], reps)
        BK.set_gemm_mode('emulated')
        t_emu, out_e = timed(dl.append_vec_tl, arms['gb300'], reps)
    finally:
        BK.set_gemm_mode(saved_mode)
    t_ref, out_r = timed(ec.append_vec_tl, arms['reference_torch_cuda'], reps)
    rel = float((out_f._data - out_r._data).abs().max() / out_r._data.abs().max())
    rel_emu = float((out_e._data - out_r._data).abs().max() / out_r._data.abs().max())
    assert torch.equal(out_f._data, out_c._data) and rel <= 1e-12, rel
    key = next(iter(dl._PROGRAMS))
    prog = dl._PROGRAMS[key]
    flops = 0
    for st in prog.steps:
        if st[0] == 'gemm':
            flops += sum(2 * Da[0] * Da[1] * Db[1] for _, _, _, Da, _, Db in st[4][0])
    # the composed-copy kernel alone: the largest gather of the program, timed in a loop
    maps = prog.maps(BK, dev)
    env = {('in', i): t._data for i, t in enumerate(arms['gb300'])}
    biggest = None
    for st in prog.steps:
        if st[0] == 'gather':
            m = maps[st[1]]
            src = env[st[2]]
            if m is not None and (biggest is None or m[0].numel() > biggest[1].numel()):
                biggest = (src, m[0], m[2])
            env[st[1]] = src if m is None else ops.map_gather(src, m[0], m[2])
        else:
            env[st[2]] = getattr(BK, st[1])(env[st[3][0]], env[st[3][1]], *st[4])
    src, gmap, conj = biggest
    ops.map_gather(src, gmap, conj)
    gms = []
    for _ in range(reps):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        ops.map_gather(src, gmap, conj)
        e1.record()
        e1.synchronize()
        gms.append(e0.elapsed_time(e1))
    t_g = float(np.median(gms))
    n_nz = int(torch.count_nonzero(gmap))
    gbytes = gmap.numel() * (4 + 8) + n_nz * 8
    peaks = {}
    try:
        with open(os.path.join(ROOT, 'MEASURED_PEAKS.json')) as f:
            peaks = json.load(f)
    except (OSError, ValueError):
        pass
    hbm = peaks.get('hbm_gbs', 6800.0)
    line = {"metric": "double-layer contraction TFLOP/s (append_vec_tl, Z2 D=6 chi=144, FP64)",
            "value": flops / t_fused / 1e9, "unit": "TFLOP/s", "n_gpus": 1, "steps": reps, "warmup": 1,
            "ms_per_step": t_fused, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (seeded normal draws as yastn.rand)",
            "config": {"workload": "append_vec_tl mode b-self, vector x [l l'] [t t'] y, chi=144, D=6, d=2, Z2",
                       "gemm_flop_per_call": flops, "vector_elements": int(vec.size),
                       "l2": "flushed between timed calls (256 MB write)",
                       "program": [st[0] for st in prog.steps]},
            "roofline": {"bound": "hbm", "kernel": "yb_map_gather", "achieved": gbytes / t_g / 1e6, "peak": hbm,
                         "unit": "GB/s", "frac": gbytes / t_g / 1e6 / hbm, "peak_source": "measured: hbm copy",
                         "traffic": None, "algorithmic_bytes": gbytes,
                         "note": "largest composed copy of the program: int32 map + 8 B store per entry, "
                                 "8 B load per mapped entry"},
            "extra": {"emulated_gemm_ms": t_emu, "emulated_tflops": flops / t_emu / 1e9,
                      "emulated_rel_err_vs_reference_torch": rel_emu,
                      "yastn_composition_gb300_ms": t_comp, "reference_torch_cuda_ms": t_ref,
                      "composition_over_fused": t_comp / t_fused, "reference_over_fused": t_ref / t_fused,
                      "rel_err_vs_reference_torch": rel, "fused_bitwise_equal_to_composition": True}}
    return line


def main():
    args = parse()
    if args.workload == 'dlayer':
        if args.impl == 'reference':
            if int(os.environ.get('RANK', '0')) == 0:
                run_reference_dlayer(args)
        else:
            run_dlayer(args)
        return
    if args.workload == 'svd144':
        if args.impl == 'reference':
            print(json.dumps({"impl": "reference", "unavailable": "svd144 compares against cuSOLVER in the GPU arm"}))
        else:
            run_svd144(args)
        return
    wl = Cfg4(args.chi, args.use_qr) if args.workload == 'cfg4' else \
        {'cfg1': Cfg1, 'cfg2': Cfg2, 'cfg3': Cfg3, 'cfg5': Cfg5}[args.workload]()
    if args.workload == 'cfg4':
        wl.checkpoint = not args.no_checkpoint
    if args.impl == 'reference':
        run_reference(args, wl)
    elif args.workload == 'cfg2':
        run_gpu_cfg2(args, wl)
    elif args.workload == 'cfg4':
        run_gpu_cfg4(args, wl)
    else:
        run_gpu(args, wl)


if __name__ == '__main__':
    main()
