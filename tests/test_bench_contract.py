"""The benchmark's reference arm on the host cores (no GPU): one JSON line with the keys of
the benchmark contract, for the default workload (DMRG Heff2 Lanczos: the reference package
itself when it is installed under baseline/_ref, else the oracle's restatement), the
tensordot workload, the CTMRG workload (its per-move checkpointed replay on the plain
per-block torch path) and the double-layer contraction (YASTN's own append_vec_tl on its
NumPy backend)."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
KEYS = {"metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
        "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e", "impl"}


def _run(*args):
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    res = subprocess.run([sys.executable, os.path.join(ROOT, 'bench.py'), '--impl', 'reference', *args],
                         capture_output=True, text=True, timeout=600, env=env, cwd=ROOT)
    assert res.returncode == 0, res.stderr[-2000:]
    lines = [ln for ln in res.stdout.splitlines() if ln.startswith('{')]
    assert len(lines) == 1
    return json.loads(lines[0])


@pytest.mark.parametrize('args', [
    ('--steps', '1', '--warmup', '0'),
    ('--workload', 'cfg1', '--steps', '1', '--warmup', '0'),
    ('--workload', 'cfg4', '--steps', '1', '--warmup', '0'),
    ('--workload', 'dlayer', '--steps', '1', '--warmup', '0'),
])
def test_reference_arm_line(args):
    if 'dlayer' in args and not os.path.isdir(os.path.join(ROOT, 'baseline', '_ref', 'yastn')):
        pytest.skip("the double-layer reference arm runs the reference package (baseline/_ref)")
    line = _run(*args)
    assert KEYS <= set(line)
    assert line["impl"] == "reference"
    assert line["value"] > 0 and line["e2e"]["value"] == line["value"]
    assert line["cpu_baseline"]["value"] == line["value"] and line["cpu_baseline"]["cores"] >= 1
    assert isinstance(line["config"]["workload"], str)
    if '--workload' not in args:  # the DMRG workload: YASTN's eigs (or its restatement) reproduces the recording
        assert line["config"]["lowest_ritz_rel_err_vs_recorded"] <= 1e-10
    if '--workload' in args and args[args.index('--workload') + 1] == 'cfg4':
        assert line["unit"] == "ms" and line["higher_is_better"] is False
        assert line["config"]["energy_rel_err_vs_reference"] <= 1e-12
    if '--workload' in args and args[args.index('--workload') + 1] == 'dlayer':
        # YASTN's own append_vec_tl on its NumPy backend; its sector GEMMs count the FLOP the
        # GPU arm counts from its compiled program (the chi=144 corner step: 1.935 GFLOP)
        assert line["cpu_baseline"]["kind"] == "reference"
        assert line["config"]["gemm_flop_per_call"] == 1934917632


def test_other_configuration_summaries_of_the_headline_line(monkeypatch):
    """The headline line's summaries of the other configurations come from this script run
    in child processes (here its reference arm, on the host): parsed into value, unit,
    workload; a failing child is recorded, not raised."""
    import importlib.util
    spec = importlib.util.spec_from_file_location('bench_mod', os.path.join(ROOT, 'bench.py'))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    monkeypatch.setenv('CUDA_VISIBLE_DEVICES', '')
    out = bench.other_config_lines(workloads=('cfg1', 'nope'), extra_args=('--impl', 'reference'))
    assert out['cfg1']['value'] > 0 and out['cfg1']['unit'] == 'TFLOP/s'
    assert 'D=64' in out['cfg1']['config']['workload']
    assert 'failed' in out['nope']
