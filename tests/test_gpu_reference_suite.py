"""YASTN's own test suites (the reference's tests/tensor, tests/mps and tests/peps, installed
unchanged under baseline/_ref/yastn_tests by baseline/install_reference.py) run against this
backend on the GPU through tests/yastn_suite_plugin.py (YASTN's 'torch' backend name resolves
to this module for the session), with pytest-xdist workers and a per-test time limit.

The whole tensor suite runs, and from the network suites the files on this backend's path:
DMRG (two-site, with YASTN's eigs), the Krylov tests, CTMRG on square and C4v lattices, the
double-layer PEPS tensor and the fixed-point CTMRG with its implicit differentiation
(torch.func.vjp through the backend's autograd Functions). Every test passes except the ones
in EXPECTED_FAILURES, each with its reason: the non-Hermitian eigensolver and the partial
Hermitian one (which the reference runs through torch.linalg.eig / SciPy's ARPACK) are not
part of this backend.
"""
import os
import subprocess
import sys
import xml.etree.ElementTree as ET

import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SUITE = os.path.join(ROOT, 'baseline', '_ref', 'yastn_tests')
FILES = ['tensor', 'mps/test_dmrg.py', 'mps/test_krylov.py', 'mps/test_environment.py', 'peps/test_ctmrg.py',
         'peps/test_ctmrg_c4v.py', 'peps/test_double_peps_tensor.py', 'peps/test_fp_c4v.py']

_NOT_PROVIDED = "decomposition not provided by this backend (the reference uses torch.linalg.eig / SciPy ARPACK)"
EXPECTED_FAILURES = {
    'test_eig.py::test_eig_basic': _NOT_PROVIDED,
    'test_eig.py::test_eig_complex': _NOT_PROVIDED,
    'test_eig.py::test_eig_degeneracy_fail': _NOT_PROVIDED,
    'test_eig.py::test_eig_transpose_meta': _NOT_PROVIDED,
    'test_eigs.py::test_eigs_arnoldi': _NOT_PROVIDED,
    'test_eighs.py::test_eigh_basic[LM]': _NOT_PROVIDED,
    'test_eighs.py::test_eigh_basic_2[LM]': _NOT_PROVIDED,
    'test_eighs.py::test_eigh_basic_2[SR]': _NOT_PROVIDED,
}


def _expected(name):
    f = name.split('::')[0]
    return name in EXPECTED_FAILURES or (f + '::*') in EXPECTED_FAILURES


def _run_suite(files, tmp_path, extra=(), env_extra=None):
    """Run YASTN's test files on this backend; returns the junit XML path."""
    xml = tmp_path / 'suite.xml'
    env = dict(os.environ)
    env['PYTHONPATH'] = os.pathsep.join([os.path.join(ROOT, 'tests'), os.path.join(ROOT, 'baseline', '_ref'), ROOT,
                                         env.get('PYTHONPATH', '')])
    env.update(env_extra or {})
    cmd = [sys.executable, '-m', 'pytest'] + list(files) + ['-p', 'yastn_suite_plugin', '--backend', 'torch_gb300',
           '--device', 'cuda', '-q', '-p', 'no:cacheprovider', '--junitxml', str(xml)] + list(extra) + \
          ['-n', '8', '--timeout', '300']
    try:
        import xdist  # noqa: F401
        import pytest_timeout  # noqa: F401
    except ImportError:
        cmd = cmd[:-4]
    proc = subprocess.run(cmd, cwd=SUITE, env=env, capture_output=True, text=True, timeout=1500)
    assert xml.exists(), proc.stdout[-3000:] + proc.stderr[-3000:]
    return xml


def _outcomes(xml):
    """{test name: passed?} of a junit XML (skipped tests left out)."""
    out = {}
    for tc in ET.parse(xml).iter('testcase'):
        if tc.find('skipped') is not None:
            continue
        name = tc.get('classname').split('.')[-1] + '.py::' + tc.get('name')
        out[name] = tc.find('failure') is None and tc.find('error') is None
    return out


# the network suites whose environments contract double-layer PEPS tensors (append_vec_*):
# CTMRG on square and C4v lattices, their measurements (fermionic ones included), the
# double-layer tensor itself and the fixed-point CTMRG
PEPS_FILES = ['peps/test_ctmrg.py', 'peps/test_ctmrg_c4v.py', 'peps/test_double_peps_tensor.py', 'peps/test_fp_c4v.py',
              'peps/test_ctmrg_measure.py', 'peps/test_fermionic_measure.py']


def test_reference_peps_suites_with_fused_double_layer(cuda_device, tmp_path):
    """YASTN's PEPS suites with the double-layer contractions run as this backend's compiled
    programs (yastn_gb300.double_layer.install()): every test passes (64 tests; with YASTN's own
    composition on this backend the same 64 pass), and the programs ran (compiled and reused,
    no contraction left to YASTN's composition)."""
    if not os.path.isdir(SUITE):
        pytest.skip("the reference's test suite is not installed (python baseline/install_reference.py <tree>)")
    (tmp_path / 'stats').mkdir()
    fused = _outcomes(_run_suite(PEPS_FILES, tmp_path, ['--gb300-double-layer'],
                                 {'YB_DOUBLE_LAYER_STATS': str(tmp_path / 'stats')}))
    failed = sorted(n for n, ok in fused.items() if not ok and not _expected(n))
    assert not failed, failed
    assert sum(fused.values()) >= 60, fused
    import json
    stats = [json.load(open(tmp_path / 'stats' / f)) for f in os.listdir(tmp_path / 'stats')]
    assert stats and sum(s['compiled'] for s in stats) > 0 and sum(s['hits'] for s in stats) > 0, stats
    assert sum(s['unfused'] for s in stats) == 0, stats
    print(f"PEPS suites with the compiled double-layer programs: {sum(fused.values())} passed; {stats}")


def test_reference_suites_on_this_backend(cuda_device, tmp_path):
    if not os.path.isdir(SUITE):
        pytest.skip("the reference's test suite is not installed (python baseline/install_reference.py <tree>)")
    xml = _run_suite(FILES, tmp_path)
    passed, failed, unexpected = 0, [], []
    for tc in ET.parse(xml).iter('testcase'):
        name = tc.get('classname').split('.')[-1] + '.py::' + tc.get('name')
        bad = tc.find('failure') is not None or tc.find('error') is not None
        if tc.find('skipped') is not None:
            continue
        if bad:
            failed.append(name)
            if not _expected(name):
                msg = (tc.find('failure') if tc.find('failure') is not None else tc.find('error')).get('message', '')
                unexpected.append(f"{name}: {msg[:300]}")
        else:
            passed += 1
    print(f"YASTN's suites on this backend: {passed} passed, {len(failed)} failed "
          f"({len(failed) - len(unexpected)} expected)")
    assert passed >= 300, passed
    assert not unexpected, "\n".join(unexpected)
