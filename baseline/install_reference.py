"""Install the unmodified YASTN reference into ``baseline/_ref`` (git-ignored).

First tries the regular offline install

    python -m pip install --no-index --no-build-isolation --find-links /opt/wheelhouse \
        --target baseline/_ref <reference tree>

(from a copy of the tree under /tmp, since the build writes next to the sources). That
fails in this image: YASTN's build backend requires ``setuptools-scm``, which is neither
installed nor in the offline wheelhouse. YASTN itself is pure Python, so the fallback does
what an install of a pure-Python package does: it copies the ``yastn`` package directory
unchanged into ``baseline/_ref``, installs ``tqdm`` there from the offline wheelhouse and
copies the pure-Python ``opt_einsum`` package of this interpreter (both are imported by
``import yastn``; the GPU machine has neither). Nothing of the reference is modified.

The reference's own test suites (tests/tensor, tests/mps and tests/peps, with their input
files) are copied unchanged to ``baseline/_ref/yastn_tests``, where
tests/test_gpu_reference_suite.py runs them against this backend.

Usage: python baseline/install_reference.py <reference tree> [wheelhouse]
"""
import os
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
TARGET = os.path.join(HERE, '_ref')


def _pip(args):
    return subprocess.run([sys.executable, '-m', 'pip', 'install', '--no-index', '--no-build-isolation'] + args,
                          capture_output=True, text=True)


def main(ref, wheelhouse='/opt/wheelhouse'):
    if os.path.exists(TARGET):
        shutil.rmtree(TARGET)
    with tempfile.TemporaryDirectory() as tmp:
        src = os.path.join(tmp, 'yastn_src')
        shutil.copytree(ref, src, ignore=shutil.ignore_patterns('.git', '__pycache__'))
        res = _pip(['--find-links', wheelhouse, '--target', TARGET, src])
    if res.returncode == 0:
        print('pip install of the reference: ok')
        return copy_tests(ref)
    print('pip install of the reference failed (metadata generation: setuptools-scm is a build requirement '
          'absent from the offline wheelhouse); installing the pure-Python package by copy')
    os.makedirs(TARGET, exist_ok=True)
    shutil.copytree(os.path.join(ref, 'yastn'), os.path.join(TARGET, 'yastn'),
                    ignore=shutil.ignore_patterns('__pycache__'))
    res = _pip(['--no-deps', '--find-links', wheelhouse, '--target', TARGET, 'tqdm'])
    if res.returncode != 0:
        print(res.stdout[-2000:], res.stderr[-2000:])
        return 1
    import opt_einsum
    shutil.copytree(os.path.dirname(opt_einsum.__file__), os.path.join(TARGET, 'opt_einsum'),
                    ignore=shutil.ignore_patterns('__pycache__'))
    print(f'installed yastn, tqdm, opt_einsum into {TARGET}')
    return copy_tests(ref)


def copy_tests(ref):
    """The reference's tests/tensor, tests/mps and tests/peps suites (with their input files),
    unchanged, beside the installed package."""
    for part in ('tensor', 'mps', 'peps'):
        dst = os.path.join(TARGET, 'yastn_tests', part)
        if os.path.exists(dst):
            shutil.rmtree(dst)
        shutil.copytree(os.path.join(ref, 'tests', part), dst, ignore=shutil.ignore_patterns('__pycache__'))
        print(f'copied the reference {part} tests into {dst}')
    return 0


if __name__ == '__main__':
    if len(sys.argv) < 2:
        print(__doc__)
        sys.exit(2)
    sys.exit(main(*sys.argv[1:]))
