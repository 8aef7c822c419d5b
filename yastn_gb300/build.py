"""Build the in-tree CUDA library ``libyastn_gb300.so`` for sm_103a with nvcc.

Each ``csrc/*.cu`` translation unit is compiled in parallel to an object file, then
linked into one shared library next to this file. No CMake, no torch extension
machinery: the library exposes only the C ABI declared in ``include/yastn_gb300.h``.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, 'csrc')
BUILD = os.path.join(HERE, '_build')
LIB = os.path.join(HERE, 'libyastn_gb300.so')
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
FLAGS = ['-O3', '-lineinfo', '-std=c++17', '-Xcompiler', '-fPIC', '--expt-relaxed-constexpr']


def nvcc():
    exe = shutil.which('nvcc')
    if exe is None:
        cand = '/usr/local/cuda/bin/nvcc'
        if os.path.exists(cand):
            return cand
        raise RuntimeError('nvcc not found: the CUDA 13 toolkit is required to build yastn_gb300')
    return exe


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith('.cu'))


def _compile(src, extra):
    obj = os.path.join(BUILD, os.path.basename(src)[:-3] + '.o')
    cmd = [nvcc()] + ARCH + FLAGS + extra + ['-c', src, '-o', obj]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{res.stderr}")
    return obj, res.stderr


def build(verbose=False, extra=()):
    """Compile every csrc/*.cu and link libyastn_gb300.so; returns the library path."""
    os.makedirs(BUILD, exist_ok=True)
    srcs = sources()
    with ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 4))) as ex:
        results = list(ex.map(lambda s: _compile(s, list(extra)), srcs))
    objs = [o for o, _ in results]
    if verbose:
        for _, err in results:
            if err.strip():
                print(err, file=sys.stderr)
    tmp = LIB + '.tmp'
    cmd = [nvcc()] + ARCH + ['-shared', '-Xcompiler', '-fPIC', '-o', tmp] + objs
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == '__main__':
    print(build(verbose='-v' in sys.argv, extra=['-Xptxas', '-v'] if '-v' in sys.argv else []))
