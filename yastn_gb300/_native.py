"""ctypes binding of ``libyastn_gb300.so`` (the C ABI in ``include/yastn_gb300.h``).

The library is required: importing the GPU ops without it raises immediately, there
is no CPU or pure-PyTorch substitute for the hot path.
"""
import ctypes
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, 'libyastn_gb300.so')
HEADER = os.path.join(os.path.dirname(HERE), 'include', 'yastn_gb300.h')

YB_OK, YB_ERR_INVALID, YB_ERR_CUDA, YB_ERR_NOT_CONVERGED, YB_ERR_TOO_LARGE = 0, 1, 2, 3, 4
YB_F64, YB_C128 = 0, 1

_vp, _i, _i64, _d = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_double

SIGNATURES = {
    'yb_abi_version': ([], _i),
    'yb_last_cuda_error': ([], _i),
    'yb_block_copy': ([_vp, _vp, _i, _vp, _i, _vp, _i, _vp], _i),
    'yb_map_gather': ([_vp, _vp, _i, _vp, _i64, _i, _vp], _i),
    'yb_gemm_reduce': ([_vp, _vp, _i, _vp, _vp, _i, _d, _d, _vp], _i),
    'yb_grouped_gemm': ([_vp, _vp, _vp, _i, _vp, _vp, _vp, _i, _d, _d, _vp], _i),
    'yb_grouped_gemm_short': ([_vp, _vp, _vp, _i, _vp, _vp, _vp, _i, _d, _d, _vp], _i),
    'yb_svd_init': ([_vp, _vp, _vp, _i, _i, _vp, _vp, _vp, _vp], _i),
    'yb_svd_qr': ([_vp, _vp, _vp, _vp, _i, _i, _vp, _vp, _vp, _i, _vp], _i),
    'yb_qr': ([_vp, _vp, _vp, _vp, _vp, _i, _i, _vp, _i, _vp], _i),
    'yb_qr_adjoint_sym': ([_vp, _vp, _i, _i, _vp], _i),
    'yb_trsm_rt': ([_vp, _vp, _vp, _i, _i, _vp], _i),
    'yb_svd_sweeps': ([_vp, _vp, _i, _vp, _i, _i, _i, _i, _i, _d, _vp, _vp], _i),
    'yb_svd_widen': ([_vp, _vp, _vp, _i, _i, _vp, _vp], _i),
    'yb_svd_block_sweeps': ([_vp, _vp, _i, _vp, _i, _i, _i, _i, _i, _i, _i, _d, _i, _vp, _vp], _i),
    'yb_svd_shift_prefill': ([_vp, _vp, _i, _i, _vp, _vp], _i),
    'yb_svd_finalize': ([_vp, _vp, _vp, _vp, _vp, _i, _i, _i, _i, _vp, _vp, _vp, _vp], _i),
    'yb_fill_candidates': ([_vp, _vp, _i, _i, _vp], _i),
    'yb_svd_adjoint_core': ([_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i, _i, _vp], _i),
    'yb_eigh_adjoint_core': ([_vp, _vp, _vp, _vp, _vp, _i, _i, _i, _d, _vp], _i),
    'yb_mask_gather': ([_vp, _vp, _i, _vp, _vp, _i, _vp, _i, _vp], _i),
    'yb_fix_signs': ([_vp, _vp, _vp, _vp, _vp, _vp, _i, _i, _i, _i, _vp], _i),
    'yb_fix_signs_adjoint': ([_vp, _vp, _vp, _vp, _vp, _vp, _vp, _i, _i, _i, _vp], _i),
    'yb_ozaki_split': ([_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i, _i, _vp], _i),
    'yb_ozaki_gemm': ([_vp, _vp, _vp, _vp, _vp, _vp, _vp, _i, _i, _vp], _i),
    'yb_ozaki_gemm_tc': ([_vp, _vp, _vp, _vp, _vp, _vp, _vp, _i, _vp, _i, _i, _i, _vp], _i),
    'yb_ozaki_device_error': ([_vp, _i, _vp], _i),
    'yb_ozaki_dot_static': ([_vp, _vp, _vp, _i, _vp, _vp, _i, _vp, _vp, _i, _vp, _vp, _vp, _i, _i,
                             _i64, _i64, _i64, _i64, _vp], _i),
    'yb_krylov_parts': ([], _i),
    'yb_krylov_dot': ([_vp, _vp, _i64, _i, _vp, _vp, _vp], _i),
    'yb_krylov_update': ([_vp, _vp, _vp, _vp, _vp, _i64, _i, _vp, _vp, _vp], _i),
    'yb_krylov_norm': ([_vp, _i64, _i, _vp, _vp, _vp], _i),
    'yb_krylov_scale': ([_vp, _vp, _i64, _i, _vp, _vp], _i),
    'yb_krylov_combine': ([_vp, _i64, _vp, _i, _i64, _i, _vp, _vp], _i),
    'yb_truncation_mask': ([_vp, _i64, _vp, _vp, _i, _d, _i64, _i, _vp, _vp, _vp], _i),
}


class NativeError(RuntimeError):
    """A yastn_gb300 C entry point returned a non-zero status."""

    def __init__(self, name, status, cuda_error=0):
        self.status = status
        self.cuda_error = cuda_error
        msg = {YB_ERR_INVALID: 'invalid argument', YB_ERR_CUDA: f'CUDA error {cuda_error}',
               YB_ERR_NOT_CONVERGED: 'not converged', YB_ERR_TOO_LARGE: 'problem too large'}.get(status, 'error')
        super().__init__(f"{name} failed: {msg} (status {status})")


_lib = None


def declared_symbols(header=HEADER):
    """Names of the functions declared in the C header."""
    with open(header) as f:
        text = f.read()
    return sorted(set(re.findall(r'^\s*(?:int|void|int64_t)\s+(yb_\w+)\s*\(', text, flags=re.M)))


def lib():
    """The loaded library; raises if it was not built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
                f"or `python yastn_gb300/build.py` (nvcc, sm_103a). yastn_gb300 has no CPU fallback.")
        L = ctypes.CDLL(LIB_PATH)
        for name, (args, res) in SIGNATURES.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
        _lib = L
    return _lib


# number of kernels launched through the library (callers state how many a call enqueues)
LAUNCHES = [0]


def call(name, *args, launches=1):
    """Call an entry point and raise NativeError on a non-zero status."""
    L = lib()
    st = getattr(L, name)(*args)
    if st != YB_OK:
        raise NativeError(name, st, L.yb_last_cuda_error() if st == YB_ERR_CUDA else 0)
    LAUNCHES[0] += launches
    return st
