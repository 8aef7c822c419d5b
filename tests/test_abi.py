"""The C-ABI library: built, loadable without a GPU, exporting every declared symbol,
and rejecting invalid arguments on the host before touching the device."""
import ctypes
import os

import pytest

from yastn_gb300 import _native as N


@pytest.fixture(scope='module')
def lib():
    if not os.path.exists(N.LIB_PATH):
        from yastn_gb300 import build
        build.build()
    return N.lib()


def test_header_declares_entry_points():
    names = N.declared_symbols()
    for must in ('yb_block_copy', 'yb_grouped_gemm', 'yb_svd_init', 'yb_svd_sweeps', 'yb_svd_widen', 'yb_svd_finalize',
                 'yb_svd_adjoint_core', 'yb_mask_gather', 'yb_fix_signs', 'yb_truncation_mask'):
        assert must in names


def test_library_exports_every_declared_symbol(lib):
    for name in N.declared_symbols():
        assert hasattr(lib, name), f"{name} declared in include/yastn_gb300.h but not exported"
        assert name in N.SIGNATURES, f"{name} has no ctypes signature"


def test_abi_version(lib):
    assert lib.yb_abi_version() == 100


def test_invalid_arguments_are_rejected_on_host(lib):
    null = ctypes.c_void_p(0)
    assert lib.yb_block_copy(null, null, 8, null, 1, null, 1, null) == N.YB_ERR_INVALID
    assert lib.yb_block_copy(null, null, 8, null, 0, null, 0, null) == N.YB_OK  # nothing to do
    assert lib.yb_grouped_gemm(null, null, null, 0, null, null, null, 3, 1.0, 0.0, null) == N.YB_ERR_INVALID
    assert lib.yb_svd_init(null, null, null, 2, 7, null, null, null, null) == N.YB_ERR_INVALID  # unknown dtype
    assert lib.yb_svd_init(null, null, null, 2, N.YB_C128, null, null, null, null) == N.YB_ERR_INVALID  # null data
    assert lib.yb_svd_sweeps(null, null, 1, null, 1, 1, 32, 7, 1, 0.0, null, null) == N.YB_ERR_INVALID
    assert lib.yb_svd_widen(null, null, null, 1, N.YB_F64, null, null) == N.YB_ERR_INVALID
    assert lib.yb_svd_block_sweeps(null, null, 1, null, 1, 1, 16, 32, N.YB_F64, 1, 1, 0.0, 0, null, null) == \
        N.YB_ERR_INVALID
    assert lib.yb_svd_qr(null, null, null, null, 1, N.YB_F64, null, null, null, 8, null) == N.YB_ERR_INVALID
    assert lib.yb_gemm_reduce(null, null, N.YB_F64, null, null, 1, 1.0, 0.0, null) == N.YB_ERR_INVALID
    assert lib.yb_qr(null, null, null, null, null, 1, N.YB_F64, null, 8, null) == N.YB_ERR_INVALID
    assert lib.yb_qr_adjoint_sym(null, null, 1, N.YB_F64, null) == N.YB_ERR_INVALID
    assert lib.yb_trsm_rt(null, null, null, 1, N.YB_C128, null) == N.YB_ERR_INVALID
    assert lib.yb_svd_finalize(null, null, null, null, null, 1, 0, 10000, 0, null, null, null, null) == N.YB_ERR_TOO_LARGE
    assert lib.yb_svd_finalize(null, null, null, null, null, 1, 0, 10, 1, null, null, null, null) == N.YB_ERR_INVALID
    assert lib.yb_truncation_mask(null, 20000, null, null, 1, 0.0, -1, 0, null, null, null) == N.YB_ERR_TOO_LARGE
    assert lib.yb_fix_signs(null, null, null, null, null, null, 1, 4, 0, 0, null) == N.YB_ERR_INVALID
    assert lib.yb_mask_gather(null, null, 8, null, null, 2, null, 0, null) == N.YB_ERR_INVALID
    # composed copies: null pointers, an unknown dtype, a misaligned complex128 pointer
    fake = ctypes.c_void_p(0x100000)
    assert lib.yb_map_gather(null, null, N.YB_F64, null, 5, 0, null) == N.YB_ERR_INVALID
    assert lib.yb_map_gather(fake, fake, 7, fake, 5, 0, null) == N.YB_ERR_INVALID
    assert lib.yb_map_gather(ctypes.c_void_p(0x100008), fake, N.YB_C128, fake, 5, 1, null) == N.YB_ERR_INVALID
    assert lib.yb_map_gather(null, null, N.YB_F64, null, 0, 0, null) == N.YB_OK  # nothing to do
    # the tcgen05 emulated GEMM takes 128 x 64 or 128 x 32 tiles only
    assert lib.yb_ozaki_gemm_tc(fake, fake, fake, fake, fake, fake, fake, 1, null, 0, 48, 8, null) == N.YB_ERR_INVALID
    assert lib.yb_ozaki_gemm_tc(null, null, null, null, null, null, null, 1, null, 0, 32, 8, null) == N.YB_ERR_INVALID


def test_backend_module_surface():
    """Every name of the reference torch backend's __all__ (backend_torch.py:32-49)."""
    from yastn_gb300 import backend
    ref_all = ['DTYPE', 'absolute', 'add', 'allclose', 'apply_mask', 'argsort', 'bitwise_not', 'checkpoint', 'clone',
               'conj', 'copy', 'cuda_is_available', 'delete', 'detach', 'detach_', 'diag_1dto2d', 'diag_2dto1d',
               'diag_create', 'diag_get', 'dot', 'dot_diag', 'eig', 'eigh', 'eigh_lowrank', 'eigs_which', 'eigvals',
               'embed_mask', 'entropy', 'exp', 'expm', 'first_element', 'fix_svd_signs', 'get_device', 'get_dtype',
               'get_shape', 'get_size', 'get_yastn_dtype', 'grad', 'imag', 'insert', 'is_complex', 'is_independent',
               'item', 'max_abs', 'maximum', 'merge_super_blocks', 'merge_to_dense', 'move_to', 'negate_blocks',
               'norm', 'norm_matrix', 'nvtx', 'ones', 'permute_dims', 'pinv', 'qr', 'rand', 'randint', 'random_seed',
               'real', 'reciprocal', 'requires_grad', 'requires_grad_', 'rsqrt', 'sqrt', 'square_matrix_from_dict',
               'sub', 'sum_elements', 'svd', 'svd_lowrank', 'svd_randomized', 'svds_scipy', 'svdvals', 'to_mask',
               'to_numpy', 'to_tensor', 'trace', 'transpose', 'transpose_and_merge', 'transpose_dot_sum', 'unmerge',
               'vdot', 'zeros']
    missing = [n for n in ref_all if not hasattr(backend, n)]
    assert not missing
    assert 'torch' in backend.BACKEND_ID and backend.BACKEND_ID != 'torch_cpp'


def test_ops_refuse_cpu_tensors():
    import torch
    from yastn_gb300 import ops
    with pytest.raises(TypeError):
        ops.merge(torch.zeros(4, dtype=torch.float64), (0,), (), (), 4)
