"""yastn_gb300 — GB300-native (sm_103a) backend for YASTN's block-sparse tensors.

    import yastn, yastn_gb300
    cfg = yastn.make_config(sym='U1', backend=yastn_gb300.backend, default_device='cuda')

``backend`` is a drop-in for ``yastn.backend.backend_torch``: the hot path
(merge/unmerge, sector GEMMs, block SVD/eigh, masks, their adjoints) runs on
hand-written CUDA kernels in ``libyastn_gb300.so``; build it with
``python yastn_gb300/build.py``. ``truncation_mask`` is a one-launch replacement for
``yastn.linalg.truncation_mask`` usable as ``mask_f``; ``eigs`` is ``yastn.eigs`` with the
hermitian Krylov expansion kept on the device (``yastn_gb300.krylov``);
``double_layer.install()`` runs YASTN's double-layer PEPS contractions as compiled programs;
``save_plans`` / ``load_plans`` write and read the compiled plans of a run (its metadata's
copy, GEMM, SVD records), so that a restarted run does not build them again.
"""
from . import backend_gb300 as backend
from .krylov import eigs
from .truncation import truncation_mask
from . import double_layer
from ._plans import save_cache as save_plans, load_cache as load_plans

__all__ = ['backend', 'eigs', 'truncation_mask', 'double_layer', 'save_plans', 'load_plans']
