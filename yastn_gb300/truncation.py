"""Device truncation of a YASTN spectrum tensor (one launch, one device->host copy).

``truncation_mask(S, ...)`` follows the rule of ``yastn/tensor/linalg.py:637-735`` and
returns the boolean mask tensor that YASTN's ``svd_with_truncation`` applies; pass it as
``mask_f=lambda S: yastn_gb300.truncation_mask(S, D_total=...)``. Ties between equal
singular values at the cut are resolved by position (the later entry of the flat
spectrum is kept first), i.e. a stable ordering.
"""
from . import ops


def truncation_mask(S, tol=0, tol_block=0, D_block=float('inf'), D_total=float('inf'),
                    truncate_multiplets=False, **kwargs):
    if not (S.isdiag and S.yastn_dtype == "float64"):
        raise ValueError("truncation_mask requires S to be real and diagonal.")
    nsym = S.config.sym.NSYM
    slices = [sl.slcs[0] for sl in S.slices]
    charges = [tuple(t[:nsym]) for t in S.struct.t]
    mask, _ = ops.truncation_mask_data(S._data.detach(), slices, charges, tol=tol, tol_block=tol_block,
                                       D_block=D_block, D_total=D_total, truncate_multiplets=truncate_multiplets)
    Smask = S.copy()
    Smask._data = mask
    return Smask
