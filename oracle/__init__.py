"""CPU oracle for the block-sparse backend hot path (test infrastructure only).

This package restates, in plain NumPy/SciPy, the reference YASTN NumPy backend
(``yastn/backend/backend_np.py``), the caller-side truncation rule
(``yastn/tensor/linalg.py``) and the reference autograd adjoints
(``yastn/backend/_backend_torch_backwards.py``,
``yastn/backend/linalg/torch_svd_gesdd.py``, ``yastn/backend/linalg/torch_eig_sym.py``).

It checks results and is never the product: only ``tests/``, ``__graft_entry__.smoke()``
and the ``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` may import it.
The GPU backend in ``yastn_gb300`` never calls into this package.

Parity pin: every function here is checked against golden vectors produced by the
reference itself (``tests/golden/make_golden.py`` imports the unmodified reference
and records inputs/outputs of its backend calls); see ``tests/test_oracle_golden.py``.
"""
from .backend_oracle import *  # noqa: F401,F403
