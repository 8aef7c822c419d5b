"""pytest plugin that runs YASTN's own tensor test suite on this backend.

YASTN's tests select their backend through the command-line options and the
``config_kwargs`` fixture of the reference's root conftest (conftest.py:4-17 of the
reference tree). This plugin offers the same options and fixture, with the extra backend
name ``torch_gb300``: YASTN resolves backends by name ('np', 'torch'), and many of its tests
gate themselves on ``config_kwargs["backend"] == "torch"`` (autograd, fixed-point CTMRG), so
for ``--backend torch_gb300`` the session makes the name 'torch' resolve to this backend
(``yastn.backend.backend_torch`` is bound to ``yastn_gb300.backend``) and the fixture passes
'torch'. Every test that asks for YASTN's torch backend then runs on this one; tests guarded
by ``'torch' not in config.getoption('--backend')`` run too.

With ``--gb300-double-layer`` the PEPS double-layer contractions (``append_vec_*``) run as
``yastn_gb300.double_layer``'s compiled programs (``double_layer.install()``).

Use: ``python -m pytest <YASTN tests/tensor files> -p yastn_suite_plugin --backend
torch_gb300 --device cuda`` with this directory, the package root and the reference install
(baseline/_ref) on PYTHONPATH.
"""
import pytest


def pytest_addoption(parser):
    parser.addoption("--backend", default="torch_gb300", choices=["np", "torch", "torch_gb300"],
                     help="backend of the YASTN tests")
    parser.addoption("--device", default="cuda", help="default device of the tensors")
    parser.addoption("--tensordot_policy", default="fuse_to_matrix",
                     choices=["fuse_to_matrix", "fuse_contracted", "no_fusion"])
    parser.addoption("--default_fusion", default="hard", choices=["hard", "meta"])
    parser.addoption("--quickstart", action="store_true", dest="quickstart", default=False)
    parser.addoption("--long_tests", action="store_true", default=False)
    parser.addoption("--ray", action="store_true", default=False)
    parser.addoption("--gb300-double-layer", action="store_true", default=False,
                     help="run the PEPS double-layer contractions as yastn_gb300's compiled programs")


def pytest_configure(config):
    if config.getoption("--backend") == "torch_gb300":
        import sys
        import yastn.backend
        import yastn_gb300
        sys.modules["yastn.backend.backend_torch"] = yastn_gb300.backend
        yastn.backend.backend_torch = yastn_gb300.backend
    if config.getoption("--gb300-double-layer"):
        from yastn_gb300 import double_layer
        double_layer.install()


def pytest_unconfigure(config):
    """With --gb300-double-layer: the compiled programs' counts of this process go to
    $YB_DOUBLE_LAYER_STATS/<worker>.json (the test that runs the suite sums them)."""
    import os
    out = os.environ.get("YB_DOUBLE_LAYER_STATS")
    if not out or not config.getoption("--gb300-double-layer"):
        return
    import json
    from yastn_gb300 import double_layer
    worker = os.environ.get("PYTEST_XDIST_WORKER", "main")
    with open(os.path.join(out, worker + ".json"), "w") as f:
        json.dump(double_layer.cache_info(), f)


@pytest.fixture
def config_kwargs(request):
    name = request.config.getoption("--backend")
    return {"backend": "torch" if name == "torch_gb300" else name,
            "default_device": request.config.getoption("--device"),
            "default_fusion": request.config.getoption("--default_fusion"),
            "tensordot_policy": request.config.getoption("--tensordot_policy")}
