"""pytest plugin that runs YASTN's own tensor test suite on this backend.

YASTN's tests select their backend through the command-line options and the
``config_kwargs`` fixture of the reference's root conftest (conftest.py:4-17 of the
reference tree). This plugin offers the same options and fixture, with the extra backend
name ``torch_gb300`` mapped to the ``yastn_gb300.backend`` module (the reference resolves
only 'np', 'torch' and 'torch_cpp' by name). Tests guarded by
``'torch' not in config.getoption('--backend')`` run for it, since it is a torch backend.

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


@pytest.fixture
def config_kwargs(request):
    name = request.config.getoption("--backend")
    backend = name
    if name == "torch_gb300":
        import yastn_gb300
        backend = yastn_gb300.backend
    return {"backend": backend,
            "default_device": request.config.getoption("--device"),
            "default_fusion": request.config.getoption("--default_fusion"),
            "tensordot_policy": request.config.getoption("--tensordot_policy")}
