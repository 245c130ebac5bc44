import pathlib
import sys

import pytest

sys.path.insert(0, str(pathlib.Path(__file__).resolve().parent))
import helpers  # noqa: E402,F401  (puts the repo root and the package on sys.path)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the CUDA library)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import ffi
    return ffi.oracle()


@pytest.fixture(scope="session")
def library():
    """The in-tree CUDA library, built if missing (nvcc cross-compiles without a GPU)."""
    import build
    build.build()
    import mpres_gb300
    return mpres_gb300


@pytest.fixture(scope="session")
def gpu(library):
    """The library with every moduli set initialised on cuda:0."""
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test collected without a GPU")
    torch.cuda.init()
    for n in (8, 16, 32):
        library.init(n)
    return library
