import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
# the reference parallelises over output blocks itself (contract.c:288-309)
os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session")
def oracle():
    """CPU restatement of the reference algorithm (the oracle the GPU results
    are compared against)."""
    import oracle.build as ob
    from libxm_gb300 import api
    lib = api.Lib(ob.build_oracle())
    blas = ob.find_blas()
    lib.dll.xmo_set_blas.argtypes = [api.C.c_char_p]
    lib.dll.xmo_set_blas(blas.encode() if blas else None)
    return lib


@pytest.fixture(scope="session")
def reference():
    """The reference libxm compiled from its own sources (only where the
    reference checkout exists)."""
    import oracle.build as ob
    from libxm_gb300 import api
    path = ob.build_reference()
    if path is None:
        pytest.skip("reference sources not present on this machine")
    lib = api.Lib(path)
    blas = ob.find_blas()
    lib.dll.xmref_set_blas.argtypes = [api.C.c_char_p]
    lib.dll.xmref_set_blas(blas.encode() if blas else None)
    return lib


@pytest.fixture(scope="session")
def engine():
    """The GB300 engine library (built in-tree)."""
    import libxm_gb300
    libxm_gb300.build()
    return libxm_gb300.load()
