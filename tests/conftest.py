import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT / "mg-cfd-app-op2_gb300"))
sys.path.insert(0, str(ROOT / "oracle"))
sys.path.insert(0, str(Path(__file__).resolve().parent))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "reference: needs the reference sources (builds oracle/_ref)")


@pytest.fixture(scope="session", autouse=True)
def built():
    """Builds the library, the oracle and (where possible) the reference binary once."""
    from mgcfd import _build
    import recipe as oracle_build  # oracle/recipe.py
    _build.build_library()
    oracle_build.build_oracle()
    oracle_build.build_reference()
    yield


@pytest.fixture(scope="session")
def reference_available():
    import recipe as oracle_build
    return oracle_build.reference_dir() is not None


@pytest.fixture(autouse=True)
def release_plans(request):
    """Per-loop execution plans are cached by map address; device buffers of
    one test may reuse the addresses of another's, so every GPU test ends by
    releasing the plans it built."""
    yield
    if request.node.get_closest_marker("gpu") is None:
        return
    from mgcfd import _lib
    if _lib._LIB is None:
        return
    import torch
    if torch.cuda.is_available():
        _lib.check(_lib._LIB.mgcfd_op_plans_release())
        _lib.check(_lib._LIB.mgcfd_op_plans_mode(1))  # MGCFD_PLANS_AUTO
        _lib.check(_lib._LIB.mgcfd_op_flux_precision(0))  # MGCFD_PRECISION_FP64
