import os
import pathlib
import sys

import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

# launch-shape tuning results of a test run go to a private cache file, not
# the user's (tuning changes speed only; the tests check that too)
if "NUMBA_CELLTREE_GB300_TUNING" not in os.environ:
    import tempfile

    os.environ["NUMBA_CELLTREE_GB300_TUNING"] = os.path.join(tempfile.mkdtemp(prefix="ct_tuning_"), "tuning.json")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libcelltree_gb300.so")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O

    O.build()
    return O


def _cuda_ok() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:  # pragma: no cover
        return False


def pytest_collection_modifyitems(config, items):
    if _cuda_ok():
        return
    skip = pytest.mark.skip(reason="no CUDA GPU in this environment")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)
