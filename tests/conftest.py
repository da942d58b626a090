import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN_DIR = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def reference_checkout():
    """The reference checkout, for the CPU tests that compile its own
    sources (FL_REFERENCE, else its usual location); None when absent."""
    path = os.environ.get("FL_REFERENCE", "/root/reference")
    return path if os.path.isfile(os.path.join(path, "src", "main.cu")) else None


def golden_names():
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN_DIR, "*.npz")))


def load_golden(name):
    with np.load(os.path.join(GOLDEN_DIR, name + ".npz"), allow_pickle=False) as z:
        return {k: (z[k].item() if z[k].ndim == 0 else z[k]) for k in z.files}


def builder():
    """fastload_gb300/_build.py loaded by path (importing the package needs
    the built library)."""
    import importlib.util

    spec = importlib.util.spec_from_file_location("fastload_gb300_build",
                                                  os.path.join(ROOT, "fastload_gb300", "_build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="session")
def built_lib():
    """Builds (if stale) and loads the CUDA library; no GPU needed to load."""
    builder().build_library()
    from fastload_gb300 import _lib

    return _lib.load()


@pytest.fixture(scope="session")
def gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    builder().build_library()
    import fastload_gb300

    return fastload_gb300
