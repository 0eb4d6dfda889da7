"""Shared test configuration.

Tests marked ``gpu`` need a CUDA device and the compiled library
(hcore_gb300/_lib/libhcore_gb300.so); the rest run on any machine.  The
oracle (oracle/, a CPU restatement of the reference) is built on demand.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the compiled hcore_gb300 library")


def _cuda_available() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if _cuda_available():
        return
    skip = pytest.mark.skip(reason="no CUDA device on this machine")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


@pytest.fixture(scope="session")
def port():
    from oracle import oracle as O

    return O.Port()


@pytest.fixture(scope="session")
def golden():
    import json

    import numpy as np

    d = os.path.join(ROOT, "tests", "golden")
    with open(os.path.join(d, "golden_meta.json")) as f:
        meta = json.load(f)
    arrs = dict(np.load(os.path.join(d, "golden_small.npz")))
    return meta, arrs


@pytest.fixture(scope="session")
def golden_tlr():
    """Reference outputs of HCORE_duncompress / dgemmbdcd / dtrsm / dpotrf."""
    import json

    import numpy as np

    d = os.path.join(ROOT, "tests", "golden")
    with open(os.path.join(d, "golden_tlr_meta.json")) as f:
        meta = json.load(f)
    return meta, dict(np.load(os.path.join(d, "golden_tlr.npz")))


@pytest.fixture(scope="session")
def golden_compress():
    """Reference outputs of the tests' compressor (generate_compress)."""
    import json

    import numpy as np

    d = os.path.join(ROOT, "tests", "golden")
    with open(os.path.join(d, "golden_compress_meta.json")) as f:
        meta = json.load(f)
    return meta, dict(np.load(os.path.join(d, "golden_compress.npz")))


@pytest.fixture(scope="session")
def golden_zgemm():
    """Reference outputs of HCORE_zgemm."""
    import json

    import numpy as np

    d = os.path.join(ROOT, "tests", "golden")
    with open(os.path.join(d, "golden_zgemm_meta.json")) as f:
        meta = json.load(f)
    return meta, dict(np.load(os.path.join(d, "golden_zgemm.npz")))


@pytest.fixture(scope="session")
def hc():
    """The GPU library, built if absent (the GPU machine builds it via build())."""
    import hcore_gb300
    from hcore_gb300 import build

    if not os.path.exists(build.LIB):
        build.build()
    hcore_gb300.lib()
    return hcore_gb300
