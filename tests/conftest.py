import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300 / sm_103a)")


@pytest.fixture(scope="session")
def kifi_lib():
    """libkifi_gpu.so, built in-tree on first use."""
    from merge_fusion_gb300 import _lib, build
    build.build()
    return _lib.load()


@pytest.fixture(scope="session")
def oracle_cpu():
    import oracle
    from oracle import cpu
    oracle.build_oracle()
    return cpu


@pytest.fixture(scope="session")
def oracle_ref():
    from oracle import build_ref, ref
    build_ref.build()
    if not ref.available():
        pytest.skip("reference CPU build not available")
    return ref


@pytest.fixture(scope="session")
def golden():
    import json
    import numpy as np
    with open(os.path.join(GOLDEN, "golden.json")) as f:
        g = json.load(f)
    frame = np.load(os.path.join(GOLDEN, "imrod_v2_frame0.npz"))
    g["depth"] = frame["depth"]
    g["view"] = frame["view"]
    g["camera"] = tuple(g["camera"])
    return g


@pytest.fixture(scope="session")
def gpu(kifi_lib):
    from merge_fusion_gb300 import _lib
    if _lib.device_count() == 0:
        pytest.fail("test marked gpu but no CUDA device is visible")
    return kifi_lib
