import importlib
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

DATA_C3 = os.path.join(ROOT, "data", "water_ti_bone")
DATA_WLB = os.path.join(ROOT, "data", "water_lung_bone")
GOLDEN = os.path.join(ROOT, "tests", "golden", "golden_water_ti_bone.npz")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def dpm():
    return importlib.import_module("dpm-g4cpp_gb300")


@pytest.fixture(scope="session")
def orc():
    m = importlib.import_module("cpu_oracle")
    m.build()
    return m


@pytest.fixture(scope="session")
def golden():
    return np.load(GOLDEN)


@pytest.fixture(scope="session")
def oracle_c3(orc):
    return orc.Oracle(DATA_C3)


@pytest.fixture(scope="session")
def oracle_wlb(orc):
    return orc.Oracle(DATA_WLB)


@pytest.fixture(scope="session")
def gpu_lib(dpm):
    """The CUDA library on a GPU; fails (does not skip) when the library is missing."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    builder = importlib.import_module("dpm-g4cpp_gb300.builder")
    builder.build()
    return dpm.library()


@pytest.fixture(scope="session")
def tables_c3(dpm, gpu_lib):
    return dpm.Tables(DATA_C3)


@pytest.fixture(scope="session")
def tables_wlb(dpm, gpu_lib):
    return dpm.Tables(DATA_WLB)
