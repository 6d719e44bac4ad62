import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libhyperflow_gpu.so")


@pytest.fixture(scope="session")
def oracle():
    import oracle as o
    o.build()
    o.set_species(9)
    return o


@pytest.fixture(scope="session")
def gpu():
    """Context on cuda:0 with the H2_Li mechanism (9 species)."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from hyperflow_gb300 import build
    build.build()
    import hyperflow_gb300 as hf
    return hf.Context("H2_Li")
