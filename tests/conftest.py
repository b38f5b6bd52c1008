import importlib.util
import json
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "temp-cat-blst_gb300")
GOLDEN = os.path.join(ROOT, "tests", "golden", "golden.json")

sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a)")
    config.addinivalue_line("markers", "slow: large-size case")


def _load_module(name, path):
    spec = importlib.util.spec_from_file_location(name, path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="session")
def golden():
    with open(GOLDEN) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def oracle():
    import oracle as om
    om.build()
    return om.Oracle()


@pytest.fixture(scope="session")
def synth():
    return _load_module("catmsm_synth", os.path.join(PKG, "synth.py"))


@pytest.fixture(scope="session")
def gpu_binding():
    return _load_module("catmsm_blst_gpu", os.path.join(PKG, "blst_gpu.py"))


@pytest.fixture(scope="session")
def gpu(gpu_binding):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    gpu_binding.load()
    return gpu_binding
