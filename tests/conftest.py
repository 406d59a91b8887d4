import importlib
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, 'tests', 'golden')


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and libniq.so")


@pytest.fixture(scope='session')
def niq():
    return importlib.import_module('neural-implicit-queries_gb300')


@pytest.fixture(scope='session')
def R():
    from oracle import ref_np
    return ref_np


def golden(name):
    return dict(np.load(os.path.join(GOLDEN, name)))


def model_from(g, prefix):
    """Rebuild a params dict stored under ``prefix/`` in a golden file."""
    p = prefix + '/'
    return {k[len(p):]: v for k, v in g.items() if k.startswith(p)}


@pytest.fixture(scope='session')
def gpu_ready(niq):
    """Skip-free guard for gpu tests: the library must load and a device must exist."""
    import torch
    assert torch.cuda.is_available(), "gpu test without a CUDA device"
    from importlib import import_module
    lib = import_module('neural-implicit-queries_gb300._lib')
    lib.load()
    return True
