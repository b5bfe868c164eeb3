import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs an sm_103a GPU (run with -m gpu)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O

    O.build()
    return O


@pytest.fixture(scope="session")
def sodlib():
    """The native library, built in-tree (nvcc cross-compiles without a GPU)."""
    from surfaceonlydeformables_gb300 import build as B
    from surfaceonlydeformables_gb300 import _lib

    B.build()
    _lib.load()
    return _lib


@pytest.fixture(scope="session")
def gpu_ctx(sodlib):
    """A library context whose work shares one CUDA stream with torch: library calls with device
    outputs return before their kernels finish (stream-ordered, as for a C++ caller), so torch's
    reads of those outputs (tensor.cpu()) must be ordered after them on the same stream."""
    import torch

    from surfaceonlydeformables_gb300.api import Context

    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    return Context(0, stream=stream)


def rel_fro(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))
