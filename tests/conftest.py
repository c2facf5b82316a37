import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def _have_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


HAVE_GPU = _have_gpu()


def pytest_collection_modifyitems(config, items):
    if HAVE_GPU:
        return
    skip = pytest.mark.skip(reason="no CUDA GPU in this environment")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


@pytest.fixture(scope="session")
def prims():
    """The product: raja_gb300 over libb200prims.so (fails loudly if absent)."""
    import raja_gb300
    raja_gb300.load()
    return raja_gb300


@pytest.fixture(scope="session")
def orc():
    """The oracle (CPU restatement of RAJA seq/omp semantics)."""
    import oracle
    oracle.lib()
    return oracle


_SIGNED = {"uint32": "int32", "uint64": "int64"}


def to_dev(a):
    """numpy array -> contiguous CUDA tensor (unsigned types via a signed view)."""
    import numpy as np
    import torch
    a = np.ascontiguousarray(a)
    if a.dtype.name in _SIGNED:
        t = torch.from_numpy(a.view(_SIGNED[a.dtype.name])).cuda()
        return t.view(getattr(torch, a.dtype.name))
    return torch.from_numpy(a).cuda()


def to_host(t):
    import numpy as np
    import torch
    name = str(t.dtype).replace("torch.", "")
    if name in _SIGNED:
        return t.view(getattr(torch, _SIGNED[name])).cpu().numpy().view(name)
    return t.cpu().numpy()
