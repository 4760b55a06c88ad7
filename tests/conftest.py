"""Shared test setup: markers, import paths, library builds, common helpers."""
import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(REPO, "naivedynamics.jl_gb300")
for p in (REPO, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the libnaivegpu kernels)")


def _build_all():
    sys.path.insert(0, PKG)
    import build as nd_build  # naivedynamics.jl_gb300/build.py
    nd_build.build()
    from oracle import naiveref
    naiveref.build()


_build_all()


def gpu_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if gpu_available():
        return
    skip = pytest.mark.skip(reason="no CUDA device in this environment")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


def canon(pi, pj, pd):
    """Canonical sorted (min, max, bits(d)) rows of a pair list."""
    pi = np.asarray(pi, np.int64)
    pj = np.asarray(pj, np.int64)
    db = np.asarray(pd, np.float32).view(np.int32).astype(np.int64)
    a = np.minimum(pi, pj)
    b = np.maximum(pi, pj)
    o = np.lexsort((db, b, a))
    return np.stack([a[o], b[o], db[o]], axis=1)


@pytest.fixture(scope="session")
def oracle():
    from oracle import naiveref
    return naiveref


@pytest.fixture(scope="session")
def nd():
    import naivedynamics
    return naivedynamics
