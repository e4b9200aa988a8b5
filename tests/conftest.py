"""Shared test setup: import paths, the gpu marker, builds on demand."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "eom-imsrg_full_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def has_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def gpu_lib():
    """Built and loaded CUDA library (GPU tests only)."""
    import build as pkg_build
    pkg_build.build()
    from imsrg_gpu import api
    return api


@pytest.fixture(scope="session")
def gpu_lib_cpu():
    """The library's Python mirror for host-only entry points (no GPU used)."""
    import build as pkg_build
    pkg_build.build()
    from imsrg_gpu import api
    return api


def make_case(emax, seed=1):
    from imsrg_gpu.layout import Layout, ho_basis
    bas = ho_basis(emax)
    return bas, Layout(**bas)


def rel_err(got, ref):
    scale = max(np.max(np.abs(ref)), 1e-300)
    return float(np.max(np.abs(got - ref)) / scale)


def elem_err(got, ref, tol, floor=1e-14):
    """Element-wise comparison: every element must satisfy
    |got_i - ref_i| <= tol * |ref_i| + floor * max|ref|.
    Returns (worst ratio of |got_i - ref_i| to that bound (<= 1 passes),
    worst relative error |got_i - ref_i| / |ref_i| over the elements with
    |ref_i| >= 1e-6 max|ref|)."""
    got, ref = np.asarray(got, np.float64), np.asarray(ref, np.float64)
    scale = max(float(np.max(np.abs(ref))), 1e-300)
    d = np.abs(got - ref)
    bound = tol * np.abs(ref) + floor * scale
    sig = np.abs(ref) >= 1e-6 * scale
    worst_rel = float(np.max(d[sig] / np.abs(ref[sig]))) if np.any(sig) else 0.0
    return float(np.max(d / bound)), worst_rel
