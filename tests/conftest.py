import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: takes more than a few seconds")


@pytest.fixture(scope="session")
def oracle():
    import ckt_oracle

    ckt_oracle.build()
    return ckt_oracle


@pytest.fixture(scope="session")
def ckt():
    """The CUDA library, built in-tree.  GPU tests fail (not skip) when no
    device is present: there is no fallback path to hide behind."""
    import legionorigins_gb300 as G
    from legionorigins_gb300 import build

    build.build()
    G.lib()
    return G


@pytest.fixture(scope="session")
def cuda(ckt):
    import torch

    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    torch.cuda.init()
    return torch


def same_bits(a, b) -> bool:
    """Bit equality of float arrays where every NaN equals every NaN (NaN
    payloads differ between CPU ISAs and the GPU)."""
    a, b = np.asarray(a), np.asarray(b)
    if a.shape != b.shape:
        return False
    na, nb = np.isnan(a), np.isnan(b)
    if not np.array_equal(na, nb):
        return False
    if a.dtype.kind != "f":
        return np.array_equal(a, b)
    ua = a[~na].view(np.uint32 if a.dtype == np.float32 else np.uint64)
    ub = b[~nb].view(np.uint32 if b.dtype == np.float32 else np.uint64)
    return np.array_equal(ua, ub)


def diff_report(a, b) -> str:
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    na, nb = np.isnan(a), np.isnan(b)
    fin = np.isfinite(a) & np.isfinite(b)
    d = np.abs(a - b)[fin]
    return (f"nan {na.sum()} vs {nb.sum()}, class mismatches {(na != nb).sum()}, "
            f"bit mismatches {(~(a == b) & ~(na & nb)).sum()}, max abs diff {d.max() if d.size else 0}")


def rel_err(a, b, tiny=1e-30):
    """|a-b| / max(|b|, tiny) over elements finite in both."""
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    fin = np.isfinite(a) & np.isfinite(b)
    r = np.abs(a - b)[fin] / np.maximum(np.abs(b[fin]), tiny)
    return r


def load_npz(name):
    return dict(np.load(os.path.join(GOLDEN, name)))
