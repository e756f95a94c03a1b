"""Shared fixtures.  GPU tests carry @pytest.mark.gpu; everything else runs on CPU."""
from __future__ import annotations

import importlib
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

import __graft_entry__ as graft  # noqa: E402


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def pkg():
    """The package, with the CUDA library and the oracle built (build() compiles both)."""
    graft.build()
    return graft.load_package()


@pytest.fixture(scope="session")
def fields(pkg):
    return importlib.import_module("oeb_gb300.fields")


@pytest.fixture(scope="session")
def orc(pkg):
    from oracle import oracle
    return oracle


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a CUDA device")
    return torch.device("cuda:0")


def bits(a: np.ndarray) -> np.ndarray:
    return a.view(np.uint64 if a.dtype == np.float64 else np.uint32)


def assert_bitwise_equal(got: np.ndarray, want: np.ndarray, what: str):
    if got.shape != want.shape:
        raise AssertionError("%s: shape %s != %s" % (what, got.shape, want.shape))
    diff = bits(got) != bits(want)
    if diff.any():
        idx = np.argwhere(diff)
        first = tuple(idx[0])
        raise AssertionError("%s: %d of %d cells differ; first [k,j,i]=%s got %r want %r" %
                             (what, len(idx), diff.size, first, got[first], want[first]))
