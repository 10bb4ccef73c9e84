"""Shared fixtures. Tests marked ``gpu`` need a CUDA device (a GB300); the rest
run on CPU. The oracle (oracle/) is the checker; liblsb.so is the product."""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "distributed-lsb_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden", "reference_lsb16.json")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU; parity tests of the CUDA path")


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<u8").tobytes()).hexdigest()


@pytest.fixture(scope="session")
def golden():
    with open(GOLDEN) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def oracle():
    import oracle as O

    O.build()
    return O


@pytest.fixture(scope="session")
def lsb():
    """The product library, built in-tree and loaded (no fallback)."""
    import lsb_gb300

    lsb_gb300.build()
    lsb_gb300.load()
    return lsb_gb300


@pytest.fixture(scope="session")
def cuda(lsb):
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.init()
    return torch


def to_np(t) -> np.ndarray:
    return t.detach().cpu().numpy().view(np.uint64)


def to_dev(a: np.ndarray, torch):
    return torch.from_numpy(np.ascontiguousarray(a).view(np.int64).copy()).cuda()
