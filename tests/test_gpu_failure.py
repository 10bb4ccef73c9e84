"""Failure detection on the GPU without a GPU fault: every device-side wait of
the sort kernels is bounded. The self-test runs the look-back wait on a
predecessor tile that never publishes (a status word nothing sets); the wait
must run out, the kernel must record LSB_ERR_DEVICE_TIMEOUT and return, and
the context must stay usable for the next sort."""
from __future__ import annotations

import time

import numpy as np
import pytest

from conftest import to_dev, to_np

pytestmark = pytest.mark.gpu


def test_lookback_wait_runs_out_and_reports(lsb, cuda, oracle):
    t0 = time.perf_counter()
    status = lsb.selftest_wait_timeout()
    elapsed = time.perf_counter() - t0
    assert status == lsb.LSB_ERR_DEVICE_TIMEOUT
    assert elapsed < 60.0
    # the same process and context sort correctly afterwards
    a = oracle.generate(100003, oracle.DIST_UNIFORM, 77)
    A = to_dev(a, cuda)
    lsb.sort_pairs(A, cuda.empty_like(A), 16)
    assert np.array_equal(to_np(A), oracle.stable_sort_by_key(a))
