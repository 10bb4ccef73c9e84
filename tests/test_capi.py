"""liblsb.so loads, exports exactly what include/lsb.h declares, and rejects
bad arguments on the host before touching a GPU (no compute calls here)."""
from __future__ import annotations

import ctypes
import os
import re

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "lsb.h")


def declared_functions() -> set[str]:
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return set(re.findall(r"\b(lsb_[a-z0-9_]+)\s*\(", text))


def test_library_exports_every_declared_symbol(lsb):
    L = lsb.load()
    names = declared_functions()
    assert names, "no declarations parsed"
    for name in names:
        assert hasattr(L, name), name
    assert names == set(lsb.SIGNATURES), names ^ set(lsb.SIGNATURES)


def test_version_and_passes(lsb):
    L = lsb.load()
    assert L.lsb_version() == 1
    assert [L.lsb_num_passes(b) for b in (1, 8, 11, 16)] == [64, 8, 6, 4]
    assert L.lsb_num_passes(0) == -1 and L.lsb_num_passes(17) == -1
    assert lsb.status_string(0) == "LSB_OK"
    assert lsb.status_string(6) == "LSB_ERR_DEVICE_TIMEOUT"
    assert lsb.status_string(99) == "LSB_ERR_UNKNOWN"


def P(x):
    return ctypes.c_void_p(x)


def test_host_validation_without_gpu(lsb):
    L = lsb.load()
    a, b = 0x7f0000000000, 0x7f1000000000  # never dereferenced: validation fails first
    null = P(0)
    assert L.lsb_sort_pairs(P(a), P(b), 10, 0, null, 0, null) == lsb.LSB_ERR_INVALID_ARG
    assert L.lsb_sort_pairs(P(a), P(b), 10, 17, null, 0, null) == lsb.LSB_ERR_INVALID_ARG
    assert L.lsb_sort_pairs(P(a), P(b), -1, 16, null, 0, null) == lsb.LSB_ERR_INVALID_ARG
    assert L.lsb_sort_pairs(P(a), P(b), 1 << 32, 16, null, 0, null) == lsb.LSB_ERR_TOO_LARGE
    assert L.lsb_sort_pairs(null, P(b), 10, 16, null, 0, null) == lsb.LSB_ERR_INVALID_ARG
    assert L.lsb_sort_pairs(P(a + 8), P(b), 10, 16, null, 0, null) == lsb.LSB_ERR_ALIGNMENT
    assert L.lsb_sort_pairs(P(a), P(a + 64), 10, 16, null, 0, null) == lsb.LSB_ERR_OVERLAP
    assert L.lsb_pass(P(a), P(b), 10, 16, 4, null, 0, null) == lsb.LSB_ERR_INVALID_ARG
    assert L.lsb_pass(P(a), P(b), 10, 16, -1, null, 0, null) == lsb.LSB_ERR_INVALID_ARG
    assert L.lsb_generate(P(a), 10, 9, 0, null) == lsb.LSB_ERR_INVALID_ARG
    assert L.lsb_generate(P(a + 4), 10, 0, 0, null) == lsb.LSB_ERR_ALIGNMENT
    out = ctypes.c_size_t(0)
    assert L.lsb_workspace_bytes(-1, 16, ctypes.byref(out)) == lsb.LSB_ERR_INVALID_ARG
    assert L.lsb_histogram(P(a), 10, 0, P(b), null) == lsb.LSB_ERR_INVALID_ARG
    # nothing to sort: succeeds without a device
    assert L.lsb_sort_pairs(null, null, 0, 16, null, 0, null) == lsb.LSB_OK
    assert L.lsb_sort_pairs(P(a), P(b), 1, 16, null, 0, null) == lsb.LSB_OK
    # piece placement: every range is checked on the host before any GPU work
    import numpy as np

    src, dst, ln = (np.array(v, dtype=np.int64) for v in ([0, 5], [5, 0], [5, 5]))
    ptrs = [P(t.ctypes.data) for t in (src, dst, ln)]
    ln[1] = 6  # runs past the received array (the valid table is not passed: it would launch)
    assert L.lsb_place_pieces(P(a), 10, P(b), 10, *ptrs, 2, null) == lsb.LSB_ERR_INVALID_ARG
    ln[1], dst[0] = 5, 6  # runs past the block
    assert L.lsb_place_pieces(P(a), 10, P(b), 10, *ptrs, 2, null) == lsb.LSB_ERR_INVALID_ARG
    dst[0] = 5
    assert L.lsb_place_pieces(P(a + 8), 10, P(b), 10, *ptrs, 2, null) == lsb.LSB_ERR_ALIGNMENT
    assert L.lsb_place_pieces(P(a), 10, P(b), 10, *ptrs, 0, null) == lsb.LSB_OK  # no pieces


def test_no_device_reports_status(lsb):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    out = ctypes.c_size_t(0)
    assert lsb.load().lsb_workspace_bytes(1000, 16, ctypes.byref(out)) == lsb.LSB_ERR_NO_DEVICE
    with pytest.raises(lsb.LsbError):
        lsb.workspace_bytes(1000, 16)


def test_driver_command_line_without_gpu(lsb):
    """lsb_sort, the counterpart of the reference's main: --help lists the flags
    and exits 0; a bad --dist value is refused before any GPU work."""
    import subprocess

    from lsb_gb300 import _build

    r = subprocess.run([_build.DRIVER_PATH, "--help"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0
    for flag in ("--n", "--print", "--verify", "--no-verify", "--digit-bits", "--dist", "--per-pass"):
        assert flag in r.stdout, flag
    r = subprocess.run([_build.DRIVER_PATH, "--dist", "bogus"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 2 and "unknown --dist" in r.stderr
    r = subprocess.run([_build.DRIVER_PATH, "--n"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 2 and "missing value" in r.stderr
    # the sharded-sort simulation refuses bad arguments before any GPU work
    for args in (["--ranks", "0"], ["--digit-bits", "17"], ["--bogus"], ["--n"]):
        r = subprocess.run([_build.SHARD_SIM_PATH, *args], capture_output=True, text=True, timeout=60)
        assert r.returncode == 2, (args, r.returncode, r.stderr)
