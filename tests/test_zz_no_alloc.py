"""lsb_sort_pairs_noalloc: the sort for callers that may not allocate device
memory (a framework that owns all GPU memory through its own arena, a path
that cannot take cudaMalloc's device-wide synchronisation). Its scratch is a
fixed array inside the library, shared by every call and left holding the
last call's contents, so this checks two calls in a row -- the second must
not be disturbed by what the first left behind -- against lsb_sort_pairs,
byte for byte. The file is named to be collected last."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

from conftest import to_dev, to_np

pytestmark = pytest.mark.gpu


def _noalloc(lsb, torch, a: np.ndarray, bits: int) -> np.ndarray:
    A = to_dev(a, torch)
    B = torch.empty_like(A)
    rc = lsb.load().lsb_sort_pairs_noalloc(ctypes.c_void_p(A.data_ptr()), ctypes.c_void_p(B.data_ptr()),
                                           a.shape[0], bits,
                                           ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == lsb.LSB_OK, lsb.status_string(rc)
    return to_np(A)


def _existing(lsb, torch, a: np.ndarray, bits: int) -> np.ndarray:
    A = to_dev(a, torch)
    B = torch.empty_like(A)
    lsb.sort_pairs(A, B, bits)
    return to_np(A)


def test_noalloc_matches_sort_pairs_twice_in_a_row(lsb, cuda, oracle):
    # large enough that the look-back ring wraps (1025 tiles of 8192 elements,
    # more than the fixed scratch's ring slots: slot reuse, completion tags,
    # tile-tagged statuses), and a smaller second call that must not see the
    # first call's ring entries
    cases = [((1 << 23) + 3, oracle.DIST_UNIFORM, 8), (70001, oracle.DIST_ZIPF, 8),
             ((1 << 23) + 3, oracle.DIST_NEARLY_SORTED, 5), (4097, oracle.DIST_LOW32, 8)]
    for call in range(2):
        for n, dist, bits in cases:
            a = oracle.generate(n, dist, seed=100 + call)
            got = _noalloc(lsb, cuda, a, bits)
            assert np.array_equal(got, _existing(lsb, cuda, a, bits)), (call, n, dist, bits)


def test_noalloc_narrow_and_wide_digits(lsb, cuda, oracle):
    # 1-bit digits: 64 passes, the widest pass and tile tags; 4-bit digits;
    # both with more tiles than the fixed scratch's ring slots (4 x grid + 64),
    # so slots are reused within every pass. Then the reference's 16-bit
    # width (and 12, 14), each digit as two half-width sub-passes, against
    # the oracle.
    n = 700 * 8192 + 5
    for call in range(2):
        for bits, dist in ((1, oracle.DIST_UNIFORM), (4, oracle.DIST_ZIPF)):
            a = oracle.generate(n, dist, seed=40 + call)
            assert np.array_equal(_noalloc(lsb, cuda, a, bits), _existing(lsb, cuda, a, bits)), (call, bits)
    for bits, dist, m in ((16, oracle.DIST_UNIFORM, (1 << 22) + 7), (16, oracle.DIST_ZIPF, 300007),
                          (12, oracle.DIST_NEARLY_SORTED, 100003), (14, oracle.DIST_LOW32, 65537)):
        a = oracle.generate(m, dist, seed=bits)
        assert np.array_equal(_noalloc(lsb, cuda, a, bits), oracle.stable_sort_by_key(a)), (bits, dist)


def test_noalloc_rejects_beyond_its_limits(lsb, cuda):
    L = lsb.load()
    A = cuda.empty((1024, 2), dtype=cuda.int64, device="cuda")
    B = cuda.empty_like(A)
    s = ctypes.c_void_p(cuda.cuda.current_stream().cuda_stream)
    pa, pb = ctypes.c_void_p(A.data_ptr()), ctypes.c_void_p(B.data_ptr())
    for bits in (0, 9, 11, 13, 15, 17, 65):
        assert L.lsb_sort_pairs_noalloc(pa, pb, 1024, bits, s) == lsb.LSB_ERR_INVALID_ARG, bits
    assert L.lsb_sort_pairs_noalloc(pa, pb, 1 << 33, 8, s) == lsb.LSB_ERR_TOO_LARGE
    assert L.lsb_sort_pairs_noalloc(pa, pb, -1, 8, s) == lsb.LSB_ERR_INVALID_ARG
    assert L.lsb_sort_pairs_noalloc(pa, pa, 1024, 8, s) == lsb.LSB_ERR_OVERLAP
