"""The oracle (oracle/, a C restatement of mpi/mpi_lsbsort.cpp) pinned against
the reference: golden digests produced by the reference program itself
(tests/golden/make_golden.py) and, where the reference checkout is present,
a live comparison with the reference compiled from its own source."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import digest



def _cases(golden, max_n):
    return [c for c in golden["cases"] if c["n"] <= max_n]


def test_generator_matches_golden_inputs(golden, oracle):
    for c in _cases(golden, 1 << 20):
        a = oracle.generate(c["n"], oracle.DIST_NAMES[c["dist"]], c["seed"])
        assert digest(a) == c["input_sha256"], (c["dist"], c["n"])


def test_mysort_matches_reference_golden(golden, oracle):
    for c in _cases(golden, 1 << 20):
        a = oracle.generate(c["n"], oracle.DIST_NAMES[c["dist"]], c["seed"])
        out = oracle.mysort(a, 16)
        assert digest(out) == c["sorted_sha256"], (c["dist"], c["n"])
        if "sorted" in c:
            exp = np.array([[int(k, 16), v] for k, v in c["sorted"]], dtype=np.uint64).reshape(-1, 2)
            assert np.array_equal(out, exp)


def test_global_shuffle_matches_reference_golden(golden, oracle):
    for c in _cases(golden, 300007):
        a = oracle.generate(c["n"], oracle.DIST_NAMES[c["dist"]], c["seed"])
        cur = a
        for d in range(4):
            assert digest(oracle.global_shuffle(a, d, 16)) == c["pass_sha256"][d], (c["dist"], c["n"], d)
            cur = oracle.global_shuffle(cur, d, 16)
            assert digest(cur) == c["after_pass_sha256"][d], (c["dist"], c["n"], d)


def test_c1_size_matches_reference_golden(golden, oracle):
    """Config: 2^24 uniform elements, 16-bit digits (the reference's own CPU-runnable case)."""
    c = [c for c in golden["cases"] if c["n"] == 1 << 24][0]
    a = oracle.generate(c["n"], oracle.DIST_NAMES[c["dist"]], c["seed"])
    assert digest(oracle.mysort(a, 16, ranks=4, threads=4)) == c["sorted_sha256"]


@pytest.mark.parametrize("bits", [1, 3, 8, 11, 12, 13, 16])
@pytest.mark.parametrize("ranks", [1, 3])
def test_any_digit_width_gives_the_stable_sort(oracle, bits, ranks):
    for dist in range(5):
        a = oracle.generate(5003, dist, seed=11)
        assert np.array_equal(oracle.mysort(a, bits, ranks=ranks, threads=ranks),
                              oracle.stable_sort_by_key(a))


def test_pass_is_stable_sort_by_digit(oracle):
    a = oracle.generate(20000, oracle.DIST_UNIFORM, 5)
    for bits in (8, 11, 16):
        for d in range(oracle.num_passes(bits)):
            out = oracle.global_shuffle(a, d, bits, ranks=2)
            mask = (1 << bits) - 1
            digits = (a[:, 0] >> np.uint64(bits * d)) & np.uint64(mask)
            assert np.array_equal(out, a[np.argsort(digits, kind="stable")])


def test_histogram_counts(oracle):
    a = oracle.generate(10000, oracle.DIST_ZIPF, 2)
    for bits in (8, 11, 16):
        h = oracle.histogram(a, bits)
        for d in range(oracle.num_passes(bits)):
            digits = (a[:, 0] >> np.uint64(bits * d)) & np.uint64((1 << bits) - 1)
            assert np.array_equal(h[d], np.bincount(digits.astype(np.int64), minlength=1 << bits))


def test_zipf_and_distributions_shape(oracle):
    a = oracle.generate(1 << 16, oracle.DIST_ZIPF, 1)
    keys, counts = np.unique(a[:, 0], return_counts=True)
    assert len(keys) < 40000 and counts.max() > 3000  # heavy duplicates (top rank ~ 9.5%)
    lo = oracle.generate(1000, oracle.DIST_LOW32, 1)
    assert int(lo[:, 0].max()) < (1 << 32)
    eq = oracle.generate(1000, oracle.DIST_EQUAL, 1)
    assert len(np.unique(eq[:, 0])) == 1
    ns = oracle.generate(1000, oracle.DIST_NEARLY_SORTED, 1)
    i = np.arange(1000, dtype=np.uint64)
    assert np.array_equal(ns[:, 0], i ^ (i >> np.uint64(3)))
    assert np.array_equal(a[:, 1], np.arange(1 << 16, dtype=np.uint64))


def test_oracle_against_live_reference(oracle):
    if not oracle.ref_available():
        pytest.skip("reference build not present (needs the reference checkout)")
    for dist in range(5):
        for n in (0, 1, 2, 9, 4097, 70001):
            a = oracle.generate(n, dist, 123)
            assert np.array_equal(oracle.mysort(a, 16, ranks=2, threads=2), oracle.ref_mysort(a))
            for d in range(4):
                assert np.array_equal(oracle.global_shuffle(a, d, 16, ranks=3), oracle.ref_global_shuffle(a, d))
