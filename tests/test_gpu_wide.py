"""Parity of the one-pass 16-bit digit family (csrc/lsb_wide.cu) with the
oracle, bit-exact: chunk and chunk-slot boundaries, buckets that need several
tiles inside one chunk, buckets that are empty in many chunks, the single
pass (globalShuffle at the reference's 16-bit width), the byte-packed digit
counters' carry repairs, and the split form kept behind LSB_WIDE_DIGITS."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import to_dev, to_np

pytestmark = pytest.mark.gpu

TILE = 8192  # elements per A tile of the wide kernel


@pytest.fixture(autouse=True)
def wide_family(monkeypatch):
    """16-bit digits through the one-pass family in every test of this file."""
    monkeypatch.setenv("LSB_WIDE_DIGITS", "wide")


def _sort(lsb, torch, a, bits=16):
    A = to_dev(a, torch)
    B = torch.empty_like(A)
    ws = lsb.alloc_workspace(a.shape[0], bits) if a.shape[0] else None
    lsb.sort_pairs(A, B, bits, workspace=ws)
    torch.cuda.synchronize()
    if ws is not None:
        assert lsb.query(ws).device_status == 0
    return to_np(A)


def _keys(keys: np.ndarray) -> np.ndarray:
    a = np.empty((keys.shape[0], 2), dtype=np.uint64)
    a[:, 0] = keys
    a[:, 1] = np.arange(keys.shape[0], dtype=np.uint64)
    return a


@pytest.mark.parametrize("tiles,slots", [(4, 2), (8, 3), (128, 3)])
def test_wide_chunk_geometry(lsb, cuda, oracle, monkeypatch, tiles, slots):
    """Sizes at tile and chunk edges, several reuses of every chunk slot."""
    monkeypatch.setenv("LSB_WIDE_CHUNK_TILES", str(tiles))
    monkeypatch.setenv("LSB_WIDE_SLOTS", str(slots))
    chunk = tiles * TILE
    sizes = [2, 3, TILE - 1, TILE, TILE + 1, chunk - 1, chunk, chunk + 1, 3 * chunk + 5]
    if tiles < 128:
        sizes.append(9 * chunk + TILE // 2 + 7)
    for n in sizes:
        for dist in (oracle.DIST_UNIFORM, oracle.DIST_ZIPF, oracle.DIST_NEARLY_SORTED, oracle.DIST_LOW32):
            a = oracle.generate(n, dist, n % 97)
            assert np.array_equal(_sort(lsb, cuda, a), oracle.stable_sort_by_key(a)), (tiles, slots, n, dist)


def test_wide_multi_tile_buckets(lsb, cuda, oracle, monkeypatch):
    """Buckets with far more than one tile of elements in a chunk: the tiles of
    a bucket resolve their offsets by look-back among themselves."""
    monkeypatch.setenv("LSB_WIDE_CHUNK_TILES", "16")
    rng = np.random.default_rng(5)
    n = 40 * TILE + 123
    # few distinct high bytes per digit, many low bytes: big buckets, long runs
    k = rng.integers(0, 1 << 63, size=n, dtype=np.uint64)
    k &= np.uint64(0x0300_FFFF_03FF_0001)
    a = _keys(k)
    assert np.array_equal(_sort(lsb, cuda, a), oracle.stable_sort_by_key(a))
    # one bucket only in every digit (high bytes all equal, low bytes vary)
    a = _keys(rng.integers(0, 1 << 63, size=n, dtype=np.uint64) & np.uint64(0x00FF_00FF_00FF_00FF))
    assert np.array_equal(_sort(lsb, cuda, a), oracle.stable_sort_by_key(a))


def test_wide_buckets_empty_in_some_chunks(lsb, cuda, oracle, monkeypatch):
    """A bucket's running prefix is handed on across chunks where it is empty."""
    monkeypatch.setenv("LSB_WIDE_CHUNK_TILES", "4")
    chunk = 4 * TILE
    rng = np.random.default_rng(11)
    n = 13 * chunk + 77
    i = np.arange(n, dtype=np.uint64)
    low = rng.integers(0, 1 << 63, size=n, dtype=np.uint64) & np.uint64(0x0000_0000_00FF_FFFF)
    # digit 1's high byte: bucket (chunk % 3) only, and bucket 200 in chunks 2 and 9
    hi = ((i // np.uint64(chunk)) % np.uint64(3)) << np.uint64(24)
    k = low | hi
    sel = ((i // np.uint64(chunk)) == 2) | ((i // np.uint64(chunk)) == 9)
    k[sel] = (k[sel] & np.uint64(0x00FF_FFFF)) | np.uint64(200 << 24)
    a = _keys(k)
    assert np.array_equal(_sort(lsb, cuda, a), oracle.stable_sort_by_key(a))


@pytest.mark.parametrize("tiles", [4, 128])
def test_wide_single_pass(lsb, cuda, oracle, monkeypatch, tiles):
    """lsb_pass at 16-bit digits (one globalShuffle) is one wide pass."""
    monkeypatch.setenv("LSB_WIDE_CHUNK_TILES", str(tiles))
    for dist in (oracle.DIST_UNIFORM, oracle.DIST_ZIPF, oracle.DIST_NEARLY_SORTED, oracle.DIST_EQUAL):
        a = oracle.generate(5 * tiles * TILE + 3, dist, 17)
        src = to_dev(a, cuda)
        for d in range(4):
            dst = cuda.empty_like(src)
            lsb.global_shuffle(src, dst, d, 16)
            assert np.array_equal(to_np(dst), oracle.global_shuffle(a, d, 16)), (tiles, dist, d)
            assert np.array_equal(to_np(src), a)


def test_wide_histogram_carries(lsb, cuda, oracle):
    """Counts of 16-bit digits held as four bytes per word: digits that share
    a word and overflow their bytes many times (carries into the neighbours)."""
    rng = np.random.default_rng(3)
    n = (1 << 22) + 9
    for span in (1, 2, 4, 6):
        d = rng.integers(0, span, size=n, dtype=np.uint64)
        k = d | (d << np.uint64(17)) | ((d + np.uint64(250)) << np.uint64(32)) | (d << np.uint64(61))
        a = _keys(k)
        h = lsb.histogram(to_dev(a, cuda), 16)
        assert np.array_equal(h.cpu().numpy(), oracle.histogram(a, 16)), span


def test_wide_and_split_agree(lsb, cuda, oracle, monkeypatch):
    """The split form (two 8-bit sub-passes per 16-bit digit) stays selectable
    and gives the same bytes."""
    for mode in ("split", "wide"):
        monkeypatch.setenv("LSB_WIDE_DIGITS", mode)
        for dist, n in ((oracle.DIST_UNIFORM, 1 << 20), (oracle.DIST_ZIPF, 300007), (oracle.DIST_LOW32, 65537)):
            a = oracle.generate(n, dist, 23)
            assert np.array_equal(_sort(lsb, cuda, a), oracle.stable_sort_by_key(a)), (mode, dist, n)
