"""Batched segmented sort (many independent arrays in one launch sequence):
every segment must come out byte-identical to the reference's stable sort of
that segment alone (oracle) and to lsb_sort_pairs on it alone."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import to_dev, to_np

pytestmark = pytest.mark.gpu


def _batch(oracle, sizes, dist, seed):
    parts = [oracle.generate(int(s), dist, seed + i) for i, s in enumerate(sizes)]
    a = np.concatenate(parts) if parts else np.empty((0, 2), dtype=np.uint64)
    off = np.zeros(len(sizes) + 1, dtype=np.int64)
    off[1:] = np.cumsum(sizes)
    return a, off


def _sizes(rng, count, lo_log, hi_log):
    s = np.floor(2.0 ** rng.uniform(lo_log, hi_log, size=count)).astype(np.int64)
    s[::17] = 0  # empty segments
    s[5::23] = 1  # one-element segments
    return s


def _check(oracle, a, off, got):
    for s in range(len(off) - 1):
        seg = a[off[s]:off[s + 1]]
        assert np.array_equal(got[off[s]:off[s + 1]], oracle.stable_sort_by_key(seg)), s


@pytest.mark.parametrize("bits,variant", [(8, 0), (11, 2), (16, 0), (4, 0), (12, 2)])
def test_segmented_matches_oracle(lsb, cuda, oracle, bits, variant):
    rng = np.random.default_rng(bits * 10 + variant)
    sizes = _sizes(rng, 300, 0, 17)
    for dist in (oracle.DIST_UNIFORM, oracle.DIST_ZIPF, oracle.DIST_NEARLY_SORTED):
        a, off = _batch(oracle, sizes, dist, 100)
        A, B = to_dev(a, cuda), cuda.empty((a.shape[0], 2), dtype=cuda.int64, device="cuda")
        offs = cuda.from_numpy(off).cuda()
        t = lsb.Tuning(digit_bits=bits, variant=variant)
        ws = lsb.alloc_segmented_workspace(a.shape[0], len(sizes), bits)
        lsb.sort_segmented(A, B, offs, tuning=t, workspace=ws)
        cuda.cuda.synchronize()
        _check(oracle, a, off, to_np(A))


def test_segmented_equals_plain_sort_per_segment(lsb, cuda, oracle):
    rng = np.random.default_rng(7)
    sizes = _sizes(rng, 40, 10, 20)
    a, off = _batch(oracle, sizes, oracle.DIST_UNIFORM, 3)
    A, B = to_dev(a, cuda), cuda.empty((a.shape[0], 2), dtype=cuda.int64, device="cuda")
    offs = cuda.from_numpy(off).cuda()
    lsb.sort_segmented(A, B, offs)  # library-managed workspace, blocking
    got = to_np(A)
    for s in range(len(sizes)):
        seg = to_dev(a[off[s]:off[s + 1]], cuda)
        if seg.shape[0] == 0:
            continue
        lsb.sort_pairs(seg, cuda.empty_like(seg), 16)
        assert np.array_equal(got[off[s]:off[s + 1]], to_np(seg)), s


def test_segmented_graph_relaunch(lsb, cuda, oracle):
    rng = np.random.default_rng(11)
    sizes = _sizes(rng, 120, 5, 16)
    a, off = _batch(oracle, sizes, oracle.DIST_ZIPF, 9)
    src = to_dev(a, cuda)
    A, B = src.clone(), cuda.empty_like(src)
    offs = cuda.from_numpy(off).cuda()
    t = lsb.Tuning(digit_bits=8, variant=0)
    ws = lsb.alloc_segmented_workspace(a.shape[0], len(sizes), 8)
    g = lsb.SegmentedGraph(A, B, offs, t, ws)
    for _ in range(3):
        A.copy_(src)
        g.launch()
        cuda.cuda.synchronize()
        _check(oracle, a, off, to_np(A))
    g.close()


def test_autotuner_returns_a_candidate(lsb, cuda):
    rng = np.random.default_rng(5)
    sizes = np.floor(2.0 ** rng.uniform(10, 18, size=200)).astype(np.int64)
    off = np.zeros(len(sizes) + 1, dtype=np.int64)
    off[1:] = np.cumsum(sizes)
    t = lsb.tune_segmented(off)
    sms = cuda.cuda.get_device_properties(0).multi_processor_count
    # digit width 8, 11 or 16; kernel shape 0 or 2; all resident CTAs, one per SM or half the SMs
    assert t.digit_bits in (8, 11, 16) and t.variant in (0, 2) and t.ctas in (0, sms, max(1, sms // 2))
    t2 = lsb.tune_segmented(off)  # cached per size class
    assert (t2.digit_bits, t2.variant, t2.ctas) == (t.digit_bits, t.variant, t.ctas)
    # the chosen configuration sorts the batch like the default one
    a = lsb.generate(int(off[-1]), lsb.DIST_UNIFORM, 3)
    A, B = a.clone(), cuda.empty_like(a)
    offs = cuda.from_numpy(off).cuda()
    ws = lsb.alloc_segmented_workspace(int(off[-1]), len(sizes), t.digit_bits)
    lsb.sort_segmented(A, B, offs, t, ws)
    A2 = a.clone()
    lsb.sort_segmented(A2, B, offs, None, lsb.alloc_segmented_workspace(int(off[-1]), len(sizes), 8))
    assert cuda.equal(A, A2)
