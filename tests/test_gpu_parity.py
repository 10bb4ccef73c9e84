"""Parity of the CUDA path (through the C ABI) with the oracle and with the
reference's golden digests, at sizes the oracle finishes in seconds.
Bit-exact: key and value arrays must be byte-identical."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import digest, to_dev, to_np

pytestmark = pytest.mark.gpu

SIZES = [0, 1, 2, 3, 17, 4095, 4096, 4097, 65535, 65537, 300007]
DISTS = [0, 1, 2, 3, 4]


def _sort(lsb, torch, a, bits, workspace=False):
    A = to_dev(a, torch)
    B = torch.empty_like(A)
    ws = lsb.alloc_workspace(a.shape[0], bits) if workspace and a.shape[0] else None
    lsb.sort_pairs(A, B, bits, workspace=ws)
    torch.cuda.synchronize()
    if ws is not None:
        assert lsb.query(ws).device_status == 0
    return to_np(A)


@pytest.mark.parametrize("bits", [8, 11, 16])
def test_sort_matches_oracle(lsb, cuda, oracle, bits):
    for dist in DISTS:
        for n in SIZES:
            a = oracle.generate(n, dist, 7)
            exp = oracle.mysort(a, bits)
            got = _sort(lsb, cuda, a, bits, workspace=(n % 2 == 1))
            assert np.array_equal(got, exp), (bits, dist, n)


@pytest.mark.parametrize("bits", [1, 4, 5, 9, 10, 12, 13, 15])
def test_other_digit_widths(lsb, cuda, oracle, bits):
    for dist in (0, 2, 4):
        a = oracle.generate(70001, dist, 3)
        assert np.array_equal(_sort(lsb, cuda, a, bits), oracle.stable_sort_by_key(a)), (bits, dist)


@pytest.mark.parametrize("variant", ["0", "4"])
@pytest.mark.parametrize("bits", [9, 10, 11])
def test_wide_bin_onesweep(lsb, cuda, oracle, monkeypatch, bits, variant):
    """Digits of 9 to 11 bits, one onesweep pass each: the default kernel
    (per-warp counters of every digit) and the two-step kernel (the tile ranked
    by the low half of the digit, then the high half; variant 4). Sizes at tile
    edges, every distribution (equal keys: one bin per tile; Zipf: a few heavy
    bins), and every single pass."""
    monkeypatch.setenv("LSB_ONESWEEP_VARIANT", variant)
    tile = 8192
    for n in (1, 2, 31, tile - 1, tile, tile + 1, 3 * tile + 17, 40 * tile + 5):
        for dist in DISTS:
            a = oracle.generate(n, dist, n % 13)
            assert np.array_equal(_sort(lsb, cuda, a, bits), oracle.stable_sort_by_key(a)), (bits, n, dist)
    a = oracle.generate(5 * tile + 3, 0, 21)
    src = to_dev(a, cuda)
    for d in range(lsb.num_passes(bits)):
        dst = cuda.empty_like(src)
        lsb.global_shuffle(src, dst, d, bits)
        assert np.array_equal(to_np(dst), oracle.global_shuffle(a, d, bits)), (bits, d)


@pytest.mark.parametrize("bits", [16, 11, 8])
def test_sort_matches_reference_golden(lsb, cuda, oracle, golden, bits):
    for c in golden["cases"]:
        if c["n"] > (1 << 20):
            continue
        a = oracle.generate(c["n"], oracle.DIST_NAMES[c["dist"]], c["seed"])
        assert digest(_sort(lsb, cuda, a, bits, workspace=True)) == c["sorted_sha256"], (c["dist"], c["n"])


def test_pass_matches_reference_golden(lsb, cuda, oracle, golden):
    for c in golden["cases"]:
        if c["n"] > 300007:
            continue
        a = oracle.generate(c["n"], oracle.DIST_NAMES[c["dist"]], c["seed"])
        src = to_dev(a, cuda)
        cur = src.clone()
        for d in range(4):
            dst = cuda.empty_like(src)
            lsb.global_shuffle(src, dst, d, 16)
            assert digest(to_np(dst)) == c["pass_sha256"][d], (c["dist"], c["n"], d)
            assert digest(to_np(src)) == c["input_sha256"]  # source untouched
            nxt = cuda.empty_like(src)
            lsb.global_shuffle(cur, nxt, d, 16)
            cur = nxt
            assert digest(to_np(cur)) == c["after_pass_sha256"][d], (c["dist"], c["n"], d)


@pytest.mark.parametrize("bits", [16, 14, 12])
def test_wide_digit_pass_workspaces(lsb, cuda, oracle, bits):
    """A wide-digit pass gives the same bytes through each of its routes: two
    half-width sub-passes through scratch the library allocates (no
    workspace) or the caller's workspace holds (lsb_pass_workspace_bytes),
    and one task-family pass (a workspace of lsb_workspace_bytes only); the
    source stays untouched. Constant sub-digits included (low32, equal)."""
    import torch

    for dist, n in ((oracle.DIST_UNIFORM, 300007), (oracle.DIST_ZIPF, 100003), (oracle.DIST_LOW32, 65537),
                    (oracle.DIST_EQUAL, 4097), (oracle.DIST_NEARLY_SORTED, 1 << 18)):
        a = oracle.generate(n, dist, 13)
        src = to_dev(a, cuda)
        big = torch.empty(lsb.pass_workspace_bytes(n, bits), dtype=torch.uint8, device="cuda")
        small = lsb.alloc_workspace(n, bits)
        for d in range(oracle.num_passes(bits)):
            exp = oracle.global_shuffle(a, d, bits)
            for ws in (None, big, small):
                dst = cuda.empty_like(src)
                lsb.global_shuffle(src, dst, d, bits, workspace=ws)
                cuda.cuda.synchronize()
                if ws is not None:
                    assert lsb.query(ws).device_status == 0
                assert np.array_equal(to_np(dst), exp), (bits, dist, d, None if ws is None else ws.numel())
            assert np.array_equal(to_np(src), a)


@pytest.mark.parametrize("bits", [8, 11])
def test_pass_matches_oracle(lsb, cuda, oracle, bits):
    for dist in DISTS:
        a = oracle.generate(100003, dist, 9)
        src = to_dev(a, cuda)
        for d in range(oracle.num_passes(bits)):
            dst = cuda.empty_like(src)
            lsb.global_shuffle(src, dst, d, bits)
            assert np.array_equal(to_np(dst), oracle.global_shuffle(a, d, bits)), (dist, d)


def test_skip_plan_and_final_copy(lsb, cuda, oracle):
    n = 50000
    cases = [
        (oracle.DIST_EQUAL, 16, 0, 0b1111),
        (oracle.DIST_LOW32, 16, 2, 0b1100),
        (oracle.DIST_LOW32, 8, 4, 0b11110000),
    ]
    for dist, bits, runs, mask in cases:
        a = oracle.generate(n, dist, 5)
        A, B = to_dev(a, cuda), cuda.empty((n, 2), dtype=cuda.int64, device="cuda")
        ws = lsb.alloc_workspace(n, bits)
        lsb.sort_pairs(A, B, bits, workspace=ws)
        st = lsb.query(ws)
        assert (st.device_status, st.passes_run, st.skipped_mask, st.final_copy) == (0, runs, mask, 0)
        assert np.array_equal(to_np(A), oracle.stable_sort_by_key(a))
    # one non-constant digit: an odd pass count, the result is copied back into A
    for bits in (16, 11, 8):
        a = oracle.generate(n, oracle.DIST_UNIFORM, 6)
        a[:, 0] &= np.uint64((1 << bits) - 1)
        A, B = to_dev(a, cuda), cuda.empty((n, 2), dtype=cuda.int64, device="cuda")
        ws = lsb.alloc_workspace(n, bits)
        lsb.sort_pairs(A, B, bits, workspace=ws)
        st = lsb.query(ws)
        assert st.passes_run == 1
        if bits != 16:  # a split 16-bit digit runs two sub-passes: even, no copy
            assert st.final_copy == 1
        assert np.array_equal(to_np(A), oracle.stable_sort_by_key(a))


def test_workspace_reuse_across_sizes(lsb, cuda, oracle):
    ws = lsb.alloc_workspace(1 << 18, 16)
    for n in (1 << 18, 1000, 1 << 17, 5):
        a = oracle.generate(n, oracle.DIST_ZIPF, n)
        A, B = to_dev(a, cuda), cuda.empty((n, 2), dtype=cuda.int64, device="cuda")
        lsb.sort_pairs(A, B, 16, workspace=ws[: max(256, lsb.workspace_bytes(n, 16))])
        assert np.array_equal(to_np(A), oracle.stable_sort_by_key(a)), n


def test_histogram_matches_oracle(lsb, cuda, oracle):
    for bits in (8, 11, 16):
        for dist in (0, 2, 3):
            a = oracle.generate(123457, dist, 4)
            h = lsb.histogram(to_dev(a, cuda), bits)
            assert np.array_equal(h.cpu().numpy(), oracle.histogram(a, bits)), (bits, dist)


@pytest.mark.parametrize("mode", ["pairs", "quads", "split"])
def test_histogram_b16_forms(lsb, cuda, oracle, monkeypatch, mode):
    """Every form of the 16-bit count: one HBM read by CTA pairs or quads, and
    one read per three digits. Sizes cover a group range with a partial round
    and more groups than the input needs."""
    monkeypatch.setenv("LSB_HIST16", mode)
    for n, dist in ((1, 0), (4097, 1), (1 << 20, 0), (3 * (1 << 20) + 11, 2), (1 << 21, 4)):
        a = oracle.generate(n, dist, 9)
        h = lsb.histogram(to_dev(a, cuda), 16)
        assert np.array_equal(h.cpu().numpy(), oracle.histogram(a, 16)), (mode, n, dist)


def test_device_generator_matches_oracle(lsb, cuda, oracle):
    for dist in DISTS:
        for n in (1, 1000, 100003):
            got = to_np(lsb.generate(n, dist, 77))
            assert np.array_equal(got, oracle.generate(n, dist, 77)), (dist, n)


def test_device_verify(lsb, cuda, oracle):
    a = oracle.generate(200000, oracle.DIST_ZIPF, 8)
    inp = to_dev(a, cuda)
    good = to_dev(oracle.stable_sort_by_key(a), cuda)
    assert lsb.verify(inp, good) == 0
    bad = good.clone()
    bad[[10, 11]] = bad[[11, 10]]  # swap two elements: order or stability broken
    assert lsb.verify(inp, bad) > 0
    dup = good.clone()
    dup[500] = dup[501]
    assert lsb.verify(inp, dup) > 0


def test_host_buffer_entry_point(lsb, cuda, oracle):
    for bits in (16, 8):
        a = oracle.generate(300007, oracle.DIST_UNIFORM, 12)
        h = a.copy()
        lsb.sort_pairs_host(h, bits)
        assert np.array_equal(h, oracle.stable_sort_by_key(a))
        t = cuda.from_numpy(a.view(np.int64).copy()).pin_memory()
        lsb.sort_pairs_host(t, bits)
        assert np.array_equal(t.numpy().view(np.uint64), oracle.stable_sort_by_key(a))


@pytest.mark.parametrize("chunks", [2, 4, 8, 16])
def test_host_buffer_pipeline(lsb, cuda, oracle, monkeypatch, chunks):
    """The chunked host-buffer sort (copies overlapped with chunk sorts, then
    stable merges) equals the stable sort: empty and one-element chunks, ties
    across chunk and slice boundaries (equal keys, Zipf), one to four output
    slices."""
    monkeypatch.setenv("LSB_HOST_CHUNKS", str(chunks))
    for n, dist, bits in ((5, oracle.DIST_UNIFORM, 16), (17, oracle.DIST_EQUAL, 8),
                          (300007, oracle.DIST_ZIPF, 16), (300007, oracle.DIST_EQUAL, 11),
                          ((1 << 21) + 3, oracle.DIST_UNIFORM, 8), ((1 << 21) + 3, oracle.DIST_ZIPF, 13),
                          ((1 << 21) + 3, oracle.DIST_NEARLY_SORTED, 16), ((1 << 22) + 5, oracle.DIST_EQUAL, 16),
                          ((1 << 22) + 5, oracle.DIST_LOW32, 8)):
        a = oracle.generate(n, dist, 21)
        h = a.copy()
        lsb.sort_pairs_host(h, bits)
        assert np.array_equal(h, oracle.stable_sort_by_key(a)), (chunks, n, dist, bits)
    a = oracle.generate(300007, oracle.DIST_LOW32, 5)
    t = cuda.from_numpy(a.view(np.int64).copy()).pin_memory()
    lsb.sort_pairs_host(t, 16)
    assert np.array_equal(t.numpy().view(np.uint64), oracle.stable_sort_by_key(a))


def test_host_buffer_pipeline_default_size(lsb, cuda, oracle, monkeypatch):
    """From 2^25 elements the host-buffer call pipelines by default (8 chunks, 16 slices)."""
    monkeypatch.delenv("LSB_HOST_CHUNKS", raising=False)
    a = oracle.generate((1 << 25) + 11, oracle.DIST_ZIPF, 3)
    t = cuda.from_numpy(a.view(np.int64).copy()).pin_memory()
    lsb.sort_pairs_host(t, 16)
    assert np.array_equal(t.numpy().view(np.uint64), oracle.stable_sort_by_key(a))


@pytest.mark.parametrize("variant", [1, 2, 3])
def test_other_kernel_shapes(lsb, cuda, oracle, monkeypatch, variant):
    """The selectable CTA shapes of the scatter kernel (LSB_ONESWEEP_VARIANT:
    the bulk-copy-load kernels 1 and 3, the two-CTA register kernel 2) sort
    like the default one."""
    monkeypatch.setenv("LSB_ONESWEEP_VARIANT", str(variant))
    for bits in (8, 16, 11, 4):
        for dist, n in ((oracle.DIST_UNIFORM, 300007), (oracle.DIST_ZIPF, 100003), (oracle.DIST_EQUAL, 4097),
                        (oracle.DIST_NEARLY_SORTED, 65537)):
            a = oracle.generate(n, dist, 31)
            assert np.array_equal(_sort(lsb, cuda, a, bits, workspace=True), oracle.stable_sort_by_key(a)), \
                (variant, bits, dist, n)


def test_cpp_driver_runs_and_verifies(lsb, cuda):
    import subprocess

    from lsb_gb300 import _build

    for bits, dist, per_pass in ((16, "uniform", False), (8, "zipf", False), (11, "nearly_sorted", False),
                                 (16, "uniform", True), (12, "zipf", True), (11, "low32", True)):
        extra = ["--per-pass"] if per_pass else []
        r = subprocess.run([_build.DRIVER_PATH, "--n", "300001", "--digit-bits", str(bits), "--dist", dist,
                            "--verify", *extra], capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stdout + r.stderr
        assert "Verification passed" in r.stdout and "Device check: 0 violations" in r.stdout
