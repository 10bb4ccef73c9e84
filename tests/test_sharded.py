"""The sharded sort's exchange (lsb_gb300.sharded): the reference's block
distribution, one all-gather of digit counts and one element all-to-all per
pass (mpi/mpi_lsbsort.cpp:339-395, :539-588), checked on the CPU against the
stable sort -- every rank simulated in one process, and world sizes 2 and 3
as gloo processes with the oracle as the local step."""
from __future__ import annotations

import os
import socket
import subprocess
import sys

import numpy as np
import pytest

from lsb_gb300 import sharded

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _simulate(oracle, a: np.ndarray, world: int, bits: int) -> np.ndarray:
    """Every rank's local pass, the exchange plans, and the placement, in one process."""
    n = a.shape[0]
    blocks = [a[slice(*sharded.block_range(n, world, r))] for r in range(world)]
    for digit in range(oracle.num_passes(bits)):
        local, counts = [], []
        for b in blocks:
            if b.shape[0]:
                local.append(oracle.global_shuffle(b, digit, bits))
                counts.append(oracle.histogram(b, bits)[digit].astype(np.int64))
            else:
                local.append(b)
                counts.append(np.zeros(1 << bits, dtype=np.int64))
        allc = np.stack(counts)
        plans = [sharded.exchange_plan(allc, n, r) for r in range(world)]
        # the all-to-all: rank r's locally sorted block cut by its send counts
        sent = [np.split(local[r], np.cumsum(plans[r].send_counts)[:-1]) for r in range(world)]
        new = []
        for q in range(world):
            recv = np.concatenate([sent[r][q] for r in range(world)]) if n else a[:0]
            assert [sent[r][q].shape[0] for r in range(world)] == plans[q].recv_counts
            lo, hi = sharded.block_range(n, world, q)
            out = np.empty((hi - lo, 2), dtype=np.uint64)
            pos = plans[q].positions()
            out[pos] = recv
            assert np.array_equal(np.sort(pos), np.arange(hi - lo))
            assert plans[q].piece_dst.shape[0] <= world << bits
            new.append(out)
        blocks = new
    return np.concatenate(blocks)


@pytest.mark.parametrize("world", [1, 2, 3, 5])
@pytest.mark.parametrize("bits", [8, 16])
def test_exchange_simulated(oracle, world, bits):
    for dist, n in ((oracle.DIST_UNIFORM, 20011), (oracle.DIST_ZIPF, 9001), (oracle.DIST_NEARLY_SORTED, 4099),
                    (oracle.DIST_LOW32, 777), (oracle.DIST_EQUAL, 100), (oracle.DIST_UNIFORM, 3),
                    (oracle.DIST_UNIFORM, 0)):
        a = oracle.generate(n, dist, 2)
        assert np.array_equal(_simulate(oracle, a, world, bits), oracle.stable_sort_by_key(a)), (world, bits, dist, n)


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


@pytest.mark.parametrize("world,n,dist,bits", [(2, 30011, 0, 16), (2, 5003, 2, 8), (3, 4097, 4, 16), (3, 2, 0, 8)])
def test_sharded_sort_gloo(oracle, world, n, dist, bits):
    port = _free_port()
    procs = []
    for r in range(world):
        env = dict(os.environ, RANK=str(r), LOCAL_RANK=str(r), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES="")
        procs.append(subprocess.Popen([sys.executable, os.path.join(ROOT, "tests", "_sharded_rank.py"), str(n),
                                       str(dist), str(bits)], cwd=ROOT, env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = []
    try:
        for p in procs:
            out, err = p.communicate(timeout=240)
            outs.append((p.returncode, out, err))
    finally:
        for p in procs:
            if p.poll() is None:
                p.kill()
    for r, (rc, out, err) in enumerate(outs):
        assert rc == 0 and f"rank {r} ok" in out, (r, rc, out, err[-2000:])


def _plan_reference(counts: np.ndarray, n: int, rank: int):
    """The exchange plan restated with numpy (the checker of lsb_exchange_plan):
    send and receive counts, and the received pieces (offset in the received
    array, block-local destination, length) in arrival order."""
    counts = np.asarray(counts, dtype=np.int64)
    world, nbins = counts.shape
    digit_start = np.concatenate(([0], np.cumsum(counts.sum(axis=0))[:-1]))
    rank_off = np.concatenate((np.zeros((1, nbins), np.int64), np.cumsum(counts, axis=0)[:-1]))
    run_start = digit_start[None, :] + rank_off
    blocks = [sharded.block_range(n, world, q) for q in range(world)]

    def pieces(r, q):
        qlo, qhi = blocks[q]
        a = np.maximum(run_start[r], qlo)
        b = np.minimum(run_start[r] + counts[r], qhi)
        keep = b > a
        return a[keep], (b - a)[keep]

    send = [int(pieces(rank, q)[1].sum()) for q in range(world)]
    lo = blocks[rank][0]
    recv, dst, ln = [], [], []
    for r in range(world):
        a, l_ = pieces(r, rank)
        recv.append(int(l_.sum()))
        dst.append(a - lo)
        ln.append(l_)
    dst, ln = np.concatenate(dst), np.concatenate(ln)
    src = np.concatenate(([0], np.cumsum(ln)[:-1])) if ln.size else ln
    return send, recv, src, dst, ln


@pytest.mark.parametrize("world,bits", [(1, 8), (2, 4), (3, 8), (4, 16), (7, 5)])
def test_native_plan_matches_reference(world, bits):
    """lsb_exchange_plan (host code in the library) against the numpy restatement:
    uniform, skewed and empty count tables, block sizes with a remainder."""
    rng = np.random.default_rng(world * 31 + bits)
    for kind in ("uniform", "skewed", "one_digit", "empty"):
        n = 0 if kind == "empty" else 3001 * world + (world - 1)
        counts = np.zeros((world, 1 << bits), dtype=np.int64)
        for r in range(world):
            lo, hi = sharded.block_range(n, world, r)
            m = hi - lo
            if kind == "uniform":
                v = rng.integers(0, 1 << bits, size=m)
            elif kind == "skewed":
                v = np.minimum(rng.zipf(1.5, size=m) - 1, (1 << bits) - 1)
            else:
                v = np.full(m, (1 << bits) // 3)
            counts[r] = np.bincount(v, minlength=1 << bits)
        for q in range(world):
            plan = sharded.exchange_plan(counts, n, q)
            send, recv, src, dst, ln = _plan_reference(counts, n, q)
            assert plan.send_counts == send and plan.recv_counts == recv, (world, bits, kind, q)
            assert np.array_equal(plan.piece_src, src) and np.array_equal(plan.piece_dst, dst), (world, bits, kind, q)
            assert np.array_equal(plan.piece_len, ln), (world, bits, kind, q)


def test_native_plan_rejects_bad_tables():
    """Counts that do not add up to n, negative counts, a rank outside the world."""
    import lsb_gb300 as lsb

    counts = np.array([[3, 1], [2, 2]], dtype=np.int64)
    with pytest.raises(RuntimeError):
        lsb.exchange_plan(counts, 9, 0)
    with pytest.raises(RuntimeError):
        lsb.exchange_plan(np.array([[3, -1], [2, 4]], dtype=np.int64), 8, 0)
    with pytest.raises(RuntimeError):
        lsb.exchange_plan(counts, 8, 2)
