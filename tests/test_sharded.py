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


@pytest.mark.parametrize("world,bits", [(1, 8), (3, 8), (4, 16)])
def test_piece_placement_expands_like_positions(world, bits):
    """GpuLocalOps.place (piece table expanded with tensor ops, here on the
    CPU) puts every received element where the plan's positions say."""
    import torch

    rng = np.random.default_rng(world * 100 + bits)
    n = 5000 + world
    counts = np.zeros((world, 1 << bits), dtype=np.int64)
    for r in range(world):
        lo, hi = sharded.block_range(n, world, r)
        counts[r] = np.bincount(rng.integers(0, 1 << bits, size=hi - lo), minlength=1 << bits)
    ops = sharded.GpuLocalOps(None, bits)
    for q in range(world):
        plan = sharded.exchange_plan(counts, n, q)
        lo, hi = sharded.block_range(n, world, q)
        total = sum(plan.recv_counts)
        recv = torch.arange(2 * total, dtype=torch.int64).reshape(total, 2)
        got = ops.place(recv, plan, hi - lo).numpy()
        exp = np.empty((hi - lo, 2), dtype=np.int64)
        exp[plan.positions()] = recv.numpy()
        assert np.array_equal(got, exp), (world, bits, q)
