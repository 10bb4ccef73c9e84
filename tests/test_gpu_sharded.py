"""The sharded sort with the library's kernels as each rank's local step
(lsb_gb300.sharded.GpuLocalOps) over NCCL, at the one GPU a run here has:
every pass's local lsb_pass + lsb_histogram, count all-gather and element
all-to-all run through the real code, and the result equals the stable sort."""
from __future__ import annotations

import socket

import numpy as np
import pytest

from conftest import to_dev, to_np

pytestmark = pytest.mark.gpu


def test_sharded_sort_one_gpu(lsb, cuda, oracle):
    import torch.distributed as dist

    from lsb_gb300 import sharded

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    dist.init_process_group("nccl", init_method=f"tcp://127.0.0.1:{port}", rank=0, world_size=1)
    try:
        for bits in (8, 16):
            for kind, n in ((oracle.DIST_UNIFORM, 300007), (oracle.DIST_ZIPF, 70001), (oracle.DIST_LOW32, 4097)):
                a = oracle.generate(n, kind, 9)
                out = sharded.sharded_sort(to_dev(a, cuda), n, bits, sharded.GpuLocalOps(lsb, bits), dist)
                assert np.array_equal(to_np(out), oracle.stable_sort_by_key(a)), (bits, kind, n)
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world,bits", [(3, 8), (5, 16)])
def test_place_pieces_matches_positions(lsb, cuda, world, bits):
    """lsb_place_pieces puts every received piece where the plan says, for
    plans of several ranks (pieces of every length, some empty ranks)."""
    from lsb_gb300 import sharded

    rng = np.random.default_rng(world + bits)
    n = 40000 * world + 3
    counts = np.zeros((world, 1 << bits), dtype=np.int64)
    for r in range(world):
        lo, hi = sharded.block_range(n, world, r)
        counts[r] = np.bincount(np.minimum(rng.zipf(1.3, size=hi - lo) - 1, (1 << bits) - 1), minlength=1 << bits)
    for q in range(world):
        plan = sharded.exchange_plan(counts, n, q)
        lo, hi = sharded.block_range(n, world, q)
        total = sum(plan.recv_counts)
        recv = cuda.arange(2 * total, dtype=cuda.int64, device="cuda").reshape(total, 2)
        out = cuda.full((hi - lo, 2), -1, dtype=cuda.int64, device="cuda")
        lsb.place_pieces(recv, out, plan.piece_src, plan.piece_dst, plan.piece_len)
        exp = np.full((hi - lo, 2), -1, dtype=np.int64)
        exp[plan.positions()] = recv.cpu().numpy()
        assert np.array_equal(out.cpu().numpy(), exp), (world, bits, q)


@pytest.mark.parametrize("world", [2, 3, 5])
def test_sharded_ranks_simulated_on_one_gpu(lsb, cuda, oracle, world):
    """Every rank of a sharded sort in one process on this GPU: each rank's
    local lsb_pass and lsb_histogram, the element all-to-all as slicing of the
    locally sorted blocks, and the library's placement kernel. The ranks run
    one after another (nothing waits on another rank's kernel)."""
    from lsb_gb300 import sharded

    for bits, (kind, n) in ((16, (oracle.DIST_UNIFORM, 200003)), (8, (oracle.DIST_ZIPF, 90001)),
                            (16, (oracle.DIST_NEARLY_SORTED, 65537))):
        a = oracle.generate(n, kind, 4)
        blocks = [to_dev(a[slice(*sharded.block_range(n, world, r))], cuda) for r in range(world)]
        ops = sharded.GpuLocalOps(lsb, bits)
        for digit in range(lsb.num_passes(bits)):
            local, counts = zip(*(ops.shuffle(b, digit, bits) for b in blocks))
            table = np.stack(counts)
            plans = [sharded.exchange_plan(table, n, q) for q in range(world)]
            sent = [cuda.split(local[r], plans[r].send_counts) for r in range(world)]
            new = []
            for q in range(world):
                recv = cuda.cat([sent[r][q] for r in range(world)])
                lo, hi = sharded.block_range(n, world, q)
                new.append(ops.place(recv, plans[q], hi - lo))
            blocks = new
        got = np.concatenate([to_np(b) for b in blocks])
        assert np.array_equal(got, oracle.stable_sort_by_key(a)), (world, bits, kind, n)


@pytest.mark.parametrize("ranks,n,bits,skew", [(1, 100003, 16, False), (2, 300007, 16, False),
                                              (3, 200003, 8, True), (5, 65537, 11, False),
                                              (8, 123457, 16, True), (4, 3, 8, False)])
def test_cpp_sharded_sort_simulated_ranks(lsb, ranks, n, bits, skew):
    """lsb_gb300::shardedSort (the C++ layer) with its ranks as host threads of
    one process on this GPU (host/lsb_shard_sim.cpp): the result equals
    std::stable_sort of the whole array, block by block in rank order."""
    import subprocess

    from lsb_gb300 import _build

    cmd = [_build.SHARD_SIM_PATH, "--ranks", str(ranks), "--n", str(n), "--digit-bits", str(bits), "--seed", "7"]
    if skew:
        cmd.append("--skew")
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), (r.returncode, r.stdout, r.stderr)
