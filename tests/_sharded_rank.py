"""One rank of the sharded sort over gloo on the CPU (run by test_sharded.py):
the exchange of lsb_gb300.sharded with the oracle as the per-rank local step.
Prints "rank R ok" when the gathered result equals the stable sort."""
from __future__ import annotations

import os
import sys

import numpy as np
import torch
import torch.distributed as dist

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "distributed-lsb_gb300")):
    sys.path.insert(0, p)

import oracle  # noqa: E402
from lsb_gb300 import sharded  # noqa: E402


class OracleLocalOps(sharded.LocalOps):
    def shuffle(self, block, digit, bits):
        a = block.numpy().view(np.uint64)
        if a.shape[0] == 0:
            return block.clone(), np.zeros(1 << bits, dtype=np.int64)
        out = oracle.global_shuffle(a, digit, bits)
        return torch.from_numpy(out.view(np.int64).copy()), oracle.histogram(a, bits)[digit].astype(np.int64)

    def place(self, received, plan, size):
        out = torch.empty((size, 2), dtype=torch.int64)
        out[torch.from_numpy(plan.positions())] = received
        return out


def main():
    n, dist_kind, bits = int(sys.argv[1]), int(sys.argv[2]), int(sys.argv[3])
    dist.init_process_group("gloo")
    world, rank = dist.get_world_size(), dist.get_rank()
    a = oracle.generate(n, dist_kind, 5)
    lo, hi = sharded.block_range(n, world, rank)
    block = torch.from_numpy(a[lo:hi].view(np.int64).copy())
    out = sharded.sharded_sort(block, n, bits, OracleLocalOps(), dist)
    sizes = [sharded.block_range(n, world, r)[1] - sharded.block_range(n, world, r)[0] for r in range(world)]
    # gloo gathers equal sizes: pad every block to the largest
    m = max(sizes)
    padded = torch.zeros((m, 2), dtype=torch.int64)
    padded[: out.shape[0]] = out
    parts = [torch.empty((m, 2), dtype=torch.int64) for _ in sizes]
    dist.all_gather(parts, padded)
    got = torch.cat([p[:s] for p, s in zip(parts, sizes)]).numpy().view(np.uint64)
    if not np.array_equal(got, oracle.stable_sort_by_key(a)):
        raise SystemExit(f"rank {rank}: sharded result differs from the stable sort")
    print(f"rank {rank} ok", flush=True)
    dist.destroy_process_group()


if __name__ == "__main__":
    main()
