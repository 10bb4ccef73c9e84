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
