"""bench.py's multi-rank plumbing (--gpus N launched one process per rank) at
world size 2 over gloo on the CPU: the barrier, the max over ranks that the
timing takes, and the rule that rank 0 alone prints the JSON line (the other
ranks of the reference arm exit 0 without work)."""
from __future__ import annotations

import json
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _launch(code_or_args: list[str], world: int = 2, timeout: int = 240):
    port = _free_port()
    procs = []
    for r in range(world):
        env = dict(os.environ, RANK=str(r), LOCAL_RANK=str(r), WORLD_SIZE=str(world),
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES="")
        procs.append(subprocess.Popen([sys.executable, *code_or_args], cwd=ROOT, env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = []
    try:
        for p in procs:
            out, err = p.communicate(timeout=timeout)
            outs.append((p.returncode, out, err))
    finally:
        for p in procs:
            if p.poll() is None:
                p.kill()
    return outs


RANKS_SNIPPET = r"""
import os, sys
sys.path.insert(0, os.getcwd())
import bench
r = bench.Ranks()
assert r.world == 2 and r.backend == "gloo"
r.barrier()
print(repr(r.max(1.5 + 10 * r.rank)))
r.barrier()
r.close()
"""


def test_ranks_barrier_and_max_over_gloo():
    outs = _launch(["-c", RANKS_SNIPPET])
    for rc, out, err in outs:
        assert rc == 0, err
        assert float(out.strip().splitlines()[-1]) == 11.5


def test_reference_arm_prints_on_rank_zero_only():
    outs = _launch(["bench.py", "--impl", "reference", "--gpus", "2", "--steps", "1",
                    "--warmup", "0", "--cpu-sample", "4096"])
    (rc0, out0, err0), (rc1, out1, err1) = outs
    assert rc0 == 0, err0
    assert rc1 == 0, err1
    lines0 = [l for l in out0.splitlines() if l.strip()]
    assert len(lines0) == 1
    rec = json.loads(lines0[0])
    assert rec["impl"] == "reference" and rec["value"] > 0 and rec["n_gpus"] == 2
    assert rec["e2e"]["h2d_bytes_per_step"] == 0
    assert not [l for l in out1.splitlines() if l.strip()]
