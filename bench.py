#!/usr/bin/env python
"""Benchmark of the GB300 LSD radix-sort pass library.

Workload (the headline configuration): one step = one full LSD sort
(lsb_sort_pairs, the reference's mySort, mpi/mpi_lsbsort.cpp:592-597) of
2^30 16-byte {uint64 key, uint64 value} elements, keys uniform from the seeded
splitmix64 stream, value = index, 16-bit digits (the reference's RADIX, 4
digits, each run as two stable 8-bit sub-passes). The input is restored from
a resident copy before every step (not timed), so every step sorts the same
unsorted 16 GiB array; arrays are far larger than L2, and the restore copy
itself sweeps L2.

Prints ONE JSON line (rank 0):
  value        M elements/s, whole job, inputs resident in HBM, CUDA events
  e2e          same metric through the host-buffer C-ABI call
               (lsb_sort_pairs_host: every step copies the 16 GiB in and out;
               chunk copies overlap chunk sorts, the sorted chunks are merged
               and copied back slice by slice), beside copy_only_ms, the two
               copies alone
  roofline     dominant kernel: algorithmic bytes per launch / mean launch time,
               against the measured HBM copy bandwidth (MEASURED_PEAKS.json)
  cpu_baseline the oracle's port of the reference algorithm on the host cores
               (bounded sample; one_rank: the same on one core), rank 0 at N=1 only
  clocks       SM clock samples taken during the timed region
  segmented    4096 arrays of floor(2^U(10,22)) elements: one batched,
               graph-captured sort against a loop of lsb_sort_pairs
  serving      10^4 Poisson-arrival requests through the request loop:
               latency p50/p99 and elements/s
  digit_bits_8 / digit_bits_11 / single_pass_task_family /
  single_pass_wide_family
               the same sort through the other digit widths and kernel
               families (all give the same bytes)
  histogram_b16
               lsb_histogram at 16-bit digits: one read per three digits
               (default) against one HBM read by CTA pairs or quads
  sharded      the sharded sort (block distribution, count all-gather and
               element all-to-all per pass) over NCCL, 2^28 elements per rank

--impl reference times the reference algorithm on the host cores instead
(see cpu_arm below). --gpus N (torchrun): the headline runs N independent
replicas, one 2^30 sort per GPU per step, value = elements of all ranks / max
rank time; the sharded leg sorts one array of N x 2^28 elements across the
N ranks (an exchange per pass).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "distributed-lsb_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "M 16-byte elems sorted/s on 1 GB300 (2^30, HBM-roofline %); batched vs plain; p50/p99"
UNIT = "M elem/s"
DIST_NAMES = {"uniform": 0, "low32": 1, "zipf": 2, "equal": 3, "nearly_sorted": 4}


def algorithmic_bytes_per_element(digit_bits: int, passes_run: int) -> int:
    """One key read for the digit counts + 32 B (read 16, write 16) per pass run."""
    return 8 + 32 * passes_run


def workload_config(n: int, bits: int, dist: str, passes: int, world: int) -> dict:
    """The `config` object of both arms: the workload the metric is quoted on."""
    return {"workload": f"lsd-sort 2^{n.bit_length() - 1} {dist} u64 keys + u64 index values, "
                        f"{bits}-bit digits ({passes} passes)",
            "n": n, "digit_bits": bits, "dist": dist, "parallelism": f"replicas x{world}",
            "l2": "inputs (16 B x n) far larger than L2; input restored by a 16 B x n copy before each step"}


def args_parse(argv=None):
    p = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["native", "reference"], default="native")
    p.add_argument("--n", type=int, default=1 << 30)
    p.add_argument("--digit-bits", type=int, default=16)
    p.add_argument("--dist", choices=sorted(DIST_NAMES), default="uniform")
    p.add_argument("--e2e-steps", type=int, default=10)
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu", action="store_true", help="skip the cpu_baseline leg")
    p.add_argument("--no-extra", action="store_true", help="skip the 8-bit-digit side measurement")
    p.add_argument("--cpu-sample", type=int, default=1 << 26)
    p.add_argument("--no-segmented", action="store_true", help="skip the batched segmented leg")
    p.add_argument("--segments", type=int, default=4096)
    p.add_argument("--seg-steps", type=int, default=3)
    p.add_argument("--seg-seed", type=int, default=2024)
    p.add_argument("--no-serving", action="store_true", help="skip the request-loop leg")
    p.add_argument("--no-configs", action="store_true",
                   help="skip the timed small (2^24) and skew (2^28) configurations")
    p.add_argument("--config-steps", type=int, default=10)
    p.add_argument("--requests", type=int, default=10000)
    p.add_argument("--rate", type=float, default=400.0, help="Poisson arrival rate, requests/s")
    p.add_argument("--serve-slots", type=int, default=4)
    p.add_argument("--no-serve-sweep", dest="serve_sweep", action="store_false",
                   help="skip the arrival-rate sweep of the serving leg")
    p.add_argument("--sweep-requests", type=int, default=1500)
    p.add_argument("--host-requests", type=int, default=1000)
    p.add_argument("--host-rate", type=float, default=1000.0)
    p.add_argument("--no-sharded", action="store_true", help="skip the sharded-sort leg")
    p.add_argument("--shard-n", type=int, default=1 << 28, help="elements per rank in the sharded leg")
    p.add_argument("--shard-steps", type=int, default=3)
    return p.parse_args(argv)


# ---------------------------------------------------------------------------
# ranks

class Ranks:
    """Process-group plumbing for --gpus N (one process per GPU, env:// rendezvous)."""

    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local_rank = int(os.environ.get("LOCAL_RANK", "0"))
        self.dist = None
        if self.world > 1:
            import torch
            import torch.distributed as dist

            from datetime import timedelta

            backend = "nccl" if torch.cuda.is_available() else "gloo"
            if backend == "nccl":
                torch.cuda.set_device(self.local_rank)
            # a rank that fails ends its peers' next collective within minutes
            dist.init_process_group(backend=backend, timeout=timedelta(minutes=5))
            self.dist = dist
            self.backend = backend

    def barrier(self):
        if self.dist is not None:
            self.dist.barrier()

    def max(self, x: float) -> float:
        if self.dist is None:
            return x
        import torch

        dev = "cuda" if self.backend == "nccl" else "cpu"
        t = torch.tensor([x], dtype=torch.float64, device=dev)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.dist is not None:
            self.dist.destroy_process_group()


# ---------------------------------------------------------------------------
# clocks

class ClockSampler:
    """nvidia-smi sampling (200 ms) of SM clock and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax.append(float(parts[2]))
                except ValueError:
                    continue
                for nm, v in zip(names, parts[5:9]):
                    if v.lower() == "active":
                        reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def measured_peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "MEASURED_PEAKS.json (measured)"}
    return {"hbm_gbs": 6800.0, "source": "fallback 6.8 TB/s"}


def committed_traffic(kernel: str, n: int, digit_bits: int):
    """DRAM bytes per launch from the committed ncu summary, scaled to n."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(p):
        return None, None
    with open(p) as f:
        d = json.load(f)
    rec = d.get(f"{kernel}/b{digit_bits}")
    if not rec:
        return None, None
    return rec["dram_bytes_per_element"] * n, rec.get("source")


# ---------------------------------------------------------------------------
# the CPU arm and the cpu_baseline leg

def cpu_sort_rate(sample: int, reps: int, warmup: int = 0, budget_s: float = 30.0, threads: int = 0):
    """Times the oracle's port of the reference algorithm (one simulated MPI
    rank per thread; all host cores unless `threads` is given) on `sample`
    uniform elements. Returns (M elem/s over the timed reps, per-rep seconds, threads)."""
    import oracle

    oracle.build(with_ref=False) if not os.path.exists(oracle.ORACLE_SO) else None
    threads = threads or os.cpu_count() or 1
    a = oracle.generate(sample, oracle.DIST_UNIFORM, 0)
    times = []
    for i in range(warmup + reps):
        t0 = time.perf_counter()
        oracle.mysort(a, 16, ranks=threads, threads=threads)
        dt = time.perf_counter() - t0
        if i >= warmup:
            times.append(dt)
        if sum(times) > budget_s:
            break
    return sample * len(times) / sum(times) / 1e6, times, threads


def cpu_arm(args, ranks: Ranks):
    """--impl reference: the reference algorithm on the host cores (the oracle's
    C port of mpi/mpi_lsbsort.cpp, one simulated rank per thread; the
    reference's own build needs its source tree, which only the development
    container has). Each step sorts a bounded sample of the workload."""
    if ranks.rank != 0:
        return None
    sample = args.cpu_sample
    value, times, threads = cpu_sort_rate(sample, max(args.steps, 1), warmup=args.warmup, budget_s=120.0)
    ms = 1e3 * statistics.mean(times)
    return {
        "impl": "reference",
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": args.gpus,
        "steps": len(times), "warmup": args.warmup, "ms_per_step": round(ms, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
        "data": "synthetic",
        # the native arm's workload; each step sorts a bounded sample of it
        "config": workload_config(args.n, 16, "uniform", (64 + 15) // 16, ranks.world),
        "cpu_baseline": {"value": round(value, 3), "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{sample} uniform elements of the workload per step, 16-bit digits, "
                                   f"{len(times)} timed steps, {threads} simulated ranks"},
        "e2e": {"value": round(value, 3), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


# ---------------------------------------------------------------------------
# the GPU arm

def configs_leg(args, lsb, torch, peaks: dict) -> dict:
    """The other single-array configurations, each timed like the headline
    (input restored from a resident copy before every step, CUDA events,
    checked with the O(n) device verifier): the reference's CPU-runnable size
    2^24, and 2^28 in the four skewed key distributions, with the sort's
    roofline on the passes it actually ran (8 B + 32 B per executed pass)."""
    bits = 16
    cases = [("small_2p24_uniform", 1 << 24, "uniform"),
             ("skew_2p28_low32", 1 << 28, "low32"), ("skew_2p28_zipf", 1 << 28, "zipf"),
             ("skew_2p28_equal", 1 << 28, "equal"), ("skew_2p28_nearly_sorted", 1 << 28, "nearly_sorted")]
    res = {}
    for name, n, dist in cases:
        inp = lsb.generate(n, DIST_NAMES[dist], seed=11)
        A = torch.empty_like(inp)
        B = torch.empty_like(inp)
        ws = lsb.alloc_workspace(n, bits)
        stream = torch.cuda.current_stream()
        times = []
        for i in range(3 + args.config_steps):
            A.copy_(inp)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            lsb.sort_pairs(A, B, bits, workspace=ws)
            e1.record(stream)
            torch.cuda.synchronize()
            if i >= 3:
                times.append(e0.elapsed_time(e1))
        st = lsb.query(ws)
        bad = lsb.verify(inp, A)
        ms = statistics.mean(times)
        per_elem = algorithmic_bytes_per_element(bits, st.passes_run)
        gbs = per_elem * n / (ms / 1e3) / 1e9
        res[name] = {"n": n, "dist": dist, "digit_bits": bits, "steps": len(times),
                     "ms_per_sort": round(ms, 4), "p50_ms": round(statistics.median(times), 4),
                     "value": round(n / (ms / 1e3) / 1e6, 3), "unit": UNIT,
                     "passes_run": st.passes_run, "skipped_mask": st.skipped_mask,
                     "final_copy": st.final_copy, "verify_violations": int(bad),
                     "sort_roofline": {"algorithmic_bytes_per_element": per_elem, "achieved_gbs": round(gbs, 1),
                                       "frac": round(gbs / peaks["hbm_gbs"], 4)}}
        del inp, A, B, ws
        torch.cuda.empty_cache()
    return res


def gpu_arm(args, ranks: Ranks):
    import torch

    import lsb_gb300 as lsb

    torch.cuda.set_device(ranks.local_rank)
    lsb.build()
    lsb.load()
    n, bits = args.n, args.digit_bits
    dist = DIST_NAMES[args.dist]
    inp = lsb.generate(n, dist, seed=ranks.rank)
    A = torch.empty_like(inp)
    B = torch.empty_like(inp)
    ws = lsb.alloc_workspace(n, bits)
    stream = torch.cuda.current_stream()

    def one_sort():
        A.copy_(inp)  # restore the unsorted input (not timed)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        lsb.sort_pairs(A, B, bits, workspace=ws)
        e1.record(stream)
        return e0, e1

    for _ in range(max(args.warmup, 0)):
        one_sort()
    torch.cuda.synchronize()
    st = lsb.query(ws)
    if st.device_status != 0:
        raise RuntimeError(f"device status {st.device_status} after warm-up")
    bad = lsb.verify(inp, A)
    if bad:
        raise RuntimeError(f"warm-up sort differs from the stable sort ({bad} violations)")
    passes_run = st.passes_run

    # timed region
    clocks = ClockSampler(torch.cuda.current_device())
    ranks.barrier()
    torch.cuda.synchronize()
    clocks.start()
    time.sleep(0.3)  # let the sampler start
    events = [one_sort() for _ in range(args.steps)]
    torch.cuda.synchronize()
    ranks.barrier()
    clk = clocks.stop()
    step_ms = [a.elapsed_time(b) for a, b in events]
    local_s = sum(step_ms) / 1e3
    t = ranks.max(local_s)
    value = n * ranks.world * args.steps / t / 1e6
    bad = lsb.verify(inp, A)
    if bad:
        raise RuntimeError(f"timed sort differs from the stable sort ({bad} violations)")
    # look-back diagnostics of the last sort (control block words 10 and 11)
    ctrl_words = ws[:64].cpu().numpy().view("<u4")
    lookback = {"windows_read": int(ctrl_words[10]), "windows_polled": int(ctrl_words[11])}

    # per-kernel device times (separate, profiled steps; same work)
    lsb.profile_read()
    lsb.profile_enable(True)
    prof_steps = min(args.steps, 5)
    for _ in range(prof_steps):
        one_sort()
    torch.cuda.synchronize()
    lsb.profile_enable(False)
    prof = lsb.profile_read()
    kernels = {k: {"launches_per_step": v[0] / prof_steps, "mean_ms": v[1] / v[0]} for k, v in prof.items()}
    launches_per_step = sum(v[0] for v in prof.values()) / prof_steps
    dom = max(prof.items(), key=lambda kv: kv[1][1])[0]
    dom_ms = prof[dom][1] / prof[dom][0]
    # algorithmic bytes per launch of the dominant kernel (per element, x n)
    per_elem = {"task_scatter": 32, "onesweep_scatter": 32, "wide_pass": 32, "task_count": 8,
                "hist_digits": 8, "hist16": 8, "final_copy": 32}.get(dom, 0)
    peaks = measured_peaks()
    achieved = per_elem * n / (dom_ms / 1e3) / 1e9
    traffic, traffic_src = committed_traffic(dom, n, bits)
    ms_per_step = t * 1e3 / args.steps
    sort_bytes = algorithmic_bytes_per_element(bits, passes_run) * n
    out = {
        "metric": METRIC,
        "value": round(value, 3),
        "unit": UNIT,
        "n_gpus": ranks.world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(ms_per_step, 4),
        "p50_ms": round(statistics.median(step_ms), 4),
        "p99_ms": round(sorted(step_ms)[min(len(step_ms) - 1, int(0.99 * len(step_ms)))], 4),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "u64",
        "data": "synthetic",
        "config": workload_config(n, bits, args.dist, passes_run, ranks.world),
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peaks["hbm_gbs"],
                     "unit": "GB/s", "frac": round(achieved / peaks["hbm_gbs"], 4),
                     "traffic": traffic, "traffic_source": traffic_src,
                     "algorithmic_bytes_per_launch": per_elem * n, "mean_launch_ms": round(dom_ms, 4),
                     "peak_source": peaks["source"]},
        "kernel_passes": int(prof.get(dom, (0, 0))[0] / prof_steps) if dom.endswith("scatter") else None,
        "sort_roofline": {"algorithmic_bytes_per_element": algorithmic_bytes_per_element(bits, passes_run),
                          "achieved_gbs": round(sort_bytes / (ms_per_step / 1e3) / 1e9, 1),
                          "frac": round(sort_bytes / (ms_per_step / 1e3) / 1e9 / peaks["hbm_gbs"], 4)},
        "kernels": {k: {kk: round(vv, 4) for kk, vv in v.items()} for k, v in kernels.items()},
        "lookback": lookback,
        "gpu_launches": int(round(launches_per_step * args.steps)),
        "clocks": clk,
    }

    # side measurements on the same input: 8-bit digits, and (for wide digits)
    # the single-pass task kernel family instead of split sub-passes
    def time_sorts(b: int, reps: int = 3, env: dict | None = None):
        old = {k: os.environ.get(k) for k in (env or {})}
        os.environ.update(env or {})
        try:
            wsx = lsb.alloc_workspace(n, b)
            ev = []
            for i in range(2 + reps):
                A.copy_(inp)
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                lsb.sort_pairs(A, B, b, workspace=wsx)
                e1.record(stream)
                if i >= 2:
                    ev.append((e0, e1))
            torch.cuda.synchronize()
            ms = statistics.mean(a.elapsed_time(b_) for a, b_ in ev)
            return {"ms_per_step": round(ms, 4), "value": round(n / (ms / 1e3) / 1e6, 3),
                    "verify_violations": lsb.verify(inp, A)}
        finally:
            for k, v in old.items():
                if v is None:
                    os.environ.pop(k, None)
                else:
                    os.environ[k] = v

    if not args.no_extra:
        if bits != 8:
            out["digit_bits_8"] = time_sorts(8)
        if bits != 11:
            out["digit_bits_11"] = time_sorts(11)
        if bits in (12, 14, 16):
            out["single_pass_task_family"] = time_sorts(bits, reps=2, env={"LSB_WIDE_DIGITS": "task"})
        if bits == 16:
            out["single_pass_wide_family"] = time_sorts(bits, reps=2, env={"LSB_WIDE_DIGITS": "wide"})
            out["histogram_b16"] = histogram_b16_leg(lsb, torch, A)

    if not args.no_configs:
        out["configs"] = configs_leg(args, lsb, torch, peaks)

    # e2e through the host-buffer entry point
    if not args.no_e2e:
        del A, B, ws
        torch.cuda.empty_cache()
        h = torch.empty((n, 2), dtype=torch.int64, pin_memory=True)
        times = []
        for i in range(1 + args.e2e_steps):
            h.copy_(inp)  # restore the unsorted input in host memory (not timed)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            lsb.sort_pairs_host(h, bits)
            dt = time.perf_counter() - t0
            if i >= 1:
                times.append(dt)
        te = ranks.max(sum(times))
        # full O(n) check of the last step's output on the device: keys in order,
        # equal keys in input order, every input index once with its key (the
        # reference's std::stable_sort comparison, mpi/mpi_lsbsort.cpp:755-784)
        dev = h.cuda()
        e2e_bad = lsb.verify(inp, dev)
        ok = e2e_bad == 0
        # the same bytes copied in and out with nothing in between: the link's floor for this call
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        dev.copy_(h, non_blocking=True)
        h.copy_(dev, non_blocking=True)
        torch.cuda.synchronize()
        floor_ms = (time.perf_counter() - t0) * 1e3
        del dev
        out["e2e"] = {"value": round(n * ranks.world * len(times) / te / 1e6, 3), "unit": UNIT,
                      "h2d_bytes_per_step": 16 * n, "d2h_bytes_per_step": 16 * n,
                      "steps": len(times), "ms_per_step": round(te * 1e3 / len(times), 3),
                      "p50_ms": round(statistics.median(times) * 1e3, 3),
                      "p99_ms": round(sorted(times)[min(len(times) - 1, int(0.99 * len(times)))] * 1e3, 3),
                      "copy_only_ms": round(floor_ms, 3),
                      "call": "lsb_sort_pairs_host (pinned host buffer): chunk copies overlapped with "
                              "chunk sorts, stable merges, merged slices copied out while the next merges",
                      "sorted_check": ok, "verify_violations": int(e2e_bad)}
        del h

    if not args.no_segmented:
        A = B = ws = None  # release the 2^30 buffers (32 GiB) before the batch
        torch.cuda.empty_cache()
        out["segmented"] = segmented_leg(args, lsb, torch, ranks)

    if not args.no_serving:
        out["serving"] = serving_leg(args, lsb, torch, ranks)

    if not args.no_sharded:
        torch.cuda.empty_cache()
        out["sharded"] = sharded_leg(args, lsb, torch, ranks)

    if ranks.rank == 0 and ranks.world == 1 and not args.no_cpu:
        val, times, threads = cpu_sort_rate(args.cpu_sample, 3, warmup=1, budget_s=30.0)
        one = args.cpu_sample // 4
        val1, times1, _ = cpu_sort_rate(one, 1, warmup=0, budget_s=30.0, threads=1)
        out["cpu_baseline"] = {"value": round(val, 3), "unit": UNIT, "cores": threads, "kind": "port",
                               "sample": f"{args.cpu_sample} uniform elements, 16-bit digits, "
                                         f"{len(times)} timed sorts, {threads} simulated ranks",
                               "one_rank": {"value": round(val1, 3), "unit": UNIT, "cores": 1,
                                            "sample": f"{one} uniform elements, 16-bit digits, one rank"}}
    return out


def histogram_b16_leg(lsb, torch, data, reps: int = 3) -> dict:
    """lsb_histogram at 16-bit digits (four digits of every key) in its three
    forms: one read of the keys per three digits (default), and one HBM read by
    CTA pairs (two digits each) or CTA quads (one digit each). Kernel time from
    the library's own launch events; the counts of all forms must agree."""
    res, counts = {}, {}
    for form in ("pairs", "quads", "split"):
        old = os.environ.get("LSB_HIST16")
        os.environ["LSB_HIST16"] = form
        try:
            lsb.histogram(data, 16)  # warm-up
            torch.cuda.synchronize()
            lsb.profile_read()
            lsb.profile_enable(True)
            for _ in range(reps):
                h = lsb.histogram(data, 16)
            torch.cuda.synchronize()
            lsb.profile_enable(False)
            prof = lsb.profile_read()
        finally:
            if old is None:
                os.environ.pop("LSB_HIST16", None)
            else:
                os.environ["LSB_HIST16"] = old
        launches, total = prof.get("hist16", (0, 0.0))
        counts[form] = h
        res[form] = {"ms": round(total / reps, 4), "launches": launches // reps,
                     "hbm_reads_of_keys": 2 if form == "split" else 1}
    res["counts_agree"] = all(bool(torch.equal(counts[f], counts["split"])) for f in ("pairs", "quads"))
    return res


def _unsigned_order(keys):
    """int64 keys mapped so that signed comparison follows the unsigned order."""
    return keys ^ (-(1 << 63))


def _pair_checksum(torch, block):
    """Sum (mod 2^64) of a mix of every key with its value: preserved exactly
    when the sort only permutes whole elements."""
    mixed = block[:, 0] ^ (block[:, 1] * -7046029254386353131)  # 0x9E3779B97F4A7C15 as int64
    return mixed.sum()


def sharded_leg(args, lsb, torch, ranks) -> dict:
    """The sharded sort (lsb_gb300.sharded) over NCCL: args.shard_n elements
    per rank (weak scaling), the reference's block distribution, one count
    all-gather and one element all-to-all per pass, 16-bit digits. With one
    GPU the group has a single rank, so the exchange is a copy to itself and
    the leg measures the sharded machinery beside lsb_sort_pairs; under
    torchrun every rank sorts with its own GPU. Checked by properties that
    hold at any size: every block sorted, blocks in order across ranks, the
    element count and a key-value checksum preserved."""
    import socket

    import torch.distributed as dist
    from lsb_gb300 import sharded

    own = ranks.dist is None
    if own:
        with socket.socket() as s:
            s.bind(("127.0.0.1", 0))
            port = s.getsockname()[1]
        dist.init_process_group("nccl", init_method=f"tcp://127.0.0.1:{port}", rank=0, world_size=1)
    try:
        world, rank = dist.get_world_size(), dist.get_rank()
        m, bits = args.shard_n, 16
        n = m * world
        block = lsb.generate(m, DIST_NAMES["uniform"], seed=1000 + rank)  # this rank's block
        ops = sharded.GpuLocalOps(lsb, bits)
        check_in = torch.stack([_pair_checksum(torch, block), torch.tensor(m, device=block.device)])
        dist.all_reduce(check_in)
        times, res = [], None
        for i in range(1 + args.shard_steps):
            dist.barrier()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            res = sharded.sharded_sort(block, n, bits, ops, dist)
            torch.cuda.synchronize()
            dt = time.perf_counter() - t0
            t = torch.tensor([dt], dtype=torch.float64, device=block.device)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            if i >= 1:
                times.append(float(t.item()))
        keys = _unsigned_order(res[:, 0])
        local_sorted = bool((keys[1:] >= keys[:-1]).all()) if keys.numel() > 1 else True
        ends = torch.stack([keys[0], keys[-1]]) if keys.numel() else torch.zeros(2, dtype=torch.int64, device=keys.device)
        all_ends = [torch.empty_like(ends) for _ in range(world)]
        dist.all_gather(all_ends, ends)
        ordered = all(int(all_ends[r][1]) <= int(all_ends[r + 1][0]) for r in range(world - 1))
        flags = torch.tensor([0 if local_sorted else 1], device=keys.device)
        dist.all_reduce(flags)
        check_out = torch.stack([_pair_checksum(torch, res), torch.tensor(res.shape[0], device=res.device)])
        dist.all_reduce(check_out)
        ms = statistics.median(times) * 1e3
        return {"n_per_rank": m, "world": world, "elements": n, "digit_bits": bits, "steps": len(times),
                "ms_per_sort": round(ms, 3), "value": round(n / (ms / 1e3) / 1e6, 3), "unit": UNIT,
                "scaling": "weak", "data": "uniform keys, one seeded stream per rank",
                "sorted_check": bool(int(flags.item()) == 0 and ordered and torch.equal(check_in, check_out)),
                "call": "lsb_gb300.sharded.sharded_sort with GpuLocalOps (lsb_pass + lsb_histogram per pass), "
                        "NCCL all_gather of counts and all_to_all_single of elements"}
    finally:
        if own:
            dist.destroy_process_group()


def segmented_leg(args, lsb, torch, ranks) -> dict:
    """Batched segmented sort: 4096 arrays with sizes floor(2^U(10, 22)) (seeded),
    uniform keys, value = index. The C++ driver (lsb_sort --segments-file)
    sorts the batch twice from the same unsorted input: by a C++ loop of
    lsb_sort_pairs over the arrays (16-bit digits, one workspace sized once for
    the largest array), and by one launch of the batched call's CUDA graph
    with the autotuned configuration; the outputs must be byte-identical."""
    import numpy as np

    from lsb_gb300 import _build

    rng = np.random.default_rng(args.seg_seed)
    sizes = np.floor(2.0 ** rng.uniform(10, 22, size=args.segments)).astype(np.int64)
    off = np.zeros(len(sizes) + 1, dtype=np.int64)
    off[1:] = np.cumsum(sizes)
    total = int(off[-1])
    fd, path = tempfile.mkstemp(suffix=".offsets")
    os.close(fd)
    try:
        off.astype("<i8").tofile(path)
        r = subprocess.run([_build.DRIVER_PATH, "--segments-file", path, "--digit-bits", "16",
                            "--seed", str(1000 + ranks.rank), "--steps", str(args.seg_steps)],
                           capture_output=True, text=True, timeout=1800)
    finally:
        os.unlink(path)
    if r.returncode != 0:
        raise RuntimeError(f"lsb_sort --segments-file failed ({r.returncode}): {r.stdout[-2000:]} {r.stderr[-2000:]}")
    d = json.loads(r.stdout.strip().splitlines()[-1])
    bms, lms = d["batched_ms"], d["loop_ms"]
    return {
        "segments": d["segments"], "elements": total, "size_law": "floor(2^U(10,22))",
        "tuning": d["tuning"], "steps": d["steps"],
        "batched_ms": round(bms, 3), "loop_ms": round(lms, 3), "speedup": round(lms / bms, 3),
        "batched_value": round(total / (bms / 1e3) / 1e6, 3), "loop_value": round(total / (lms / 1e3) / 1e6, 3),
        "unit": UNIT, "identical_outputs": d["identical_outputs"],
        "loop_call": "C++ loop of lsb_sort_pairs per array (lsb_sort --segments-file), 16-bit digits, "
                     "one workspace sized once for the largest array",
        "batched_call": "lsb_graph_launch of lsb_graph_capture_segmented with lsb_tune_segmented's choice",
    }


def _serve_run(lsb, srv_kwargs: dict, n_req: int, arrivals, submit) -> dict:
    """One open-loop run: submits request i at arrivals[i] (seconds after the
    start) through `submit(srv, i)`, waits for every result, and returns the
    host-side and device-side statistics."""
    with lsb.Server(**srv_kwargs) as srv:
        t0 = time.perf_counter()
        ids = []
        for i in range(n_req):
            delay = t0 + arrivals[i] - time.perf_counter()
            if delay > 0.002:
                time.sleep(delay - 0.001)
            while time.perf_counter() < t0 + arrivals[i]:
                pass
            ids.append(submit(srv, i))
        for r in ids:
            info = srv.wait(r)
            if info.status != 0:
                raise RuntimeError(f"request {r} failed with status {info.status}")
        return {"stats": srv.stats(), "device": srv.device_stats()}


def _serve_summary(res: dict, n_req: int, rate: float, elements: int, size_law: str) -> dict:
    st, dv = res["stats"], res["device"]
    return {"requests": n_req, "rate_per_s": rate, "size_law": size_law, "elements": int(elements),
            "latency_p50_ms": round(st.latency_p50_ms, 3), "latency_p99_ms": round(st.latency_p99_ms, 3),
            "service_p50_ms": round(st.service_p50_ms, 3), "service_p99_ms": round(st.service_p99_ms, 3),
            "value": round(st.elements_per_s / 1e6, 3), "unit": UNIT, "wall_ms": round(st.wall_ms, 1),
            "batched_requests": int(st.batched_requests), "units": int(st.units),
            "peak_hbm_gb": round(st.peak_bytes / 1e9, 3), "budget_hbm_gb": round(st.budget_bytes / 1e9, 3),
            "device_overlap": round(dv.overlap, 3), "device_max_concurrent_units": int(dv.max_concurrent),
            "device_busy_ms": round(dv.busy_ms, 1)}


def serving_leg(args, lsb, torch, ranks) -> dict:
    """Open-loop request streams through the request loop (lsb_server_*),
    16-bit digits:
      - the configuration: Poisson arrivals at args.rate, args.requests
        requests, sizes floor(2^U(10, 27)) elements of uniform keys generated
        on the device per request;
      - a sweep of the arrival rate with the same size law up to saturation
        (served against offered load and p99 per rate);
      - host-buffer requests (pinned host memory copied in and out by the
        loop), sizes floor(2^U(10, 20)).
    The units' device spans (CUDA events on their streams) show whether units
    on different stream slots overlap on the GPU (device_overlap > 1)."""
    import numpy as np

    kw = {"slots": args.serve_slots, "digit_bits": 16}
    rng = np.random.default_rng(7 + ranks.rank)
    sizes = np.floor(2.0 ** rng.uniform(10, 27, size=args.requests)).astype(np.int64)
    arrivals = np.cumsum(rng.exponential(1.0 / args.rate, size=args.requests))
    res = _serve_run(lsb, kw, args.requests, arrivals,
                     lambda srv, i: srv.submit_generated(int(sizes[i]), 0, 1 + i))
    out = _serve_summary(res, args.requests, args.rate, sizes.sum(), "floor(2^U(10,27))")
    out["offered_melem_s"] = round(float(sizes.mean()) * args.rate / 1e6, 1)
    out["slots"] = args.serve_slots
    out["digit_bits"] = 16

    if args.serve_sweep:
        sweep = []
        for rate in (200.0, 400.0, 800.0, 1600.0, 3200.0, 6400.0):
            m = args.sweep_requests
            rs = np.random.default_rng(100 + int(rate))
            sz = np.floor(2.0 ** rs.uniform(10, 27, size=m)).astype(np.int64)
            arr = np.cumsum(rs.exponential(1.0 / rate, size=m))
            r = _serve_run(lsb, kw, m, arr, lambda srv, i, sz=sz: srv.submit_generated(int(sz[i]), 0, 1 + i))
            row = _serve_summary(r, m, rate, sz.sum(), "floor(2^U(10,27))")
            row["offered_melem_s"] = round(float(sz.mean()) * rate / 1e6, 1)
            sweep.append(row)
        out["sweep"] = sweep
        out["saturation_melem_s"] = max(x["value"] for x in sweep)
        base_p99 = sweep[0]["latency_p99_ms"]
        out["p99_knee_rate_per_s"] = next(
            (x["rate_per_s"] for x in sweep
             if x["latency_p99_ms"] > 10 * base_p99 or x["value"] < 0.9 * x["offered_melem_s"]), None)

    # requests whose data lives in host memory (pinned), copied in and out by the loop
    m = args.host_requests
    rh = np.random.default_rng(9)
    hs = np.floor(2.0 ** rh.uniform(10, 20, size=m)).astype(np.int64)
    off = np.zeros(m + 1, dtype=np.int64)
    off[1:] = np.cumsum(hs)
    host = torch.empty((int(off[-1]), 2), dtype=torch.int64, pin_memory=True)
    # non-negative keys, so that the signed check below agrees with the unsigned order
    host[:, 0] = torch.randint(0, 1 << 62, (int(off[-1]),), dtype=torch.int64)
    host[:, 1] = torch.arange(int(off[-1]), dtype=torch.int64)
    arr = np.cumsum(rh.exponential(1.0 / args.host_rate, size=m))
    views = [host[off[i]:off[i + 1]] for i in range(m)]
    r = _serve_run(lsb, kw, m, arr, lambda srv, i: srv.submit_host(views[i]))
    hrow = _serve_summary(r, m, args.host_rate, hs.sum(), "floor(2^U(10,20)), pinned host buffers")
    hrow["sorted_check"] = all(bool((v[1:, 0] >= v[:-1, 0]).all()) for v in views[:: max(1, m // 50)])
    out["host_buffers"] = hrow
    del host, views
    return out


def main(argv=None):
    args = args_parse(argv)
    ranks = Ranks()
    try:
        out = cpu_arm(args, ranks) if args.impl == "reference" else gpu_arm(args, ranks)
        if ranks.rank == 0 and out is not None:
            print(json.dumps(out), flush=True)
    finally:
        ranks.close()


if __name__ == "__main__":
    main()
