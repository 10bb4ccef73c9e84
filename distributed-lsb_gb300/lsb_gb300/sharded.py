"""Sharded LSD sort: one array split over several processes (one per GPU),
the reference's own distributed structure (mpi/mpi_lsbsort.cpp).

Partitioning (DistributedArray, mpi/mpi_lsbsort.cpp:97-171): block
distribution, rank r holds the global elements [r*B, min((r+1)*B, n)) with
B = ceil(n / R) (:154-159); every rank holds its block before and after every
pass, and after the last pass the blocks concatenated are the stable sort.

One pass (globalShuffle, :493-589), for digit d:
  1. local: the block stably sorted by d, and the block's count of every digit
     value (localShuffle, :225-259);
  2. counts: one all-gather of the R x 2^b count table. Every rank then knows
     every count, and the start of the run of (digit v, rank r) in the global
     order, start(v, r) = sum of the counts of digits below v over all ranks +
     the counts of digit v on ranks below r (digit-major, like
     GlobalCounts[digit * R + rank], :362). This one collective replaces the
     reference's count transpose, exclusive scan and start redistribution
     (copyCountsToGlobalCounts / exclusiveScan / copyStartsFromGlobalStarts,
     :339-491);
  3. elements: one all-to-all. Rank r's locally sorted block is a sequence of
     runs, one per digit value; each run's destination range
     [start(v, r), start(v, r) + count(r, v)) is cut at the block boundaries
     and every piece goes to the rank owning it, in run order (:539-588). The
     receiver derives every received element's position from the same count
     table, so no index travels with the elements (the reference sends 24-byte
     records with a destination index, :550-575).

Each rank sends and receives about (R-1)/R of its block per pass. The local
step is the caller's: on GPUs the library's pass and histogram kernels
(`GpuLocalOps`). The exchange plan is integer arithmetic over the count table,
the same on every rank, done by the library (lsb_exchange_plan): what a rank
sends to each rank, and what it receives as pieces (offset in the received
array, block-local destination, length), at most R x 2^b of them, which the
library's placement kernel copies into place (lsb_place_pieces).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


def block_range(n: int, world: int, rank: int) -> tuple[int, int]:
    """[lo, hi) of rank's block: blocks of ceil(n / world) elements
    (mpi/mpi_lsbsort.cpp:154-159)."""
    b = (n + world - 1) // world if world else 0
    lo = min(n, rank * b)
    return lo, min(n, lo + b)


@dataclass
class ExchangePlan:
    send_counts: list[int]   # elements this rank sends to each rank, in rank order
    recv_counts: list[int]   # elements this rank receives from each rank
    piece_src: np.ndarray    # offset of every received piece in the received array
    piece_dst: np.ndarray    # block-local start of every received piece, in arrival order
    piece_len: np.ndarray    # length of every received piece

    def positions(self) -> np.ndarray:
        """Block-local position of every received element, in arrival order."""
        total = int(self.piece_len.sum())
        if total == 0:
            return np.zeros(0, dtype=np.int64)
        return np.repeat(self.piece_dst - self.piece_src, self.piece_len) + np.arange(total, dtype=np.int64)


def exchange_plan(counts: np.ndarray, n: int, rank: int) -> ExchangePlan:
    """The element exchange of one pass for `rank`, from the all-gathered count
    table counts[r][v] (elements of digit value v in rank r's block), by the
    library (lsb_exchange_plan, host arithmetic). Rank r's run of digit v
    occupies the global range [start(v, r), start(v, r) + counts[r][v]) of the
    pass's output, start digit-major over (v, r); the slice sent to rank q is
    the part of every run inside q's block, runs in order, and the receiver
    lays out what it gets the same way."""
    from . import exchange_plan as native_plan

    send, recv, src, dst, ln = native_plan(counts, n, rank)
    return ExchangePlan([int(x) for x in send], [int(x) for x in recv], src, dst, ln)


class LocalOps:
    """The per-rank work of a pass. shuffle(block, digit, bits) returns the
    block stably sorted by the digit and the count of every digit value
    (int64 numpy array of 2^bits); place(received, plan, size) returns a block
    of `size` elements with the received pieces at their destinations
    (plan.piece_dst, plan.piece_len, in arrival order)."""

    def shuffle(self, block, digit: int, bits: int):
        raise NotImplementedError

    def place(self, received, plan: ExchangePlan, size: int):
        raise NotImplementedError


class GpuLocalOps(LocalOps):
    """The library's kernels on this rank's GPU: one lsb_pass (globalShuffle
    of the block) and one lsb_histogram per pass."""

    def __init__(self, lsb, digit_bits: int):
        self.lsb = lsb
        self.bits = digit_bits

    def shuffle(self, block, digit: int, bits: int):
        import torch

        out = torch.empty_like(block)
        if block.shape[0]:
            self.lsb.global_shuffle(block, out, digit, bits)
            counts = self.lsb.histogram(out, bits)[digit].cpu().numpy()
        else:
            counts = np.zeros(1 << bits, dtype=np.int64)
        return out, counts

    def place(self, received, plan: ExchangePlan, size: int):
        import torch

        if received.shape[0] == size and np.array_equal(plan.piece_dst, plan.piece_src):
            return received  # the pieces arrive in destination order (e.g. one rank): nothing to move
        out = torch.empty((size, 2), dtype=received.dtype, device=received.device)
        self.lsb.place_pieces(received, out, plan.piece_src, plan.piece_dst, plan.piece_len)
        return out


def sharded_sort(block, n: int, digit_bits: int, ops: LocalOps, dist, group=None):
    """Stably sorts the array whose rank-local block (this rank's
    block_range(n, world, rank)) is `block` (int64 tensor (m, 2), key then
    value), across all ranks of `group`; returns this rank's block of the
    result. Collectives: one all-gather of counts and one all-to-all of
    elements per pass (dist: torch.distributed, any backend that has
    all_to_all_single; tensors on the backend's device)."""
    import torch

    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    lo, hi = block_range(n, world, rank)
    if block.shape[0] != hi - lo:
        raise ValueError(f"rank {rank}: block of {block.shape[0]} elements, expected {hi - lo}")
    nbins = 1 << digit_bits
    passes = (64 + digit_bits - 1) // digit_bits
    dev = block.device
    for digit in range(passes):
        local, counts = ops.shuffle(block, digit, digit_bits)
        table = torch.from_numpy(np.ascontiguousarray(counts, dtype=np.int64)).to(dev)
        gathered = [torch.empty(nbins, dtype=torch.int64, device=dev) for _ in range(world)]
        dist.all_gather(gathered, table, group=group)
        allc = np.stack([g.cpu().numpy() for g in gathered])
        if (allc.sum(axis=0) == n).any():
            block = local  # one digit value holds every element: the pass is the identity
            continue
        plan = exchange_plan(allc, n, rank)
        recv = torch.empty((sum(plan.recv_counts), 2), dtype=block.dtype, device=dev)
        dist.all_to_all_single(recv, local.contiguous(), output_split_sizes=plan.recv_counts,
                               input_split_sizes=plan.send_counts, group=group)
        block = ops.place(recv, plan, hi - lo)
    return block
