"""The request loop (continuous batching): requests that arrive while others
are on the GPU are admitted as slots and memory free up, small ones are sorted
together, and every result must be byte-identical to the same input sorted
alone (and to the reference's stable sort)."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import to_np

pytestmark = pytest.mark.gpu


def _alone(lsb, torch, n, dist, seed):
    a = lsb.generate(n, dist, seed)
    lsb.sort_pairs(a, torch.empty_like(a), 16)
    return to_np(a)


def test_results_same_alone_and_in_the_mix(lsb, cuda, oracle):
    rng = np.random.default_rng(3)
    sizes = [int(s) for s in np.floor(2.0 ** rng.uniform(4, 20, size=60))] + [1, 0, 3 << 20]
    dists = [int(d) for d in rng.integers(0, 5, size=len(sizes))]
    with lsb.Server(slots=4, digit_bits=16, batch_max_elems=1 << 18) as srv:
        ids = [srv.submit_generated(n, d, 500 + i, keep=True) for i, (n, d) in enumerate(zip(sizes, dists))]
        infos = [srv.wait(r) for r in ids]
        outs = [srv.fetch(r, n) for r, n in zip(ids, sizes)]
        st = srv.stats()
    assert all(i.status == 0 for i in infos)
    assert any(i.batch > 1 for i in infos), "small requests were batched"
    assert st.requests_done == len(sizes) and st.units < len(sizes)
    for i, (n, d) in enumerate(zip(sizes, dists)):
        assert np.array_equal(outs[i], _alone(lsb, cuda, n, d, 500 + i)), i
        if n <= 100000:
            assert np.array_equal(outs[i], oracle.stable_sort_by_key(oracle.generate(n, d, 500 + i))), i
    assert st.latency_p50_ms > 0 and st.latency_p99_ms >= st.latency_p50_ms


def test_host_buffer_requests(lsb, cuda, oracle):
    arrays = [oracle.generate(n, oracle.DIST_ZIPF, 40 + n) for n in (5, 1000, 70001, 300007, 17)]
    expect = [oracle.stable_sort_by_key(a) for a in arrays]
    bufs = [cuda.from_numpy(a.view(np.int64).copy()).pin_memory() for a in arrays]
    with lsb.Server(slots=3, batch_max_elems=1 << 17) as srv:
        ids = [srv.submit_host(b) for b in bufs]
        for r in ids:
            assert srv.wait(r).status == 0
    for b, e in zip(bufs, expect):
        assert np.array_equal(b.numpy().view(np.uint64), e)


def test_admission_respects_memory_budget(lsb, cuda):
    budget = 96 << 20
    with lsb.Server(slots=4, hbm_budget_bytes=budget, batch_max_elems=1 << 16) as srv:
        ids = [srv.submit_generated(1 << 20, 0, s) for s in range(12)]  # ~33 MB each with scratch
        for r in ids:
            assert srv.wait(r).status == 0
        st = srv.stats()
    assert st.requests_done == 12
    assert 0 < st.peak_bytes <= budget
