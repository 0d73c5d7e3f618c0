"""The serving form: requests submitted concurrently are continuously batched,
and each request's result is identical to the same reads searched alone (and to
the oracle), whatever else shares its batch."""
from __future__ import annotations

import threading
import time

import numpy as np
import pytest

from hpgbwt import lib, synth
from oracle.pyoracle import PortOracle

pytestmark = pytest.mark.gpu


def _same(a: lib.Result, b: lib.Result):
    assert np.array_equal(a.rs_count, b.rs_count)
    assert np.array_equal(a.rs_truncated, b.rs_truncated)
    assert np.array_equal(a.hits, b.hits)
    assert np.array_equal(a.locs, b.locs)


def _requests(genome, sizes, seed):
    out = []
    for i, n in enumerate(sizes):
        if n == 0:
            out.append(synth.from_strings([]))
        else:
            out.append(synth.reads(genome, n, seed + i, length=(36, 250), edits="mix_30_50_20"))
    return out


@pytest.mark.parametrize("max_results", [1 << 16, 3])
def test_alone_equals_in_mix(case_factory, max_results):
    c = case_factory("repeats", 300_000, 3, 3)
    sizes = [3000, 1, 0, 250, 7000, 64, 4096, 1200, 9000, 17, 2500, 600]
    reqs = _requests(c.genome, sizes, 300)
    ora = PortOracle(c.index)
    with lib.GpuIndex(c.index) as g:
        alone = [g.search(r, mode=lib.MODE_SEARCH1, form=lib.FORM_BATCHED, max_results=max_results) for r in reqs]
        with lib.Server(g, max_batch_reads=16384, max_results=max_results) as srv:
            tickets = [None] * len(reqs)

            def client(ids):  # requests arrive from several threads, some while batches run
                for i in ids:
                    time.sleep(0.001 * (i % 3))
                    tickets[i] = srv.submit(reqs[i].seq, reqs[i].offsets)

            th = [threading.Thread(target=client, args=(list(range(k, len(reqs), 3)),)) for k in range(3)]
            for t in th:
                t.start()
            for t in th:
                t.join()
            got = [srv.wait(t) for t in tickets]
            st = srv.stats()
    assert st["requests"] == len(reqs) and st["reads"] == sum(sizes)
    for i, (res, lat) in enumerate(got):
        assert lat is not None and lat >= 0
        _same(res, alone[i])
    for i in (0, 4, 9):
        _same(got[i][0], ora.search(reqs[i], mode=lib.MODE_SEARCH1, max_results=max_results, threads=8))


def test_batches_share_requests_and_budget_splits_them(case_factory):
    c = case_factory("repeats", 300_000, 3, 3)
    reqs = _requests(c.genome, [2000] * 8, 400)
    with lib.GpuIndex(c.index) as g:
        alone = [g.search(r, form=lib.FORM_BATCHED) for r in reqs]
        for budget, expect_shared in ((1 << 30, True), (1, False)):
            with lib.Server(g, max_batch_reads=65536, hbm_budget=budget) as srv:
                tickets = [srv.submit(r.seq, r.offsets) for r in reqs]
                got = [srv.wait(t)[0] for t in tickets]
                st = srv.stats()
            for a, b in zip(got, alone):
                _same(a, b)
            if expect_shared:
                assert st["max_batch_requests"] > 1
            else:  # a budget below any request admits one request per batch
                assert st["max_batch_requests"] == 1 and st["batches"] == len(reqs)


def test_serving_pools_grow(tmp_path_factory):
    """Requests whose hits and rows overflow the first pools of their plan."""
    rng = np.random.default_rng(8)
    g0 = synth.genome("iid", 60_000, 45)
    elem = rng.integers(0, 4, 300, dtype=np.uint8)
    for k in range(150):
        cp = elem.copy()
        m = rng.random(300) < 0.02
        cp[m] = rng.integers(0, 4, int(m.sum()), dtype=np.uint8)
        g0[12_000 + k * 300: 12_000 + (k + 1) * 300] = cp
    d = tmp_path_factory.mktemp("serve_copies")
    synth.write_fasta(str(d / "g.fa"), g0, [30_000, 30_000])
    lib.build_index(str(d / "g.fa"), str(d / "idx"), 16)
    reqs = [synth.reads(g0, n, 500 + i, length=(30, 100), edits="mix_30_50_20") for i, n in enumerate([4000, 3000])]
    ora = PortOracle(str(d / "idx"))
    with lib.GpuIndex(str(d / "idx")) as g:
        with lib.Server(g, max_batch_reads=8192) as srv:
            tickets = [srv.submit(r.seq, r.offsets) for r in reqs]
            got = [srv.wait(t)[0] for t in tickets]
            assert srv.stats()["regrowths"] >= 1
    for r, res in zip(reqs, got):
        _same(res, ora.search(r, mode=lib.MODE_SEARCH1, max_results=1 << 16, threads=8))


def test_server_rejects_and_releases(case_factory):
    c = case_factory("repeats", 300_000, 3, 3)
    big = synth.reads(c.genome, 5000, 601, length=100)
    small = synth.reads(c.genome, 10, 602, length=100)
    with lib.GpuIndex(c.index) as g:
        with lib.Server(g, max_batch_reads=4096) as srv:
            with pytest.raises(RuntimeError, match="batch capacity"):
                srv.submit(big.seq, big.offsets)
            t = srv.submit(small.seq, small.offsets)
            view, lat = srv.wait(t, copy=False)
            assert view.n_reads == 10 and lat >= 0
            srv.release(t)
            with pytest.raises(RuntimeError, match="unknown or released"):
                srv.release(t)


def test_serving_locate_limit(tmp_path_factory):
    """The serving form applies the index's locate limit like the batched call: lists over
    the limit keep their hits, get no rows and truncation bit 1, as the oracle's limit."""
    import sys
    from pathlib import Path
    sys.path.insert(0, str(Path(__file__).resolve().parent))
    from low_complexity import low_complexity_case
    index, reads = low_complexity_case(tmp_path_factory.mktemp("serve_limit"))
    # requests of the low-complexity reads in three slices
    n = len(reads.offsets) - 1
    cuts = [0, 7, 60, n]
    reqs = [reads.subset(np.arange(a, b)) for a, b in zip(cuts, cuts[1:])]
    ora = PortOracle(index)
    with lib.GpuIndex(index) as g:
        g.set_locate_limit(5000)
        with lib.Server(g, max_batch_reads=4096, max_results=100) as srv:
            tickets = [srv.submit(r.seq, r.offsets) for r in reqs]
            got = [srv.wait(t)[0] for t in tickets]
    for r, res in zip(reqs, got):
        want = ora.search(r, mode=lib.MODE_SEARCH1, max_results=100, threads=8, locate_limit=5000)
        _same(res, want)
    assert any((res.rs_truncated & 2).any() for res in got)
