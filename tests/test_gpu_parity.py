"""GPU parity: the CUDA pipeline (through the C ABI) against the CPU oracle, bit-exact."""
from __future__ import annotations

import numpy as np
import pytest

from hpgbwt import lib, synth
from low_complexity import low_complexity_case
from oracle.pyoracle import PortOracle

pytestmark = pytest.mark.gpu


def _assert_same(gpu: lib.Result, ref: lib.Result):
    assert np.array_equal(gpu.rs_count, ref.rs_count), "per-strand hit counts differ"
    assert np.array_equal(gpu.rs_truncated, ref.rs_truncated), "truncation flags differ"
    assert len(gpu.hits) == len(ref.hits)
    assert np.array_equal(gpu.hits, ref.hits), "hits differ"
    assert len(gpu.locs) == len(ref.locs)
    assert np.array_equal(gpu.locs, ref.locs), "located rows differ"


@pytest.mark.parametrize("form", [lib.FORM_PLAIN, lib.FORM_BATCHED])
@pytest.mark.parametrize("mode", [lib.MODE_EXACT, lib.MODE_SEARCH1])
@pytest.mark.parametrize("kind,n,chroms,edits,length", [
    ("iid", 200_000, 1, "none", 100),
    ("repeats", 300_000, 3, "per_base_capped", 100),
    ("repeats", 300_000, 3, "mix_30_50_20", (36, 250)),
    ("human_like", 200_000, 5, "mix_30_50_20", (20, 150)),
])
def test_gpu_matches_oracle(case_factory, mode, form, kind, n, chroms, edits, length):
    c = case_factory(kind, n, 3, chroms)
    reads = synth.reads(c.genome, 4000, 17, length=length, edits=edits)
    ora = PortOracle(c.index)
    with lib.GpuIndex(c.index) as g:
        got = g.search(reads, mode=mode, form=form, max_results=1 << 16)
    want = ora.search(reads, mode=mode, max_results=1 << 16, threads=8)
    _assert_same(got, want)


@pytest.mark.parametrize("form", [lib.FORM_PLAIN, lib.FORM_BATCHED])
@pytest.mark.parametrize("max_results", [0, 1, 2, 3, 9, 17])
def test_truncation_matches_oracle(case_factory, max_results, form):
    c = case_factory("human_like", 100_000, 5, 2)
    reads = synth.reads(c.genome, 3000, 23, length=(20, 120), edits="mix_30_50_20")
    ora = PortOracle(c.index)
    with lib.GpuIndex(c.index) as g:
        got = g.search(reads, mode=lib.MODE_SEARCH1, form=form, max_results=max_results)
    want = ora.search(reads, mode=lib.MODE_SEARCH1, max_results=max_results, threads=8)
    assert want.rs_truncated.any() or max_results > 3
    _assert_same(got, want)


def test_edge_reads(case_factory):
    c = case_factory("iid", 50_000, 9, 1)
    g0 = c.genome
    A = np.frombuffer(b"ACGT", dtype=np.uint8)
    seqs = [b"", b"A", b"AC", b"ACG", A[g0[100:105]].tobytes(), b"ACGTN" * 10, b"acgt" * 20,
            A[g0[1000:1100]].tobytes(), A[g0[-80:]].tobytes(), A[g0[:64]].tobytes(),
            A[g0[5000:6000]].tobytes(), b"T" * 300]
    reads = synth.from_strings(seqs)
    ora = PortOracle(c.index)
    with lib.GpuIndex(c.index) as g:
        for mode in (lib.MODE_EXACT, lib.MODE_SEARCH1):
            for form in (lib.FORM_PLAIN, lib.FORM_BATCHED):
                got = g.search(reads, mode=mode, form=form)
                want = ora.search(reads, mode=mode, threads=1)
                _assert_same(got, want)


def test_chunked_equals_single_pass(case_factory):
    c = case_factory("repeats", 300_000, 3, 3)
    reads = synth.reads(c.genome, 5000, 29, length=(36, 250), edits="mix_30_50_20")
    with lib.GpuIndex(c.index) as g:
        whole = g.search(reads)
        g.set_chunk(777)
        parts = g.search(reads)
    assert whole.equal(parts)


@pytest.mark.parametrize("stack,chunk,per_sm,minb", [(2, 1, 0, 1), (4, 2, 0, 12), (8, 4, 0, 16), (2, 8, 1, 1),
                                                     (4, 1, 3, 16), (0, 4, 0, 1), (0, 1, 2, 12), (-1, 1, 0, 1),
                                                     (-1, 1, 0, 12), (-1, 1, 2, 16)])
def test_batched_tunings_agree(case_factory, stack, chunk, per_sm, minb):
    """Every autotuner setting gives the oracle's answer; depth 2 forces spills to the drain path."""
    c = case_factory("human_like", 200_000, 5, 5)
    reads = synth.reads(c.genome, 4000, 37, length=(20, 150), edits="mix_30_50_20")
    want = PortOracle(c.index).search(reads, mode=lib.MODE_SEARCH1, max_results=1 << 16, threads=8)
    with lib.GpuIndex(c.index) as g:
        g.set_tuning(per_sm, stack, chunk, minb)
        got = g.search(reads, mode=lib.MODE_SEARCH1, form=lib.FORM_BATCHED)
    _assert_same(got, want)


def test_autotuner_keeps_results(case_factory):
    torch = pytest.importorskip("torch")
    c = case_factory("repeats", 300_000, 3, 3)
    reads = synth.reads(c.genome, 6000, 39, length=(36, 250), edits="mix_30_50_20")
    want = PortOracle(c.index).search(reads, mode=lib.MODE_SEARCH1, max_results=64, threads=8)
    d_seq = torch.from_numpy(reads.seq).cuda()
    d_off = torch.from_numpy(reads.offsets.view(np.int64)).cuda()
    with lib.GpuIndex(c.index) as g:
        table = g.autotune(d_seq.data_ptr(), d_off.data_ptr(), len(reads), int(reads.offsets[-1]),
                           int(np.diff(reads.offsets).max()), 64)
        # 60 fused/split/lockstep settings, 12 warp-cooperative ones, 4 load forms,
        # 3 direction splits (fused form only), 5 start tables, 4 idle batches
        assert len(table) in (85, 88) and all(r["search_us"] > 0 for r in table)
        chosen = g.get_tuning()
        best_us = min(r["search_us"] for r in table[:72])
        mine = [r["search_us"] for r in table[:72]
                if (r["stack"], r["chains_per_claim"], r["register_bound_blocks"]) ==
                (chosen["stack"], chosen["chains_per_claim"], chosen["register_bound_blocks"])]
        assert mine and min(mine) <= best_us + 1  # the fastest setting (ties rounded to 1 us) was kept
        got = g.search(reads, mode=lib.MODE_SEARCH1, form=lib.FORM_BATCHED, max_results=64)
    _assert_same(got, want)


def test_batched_golden(tmp_path_factory):
    """The batched form reproduces the reference's own outputs in the golden fixtures."""
    from golden_cases import GoldenCase, names
    for name in names():
        gc = GoldenCase(name)
        index = gc.build(tmp_path_factory.mktemp(name))
        with lib.GpuIndex(index) as g:
            for tag in gc.tags():
                mode, mr = int(tag[1]), int(tag.split("_r")[1])
                for form in (lib.FORM_PLAIN, lib.FORM_BATCHED):
                    _assert_same(g.search(gc.reads, mode=mode, form=form, max_results=mr), gc.expected(tag))


@pytest.mark.parametrize("load_mode", [0, 1, 2, 3])
def test_block_load_modes_agree(case_factory, load_mode):
    c = case_factory("repeats", 300_000, 3, 3)
    reads = synth.reads(c.genome, 3000, 41, length=(36, 250), edits="mix_30_50_20")
    want = PortOracle(c.index).search(reads, mode=lib.MODE_SEARCH1, max_results=1 << 16, threads=8)
    with lib.GpuIndex(c.index) as g:
        g.set_load_mode(load_mode)
        assert g.load_mode() == load_mode
        for form in (lib.FORM_PLAIN, lib.FORM_BATCHED):
            _assert_same(g.search(reads, mode=lib.MODE_SEARCH1, form=form), want)


@pytest.mark.parametrize("symbols", [0, 8, 10, 12])
def test_start_table_lengths_agree(case_factory, symbols):
    """Chains that start with one start-table lookup give the oracle's answer;
    reads shorter than 2L+2 bases take the step-by-step start."""
    c = case_factory("human_like", 200_000, 5, 5)
    reads = synth.reads(c.genome, 4000, 43, length=(12, 150), edits="mix_30_50_20")
    want = PortOracle(c.index).search(reads, mode=lib.MODE_SEARCH1, max_results=1 << 16, threads=8)
    with lib.GpuIndex(c.index) as g:
        g.set_start_table(symbols)
        assert g.start_table() == symbols
        for stack in (0, 2, 4):  # split form (chain-only kernel) and fused
            g.set_tuning(0, stack, 1, 1)
            _assert_same(g.search(reads, mode=lib.MODE_SEARCH1, form=lib.FORM_BATCHED), want)
        g.set_graph(False)
        _assert_same(g.search(reads, mode=lib.MODE_SEARCH1, form=lib.FORM_BATCHED), want)


@pytest.mark.parametrize("batch", [1, 4, 8, 16, 32])
@pytest.mark.parametrize("split", [0, 2])
def test_idle_batch_agrees(case_factory, batch, split):
    """Idle lanes moving on together (any batch size, both direction modes) give the same results."""
    c = case_factory("repeats", 300_000, 3, 3)
    main = synth.reads(c.genome, 5000, 53, length=(3, 250), edits="mix_30_50_20")
    odd = synth.from_strings([b"", b"AC", b"ACGTN" * 5, b"GATTACA", b""] * 40)
    seq = np.concatenate([odd.seq, main.seq])
    offs = np.concatenate([odd.offsets, main.offsets[1:] + odd.offsets[-1]]).astype(np.uint64)
    reads = synth.ReadSet(seq, offs, np.zeros(1), np.zeros(1), np.zeros(1))
    want = PortOracle(c.index).search(reads, mode=lib.MODE_SEARCH1, max_results=1 << 16, threads=8)
    with lib.GpuIndex(c.index) as g:
        g.set_tuning(0, 4, 2, 12)
        g.set_direction_split(split)
        g.set_idle_batch(batch)
        assert g.idle_batch() == batch
        _assert_same(g.search(reads, mode=lib.MODE_SEARCH1, form=lib.FORM_BATCHED), want)
        g.set_graph(False)
        _assert_same(g.search(reads, mode=lib.MODE_SEARCH1, form=lib.FORM_BATCHED), want)


@pytest.mark.parametrize("split", [0, 1, 2])
@pytest.mark.parametrize("stack,minb", [(2, 10), (4, 1), (8, 12)])
def test_direction_split_agrees(case_factory, split, stack, minb):
    c = case_factory("repeats", 300_000, 3, 3)
    main = synth.reads(c.genome, 5000, 47, length=(3, 250), edits="mix_30_50_20")
    odd = synth.from_strings([b"", b"AC", b"ACGTN" * 5, b"GATTACA", b""] * 40)  # skipped and short reads
    seq = np.concatenate([odd.seq, main.seq, odd.seq])
    offs = np.concatenate([odd.offsets, main.offsets[1:] + odd.offsets[-1],
                           odd.offsets[1:] + odd.offsets[-1] + main.offsets[-1]]).astype(np.uint64)
    reads = synth.ReadSet(seq, offs, np.zeros(1), np.zeros(1), np.zeros(1))
    want = PortOracle(c.index).search(reads, mode=lib.MODE_SEARCH1, max_results=1 << 16, threads=8)
    with lib.GpuIndex(c.index) as g:
        g.set_tuning(0, stack, 2, minb)
        g.set_direction_split(split)
        assert g.direction_split() == split
        _assert_same(g.search(reads, mode=lib.MODE_SEARCH1, form=lib.FORM_BATCHED), want)
        g.set_graph(False)
        _assert_same(g.search(reads, mode=lib.MODE_SEARCH1, form=lib.FORM_BATCHED), want)


@pytest.mark.parametrize("form", [lib.FORM_PLAIN, lib.FORM_BATCHED])
@pytest.mark.parametrize("max_results", [100, 1024])
def test_large_intervals_match_oracle(tmp_path_factory, form, max_results):
    """Every row of every hit is located when intervals hold thousands of rows and
    the hit lists are cut at max_results (low-complexity reads)."""
    index, reads = low_complexity_case(tmp_path_factory.mktemp(f"lowcx_{form}_{max_results}"))
    ora = PortOracle(index)
    with lib.GpuIndex(index) as g:
        got = g.search(reads, mode=lib.MODE_SEARCH1, form=form, max_results=max_results)
    want = ora.search(reads, mode=lib.MODE_SEARCH1, max_results=max_results, threads=8)
    sz = np.maximum(want.hits["l"] - want.hits["k"] + 1, 0)
    assert sz.max() > 1000 and len(want.locs) == int(sz.sum())
    assert want.rs_truncated.any() or max_results > 100
    _assert_same(got, want)


@pytest.mark.parametrize("form,graph", [(lib.FORM_PLAIN, True), (lib.FORM_BATCHED, True), (lib.FORM_BATCHED, False)])
def test_locate_limit_matches_oracle(tmp_path_factory, form, graph):
    """With a locate limit, lists covering more rows keep their hits, lose their
    located rows and carry truncation bit 1, exactly as the oracle's limit."""
    index, reads = low_complexity_case(tmp_path_factory.mktemp(f"lowcx_limit_{form}_{graph}"))
    ora = PortOracle(index)
    with lib.GpuIndex(index) as g:
        g.set_graph(graph)
        g.set_locate_limit(5000)
        assert g.locate_limit() == 5000
        got = g.search(reads, mode=lib.MODE_SEARCH1, form=form, max_results=100)
        g.set_locate_limit(0)
        again = g.search(reads, mode=lib.MODE_SEARCH1, form=form, max_results=100)
    want = ora.search(reads, mode=lib.MODE_SEARCH1, max_results=100, threads=8, locate_limit=5000)
    assert (want.rs_truncated & 2).any() and len(want.locs) > 0
    _assert_same(got, want)
    _assert_same(again, ora.search(reads, mode=lib.MODE_SEARCH1, max_results=100, threads=8))


def _mixed_reads(c, n, seed, lo=3, hi=250):
    """Skipped, short and odd reads around a main batch of mixed lengths and edits."""
    main = synth.reads(c.genome, n, seed, length=(lo, hi), edits="mix_30_50_20")
    odd = synth.from_strings([b"", b"AC", b"ACGTN" * 5, b"GATTACA", b""] * 40)
    seq = np.concatenate([odd.seq, main.seq, odd.seq])
    offs = np.concatenate([odd.offsets, main.offsets[1:] + odd.offsets[-1],
                           odd.offsets[1:] + odd.offsets[-1] + main.offsets[-1]]).astype(np.uint64)
    return synth.ReadSet(seq, offs, np.zeros(1), np.zeros(1), np.zeros(1))


@pytest.mark.parametrize("group", [1, 8, 32])
@pytest.mark.parametrize("split", [0, 2])
@pytest.mark.parametrize("idle,minb", [(1, 12), (8, 12), (16, 8), (4, 1)])
def test_wave_form_agrees(case_factory, group, split, idle, minb):
    """The warp-cooperative form (reads per warp group x direction split x idle
    batch x register bound) gives the oracle's answer, direct and from the graph."""
    c = case_factory("repeats", 300_000, 3, 3)
    reads = _mixed_reads(c, 5000, 61)
    want = PortOracle(c.index).search(reads, mode=lib.MODE_SEARCH1, max_results=1 << 16, threads=8)
    with lib.GpuIndex(c.index) as g:
        g.set_tuning(0, 4, 1, minb)
        g.set_wave_group(group)
        g.set_direction_split(split)
        g.set_idle_batch(idle)
        assert g.wave_group() == group and g.get_tuning()["stack"] == -2
        _assert_same(g.search(reads, mode=lib.MODE_SEARCH1, form=lib.FORM_BATCHED), want)
        g.set_graph(False)
        _assert_same(g.search(reads, mode=lib.MODE_SEARCH1, form=lib.FORM_BATCHED), want)


@pytest.mark.parametrize("symbols", [0, 8, 11])
def test_wave_start_table_and_truncation(case_factory, symbols):
    c = case_factory("human_like", 200_000, 5, 5)
    reads = synth.reads(c.genome, 4000, 67, length=(12, 150), edits="mix_30_50_20")
    ora = PortOracle(c.index)
    with lib.GpuIndex(c.index) as g:
        g.set_start_table(symbols)
        g.set_wave_group(16)
        for mr in (0, 3, 1 << 16):
            _assert_same(g.search(reads, mode=lib.MODE_SEARCH1, form=lib.FORM_BATCHED, max_results=mr),
                         ora.search(reads, mode=lib.MODE_SEARCH1, max_results=mr, threads=8))


def test_wave_long_reads(case_factory):
    """Reads too long for a warp's 4096-base group buffer go to the fused kernel
    through the long-read list; the rest of the batch stays warp-cooperative."""
    c = case_factory("iid", 200_000, 71, 1)
    A = np.frombuffer(b"ACGT", dtype=np.uint8)
    g0 = c.genome
    long = [A[g0[1000:5100]].tobytes(), A[g0[20000:30000]].tobytes(), A[g0[50000:54065]].tobytes(),
            A[g0[60000:64050]].tobytes(), A[g0[90000:122767]].tobytes()]
    short = synth.reads(c.genome, 300, 73, length=(36, 250), edits="mix_30_50_20")
    seqs = []
    for i in range(len(short)):
        seqs.append(short.read(i))
        if i % 60 == 0:
            seqs.append(long[(i // 60) % len(long)])
    reads = synth.from_strings(seqs)
    assert np.diff(reads.offsets).max() == 32767
    want = PortOracle(c.index).search(reads, mode=lib.MODE_SEARCH1, max_results=1 << 16, threads=8)
    with lib.GpuIndex(c.index) as g:
        for split in (0, 2):
            g.set_wave_group(32)
            g.set_direction_split(split)
            _assert_same(g.search(reads, mode=lib.MODE_SEARCH1, form=lib.FORM_BATCHED), want)
            g.set_graph(False)
            _assert_same(g.search(reads, mode=lib.MODE_SEARCH1, form=lib.FORM_BATCHED), want)
            g.set_graph(True)


@pytest.mark.parametrize("max_results", [100, 1024])
def test_wave_overflowing_stacks(tmp_path_factory, max_results):
    """Low-complexity reads find more change points than a warp's stack holds:
    the rest go through the device queue and the branch launch."""
    index, reads = low_complexity_case(tmp_path_factory.mktemp(f"lowcx_wave_{max_results}"))
    want = PortOracle(index).search(reads, mode=lib.MODE_SEARCH1, max_results=max_results, threads=8)
    with lib.GpuIndex(index) as g:
        g.set_wave_group(32)
        _assert_same(g.search(reads, mode=lib.MODE_SEARCH1, form=lib.FORM_BATCHED, max_results=max_results), want)
