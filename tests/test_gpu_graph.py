"""The batched form replayed from a captured CUDA graph: identical to the
stage-by-stage launch and to the oracle, across capacity classes, pool growth
(result, spill and locate pools sized too small on purpose by the data) and
both the host and the device entry points."""
from __future__ import annotations

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


@pytest.fixture(scope="module")
def copies_case(tmp_path_factory):
    """60 kbp with 150 copies of one 300 bp element at ~98 % identity: reads
    there carry dozens of 1-error hits and hundreds of located rows, more than
    the first capture of a 4096-read plan holds."""
    rng = np.random.default_rng(8)
    g = synth.genome("iid", 60_000, 45)
    elem = rng.integers(0, 4, 300, dtype=np.uint8)
    for c in range(150):
        cp = elem.copy()
        m = rng.random(300) < 0.02
        cp[m] = rng.integers(0, 4, int(m.sum()), dtype=np.uint8)
        g[12_000 + c * 300: 12_000 + (c + 1) * 300] = cp
    d = tmp_path_factory.mktemp("copies")
    synth.write_fasta(str(d / "g.fa"), g, [30_000, 30_000])
    lib.build_index(str(d / "g.fa"), str(d / "idx"), 16)
    return g, str(d / "idx")


@pytest.mark.parametrize("stack", [4, 2, 0, -1])
def test_graph_pools_grow(copies_case, stack):
    g0, index = copies_case
    reads = synth.reads(g0, 4000, 9, length=(30, 100), edits="mix_30_50_20")
    want = PortOracle(index).search(reads, mode=lib.MODE_SEARCH1, max_results=1 << 16, threads=8)
    assert len(want.hits) > 4 * 4096 + 4096 and len(want.locs) > 8 * 4096 + 4096  # both first pools overflow
    with lib.GpuIndex(index) as g:
        g.set_tuning(0, stack, 1, 1)
        assert g.graph()
        got = g.search(reads, mode=lib.MODE_SEARCH1, form=lib.FORM_BATCHED)
        _same(got, want)
        again = g.search(reads, mode=lib.MODE_SEARCH1, form=lib.FORM_BATCHED)  # grown plan reused
        _same(again, want)
        g.set_graph(False)
        _same(g.search(reads, mode=lib.MODE_SEARCH1, form=lib.FORM_BATCHED), want)


def test_graph_batches_of_every_size(case_factory):
    """One engine, batches of changing size (same class, new class, empty):
    each equals the oracle on its own reads."""
    c = case_factory("repeats", 300_000, 3, 3)
    ora = PortOracle(c.index)
    with lib.GpuIndex(c.index) as g:
        for i, n in enumerate([3000, 100, 0, 3000, 5000, 1, 4096, 4097]):
            reads = synth.reads(c.genome, n, 50 + i, length=(36, 250), edits="mix_30_50_20") if n else \
                synth.from_strings([])
            for mr in (1 << 16, 3):
                got = g.search(reads, mode=lib.MODE_SEARCH1, form=lib.FORM_BATCHED, max_results=mr)
                _same(got, ora.search(reads, mode=lib.MODE_SEARCH1, max_results=mr, threads=8))


def test_graph_device_entry(case_factory):
    torch = pytest.importorskip("torch")
    c = case_factory("human_like", 200_000, 5, 5)
    reads = synth.reads(c.genome, 6000, 61, length=(20, 150), edits="mix_30_50_20")
    want = PortOracle(c.index).search(reads, mode=lib.MODE_SEARCH1, max_results=1 << 16, threads=8)
    d_seq = torch.from_numpy(reads.seq).cuda()
    d_off = torch.from_numpy(reads.offsets.view(np.int64)).cuda()
    with lib.GpuIndex(c.index) as g:
        for graph in (True, False, True):
            g.set_graph(graph)
            rs = g.search_device(d_seq.data_ptr(), d_off.data_ptr(), len(reads), int(reads.offsets[-1]),
                                 int(np.diff(reads.offsets).max()), form=lib.FORM_BATCHED)
            hits = np.zeros(rs.n_hits, lib.HIT_DTYPE)
            locs = np.zeros(rs.n_locs, lib.LOC_DTYPE)
            cnt = np.zeros(2 * len(reads), np.uint32)
            tr = np.zeros(2 * len(reads), np.uint8)
            g.copy_result(rs, hits.ctypes.data, locs.ctypes.data, cnt.ctypes.data, tr.ctypes.data)
            assert np.array_equal(cnt, want.rs_count) and np.array_equal(tr, want.rs_truncated)
            assert np.array_equal(hits, want.hits) and np.array_equal(locs, want.locs)
            ms = g.stage_ms()
            assert ms[1] > 0 and ms[3] >= 0


def test_graph_replay_launches_counted(case_factory):
    """A replay adds its captured kernel nodes to the launch count."""
    c = case_factory("repeats", 300_000, 3, 3)
    reads = synth.reads(c.genome, 2000, 71, length=100, edits="per_base_capped")
    with lib.GpuIndex(c.index) as g:
        g.search(reads, form=lib.FORM_BATCHED)  # captures
        n0 = lib.launch_count()
        g.search(reads, form=lib.FORM_BATCHED)
        per_replay = lib.launch_count() - n0
        g.search(reads, form=lib.FORM_BATCHED)
        assert lib.launch_count() - n0 == 2 * per_replay and per_replay >= 10


def test_graph_rejects_bad_offsets(case_factory):
    """The graph checks read offsets on the device: bad reads are switched off
    before any kernel reads them and the call fails; the next call is clean."""
    c = case_factory("repeats", 300_000, 3, 3)
    good = synth.reads(c.genome, 500, 81, length=100)
    want = PortOracle(c.index).search(good, mode=lib.MODE_SEARCH1, max_results=1 << 16, threads=8)
    seq = np.frombuffer(b"ACGT" * 20000, dtype=np.uint8)
    bad_sets = [np.array([0, 100, 50, 150], dtype=np.uint64),        # decreasing inside the batch
                np.array([0, 40_000, 40_100], dtype=np.uint64)]      # a read longer than 32767 bases

    class RS:
        pass
    with lib.GpuIndex(c.index) as g:
        for offs in bad_sets:
            rs = RS()
            rs.seq, rs.offsets = seq, offs
            with pytest.raises(RuntimeError, match="non-decreasing"):
                g.search(rs, form=lib.FORM_BATCHED)
            _same(g.search(good, form=lib.FORM_BATCHED), want)


def test_pipelined_host_batches(tmp_path_factory):
    """Host batches of 2+ chunks run with their copies overlapping other chunks'
    replays; a chunk whose pools overflow (read-dense repeat copies) is grown and
    rerun inside the pipeline.  Equal to the stage-by-stage form and the oracle."""
    rng = np.random.default_rng(18)
    g0 = synth.genome("repeats", 400_000, 61)
    elem = rng.integers(0, 4, 300, dtype=np.uint8)
    for k in range(150):
        cp = elem.copy()
        m = rng.random(300) < 0.02
        cp[m] = rng.integers(0, 4, int(m.sum()), dtype=np.uint8)
        g0[200_000 + k * 300: 200_000 + (k + 1) * 300] = cp
    d = tmp_path_factory.mktemp("pipe")
    synth.write_fasta(str(d / "g.fa"), g0, [200_000, 200_000])
    lib.build_index(str(d / "g.fa"), str(d / "idx"), 16)
    normal = synth.reads_fast(g0[:190_000], 480_000, 71, 100, "per_base_capped")
    heavy = synth.reads(g0[200_000:245_000], 60_000, 72, length=(60, 100), edits="mix_30_50_20")
    seqs = [normal.seq[:int(normal.offsets[300_000])], heavy.seq, normal.seq[int(normal.offsets[300_000]):]]
    offs = np.concatenate([normal.offsets[:300_001],
                           heavy.offsets[1:] + normal.offsets[300_000],
                           normal.offsets[300_001:] - normal.offsets[300_000] + normal.offsets[300_000]
                           + heavy.offsets[-1]]).astype(np.uint64)
    reads = synth.ReadSet(np.concatenate(seqs), offs, np.zeros(1), np.zeros(1), np.zeros(1))
    assert len(reads) == 540_000
    want = PortOracle(str(d / "idx")).search(reads, mode=lib.MODE_SEARCH1, max_results=1 << 16, threads=16)
    with lib.GpuIndex(str(d / "idx")) as g:
        g.set_pipeline_chunk(262144)  # 3 chunks
        for _ in range(2):  # the second call reuses grown plans and result sizing
            _same(g.search(reads, mode=lib.MODE_SEARCH1, form=lib.FORM_BATCHED), want)
        g.set_graph(False)
        _same(g.search(reads, mode=lib.MODE_SEARCH1, form=lib.FORM_BATCHED), want)


def test_device_bases_at_any_address(case_factory):
    """The graph form encodes a caller's device bases where they are: a buffer
    that starts one byte past an aligned address (16-byte vector loads cannot
    be used) gives the same records as the plain form and the oracle."""
    torch = pytest.importorskip("torch")
    c = case_factory("repeats", 300_000, 3, 3)
    reads = synth.reads(c.genome, 5000, 62, length=(36, 250), edits="mix_30_50_20")
    want = PortOracle(c.index).search(reads, mode=lib.MODE_SEARCH1, max_results=1 << 16, threads=8)
    buf = torch.zeros(len(reads.seq) + 64, dtype=torch.uint8, device="cuda")
    buf[1:1 + len(reads.seq)] = torch.from_numpy(reads.seq).cuda()
    d_off = torch.from_numpy(reads.offsets.view(np.int64)).cuda()
    with lib.GpuIndex(c.index) as g:
        for form in (lib.FORM_BATCHED, lib.FORM_PLAIN, lib.FORM_BATCHED):
            rs = g.search_device(buf.data_ptr() + 1, d_off.data_ptr(), len(reads), int(reads.offsets[-1]),
                                 int(np.diff(reads.offsets).max()), form=form)
            hits = np.zeros(rs.n_hits, lib.HIT_DTYPE)
            locs = np.zeros(rs.n_locs, lib.LOC_DTYPE)
            cnt = np.zeros(2 * len(reads), np.uint32)
            tr = np.zeros(2 * len(reads), np.uint8)
            g.copy_result(rs, hits.ctypes.data, locs.ctypes.data, cnt.ctypes.data, tr.ctypes.data)
            assert np.array_equal(cnt, want.rs_count) and np.array_equal(tr, want.rs_truncated)
            assert np.array_equal(hits, want.hits) and np.array_equal(locs, want.locs)
