"""The k-error block search on the GPU (bwt_gpu_block_search: BWSearchCPU as
bwt_map_inexact_read_2 runs it) against the reference's recorded outputs and
the CPU oracle, and bwt_map_inexact_read_2's array-list form against its
per-read calls."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

import api_lists as al
from golden_cases import GoldenCase, names
from hpgbwt import lib, synth
from oracle.pyoracle import PortOracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def golden(tmp_path_factory):
    out = {}
    for name in names():
        gc = GoldenCase(name)
        out[name] = (gc, gc.build(tmp_path_factory.mktemp("blk_" + name)))
    return out


@pytest.mark.parametrize("name", names())
def test_block_search_matches_reference_fixtures(golden, name):
    """Results, located rows and anchors equal the reference's at every recorded
    capacity; the refused-result bits equal the oracle's."""
    gc, index = golden[name]
    ora = PortOracle(index)
    with lib.GpuIndex(index) as g:
        for mr in gc.block_capacities():
            got = g.block_search(gc.reads, max_results=mr)
            assert got.equal(gc.block_expected(mr), truncation=False), mr
            assert got.equal(ora.block_search(gc.reads, max_results=mr, threads=8)), mr
            assert g.block_search_ms() > 0
    ora.close()


@pytest.mark.parametrize("kind,n,seed,chroms,length,edits,caps", [
    ("repeats", 300_000, 3, 3, (3, 250), "mix_30_50_20", [1 << 16, 0, 1, 3, 8]),
    ("iid", 200_000, 4, 1, (55, 130), "per_base_capped", [1 << 16, 2]),
    ("human_like", 120_000, 5, 2, (20, 400), "mix_30_50_20", [1 << 16, 5]),
])
def test_block_search_matches_oracle(case_factory, kind, n, seed, chroms, length, edits, caps):
    c = case_factory(kind, n, seed, chroms)
    main = synth.reads(c.genome, 4000, seed + 60, length=length, edits=edits)
    odd = synth.from_strings([b"", b"AC", b"ACGTN" * 5, b"GATTACA", b"A" * 61, b""] * 20)
    seq = np.concatenate([odd.seq, main.seq])
    offs = np.concatenate([odd.offsets, main.offsets[1:] + odd.offsets[-1]]).astype(np.uint64)
    reads = synth.ReadSet(seq, offs, np.zeros(1), np.zeros(1), np.zeros(1))
    ora = PortOracle(c.index)
    with lib.GpuIndex(c.index) as g:
        for mr in caps:
            want = ora.block_search(reads, max_results=mr, threads=8)
            got = g.block_search(reads, max_results=mr)
            assert got.equal(want), mr
    ora.close()


def test_block_search_repetitive_reads_and_locate_limit(tmp_path):
    """Homopolymer and tandem reads: many results per list (the slot overflow
    path), lists cut by their capacity, and the locate limit."""
    from low_complexity import low_complexity_case
    index, reads = low_complexity_case(tmp_path)
    ora = PortOracle(index)
    with lib.GpuIndex(index) as g:
        for mr in (1 << 16, 100, 7):
            want = ora.block_search(reads, max_results=mr, threads=8)
            got = g.block_search(reads, max_results=mr)
            assert got.equal(want), mr
            if mr >= 100:
                assert (got.result.rs_count > 4).any()  # more results than first-pass slots
        # at 7, a homopolymer read's ~75 branch points per block overflow the list:
        # the reference drops the block's branches
        assert (want.result.rs_truncated & 1).any()
        g.set_locate_limit(5000)
        lim = g.block_search(reads, max_results=100)
        want = ora.block_search(reads, max_results=100, threads=8, locate_limit=5000)
        assert lim.equal(want)
        assert (lim.result.rs_truncated & 2).any()
    ora.close()


def test_block_search_empty_batch(golden):
    gc, index = golden[names()[0]]
    empty = synth.from_strings([])
    with lib.GpuIndex(index) as g:
        got = g.block_search(empty)
    assert len(got.result.hits) == 0 and len(got.n_anchors) == 0


@pytest.mark.parametrize("filt,flag", [(200, 0), (3, 1), (0, 1)])
def test_array_list_2_equals_per_read(golden, filt, flag):
    """bwt_map_inexact_array_list_2: every read as bwt_map_inexact_read_2 maps it
    (the reference's own lists, recorded in the fixtures)."""
    L = lib.load()
    al.bind(L)
    gc, index = golden["repeats_3chr"]
    fq = gc.api_fastq()
    want = gc.api_expected(al.API_INEXACT_READ2, filt, flag, fq.n)
    reads = L.array_list_new(fq.n + 1, 1.25, 2)
    lists = (ctypes.c_void_p * fq.n)()
    keep = []
    for i in range(fq.n):
        r = al.FastqRead()
        o = int(fq.offs[i])
        r.id = fq.ids.ctypes.data + int(fq.id_offs[i])
        r.sequence = fq.seq.ctypes.data + o
        r.quality = fq.qual.ctypes.data + o
        r.length = len(fq.seqs[i])
        keep.append(r)
        L.array_list_insert(ctypes.addressof(r), reads)
        lists[i] = L.array_list_new(16, 1.25, 2)
        L.array_list_set_flag(flag, lists[i])
    unmapped = (ctypes.c_size_t * fq.n)()
    n_un = ctypes.c_size_t()
    opt = L.bwt_optarg_new(1, 1, filt, filt)
    with lib.GpuIndex(index) as g:
        L.bwt_map_inexact_array_list_2(reads, opt, g.handle, lists, ctypes.byref(n_un), unmapped)
    L.bwt_optarg_free(opt)
    got_unmapped = []
    for i in range(fq.n):
        L_i = len(fq.seqs[i])
        anchors = L_i >= 5 and L.array_list_get_flag(lists[i]) == 1
        got = al.walk_list(L, lists[i], want[i]["ret"], anchors, qmax=L_i)
        assert got["flag"] == want[i]["flag"] and got["items"] == want[i]["items"], i
        if not any(it[0] == "aln" and it[6] for it in got["items"]):
            got_unmapped.append(i)
    assert list(unmapped[:n_un.value]) == got_unmapped
    L.array_list_free(reads, None)
