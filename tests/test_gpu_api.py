"""The alignment-list entry points (bwt_map_exact_*, bwt_map_inexact_*) on the
GPU against the reference's own lists recorded in the golden fixtures: every
field of every alignment and anchor, list flags, return values, unmapped
batches."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

import api_lists as al
from golden_cases import GoldenCase, names
from hpgbwt import lib

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def loaded(tmp_path_factory):
    L = lib.load()
    al.bind(L)
    out = {}
    for name in names():
        gc = GoldenCase(name)
        out[name] = (gc, gc.build(tmp_path_factory.mktemp("api_" + name)))
    return L, out


@pytest.mark.parametrize("name", names())
def test_entry_points_match_reference(loaded, name):
    L, cases = loaded
    gc, index = cases[name]
    fq = gc.api_fastq()
    with lib.GpuIndex(index) as g:
        for api, filt, flag in gc.api_runs():
            want = gc.api_expected(api, filt, flag, fq.n)
            got = al.product_map(L, g.handle, api, fq, filt, flag)
            if isinstance(want, list):
                assert len(got) == len(want)
                for i, (a, b) in enumerate(zip(got, want)):
                    assert a == b, f"api {api} filter {filt} flag {flag} read {i}: {a} != {b}"
            else:
                assert got == want, f"api {api} filter {filt} flag {flag}"


@pytest.mark.parametrize("name", names())
def test_batch_forms_equal_per_read(loaded, name):
    """bwt_map_inexact_batch / _array_list: each read as bwt_map_inexact_read maps it."""
    L, cases = loaded
    gc, index = cases[name]
    fq = gc.api_fastq()
    for filt in (200, 3):
        per_read = gc.api_expected(al.API_INEXACT_READ, filt, 0, fq.n)
        with lib.GpuIndex(index) as g:
            got = al.product_map(L, g.handle, al.API_INEXACT_BATCH, fq, filt)
        items = [it for r in per_read for it in r["items"]]
        assert got["list"]["items"] == items
        unmapped = [i for i, r in enumerate(per_read) if not any(it[6] for it in r["items"])]
        assert len(got["unmapped"]) == len(unmapped)
        for (h, s, q), i in zip(got["unmapped"], unmapped):
            assert h == fq.idl[i] + b"\0" and s == fq.seqs[i] + b"\0" and q == fq.quals[i] + b"\0"


@pytest.mark.parametrize("name", names())
def test_array_list_form(loaded, name):
    L, cases = loaded
    gc, index = cases[name]
    fq = gc.api_fastq()
    want = gc.api_expected(al.API_INEXACT_READ, 200, 1, fq.n)
    keep = []
    reads = L.array_list_new(fq.n + 1, 1.25, 2)
    lists = (ctypes.c_void_p * fq.n)()
    for i in range(fq.n):
        r = al.FastqRead()
        o = int(fq.offs[i])
        r.id = fq.ids.ctypes.data + int(fq.id_offs[i])
        r.sequence = fq.seq.ctypes.data + o
        r.quality = fq.qual.ctypes.data + o
        rc = ctypes.create_string_buffer(al._revcomp(fq.seqs[i]), len(fq.seqs[i]) + 1)
        r.revcomp = ctypes.addressof(rc)
        keep += [r, rc]
        L.array_list_insert(ctypes.addressof(r), reads)
        lists[i] = L.array_list_new(8, 1.25, 2)
        L.array_list_set_flag(1, lists[i])
    opt = L.bwt_optarg_new(1, 1, 200, 200)
    n_un = ctypes.c_size_t()
    un = (ctypes.c_size_t * fq.n)()
    with lib.GpuIndex(index) as g:
        L.bwt_map_inexact_array_list(reads, opt, g.handle, lists, ctypes.byref(n_un), un)
    L.bwt_optarg_free(opt)
    for i in range(fq.n):
        anchors = len(fq.seqs[i]) >= 5 and L.array_list_get_flag(lists[i]) == 1
        got = al.walk_list(L, lists[i], want[i]["ret"], anchors, qmax=len(fq.seqs[i]))
        assert got == want[i], f"read {i}"
    assert list(un[:n_un.value]) == [i for i, r in enumerate(want) if not any(
        it[0] == "aln" and it[6] for it in r["items"])]
    L.array_list_free(reads, None)


@pytest.mark.parametrize("name", names())
def test_array_list_form_shared_list(loaded, name):
    """bwt_map_inexact_array_list with one list named for every read maps them as
    bwt_map_inexact_read called read after read on that list (the records of a read
    can depend on what the list already holds: bwt.c:2234-2237 re-marks its first
    alignment), so the records are built in read order on one thread."""
    L, cases = loaded
    gc, index = cases[name]
    fq = gc.api_fastq()
    keep = []
    reads = L.array_list_new(fq.n + 1, 1.25, 2)
    shared = L.array_list_new(64, 1.25, 2)
    one_by_one = L.array_list_new(64, 1.25, 2)
    lists = (ctypes.c_void_p * fq.n)(*([shared] * fq.n))
    opt = L.bwt_optarg_new(1, 1, 3, 3)  # a small filter: some strands pass it and set the flag
    with lib.GpuIndex(index) as g:
        for i in range(fq.n):
            r = al.FastqRead()
            o = int(fq.offs[i])
            r.id = fq.ids.ctypes.data + int(fq.id_offs[i])
            r.sequence = fq.seq.ctypes.data + o
            r.quality = fq.qual.ctypes.data + o
            rc = ctypes.create_string_buffer(al._revcomp(fq.seqs[i]), len(fq.seqs[i]) + 1)
            r.revcomp = ctypes.addressof(rc)
            r.length = len(fq.seqs[i])
            keep += [r, rc]
            L.array_list_insert(ctypes.addressof(r), reads)
            L.bwt_map_inexact_read(ctypes.byref(r), opt, g.handle, one_by_one)
        n_un = ctypes.c_size_t()
        un = (ctypes.c_size_t * fq.n)()
        L.bwt_map_inexact_array_list(reads, opt, g.handle, lists, ctypes.byref(n_un), un)
    L.bwt_optarg_free(opt)
    got = al.walk_list(L, shared, 0, False)
    want = al.walk_list(L, one_by_one, 0, False)
    assert len(got["items"]) > fq.n // 4
    assert got == want
    L.array_list_free(reads, None)


def test_edge_reads_do_not_break(loaded):
    """Reads the reference cannot take (empty, 1-3 bases, N, lower case) map without faults."""
    L, cases = loaded
    gc, index = cases[names()[0]]
    fq = al.FastqSet([b"", b"A", b"AC", b"ACG", b"ACGTN" * 8, b"acgtacgtacgtacgtacgt", b"NNNN"])
    with lib.GpuIndex(index) as g:
        ex = al.product_map(L, g.handle, al.API_EXACT_READ, fq, 200)
        inx = al.product_map(L, g.handle, al.API_INEXACT_READ, fq, 200, 1)
    assert all(r["ret"] == len(r["items"]) for r in ex)
    for i in range(4):  # under 5 bases: one unmapped record
        assert inx[i]["ret"] == 1 and inx[i]["items"][0][4] == 1 and inx[i]["items"][0][6] == 0
        assert inx[i]["items"][0][14] == b"%dX" % len(fq.seqs[i])
