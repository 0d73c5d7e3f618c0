"""Host side of the alignment-list layer (CPU): the library's own container
fallbacks, the bwt.h string helpers, and the recorded reference lists."""
from __future__ import annotations

import ctypes

import numpy as np

import api_lists as al
from golden_cases import GoldenCase, names
from hpgbwt import lib


def _lib():
    L = lib.load()
    al.bind(L)
    L.seq_reverse_complementary.argtypes = [ctypes.c_char_p, ctypes.c_uint]
    L.reverse_str.restype = ctypes.c_void_p
    L.reverse_str.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_size_t]
    L.bwt_anchor_new.restype = ctypes.c_void_p
    L.bwt_anchor_new.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_int]
    L.alignment_new.restype = ctypes.c_void_p
    return L


def test_array_list_fallback():
    L = _lib()
    for mode in (1, 2):
        lst = L.array_list_new(2, 1.25, mode)
        vals = [ctypes.c_int(i) for i in range(50)]
        for v in vals:
            assert L.array_list_insert(ctypes.addressof(v), lst) == 1
        assert L.array_list_size(lst) == 50
        assert [L.array_list_get(i, lst) for i in range(50)] == [ctypes.addressof(v) for v in vals]
        assert L.array_list_get(50, lst) is None
        assert L.array_list_remove_at(3, lst) == ctypes.addressof(vals[3])
        assert L.array_list_size(lst) == 49 and L.array_list_get(3, lst) == ctypes.addressof(vals[4])
        L.array_list_set_flag(7, lst)
        assert L.array_list_get_flag(lst) == 7
        L.array_list_free(lst, None)


def test_alignment_and_anchor_objects():
    L = _lib()
    a = L.alignment_new()
    aln = al.Alignment.from_address(a)
    assert aln.position == 0 and not aln.sequence
    L.alignment_free(a)
    p = L.bwt_anchor_new(1, 3, 100, 150, 0)
    x = al.Anchor.from_address(p)
    assert (x.strand, x.chromosome, x.start, x.end, x.type) == (1, 3, 100, 150, 0)
    L.bwt_anchor_free(p)


def test_string_helpers():
    L = _lib()
    for s in (b"ACGTTGCA", b"acgtN", b"A", b"GATTACA"):
        b = ctypes.create_string_buffer(s, len(s) + 1)
        L.seq_reverse_complementary(b, len(s))
        assert b.raw[:len(s)] == al._revcomp(s)
    d = ctypes.create_string_buffer(16)
    L.reverse_str(b"hello", d, 5)
    assert d.value == b"olleh"


def test_recorded_lists_parse():
    """Every recorded reference list parses to the end of its bytes."""
    for name in names():
        gc = GoldenCase(name)
        fq = gc.api_fastq()
        assert fq.n > 100
        for api, filt, flag in gc.api_runs():
            blob = gc.arrays[f"api{api}_f{filt}_g{flag}"].tobytes()
            r = al._Rd(blob)
            if api in al.PER_READ_APIS:
                lists = [al._parse_list(r) for _ in range(fq.n)]
                assert r.o == len(blob)
                assert all(x["ret"] == len(x["items"]) for x in lists)  # fresh lists: return = list size
            else:
                out = al.parse_blob(api, blob, fq.n)
                assert out["list"]["ret"] == len(out["list"]["items"])
        # the recorded runs exercise the filter flag and the anchors
        flags = {x["flag"] for x in gc.api_expected(al.API_INEXACT_READ, 3, 0, fq.n)}
        anchors = sum(it[0] == "anchor" for x in gc.api_expected(al.API_INEXACT_READ, 200, 1, fq.n)
                      for it in x["items"])
        assert anchors > 0 and (2 in flags or name == "iid_1chr")
        # and those of bwt_map_inexact_read_2 (block search): filter flag, anchors, every cigar shape
        flags2 = {x["flag"] for x in gc.api_expected(al.API_INEXACT_READ2, 3, 1, fq.n)}
        items2 = [it for x in gc.api_expected(al.API_INEXACT_READ2, 200, 1, fq.n) for it in x["items"]]
        cigars = {it[14].rstrip(b"0123456789") for it in items2 if it[0] == "aln"}
        assert flags2 == {0, 1, 2} and any(it[0] == "anchor" for it in items2)
        assert {b"=", b"M", b"X"} <= {c[-1:] for c in cigars}


def test_result_arrays_past_2gib():
    """Result arrays above 2 GiB come back whole (ctypes.string_at would wrap the size)."""
    from hpgbwt.lib import _arr, LOC_DTYPE
    n = (1 << 31) // LOC_DTYPE.itemsize + 1000
    buf = np.zeros(n, dtype=LOC_DTYPE)
    buf["hit"][-1] = 7
    out = _arr(buf.ctypes.data, n, LOC_DTYPE)
    assert len(out) == n and out["hit"][-1] == 7


def test_linked_list_fallback():
    """linked_list_* of the library (processes without hpg-libs): insert at the
    head, insert_last at the tail, iteration first to last."""
    import seed_lists as sl
    L = _lib()
    sl.bind(L)
    L.linked_list_new.restype = ctypes.c_void_p
    L.linked_list_new.argtypes = [ctypes.c_int]
    L.linked_list_insert.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    L.linked_list_insert_last.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    L.linked_list_size.restype = ctypes.c_size_t
    L.linked_list_size.argtypes = [ctypes.c_void_p]
    for f in ("linked_list_get_first", "linked_list_get_last"):
        getattr(L, f).restype = ctypes.c_void_p
        getattr(L, f).argtypes = [ctypes.c_void_p]
    L.linked_list_free.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    for mode in (1, 2):
        lst = L.linked_list_new(mode)
        vals = [ctypes.c_int(i) for i in range(6)]
        for v in vals[:3]:
            L.linked_list_insert(ctypes.addressof(v), lst)
        for v in vals[3:]:
            L.linked_list_insert_last(ctypes.addressof(v), lst)
        assert L.linked_list_size(lst) == 6
        it = L.linked_list_iterator_new(lst)
        got = []
        p = L.linked_list_iterator_curr(it)
        while p:
            got.append(p)
            p = L.linked_list_iterator_next(it)
        L.linked_list_iterator_free(it)
        want = [ctypes.addressof(vals[i]) for i in (2, 1, 0, 3, 4, 5)]
        assert got == want
        assert L.linked_list_get_first(lst) == want[0] and L.linked_list_get_last(lst) == want[-1]
        L.linked_list_free(lst, None)


def test_seed_and_cal_objects():
    """cal_new / seed_region_new / region_bwt_new / cal_optarg_new (bwt.c:128-409):
    fields as given, the CAL's read area from its first and last seed."""
    import seed_lists as sl
    L = _lib()
    sl.bind(L)
    L.seed_region_new.restype = ctypes.c_void_p
    L.seed_region_new.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_int,
                                  ctypes.c_int, ctypes.c_int]
    L.region_bwt_new.restype = ctypes.c_void_p
    L.region_bwt_new.argtypes = [ctypes.c_size_t, ctypes.c_short] + [ctypes.c_size_t] * 5 + [ctypes.c_int]
    L.cal_new.restype = ctypes.c_void_p
    L.cal_new.argtypes = [ctypes.c_size_t, ctypes.c_short, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_size_t,
                          ctypes.c_void_p, ctypes.c_void_p]
    L.linked_list_new.restype = ctypes.c_void_p
    L.linked_list_new.argtypes = [ctypes.c_int]
    L.linked_list_insert_last.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    r = sl.Region.from_address(L.region_bwt_new(3, 1, 100, 115, 4, 19, 120, 7))
    assert (r.chromosome_id, r.strand, r.start, r.end, r.seq_start, r.seq_end, r.seq_len, r.id) == \
        (3, 1, 100, 115, 4, 19, 120, 7)
    L.region_bwt_free(ctypes.addressof(r))
    sr = L.linked_list_new(2)
    L.linked_list_insert_last(L.seed_region_new(5, 30, 1000, 1025, 2, 0, 0), sr)
    L.linked_list_insert_last(L.seed_region_new(40, 90, 1035, 1085, 4, 0, 0), sr)
    c = sl.Cal.from_address(L.cal_new(1, 0, 1000, 1085, 6, sr, L.linked_list_new(2)))
    assert (c.chromosome_id, c.strand, c.start, c.end, c.num_seeds, c.read_area) == (1, 0, 1000, 1085, 6, 85)
    assert L.array_list_size(c.candidates_seeds_start) == 0 and L.array_list_size(c.candidates_seeds_end) == 0
    seeds = [(s.read_start, s.read_end, s.genome_start, s.genome_end, s.id) for s in sl._linked(L, c.sr_list)]
    assert seeds == [(5, 30, 1000, 1025, 2), (40, 90, 1035, 1085, 4)]
    L.cal_free(ctypes.addressof(c))
    o = L.cal_optarg_new(20, 0, 0, 0, 16, 0, 0, 500000, 0)
    L.cal_optarg_free(o)


def test_recorded_seed_runs_parse():
    """Every case records the reference's seeds and CALs for each run, one R line per read."""
    for name in names():
        gc = GoldenCase(name)
        reads = gc.seed_reads()
        assert len(reads) > 100 and all(len(r) >= 40 for r in reads)
        runs = gc.seed_runs()
        assert {m for m, *_ in runs} == {0, 1, 2}
        for run in runs:
            text = gc.seed_expected(*run).decode()
            assert sum(1 for line in text.splitlines() if line.startswith("R ")) == len(reads)
