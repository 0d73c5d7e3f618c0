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
            if api in (al.API_EXACT_READ, al.API_INEXACT_READ):
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


def test_result_arrays_past_2gib():
    """Result arrays above 2 GiB come back whole (ctypes.string_at would wrap the size)."""
    from hpgbwt.lib import _arr, LOC_DTYPE
    n = (1 << 31) // LOC_DTYPE.itemsize + 1000
    buf = np.zeros(n, dtype=LOC_DTYPE)
    buf["hit"][-1] = 7
    out = _arr(buf.ctypes.data, n, LOC_DTYPE)
    assert len(out) == n and out["hit"][-1] == 7
