"""Seeds and CALs of the product (bwt_map_exact_seeds_seq, bwt_generate_cals and
the batch form) written as the text that oracle/ref/ref_harness.c:ref_seeds_cals
writes for the reference's own records."""
from __future__ import annotations

import ctypes

import numpy as np

MODE_SEEDS, MODE_CALS, MODE_WINDOW = 0, 1, 2  # MODE_WINDOW: bwt_map_exact_seeds_by_region


class Region(ctypes.Structure):  # bwt.h:185-198
    _fields_ = [("chromosome_id", ctypes.c_size_t), ("strand", ctypes.c_short), ("start", ctypes.c_size_t),
                ("end", ctypes.c_size_t), ("seq_start", ctypes.c_size_t), ("seq_end", ctypes.c_size_t),
                ("seq_len", ctypes.c_size_t), ("id", ctypes.c_int), ("pos_err", ctypes.c_int),
                ("type_err", ctypes.c_int)]


class SeedRegion(ctypes.Structure):  # bwt.h:93-111
    _fields_ = [("read_start", ctypes.c_int), ("read_end", ctypes.c_int), ("genome_start", ctypes.c_size_t),
                ("genome_end", ctypes.c_size_t), ("id", ctypes.c_int), ("fusion_left", ctypes.c_int),
                ("fusion_right", ctypes.c_int), ("strand", ctypes.c_int), ("chromosome_id", ctypes.c_int),
                ("num_mismatches", ctypes.c_int), ("pos_err", ctypes.c_int), ("type_err", ctypes.c_int),
                ("errors_list", ctypes.c_void_p), ("info", ctypes.c_void_p)]


class Cal(ctypes.Structure):  # bwt.h:123-142
    _fields_ = [("chromosome_id", ctypes.c_size_t), ("strand", ctypes.c_short), ("start", ctypes.c_size_t),
                ("end", ctypes.c_size_t), ("num_seeds", ctypes.c_size_t), ("read_area", ctypes.c_int),
                ("l_flank", ctypes.c_int), ("r_flank", ctypes.c_int), ("fill_gaps", ctypes.c_int),
                ("num_targets", ctypes.c_int), ("type_seeds", ctypes.c_int), ("num_mismatches", ctypes.c_int),
                ("sr_list", ctypes.c_void_p), ("sr_duplicate_list", ctypes.c_void_p),
                ("candidates_seeds_start", ctypes.c_void_p), ("candidates_seeds_end", ctypes.c_void_p),
                ("info", ctypes.c_void_p)]


def bind(lib) -> None:
    vp, sz = ctypes.c_void_p, ctypes.c_size_t
    lib.bwt_optarg_new.restype = vp
    lib.bwt_optarg_new.argtypes = [sz, sz, ctypes.c_int, ctypes.c_int]
    lib.bwt_optarg_free.argtypes = [vp]
    lib.cal_optarg_new.restype = vp
    lib.cal_optarg_new.argtypes = [sz] * 9
    lib.cal_optarg_free.argtypes = [vp]
    lib.array_list_new.restype = vp
    lib.array_list_new.argtypes = [sz, ctypes.c_float, ctypes.c_int]
    lib.array_list_size.restype = sz
    lib.array_list_size.argtypes = [vp]
    lib.array_list_get.restype = vp
    lib.array_list_get.argtypes = [sz, vp]
    lib.array_list_free.argtypes = [vp, vp]
    lib.linked_list_iterator_new.restype = vp
    lib.linked_list_iterator_new.argtypes = [vp]
    lib.linked_list_iterator_curr.restype = vp
    lib.linked_list_iterator_curr.argtypes = [vp]
    lib.linked_list_iterator_next.restype = vp
    lib.linked_list_iterator_next.argtypes = [vp]
    lib.linked_list_iterator_free.argtypes = [vp]
    lib.region_bwt_free.argtypes = [vp]
    lib.cal_free.argtypes = [vp]
    lib.bwt_map_exact_seeds_seq.restype = sz
    lib.bwt_map_exact_seeds_seq.argtypes = [ctypes.c_int, ctypes.c_int, vp, sz, sz, vp, vp, vp, ctypes.c_ubyte]
    lib.bwt_map_exact_seeds_by_region.restype = sz
    lib.bwt_map_exact_seeds_by_region.argtypes = [ctypes.c_int, ctypes.c_int, vp, ctypes.c_int, ctypes.c_int, vp, vp,
                                                  vp]
    lib.bwt_generate_cals.restype = sz
    lib.bwt_generate_cals.argtypes = [vp, sz, vp, vp, vp, vp, ctypes.c_uint]
    lib.bwt_generate_cals_batch.restype = sz
    lib.bwt_generate_cals_batch.argtypes = [vp, sz, sz, vp, vp, vp, vp, ctypes.c_uint]


def pack(reads: list[bytes]) -> tuple[np.ndarray, np.ndarray]:
    """NUL-terminated reads back to back and their offsets (ref_seeds_cals' input)."""
    offs = [0]
    for r in reads:
        offs.append(offs[-1] + len(r) + 1)
    buf = np.frombuffer(b"".join(r + b"\0" for r in reads) or b"\0", dtype=np.uint8).copy()
    return buf, np.array(offs, dtype=np.uint64)


def _seed(tag: str, s: SeedRegion) -> str:
    return f"{tag} {s.read_start} {s.read_end} {s.genome_start} {s.genome_end} {s.id}\n"


def _linked(lib, lst: int):
    it = lib.linked_list_iterator_new(lst)
    p = lib.linked_list_iterator_curr(it)
    while p:
        yield SeedRegion.from_address(p)
        p = lib.linked_list_iterator_next(it)
    lib.linked_list_iterator_free(it)


def _arr(lib, lst: int):
    for a in range(lib.array_list_size(lst)):
        yield SeedRegion.from_address(lib.array_list_get(a, lst))


def _write(lib, mode: int, ret: int, lst: int, out: list[str]) -> None:
    n = lib.array_list_size(lst)
    out.append(f"R {ret} {n}\n")
    for k in range(n):
        p = lib.array_list_get(k, lst)
        if mode in (MODE_SEEDS, MODE_WINDOW):
            r = Region.from_address(p)
            out.append(f"G {r.chromosome_id} {r.strand} {r.start} {r.end} {r.seq_start} {r.seq_end} {r.seq_len} "
                       f"{r.id}\n")
            lib.region_bwt_free(p)
        else:
            c = Cal.from_address(p)
            out.append(f"C {c.chromosome_id} {c.strand} {c.start} {c.end} {c.num_seeds} {c.read_area}\n")
            out.extend(_seed("S", s) for s in _linked(lib, c.sr_list))
            out.extend(_seed("D", s) for s in _linked(lib, c.sr_duplicate_list))
            out.extend(_seed("A", s) for s in _arr(lib, c.candidates_seeds_start))
            out.extend(_seed("B", s) for s in _arr(lib, c.candidates_seeds_end))
            lib.cal_free(p)
    lib.array_list_free(lst, None)


def product_seeds_cals(lib, index_handle: int, mode: int, reads: list[bytes], seed_size: int, filter_seed: int,
                       min_cal_size: int, max_intron: int, nchrom: int, batch: bool = False) -> bytes:
    """The product's records for every read in ref_seeds_cals' text form; with
    batch, the CALs of all reads come from one bwt_generate_cals_batch call."""
    opt = lib.bwt_optarg_new(1, 1, 200, filter_seed)
    copt = lib.cal_optarg_new(min_cal_size, 0, 0, 0, seed_size, 0, 0, max_intron, 0)
    bufs = [ctypes.create_string_buffer(r, len(r) + 1) for r in reads]
    out: list[str] = []
    try:
        if batch:
            arr = (ctypes.c_void_p * max(1, len(reads)))(*[ctypes.addressof(b) for b in bufs])
            lists = (ctypes.c_void_p * max(1, len(reads)))(*[lib.array_list_new(16, 1.25, 2) for _ in reads])
            lib.bwt_generate_cals_batch(arr, len(reads), seed_size, opt, copt, index_handle, lists, nchrom)
            for i in range(len(reads)):
                _write(lib, MODE_CALS, lib.array_list_size(lists[i]), lists[i], out)
        else:
            for b in bufs:
                lst = lib.array_list_new(16, 1.25, 2)
                if mode == MODE_SEEDS:
                    ret = lib.bwt_map_exact_seeds_seq(0, 0, ctypes.addressof(b), seed_size, 0, opt, index_handle,
                                                      lst, 0)
                elif mode == MODE_WINDOW:  # window [min_cal_size, len - max_intron), as ref_seeds_cals mode 2
                    L = len(b.value)
                    ret = lib.bwt_map_exact_seeds_by_region(min_cal_size, L - max_intron, ctypes.addressof(b),
                                                            seed_size, 0, opt, index_handle, lst)
                else:
                    ret = lib.bwt_generate_cals(ctypes.addressof(b), seed_size, opt, copt, index_handle, lst, nchrom)
                _write(lib, mode, ret, lst, out)
    finally:
        lib.bwt_optarg_free(opt)
        lib.cal_optarg_free(copt)
    return "".join(out).encode()
