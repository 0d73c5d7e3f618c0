"""Alignment lists of the hpg-libs entry points (bwt_map_exact_*, bwt_map_inexact_*),
as comparable Python values: from the reference (serialised by
oracle/ref/ref_harness.c:ref_map_api, stored in the golden fixtures) and from the
product (walked through ctypes over the library's own array_list_t and
alignment_t)."""
from __future__ import annotations

import ctypes
import struct

import numpy as np

API_EXACT_READ, API_EXACT_SEQS, API_EXACT_BATCH, API_INEXACT_READ, API_INEXACT_BATCH = 0, 1, 2, 3, 4
API_INEXACT_READ2 = 5  # bwt_map_inexact_read_2 per read
PER_READ_APIS = (API_EXACT_READ, API_INEXACT_READ, API_INEXACT_READ2)


class FastqSet:
    """Reads as NUL-terminated sequence / quality / id strings; offs[i+1]-offs[i] = len+1."""

    def __init__(self, seqs: list[bytes], ids: list[bytes] | None = None, quals: list[bytes] | None = None):
        n = len(seqs)
        if ids is None:
            ids = [(b"@read%d desc/%d" % (i, i % 2 + 1)) if i % 3 else (b"read%d" % i) for i in range(n)]
        if quals is None:
            quals = [bytes(33 + (7 * i + j) % 40 for j in range(len(s))) for i, s in enumerate(seqs)]
        self.n = n
        self.seqs, self.quals, self.idl = seqs, quals, ids
        self.seq = np.frombuffer(b"".join(s + b"\0" for s in seqs) + b"\0", dtype=np.uint8).copy()
        self.qual = np.frombuffer(b"".join(q + b"\0" for q in quals) + b"\0", dtype=np.uint8).copy()
        self.offs = np.zeros(n + 1, dtype=np.uint64)
        np.cumsum([len(s) + 1 for s in seqs], out=self.offs[1:]) if n else None
        self.ids = np.frombuffer(b"".join(i + b"\0" for i in ids) + b"\0", dtype=np.uint8).copy()
        self.id_offs = np.zeros(n + 1, dtype=np.uint64)
        np.cumsum([len(i) + 1 for i in ids], out=self.id_offs[1:]) if n else None


# ---------------------------------------------------------------- parsing --

class _Rd:
    def __init__(self, b: bytes):
        self.b, self.o = b, 0

    def take(self, fmt: str):
        v = struct.unpack_from("<" + fmt, self.b, self.o)
        self.o += struct.calcsize("<" + fmt)
        return v if len(v) > 1 else v[0]

    def str(self):
        n = self.take("I")
        if n == 0xFFFFFFFF:
            return None
        s = self.b[self.o:self.o + n]
        self.o += n
        return s


def _parse_list(r: _Rd):
    n, flag, ret, anchors = r.take("IiQB")
    items = []
    for _ in range(n):
        if anchors:
            items.append(("anchor",) + tuple(r.take("iiQQi")))
        else:
            head = r.take("IiiiBBBiii")
            qn, sq, ql, cg = r.str(), r.str(), r.str(), r.str()
            ol = r.take("i")
            opt = r.b[r.o:r.o + max(ol, 0)]
            r.o += max(ol, 0)
            items.append(("aln",) + tuple(head) + (qn, sq, ql, cg, ol, opt))
    return {"flag": flag, "ret": ret, "items": items}


def parse_blob(api: int, blob: bytes, n_reads: int):
    r = _Rd(blob)
    if api in PER_READ_APIS:
        return [_parse_list(r) for _ in range(n_reads)]
    out = {"list": _parse_list(r)}
    if api == API_EXACT_SEQS:
        out["status"] = list(r.b[r.o:r.o + n_reads])
    else:
        u = r.take("I")
        out["unmapped"] = [(r.str(), r.str(), r.str()) for _ in range(u)]
    return out


# ---------------------------------------------------------------- product --

class FastqRead(ctypes.Structure):
    _fields_ = [("id", ctypes.c_void_p), ("sequence", ctypes.c_void_p), ("revcomp", ctypes.c_void_p),
                ("quality", ctypes.c_void_p), ("rev_quality", ctypes.c_void_p), ("adapter", ctypes.c_void_p),
                ("adapter_revcomp", ctypes.c_void_p), ("adapter_quality", ctypes.c_void_p),
                ("length", ctypes.c_int), ("adapter_length", ctypes.c_int), ("adapter_strand", ctypes.c_int)]


class FastqBatch(ctypes.Structure):
    _fields_ = [("num_reads", ctypes.c_ulong), ("data_indices_size", ctypes.c_ulong), ("data_size", ctypes.c_ulong),
                ("source_id", ctypes.c_int), ("header_indices", ctypes.c_void_p), ("header", ctypes.c_void_p),
                ("data_indices", ctypes.c_void_p), ("seq", ctypes.c_void_p), ("quality", ctypes.c_void_p)]


class Alignment(ctypes.Structure):
    _fields_ = [("optional_fields_length", ctypes.c_int), ("chromosome", ctypes.c_uint), ("position", ctypes.c_int),
                ("mate_position", ctypes.c_int), ("mate_chromosome", ctypes.c_int),
                ("template_length", ctypes.c_int), ("map_quality", ctypes.c_int), ("mapq", ctypes.c_int),
                ("num_cigar_operations", ctypes.c_int), ("map_len", ctypes.c_int),
                ("is_paired_end", ctypes.c_uint8), ("is_paired_end_mapped", ctypes.c_uint8),
                ("is_seq_mapped", ctypes.c_uint8), ("is_mate_mapped", ctypes.c_uint8),
                ("seq_strand", ctypes.c_uint8), ("mate_strand", ctypes.c_uint8), ("pair_num", ctypes.c_uint8),
                ("secondary_alignment", ctypes.c_uint8), ("fails_quality_check", ctypes.c_uint8),
                ("pc_optical_duplicate", ctypes.c_uint8), ("query_name", ctypes.c_void_p),
                ("sequence", ctypes.c_void_p), ("quality", ctypes.c_void_p), ("cigar", ctypes.c_void_p),
                ("optional_fields", ctypes.c_void_p), ("alig_data", ctypes.c_void_p)]


class Anchor(ctypes.Structure):
    _fields_ = [("strand", ctypes.c_int), ("chromosome", ctypes.c_int), ("start", ctypes.c_size_t),
                ("end", ctypes.c_size_t), ("type", ctypes.c_int)]


def bind(lib) -> None:
    vp, sz = ctypes.c_void_p, ctypes.c_size_t
    lib.bwt_optarg_new.restype = vp
    lib.bwt_optarg_new.argtypes = [sz, sz, ctypes.c_int, ctypes.c_int]
    lib.bwt_optarg_free.argtypes = [vp]
    lib.array_list_new.restype = vp
    lib.array_list_new.argtypes = [sz, ctypes.c_float, ctypes.c_int]
    lib.array_list_size.restype = sz
    lib.array_list_size.argtypes = [vp]
    lib.array_list_get.restype = vp
    lib.array_list_get.argtypes = [sz, vp]
    lib.array_list_get_flag.argtypes = [vp]
    lib.array_list_set_flag.argtypes = [ctypes.c_int, vp]
    lib.array_list_insert.argtypes = [vp, vp]
    lib.array_list_remove_at.restype = vp
    lib.array_list_remove_at.argtypes = [sz, vp]
    lib.array_list_free.argtypes = [vp, vp]
    lib.alignment_free.argtypes = [vp]
    lib.bwt_anchor_free.argtypes = [vp]
    for f in ("bwt_map_exact_read", "bwt_map_inexact_read", "bwt_map_inexact_read_2"):
        getattr(lib, f).restype = sz
        getattr(lib, f).argtypes = [vp, vp, vp, vp]
    lib.bwt_map_exact_seqs.restype = sz
    lib.bwt_map_exact_seqs.argtypes = [vp, sz, vp, vp, vp, vp]
    for f in ("bwt_map_exact_batch", "bwt_map_inexact_batch"):
        getattr(lib, f).restype = sz
        getattr(lib, f).argtypes = [vp, vp, vp, vp, vp]
    for f in ("bwt_map_inexact_array_list", "bwt_map_inexact_array_list_2"):
        getattr(lib, f).restype = sz
        getattr(lib, f).argtypes = [vp, vp, vp, vp, vp, vp]


def _cstr(p, maxlen=None):
    if not p:
        return None
    s = ctypes.string_at(p)
    return s if maxlen is None else s[:maxlen]


def walk_list(lib, lst: int, ret: int, anchors: bool, qmax=None, free: bool = True):
    n = lib.array_list_size(lst)
    items = []
    for i in range(n):
        p = lib.array_list_get(i, lst)
        if anchors:
            a = Anchor.from_address(p)
            items.append(("anchor", a.strand, a.chromosome, a.start, a.end, a.type))
            if free:
                lib.bwt_anchor_free(p)
        else:
            a = Alignment.from_address(p)
            ol = a.optional_fields_length
            opt = ctypes.string_at(a.optional_fields, ol) if ol > 0 and a.optional_fields else b""
            items.append(("aln", a.chromosome, a.position, a.map_quality, a.num_cigar_operations, a.seq_strand,
                          a.is_seq_mapped, a.secondary_alignment, a.mate_position, a.mate_chromosome,
                          a.template_length, _cstr(a.query_name), _cstr(a.sequence), _cstr(a.quality, qmax),
                          _cstr(a.cigar), ol, opt))
            if free:
                lib.alignment_free(p)
    flag = lib.array_list_get_flag(lst)
    if free:
        lib.array_list_free(lst, None)
    return {"flag": flag, "ret": ret, "items": items}


def product_map(lib, index_handle: int, api: int, fq: FastqSet, filter_read_mappings: int, flag: int = 0):
    """The product's entry point on the same reads, shaped like parse_blob's output."""
    inexact = api in (API_INEXACT_READ, API_INEXACT_READ2)
    opt = lib.bwt_optarg_new(1 if inexact else 0, 1, filter_read_mappings, filter_read_mappings)
    try:
        if api in PER_READ_APIS:
            out = []
            for i in range(fq.n):
                o = int(fq.offs[i])
                r = FastqRead()
                r.id = fq.ids.ctypes.data + int(fq.id_offs[i])
                r.sequence = fq.seq.ctypes.data + o
                r.quality = fq.qual.ctypes.data + o
                L = len(fq.seqs[i])
                rc = ctypes.create_string_buffer(_revcomp(fq.seqs[i]), L + 1)
                r.revcomp = ctypes.addressof(rc)
                r.length = L
                lst = lib.array_list_new(16, 1.25, 2)
                lib.array_list_set_flag(flag if inexact else 0, lst)
                f = {API_EXACT_READ: lib.bwt_map_exact_read, API_INEXACT_READ: lib.bwt_map_inexact_read,
                     API_INEXACT_READ2: lib.bwt_map_inexact_read_2}[api]
                ret = f(ctypes.byref(r), opt, index_handle, lst)
                anchors = inexact and L >= 5 and lib.array_list_get_flag(lst) == 1
                out.append(walk_list(lib, lst, ret, anchors, qmax=L))
            return out
        if api == API_EXACT_SEQS:
            arr = (ctypes.c_void_p * max(1, fq.n))(*[fq.seq.ctypes.data + int(fq.offs[i]) for i in range(fq.n)])
            status = ctypes.create_string_buffer(fq.n + 1)
            lst = lib.array_list_new(16, 1.25, 1)
            ret = lib.bwt_map_exact_seqs(arr, fq.n, opt, index_handle, status, lst)
            return {"list": walk_list(lib, lst, ret, False), "status": list(status.raw[:fq.n])}
        # batch forms
        hidx = np.ascontiguousarray(fq.id_offs.astype(np.int32))
        didx = np.ascontiguousarray(fq.offs.astype(np.int32))
        b = FastqBatch(num_reads=fq.n, header_indices=hidx.ctypes.data, header=fq.ids.ctypes.data,
                       data_indices=didx.ctypes.data, seq=fq.seq.ctypes.data, quality=fq.qual.ctypes.data)
        uh = np.zeros(fq.n + 1, np.int32)
        ud = np.zeros(fq.n + 1, np.int32)
        ubuf = [np.zeros(int(fq.id_offs[-1]) + 1, np.uint8), np.zeros(int(fq.offs[-1]) + 1, np.uint8),
                np.zeros(int(fq.offs[-1]) + 1, np.uint8)]
        u = FastqBatch(header_indices=uh.ctypes.data, header=ubuf[0].ctypes.data, data_indices=ud.ctypes.data,
                       seq=ubuf[1].ctypes.data, quality=ubuf[2].ctypes.data)
        lst = lib.array_list_new(16, 1.25, 1)
        f = lib.bwt_map_exact_batch if api == API_EXACT_BATCH else lib.bwt_map_inexact_batch
        ret = f(ctypes.byref(b), opt, index_handle, ctypes.byref(u), lst)
        um = []
        for k in range(u.num_reads):
            um.append((ubuf[0][uh[k]:uh[k + 1]].tobytes(), ubuf[1][ud[k]:ud[k + 1]].tobytes(),
                       ubuf[2][ud[k]:ud[k + 1]].tobytes()))
        return {"list": walk_list(lib, lst, ret, False), "unmapped": um}
    finally:
        lib.bwt_optarg_free(opt)


_COMP = {ord(a): ord(b) for a, b in zip("ACGTacgt", "TGCATGCA")}


def _revcomp(s: bytes) -> bytes:
    """seq_reverse_complementary (bwt.c:653-680): complement, reverse, anything else to 'N'."""
    return bytes(_COMP.get(c, ord("N")) for c in s[::-1])
