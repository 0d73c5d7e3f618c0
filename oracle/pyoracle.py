"""TEST INFRASTRUCTURE ONLY: Python loaders for the CPU oracles.

- ``PortOracle``: oracle/liboracle.so, the C restatement in oracle/fm_oracle.c.
- ``RefOracle``: oracle/_ref/libhpgref.so, the reference's own sources driven by
  oracle/ref/ref_harness.c (exists only where the reference tree was present
  at build time).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
module; the product never does.
"""
from __future__ import annotations

import ctypes
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT / "hpg-libs_gb300"))
from hpgbwt.lib import ANCHOR_DTYPE, BlockResult, ResultSetC, Result, result_from_c  # noqa: E402

PORT_LIB = ROOT / "oracle" / "liboracle.so"
REF_LIB = ROOT / "oracle" / "_ref" / "libhpgref.so"


class PortOracle:
    def __init__(self, index_dir: str):
        if not PORT_LIB.exists():
            raise RuntimeError(f"{PORT_LIB} missing; run hpg-libs_gb300/hpgbwt/build.py")
        self.lib = ctypes.CDLL(str(PORT_LIB))
        self.lib.fmo_index_load.restype = ctypes.c_void_p
        self.lib.fmo_index_load.argtypes = [ctypes.c_char_p]
        self.lib.fmo_index_free.argtypes = [ctypes.c_void_p]
        self.lib.fmo_search.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.c_size_t, ctypes.c_uint32, ctypes.c_int, ctypes.POINTER(ResultSetC)]
        self.lib.fmo_search_limit.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                              ctypes.c_size_t, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int,
                                              ctypes.POINTER(ResultSetC)]
        self.lib.fmo_block_search.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                                              ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int,
                                              ctypes.POINTER(ResultSetC), ctypes.c_void_p, ctypes.c_void_p]
        self.lib.fmo_result_free.argtypes = [ctypes.POINTER(ResultSetC)]
        self.lib.fmo_max_threads.restype = ctypes.c_int
        self.h = self.lib.fmo_index_load(index_dir.encode())
        if not self.h:
            raise RuntimeError(f"oracle cannot load index {index_dir}")

    def max_threads(self) -> int:
        return int(self.lib.fmo_max_threads())

    def search(self, reads, mode: int = 1, max_results: int = 1 << 16, threads: int = 1,
               locate_limit: int = 0) -> Result:
        seq = np.ascontiguousarray(reads.seq, dtype=np.uint8)
        offs = np.ascontiguousarray(reads.offsets, dtype=np.uint64)
        n = len(offs) - 1
        rs = ResultSetC()
        self.lib.fmo_search_limit(self.h, mode, seq.ctypes.data, offs.ctypes.data, n, max_results, locate_limit,
                                  threads, ctypes.byref(rs))
        try:
            return result_from_c(rs, n)
        finally:
            self.lib.fmo_result_free(ctypes.byref(rs))

    def block_search(self, reads, max_results: int = 1 << 16, threads: int = 1,
                     locate_limit: int = 0) -> BlockResult:
        """k-error block search (BWSearchCPU as bwt_map_inexact_read_2 drives it), with anchors."""
        seq = np.ascontiguousarray(reads.seq, dtype=np.uint8)
        offs = np.ascontiguousarray(reads.offsets, dtype=np.uint64)
        n = len(offs) - 1
        anchors = np.zeros(4 * n + 1, dtype=ANCHOR_DTYPE)
        n_anchors = np.zeros(2 * n + 1, dtype=np.uint8)
        rs = ResultSetC()
        self.lib.fmo_block_search(self.h, seq.ctypes.data, offs.ctypes.data, n, max_results, locate_limit, threads,
                                  ctypes.byref(rs), anchors.ctypes.data, n_anchors.ctypes.data)
        try:
            return BlockResult(result_from_c(rs, n), anchors[:4 * n], n_anchors[:2 * n])
        finally:
            self.lib.fmo_result_free(ctypes.byref(rs))

    def close(self) -> None:
        if self.h:
            self.lib.fmo_index_free(self.h)
            self.h = None


def ref_available() -> bool:
    return REF_LIB.exists()


class RefOracle:
    def __init__(self, index_dir: str | None = None):
        self.lib = ctypes.CDLL(str(REF_LIB))
        self.lib.ref_index_load.restype = ctypes.c_void_p
        self.lib.ref_index_load.argtypes = [ctypes.c_char_p]
        self.lib.ref_index_free.argtypes = [ctypes.c_void_p]
        self.lib.ref_build_index.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_uint]
        self.lib.ref_search.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.c_size_t, ctypes.c_uint32, ctypes.POINTER(ResultSetC)]
        self.lib.ref_result_free.argtypes = [ctypes.POINTER(ResultSetC)]
        self.lib.ref_map_api.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                         ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                                         ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p),
                                         ctypes.POINTER(ctypes.c_size_t)]
        self.lib.ref_seeds_cals.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                            ctypes.c_size_t, ctypes.c_size_t, ctypes.c_int, ctypes.c_size_t,
                                            ctypes.c_size_t, ctypes.c_uint, ctypes.POINTER(ctypes.c_void_p),
                                            ctypes.POINTER(ctypes.c_size_t)]
        self.lib.ref_blob_free.argtypes = [ctypes.c_void_p]
        self.lib.ref_block_search.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                                              ctypes.c_uint32, ctypes.POINTER(ResultSetC), ctypes.c_void_p,
                                              ctypes.c_void_p]
        self.h = self.lib.ref_index_load(index_dir.encode()) if index_dir else None

    def build_index(self, fasta: str, outdir: str, ratio: int = 16) -> None:
        Path(outdir).mkdir(parents=True, exist_ok=True)
        self.lib.ref_build_index(fasta.encode(), outdir.encode(), ratio)

    def search(self, reads, mode: int = 1, max_results: int = 1 << 16) -> Result:
        seq = np.ascontiguousarray(reads.seq, dtype=np.uint8)
        offs = np.ascontiguousarray(reads.offsets, dtype=np.uint64)
        n = len(offs) - 1
        rs = ResultSetC()
        self.lib.ref_search(self.h, mode, seq.ctypes.data, offs.ctypes.data, n, max_results, ctypes.byref(rs))
        try:
            return result_from_c(rs, n)
        finally:
            self.lib.ref_result_free(ctypes.byref(rs))

    def block_search(self, reads, max_results: int = 1 << 16) -> BlockResult:
        """The reference's BWSearchCPU per strand as bwt_map_inexact_read_2 calls it (rs_truncated all 0)."""
        seq = np.ascontiguousarray(reads.seq, dtype=np.uint8)
        offs = np.ascontiguousarray(reads.offsets, dtype=np.uint64)
        n = len(offs) - 1
        anchors = np.zeros(4 * n + 1, dtype=ANCHOR_DTYPE)
        n_anchors = np.zeros(2 * n + 1, dtype=np.uint8)
        rs = ResultSetC()
        self.lib.ref_block_search(self.h, seq.ctypes.data, offs.ctypes.data, n, max_results, ctypes.byref(rs),
                                  anchors.ctypes.data, n_anchors.ctypes.data)
        try:
            return BlockResult(result_from_c(rs, n), anchors[:4 * n], n_anchors[:2 * n])
        finally:
            self.lib.ref_result_free(ctypes.byref(rs))

    def map_api(self, api: int, fq, filter_read_mappings: int, flag: int = 0) -> bytes:
        """The reference's alignment-list functions on a fastq set (see ref_map_api), serialised."""
        p = ctypes.c_void_p()
        n = ctypes.c_size_t()
        self.lib.ref_map_api(self.h, api, fq.seq.ctypes.data, fq.qual.ctypes.data, fq.offs.ctypes.data,
                             fq.ids.ctypes.data, fq.id_offs.ctypes.data, fq.n, filter_read_mappings, flag,
                             ctypes.byref(p), ctypes.byref(n))
        try:
            return bytes((ctypes.c_uint8 * n.value).from_address(p.value)) if n.value else b""
        finally:
            self.lib.ref_blob_free(p)

    def seeds_cals(self, mode: int, reads: list[bytes], seed_size: int, filter_seed: int, min_cal_size: int,
                   max_intron: int, nchrom: int) -> bytes:
        """The reference's bwt_map_exact_seeds_seq (mode 0) or bwt_generate_cals (mode 1) per
        read, as text (see ref_seeds_cals)."""
        sys.path.insert(0, str(ROOT / "tests"))
        from seed_lists import pack
        buf, offs = pack(reads)
        p = ctypes.c_void_p()
        n = ctypes.c_size_t()
        self.lib.ref_seeds_cals(self.h, mode, buf.ctypes.data, offs.ctypes.data, len(reads), seed_size, filter_seed,
                                min_cal_size, max_intron, nchrom, ctypes.byref(p), ctypes.byref(n))
        try:
            return bytes((ctypes.c_uint8 * n.value).from_address(p.value)) if n.value else b""
        finally:
            self.lib.ref_blob_free(p)

    def close(self) -> None:
        if self.h:
            self.lib.ref_index_free(self.h)
            self.h = None
