"""ctypes binding of libhpgbwt.so (the C ABI declared in include/hpg_bwt.h).

This is how the tests and the benchmark drive the library; C callers link the
shared library directly.  There is no Python compute path: every search runs
in the CUDA kernels behind the C ABI, and opening an index without a CUDA
device fails.
"""
from __future__ import annotations

import ctypes
import time
from dataclasses import dataclass
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent.parent / "libhpgbwt.so"

MODE_EXACT = 0
MODE_SEARCH1 = 1
MODE_BLOCK = 2
FORM_PLAIN = 0
FORM_BATCHED = 1

HIT_DTYPE = np.dtype([("read", "<u4"), ("strand", "u1"), ("dir", "u1"), ("nm", "u1"), ("err_kind", "u1"),
                      ("err_base", "u1"), ("pad0", "u1"), ("err_pos", "<i2"), ("pad1", "<u4"), ("k", "<i8"),
                      ("l", "<i8")])
LOC_DTYPE = np.dtype([("key", "<u8"), ("position", "<u8"), ("hit", "<u4"), ("chrom", "<u4"), ("valid", "<u4"),
                      ("pad", "<u4")])
ANCHOR_DTYPE = np.dtype([("k", "<i8"), ("l", "<i8"), ("start", "<i2"), ("end", "<i2"), ("pos", "<i2"),
                         ("dir", "u1"), ("pad", "u1")])
assert HIT_DTYPE.itemsize == 32 and LOC_DTYPE.itemsize == 32 and ANCHOR_DTYPE.itemsize == 24


class ResultSetC(ctypes.Structure):
    _fields_ = [("n_reads", ctypes.c_size_t), ("n_hits", ctypes.c_size_t), ("hits", ctypes.c_void_p),
                ("n_locs", ctypes.c_size_t), ("locs", ctypes.c_void_p), ("rs_count", ctypes.c_void_p),
                ("rs_truncated", ctypes.c_void_p)]


@dataclass
class Result:
    """Flat search output (see include/hpg_bwt_records.h for the ordering)."""
    hits: np.ndarray
    locs: np.ndarray
    rs_count: np.ndarray
    rs_truncated: np.ndarray

    def equal(self, other: "Result") -> bool:
        return (np.array_equal(self.hits, other.hits) and np.array_equal(self.locs, other.locs)
                and np.array_equal(self.rs_count, other.rs_count)
                and np.array_equal(self.rs_truncated, other.rs_truncated))

    def subset(self, reads: np.ndarray) -> "Result":
        """The records of the given reads (ascending batch indices), renumbered as
        the result of a batch holding only those reads: read ids become their
        positions in `reads`, hit ids count the kept hits."""
        reads = np.asarray(reads, dtype=np.int64)
        n = len(self.rs_count) // 2
        new_read = np.full(n, -1, dtype=np.int64)
        new_read[reads] = np.arange(len(reads))
        keep_hit = new_read[self.hits["read"].astype(np.int64)] >= 0
        hits = self.hits[keep_hit].copy()
        hits["read"] = new_read[hits["read"].astype(np.int64)].astype(np.uint32)
        new_hit = np.cumsum(keep_hit, dtype=np.int64) - 1
        keep_loc = keep_hit[self.locs["hit"].astype(np.int64)] if len(self.locs) else np.zeros(0, dtype=bool)
        locs = self.locs[keep_loc].copy()
        locs["hit"] = new_hit[locs["hit"].astype(np.int64)].astype(np.uint32)
        rows = np.stack([2 * reads, 2 * reads + 1], axis=1).ravel()
        return Result(hits, locs, self.rs_count[rows].copy(), self.rs_truncated[rows].copy())


@dataclass
class BlockResult:
    """k-error block search output: the result set plus the anchors, anchors[2 * (2 * read + strand) + a]
    valid for a < n_anchors[2 * read + strand]."""
    result: Result
    anchors: np.ndarray
    n_anchors: np.ndarray

    def used_anchors(self) -> np.ndarray:
        """The valid anchors in (read, strand, order) order, unused slots dropped."""
        keep = np.arange(2)[None, :] < self.n_anchors[:, None]
        return self.anchors.reshape(-1, 2)[keep]

    def equal(self, other: "BlockResult", truncation: bool = True) -> bool:
        a, b = self.result, other.result
        same = (np.array_equal(a.hits, b.hits) and np.array_equal(a.locs, b.locs)
                and np.array_equal(a.rs_count, b.rs_count))
        if truncation:
            same = same and np.array_equal(a.rs_truncated, b.rs_truncated)
        return (same and np.array_equal(self.n_anchors, other.n_anchors)
                and np.array_equal(self.used_anchors(), other.used_anchors()))


def _arr(ptr: int | None, n: int, dt: np.dtype) -> np.ndarray:
    if n == 0 or not ptr:
        return np.zeros(0, dtype=dt)
    # a ctypes array view, not ctypes.string_at, whose size argument is a C int (wraps past 2 GiB)
    return np.frombuffer((ctypes.c_uint8 * (n * dt.itemsize)).from_address(ptr), dtype=dt).copy()


def result_from_c(rs: ResultSetC, n_reads: int) -> Result:
    return Result(_arr(rs.hits, rs.n_hits, HIT_DTYPE), _arr(rs.locs, rs.n_locs, LOC_DTYPE),
                  _arr(rs.rs_count, 2 * n_reads, np.dtype("<u4")), _arr(rs.rs_truncated, 2 * n_reads, np.dtype("u1")))


_lib = None


def load() -> ctypes.CDLL:
    """Load the shared library (it must have been built; see build.py)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(f"{LIB_PATH} is missing: build it with hpg-libs_gb300/hpgbwt/build.py")
    lib = ctypes.CDLL(str(LIB_PATH), mode=ctypes.RTLD_LOCAL)
    vp, sz, u32, u64 = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_uint32, ctypes.c_uint64
    lib.bwt_index_open.restype = vp
    lib.bwt_index_open.argtypes = [ctypes.c_char_p, ctypes.c_bool, ctypes.c_int, ctypes.c_char_p, sz]
    lib.bwt_index_free.argtypes = [vp]
    lib.bwt_gpu_search_batch.argtypes = [vp, ctypes.c_int, ctypes.c_int, vp, vp, sz, u32, ctypes.POINTER(ResultSetC)]
    lib.bwt_gpu_search_device.argtypes = [vp, ctypes.c_int, ctypes.c_int, vp, vp, sz, u64, u32, u32,
                                          ctypes.POINTER(ResultSetC)]
    lib.bwt_gpu_copy_result.argtypes = [vp, ctypes.POINTER(ResultSetC), vp, vp, vp, vp]
    lib.bwt_gpu_result_free.argtypes = [ctypes.POINTER(ResultSetC)]
    lib.bwt_gpu_stream.restype = vp
    lib.bwt_gpu_stream.argtypes = [vp]
    lib.bwt_gpu_stage_ms.argtypes = [vp, ctypes.POINTER(ctypes.c_float), ctypes.c_int]
    lib.bwt_gpu_set_census.argtypes = [vp, ctypes.c_int]
    lib.bwt_gpu_census.restype = ctypes.c_ulonglong
    lib.bwt_gpu_census.argtypes = [vp]
    lib.bwt_gpu_set_chunk.argtypes = [vp, sz]
    lib.bwt_gpu_set_tuning.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    lib.bwt_gpu_get_tuning.argtypes = [vp, ctypes.POINTER(ctypes.c_int)]
    lib.bwt_gpu_set_load_mode.argtypes = [vp, ctypes.c_int]
    lib.bwt_gpu_load_mode.argtypes = [vp]
    lib.bwt_gpu_server_new.restype = vp
    lib.bwt_gpu_server_new.argtypes = [vp, sz, u64, u64, u32]
    lib.bwt_gpu_server_submit.argtypes = [vp, vp, vp, sz, ctypes.POINTER(ctypes.c_uint64)]
    lib.bwt_gpu_server_wait.argtypes = [vp, u64, ctypes.POINTER(ResultSetC), ctypes.POINTER(ctypes.c_double),
                                        ctypes.c_int]
    lib.bwt_gpu_server_release.argtypes = [vp, u64]
    lib.bwt_gpu_server_stats.argtypes = [vp, ctypes.POINTER(ctypes.c_double), ctypes.c_int]
    lib.bwt_gpu_server_free.argtypes = [vp]
    lib.bwt_gpu_set_graph.argtypes = [vp, ctypes.c_int]
    lib.bwt_gpu_graph.argtypes = [vp]
    lib.bwt_gpu_set_pipeline_chunk.argtypes = [vp, sz]
    lib.bwt_gpu_set_start_table.argtypes = [vp, ctypes.c_int]
    lib.bwt_gpu_set_direction_split.argtypes = [vp, ctypes.c_int]
    lib.bwt_gpu_direction_split.argtypes = [vp]
    lib.bwt_gpu_map_device_seconds.restype = ctypes.c_double
    lib.bwt_gpu_map_device_seconds.argtypes = [vp]
    lib.bwt_gpu_set_wave_group.argtypes = [vp, ctypes.c_int]
    lib.bwt_gpu_wave_group.argtypes = [vp]
    lib.bwt_gpu_set_idle_batch.argtypes = [vp, ctypes.c_int]
    lib.bwt_gpu_idle_batch.argtypes = [vp]
    lib.bwt_gpu_set_locate_limit.argtypes = [vp, u64]
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
    lib.cal_free.argtypes = [vp]
    lib.bwt_map_inexact_batch.restype = sz
    lib.bwt_map_inexact_batch.argtypes = [vp, vp, vp, vp, vp]
    lib.bwt_map_inexact_array_list_2.restype = sz
    lib.bwt_map_inexact_array_list_2.argtypes = [vp, vp, vp, vp, vp, vp]
    lib.array_list_insert.argtypes = [vp, vp]
    lib.bwt_gpu_block_search.argtypes = [vp, vp, vp, sz, u32, ctypes.POINTER(ResultSetC), vp, vp]
    lib.bwt_gpu_block_search_ms.restype = ctypes.c_float
    lib.bwt_gpu_block_search_ms.argtypes = [vp]
    lib.alignment_free.argtypes = [vp]
    lib.bwt_generate_cals_batch.restype = sz
    lib.bwt_generate_cals_batch.argtypes = [vp, sz, sz, vp, vp, vp, vp, ctypes.c_uint]
    lib.bwt_gpu_locate_limit.argtypes = [vp]
    lib.bwt_gpu_locate_limit.restype = u64
    lib.bwt_gpu_start_table.argtypes = [vp]
    lib.bwt_gpu_autotune.argtypes = [vp, vp, vp, sz, u64, u32, u32, ctypes.POINTER(ctypes.c_int), ctypes.c_int,
                                     ctypes.POINTER(ctypes.c_int)]
    lib.bwt_gpu_last_error.restype = ctypes.c_char_p
    lib.bwt_gpu_launch_count.restype = ctypes.c_ulonglong
    lib.bwt_gpu_index_bytes.restype = sz
    lib.bwt_gpu_index_bytes.argtypes = [vp]
    lib.bwt_gpu_gather_ceiling.argtypes = [ctypes.c_int, sz, u32, u32, ctypes.POINTER(ctypes.c_double)]
    lib.hpg_bwt_build_index.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_uint, ctypes.c_int,
                                        ctypes.c_char_p, ctypes.c_char_p, sz]
    lib.hpg_bwt_build_index_on.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_uint, ctypes.c_int,
                                           ctypes.c_char_p, ctypes.c_int, ctypes.c_char_p, sz]
    _lib = lib
    return lib


def launch_count() -> int:
    return int(load().bwt_gpu_launch_count())


def gather_ceiling(device: int, nbytes: int, blocks: int, steps: int) -> float:
    lib = load()
    v = ctypes.c_double()
    if lib.bwt_gpu_gather_ceiling(device, nbytes, blocks, steps, ctypes.byref(v)) != 0:
        raise RuntimeError(lib.bwt_gpu_last_error().decode())
    return v.value


def build_index(fasta: str, outdir: str, ratio: int = 16, bases: str = "ACGT", device: int = -1) -> None:
    """Write the reference's index files for a FASTA; suffix arrays on the host, or on CUDA device `device`."""
    lib = load()
    err = ctypes.create_string_buffer(1024)
    if lib.hpg_bwt_build_index_on(fasta.encode(), outdir.encode(), ratio, 0, bases.encode(), device, err, 1024) != 0:
        raise RuntimeError(err.value.decode())


class GpuIndex:
    """An index loaded into GPU memory through bwt_index_open."""

    def __init__(self, index_dir: str, device: int = -1, inverse_sa: bool = False):
        self.lib = load()
        err = ctypes.create_string_buffer(2048)
        h = self.lib.bwt_index_open(index_dir.encode(), inverse_sa, device, err, 2048)
        if not h:
            raise RuntimeError(err.value.decode())
        self.handle = h

    def close(self) -> None:
        if self.handle:
            self.lib.bwt_index_free(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, rc: int) -> None:
        if rc != 0:
            raise RuntimeError(self.lib.bwt_gpu_last_error().decode())

    def search(self, reads, mode: int = MODE_SEARCH1, form: int = FORM_PLAIN, max_results: int = 1 << 16) -> Result:
        """Search a synth.ReadSet-like object (seq: uint8 ASCII, offsets: uint64)."""
        seq = np.ascontiguousarray(reads.seq, dtype=np.uint8)
        offs = np.ascontiguousarray(reads.offsets, dtype=np.uint64)
        n = len(offs) - 1
        rs = ResultSetC()
        self._check(self.lib.bwt_gpu_search_batch(self.handle, mode, form, seq.ctypes.data, offs.ctypes.data, n,
                                                  max_results, ctypes.byref(rs)))
        try:
            return result_from_c(rs, n)
        finally:
            self.lib.bwt_gpu_result_free(ctypes.byref(rs))

    def block_search(self, reads, max_results: int = 1 << 16) -> BlockResult:
        """k-error block search (bwt_gpu_block_search) of a synth.ReadSet-like object, with anchors."""
        seq = np.ascontiguousarray(reads.seq, dtype=np.uint8)
        offs = np.ascontiguousarray(reads.offsets, dtype=np.uint64)
        n = len(offs) - 1
        anchors = np.zeros(4 * n + 1, dtype=ANCHOR_DTYPE)
        n_anchors = np.zeros(2 * n + 1, dtype=np.uint8)
        rs = ResultSetC()
        self._check(self.lib.bwt_gpu_block_search(self.handle, seq.ctypes.data, offs.ctypes.data, n, max_results,
                                                  ctypes.byref(rs), anchors.ctypes.data, n_anchors.ctypes.data))
        try:
            return BlockResult(result_from_c(rs, n), anchors[:4 * n], n_anchors[:2 * n])
        finally:
            self.lib.bwt_gpu_result_free(ctypes.byref(rs))

    def block_search_ms(self) -> float:
        """Device time of the last block search's kernel(s)."""
        return float(self.lib.bwt_gpu_block_search_ms(self.handle))

    def search_device(self, d_seqs: int, d_offs: int, n_reads: int, total_bases: int, max_len: int,
                      mode: int = MODE_SEARCH1, form: int = FORM_PLAIN, max_results: int = 1 << 16) -> ResultSetC:
        rs = ResultSetC()
        self._check(self.lib.bwt_gpu_search_device(self.handle, mode, form, d_seqs, d_offs, n_reads, total_bases,
                                                   max_len, max_results, ctypes.byref(rs)))
        return rs

    def copy_result(self, rs: ResultSetC, hits: int, locs: int, rs_count: int, rs_trunc: int) -> None:
        self._check(self.lib.bwt_gpu_copy_result(self.handle, ctypes.byref(rs), hits, locs, rs_count, rs_trunc))

    def stream(self) -> int:
        return self.lib.bwt_gpu_stream(self.handle)

    def stage_ms(self) -> list[float]:
        """encode, search, finalize, locate, and the drain launch's share of search."""
        a = (ctypes.c_float * 5)()
        self.lib.bwt_gpu_stage_ms(self.handle, a, 5)
        return list(a)

    def set_census(self, on: bool) -> None:
        self.lib.bwt_gpu_set_census(self.handle, 1 if on else 0)

    def census(self) -> int:
        return int(self.lib.bwt_gpu_census(self.handle))

    def set_tuning(self, blocks_per_sm: int, stack: int, chunk: int, min_blocks: int = 1) -> None:
        self.lib.bwt_gpu_set_tuning(self.handle, min_blocks, blocks_per_sm, stack, chunk)

    def get_tuning(self) -> dict:
        a = (ctypes.c_int * 5)()
        self.lib.bwt_gpu_get_tuning(self.handle, a)
        return {"threads_per_block": a[0], "blocks_per_sm": a[1], "stack": a[2], "chains_per_claim": a[3],
                "register_bound_blocks": a[4]}

    def autotune(self, d_seqs: int, d_offs: int, n_reads: int, total_bases: int, max_len: int,
                 max_results: int = 1 << 16) -> list[dict]:
        table = (ctypes.c_int * (5 * 128))()
        rows = ctypes.c_int()
        self._check(self.lib.bwt_gpu_autotune(self.handle, d_seqs, d_offs, n_reads, total_bases, max_len,
                                              max_results, table, 128, ctypes.byref(rows)))
        rows.value = min(rows.value, 128)
        return [{"register_bound_blocks": table[5 * i], "blocks_per_sm": table[5 * i + 1], "stack": table[5 * i + 2],
                 "chains_per_claim": table[5 * i + 3], "search_us": table[5 * i + 4]} for i in range(rows.value)]

    def set_load_mode(self, mode: int) -> None:
        self.lib.bwt_gpu_set_load_mode(self.handle, mode)

    def load_mode(self) -> int:
        return int(self.lib.bwt_gpu_load_mode(self.handle))

    def set_graph(self, on: bool) -> None:
        """Batched form from the captured CUDA graph (default) or launched stage by stage."""
        self.lib.bwt_gpu_set_graph(self.handle, 1 if on else 0)

    def set_direction_split(self, mode: int) -> None:
        """Fused batched search: 0 mixed, 1 index direction by SM half, 2 one launch per direction."""
        self.lib.bwt_gpu_set_direction_split(self.handle, int(mode))

    def direction_split(self) -> int:
        return int(self.lib.bwt_gpu_direction_split(self.handle))

    def set_wave_group(self, reads: int) -> None:
        """Warp-cooperative batched search with `reads` reads per warp group (0: back to the fused form)."""
        self.lib.bwt_gpu_set_wave_group(self.handle, int(reads))

    def wave_group(self) -> int:
        return int(self.lib.bwt_gpu_wave_group(self.handle))

    def set_idle_batch(self, lanes: int) -> None:
        """Fused batched search: idle lanes of a warp take their next work item together, `lanes` at a time."""
        self.lib.bwt_gpu_set_idle_batch(self.handle, int(lanes))

    def idle_batch(self) -> int:
        return int(self.lib.bwt_gpu_idle_batch(self.handle))

    def generate_cals(self, reads: list[bytes], nchromosomes: int, seed_size: int = 16,
                      filter_seed_mappings: int = 300, min_cal_size: int = 20,
                      max_intron_size: int = 500_000) -> list[int]:
        """bwt_generate_cals_batch over the reads (ASCII): the number of CALs of each
        read (the cal_t records are built and freed)."""
        n = len(reads)
        bufs = [ctypes.create_string_buffer(r, len(r) + 1) for r in reads]
        arr = (ctypes.c_void_p * max(1, n))(*[ctypes.addressof(b) for b in bufs])
        lists = (ctypes.c_void_p * max(1, n))(*[self.lib.array_list_new(16, 1.25, 2) for _ in range(n)])
        opt = self.lib.bwt_optarg_new(1, 1, 200, filter_seed_mappings)
        copt = self.lib.cal_optarg_new(min_cal_size, 0, 0, 0, seed_size, 0, 0, max_intron_size, 0)
        try:
            t0 = time.perf_counter()
            self.lib.bwt_generate_cals_batch(arr, n, seed_size, opt, copt, self.handle, lists, nchromosomes)
            self.last_cal_seconds = time.perf_counter() - t0
            counts = [int(self.lib.array_list_size(lists[i])) for i in range(n)]
        finally:
            free = ctypes.cast(self.lib.cal_free, ctypes.c_void_p)
            for i in range(n):
                self.lib.array_list_free(lists[i], free)
            self.lib.bwt_optarg_free(opt)
            self.lib.cal_optarg_free(copt)
        return counts

    def map_inexact_batch(self, reads: list[bytes], filter_read_mappings: int = 200) -> int:
        """bwt_map_inexact_batch (the reference's alignment-list entry point) over the
        reads: the number of alignment records (built and freed); the C call's wall
        time is left in last_map_seconds."""

        class FastqBatch(ctypes.Structure):  # c/src/bioformats/fastq/fastq_batch.h:24-34
            _fields_ = [("num_reads", ctypes.c_ulong), ("data_indices_size", ctypes.c_ulong),
                        ("data_size", ctypes.c_ulong), ("source_id", ctypes.c_int),
                        ("header_indices", ctypes.c_void_p), ("header", ctypes.c_void_p),
                        ("data_indices", ctypes.c_void_p), ("seq", ctypes.c_void_p), ("quality", ctypes.c_void_p)]
        n = len(reads)
        seq = b"".join(r + b"\0" for r in reads)
        qual = b"".join(b"I" * len(r) + b"\0" for r in reads)
        ids = b"".join(b"@r%d\0" % i for i in range(n))
        didx = np.zeros(n + 1, np.int32)
        didx[1:] = np.cumsum([len(r) + 1 for r in reads])
        hidx = np.zeros(n + 1, np.int32)
        hidx[1:] = np.cumsum([len(b"@r%d" % i) + 1 for i in range(n)])
        sbuf, qbuf, ibuf = (ctypes.create_string_buffer(x, len(x)) for x in (seq, qual, ids))
        b = FastqBatch(num_reads=n, header_indices=hidx.ctypes.data, header=ctypes.addressof(ibuf),
                       data_indices=didx.ctypes.data, seq=ctypes.addressof(sbuf), quality=ctypes.addressof(qbuf))
        uh, ud = np.zeros(n + 1, np.int32), np.zeros(n + 1, np.int32)
        ub = [ctypes.create_string_buffer(len(ids) + 1), ctypes.create_string_buffer(len(seq) + 1),
              ctypes.create_string_buffer(len(seq) + 1)]
        u = FastqBatch(header_indices=uh.ctypes.data, header=ctypes.addressof(ub[0]), data_indices=ud.ctypes.data,
                       seq=ctypes.addressof(ub[1]), quality=ctypes.addressof(ub[2]))
        opt = self.lib.bwt_optarg_new(1, 1, filter_read_mappings, filter_read_mappings)
        lst = self.lib.array_list_new(max(16, n), 1.25, 2)
        try:
            t0 = time.perf_counter()
            self.lib.bwt_map_inexact_batch(ctypes.byref(b), opt, self.handle, ctypes.byref(u), lst)
            self.last_map_seconds = time.perf_counter() - t0
            self.last_map_device_seconds = float(self.lib.bwt_gpu_map_device_seconds(self.handle))
            count = int(self.lib.array_list_size(lst))
        finally:
            self.lib.array_list_free(lst, ctypes.cast(self.lib.alignment_free, ctypes.c_void_p))
            self.lib.bwt_optarg_free(opt)
        return count

    def map_inexact_batch_arrays(self, seq: np.ndarray, offsets: np.ndarray, filter_read_mappings: int = 200) -> int:
        """map_inexact_batch over reads given as concatenated bases and n+1 offsets
        (fastq_batch buffers built with numpy: large batches)."""
        n = len(offsets) - 1

        class FastqBatch(ctypes.Structure):  # c/src/bioformats/fastq/fastq_batch.h:24-34
            _fields_ = [("num_reads", ctypes.c_ulong), ("data_indices_size", ctypes.c_ulong),
                        ("data_size", ctypes.c_ulong), ("source_id", ctypes.c_int),
                        ("header_indices", ctypes.c_void_p), ("header", ctypes.c_void_p),
                        ("data_indices", ctypes.c_void_p), ("seq", ctypes.c_void_p), ("quality", ctypes.c_void_p)]
        offs = np.asarray(offsets, dtype=np.int64)
        if int(offs[-1]) + n >= 2 ** 31:  # fastq_batch_t's data_indices are C ints
            raise ValueError("a fastq batch holds less than 2^31 bytes of bases (its indices are int)")
        data = np.insert(np.asarray(seq, dtype=np.uint8), offs[1:], 0)
        qual = np.where(data == 0, 0, ord("I")).astype(np.uint8)
        didx = (offs + np.arange(n + 1)).astype(np.int32)
        ids = np.frombuffer(b"".join(b"@r%09d\0" % i for i in range(n)), dtype=np.uint8)
        hidx = (np.arange(n + 1) * 12).astype(np.int32)
        b = FastqBatch(num_reads=n, header_indices=hidx.ctypes.data, header=ids.ctypes.data,
                       data_indices=didx.ctypes.data, seq=data.ctypes.data, quality=qual.ctypes.data)
        uh, ud = np.zeros(n + 1, np.int32), np.zeros(n + 1, np.int32)
        ub = [np.zeros(len(ids) + 1, np.uint8), np.zeros(len(data) + 1, np.uint8), np.zeros(len(data) + 1, np.uint8)]
        u = FastqBatch(header_indices=uh.ctypes.data, header=ub[0].ctypes.data, data_indices=ud.ctypes.data,
                       seq=ub[1].ctypes.data, quality=ub[2].ctypes.data)
        opt = self.lib.bwt_optarg_new(1, 1, filter_read_mappings, filter_read_mappings)
        lst = self.lib.array_list_new(max(16, n), 1.25, 2)
        try:
            t0 = time.perf_counter()
            self.lib.bwt_map_inexact_batch(ctypes.byref(b), opt, self.handle, ctypes.byref(u), lst)
            self.last_map_seconds = time.perf_counter() - t0
            self.last_map_device_seconds = float(self.lib.bwt_gpu_map_device_seconds(self.handle))
            count = int(self.lib.array_list_size(lst))
        finally:
            self.lib.array_list_free(lst, ctypes.cast(self.lib.alignment_free, ctypes.c_void_p))
            self.lib.bwt_optarg_free(opt)
        return count

    def map_block_array_list(self, reads: list[bytes], filter_read_mappings: int = 200) -> int:
        """bwt_map_inexact_array_list_2 (every read as bwt_map_inexact_read_2 maps it) over the
        reads: the number of alignment records (built and freed); the C call's wall time
        is left in last_map_seconds."""

        class FastqRead(ctypes.Structure):  # c/src/bioformats/fastq/fastq_read.h:20-32
            _fields_ = [("id", ctypes.c_void_p), ("sequence", ctypes.c_void_p), ("revcomp", ctypes.c_void_p),
                        ("quality", ctypes.c_void_p), ("rev_quality", ctypes.c_void_p),
                        ("adapter", ctypes.c_void_p), ("adapter_revcomp", ctypes.c_void_p),
                        ("adapter_quality", ctypes.c_void_p), ("length", ctypes.c_int),
                        ("adapter_length", ctypes.c_int), ("adapter_strand", ctypes.c_int)]
        n = len(reads)
        seq = ctypes.create_string_buffer(b"".join(r + b"\0" for r in reads))
        qual = ctypes.create_string_buffer(b"".join(b"I" * len(r) + b"\0" for r in reads))
        ids = ctypes.create_string_buffer(b"".join(b"r%d\0" % i for i in range(n)))
        so, io = 0, 0
        recs = (FastqRead * max(1, n))()
        for i, r in enumerate(reads):
            recs[i].id = ctypes.addressof(ids) + io
            recs[i].sequence = ctypes.addressof(seq) + so
            recs[i].quality = ctypes.addressof(qual) + so
            recs[i].length = len(r)
            so += len(r) + 1
            io += len(b"r%d" % i) + 1
        rl = self.lib.array_list_new(max(16, n), 1.25, 2)
        for i in range(n):
            self.lib.array_list_insert(ctypes.addressof(recs[i]), rl)
        lists = (ctypes.c_void_p * max(1, n))(*[self.lib.array_list_new(4, 1.25, 2) for _ in range(n)])
        unmapped = (ctypes.c_size_t * max(1, n))()
        n_un = ctypes.c_size_t()
        opt = self.lib.bwt_optarg_new(1, 1, filter_read_mappings, filter_read_mappings)
        try:
            t0 = time.perf_counter()
            total = self.lib.bwt_map_inexact_array_list_2(rl, opt, self.handle, lists, ctypes.byref(n_un), unmapped)
            self.last_map_seconds = time.perf_counter() - t0
        finally:
            free = ctypes.cast(self.lib.alignment_free, ctypes.c_void_p)
            for i in range(n):
                self.lib.array_list_free(lists[i], free)
            self.lib.array_list_free(rl, None)
            self.lib.bwt_optarg_free(opt)
        return int(total)

    def set_locate_limit(self, max_rows: int) -> None:
        """Lists (read, strand) covering more than max_rows rows are not located (rs_truncated bit 1); 0 = none."""
        self.lib.bwt_gpu_set_locate_limit(self.handle, int(max_rows))

    def locate_limit(self) -> int:
        return int(self.lib.bwt_gpu_locate_limit(self.handle))

    def set_start_table(self, symbols: int) -> None:
        """Start-table length of the batched search (0 = none)."""
        self._check(self.lib.bwt_gpu_set_start_table(self.handle, symbols))

    def start_table(self) -> int:
        return int(self.lib.bwt_gpu_start_table(self.handle))

    def set_pipeline_chunk(self, reads: int) -> None:
        """Reads per chunk of pipelined host batches (0 or -1: not pipelined, the default)."""
        self.lib.bwt_gpu_set_pipeline_chunk(self.handle, reads if reads >= 0 else (1 << 64) - 1)

    def graph(self) -> bool:
        return bool(self.lib.bwt_gpu_graph(self.handle))

    def index_bytes(self) -> int:
        return int(self.lib.bwt_gpu_index_bytes(self.handle))

    def set_chunk(self, reads: int) -> None:
        self.lib.bwt_gpu_set_chunk(self.handle, reads)


SERVER_STATS = ("batches", "requests", "reads", "mean_batch_reads", "batch_wall_ms", "regrowths", "plan_bytes",
                "hbm_budget", "max_batch_reads", "max_batch_requests", "queued", "hits_per_read", "rows_per_read")


class Server:
    """The serving form of an index (bwt_gpu_server_*): submit read sets from
    any thread, wait for each; results of a request equal a lone search of it."""

    def __init__(self, index: GpuIndex, max_batch_reads: int, max_batch_bases: int = 0, hbm_budget: int = 0,
                 max_results: int = 1 << 16):
        self.lib = index.lib
        self.handle = self.lib.bwt_gpu_server_new(index.handle, max_batch_reads, max_batch_bases, hbm_budget,
                                                  max_results)
        if not self.handle:
            raise RuntimeError(self.lib.bwt_gpu_last_error().decode())
        self._held = {}  # submitted arrays stay alive until their request is released

    def submit(self, seq: np.ndarray, offsets: np.ndarray) -> int:
        seq = np.ascontiguousarray(seq, dtype=np.uint8)
        offsets = np.ascontiguousarray(offsets, dtype=np.uint64)
        t = ctypes.c_uint64()
        rc = self.lib.bwt_gpu_server_submit(self.handle, seq.ctypes.data, offsets.ctypes.data, len(offsets) - 1,
                                            ctypes.byref(t))
        if rc != 0:
            raise RuntimeError(self.lib.bwt_gpu_last_error().decode())
        self._held[t.value] = (seq, offsets)
        return t.value

    def wait(self, ticket: int, timeout_ms: int = -1, copy: bool = True, release: bool = True):
        """(Result or None if timed out, latency ms).  With copy the view is copied out and released."""
        rs = ResultSetC()
        lat = ctypes.c_double()
        rc = self.lib.bwt_gpu_server_wait(self.handle, ticket, ctypes.byref(rs), ctypes.byref(lat), timeout_ms)
        if rc < 0:
            self._held.pop(ticket, None)
            raise RuntimeError(self.lib.bwt_gpu_last_error().decode())
        if rc == 1:
            return None, None
        res = result_from_c(rs, rs.n_reads) if copy else rs
        if copy and release:
            self.release(ticket)
        return res, lat.value

    def release(self, ticket: int) -> None:
        self._held.pop(ticket, None)
        if self.lib.bwt_gpu_server_release(self.handle, ticket) != 0:
            raise RuntimeError(self.lib.bwt_gpu_last_error().decode())

    def stats(self) -> dict:
        a = (ctypes.c_double * len(SERVER_STATS))()
        self.lib.bwt_gpu_server_stats(self.handle, a, len(SERVER_STATS))
        return dict(zip(SERVER_STATS, list(a)))

    def close(self) -> None:
        if self.handle:
            self.lib.bwt_gpu_server_free(self.handle)
            self.handle = None
            self._held.clear()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
