"""The allocation-free BWSearch1 entry point against the regular batch entry point.

bwt_gpu_search1_noalloc serves callers that may not allocate device memory
(a process whose HBM belongs to another allocator, or a latency-critical
thread that cannot afford a cudaMalloc): it keeps its scratch in a fixed
array inside the library.  These tests give it caller-owned device buffers,
call it twice in a row on different read batches, and check every
per-strand hit list, count and truncation flag against bwt_gpu_search_batch
on the same reads, bit for bit; then the odd reads (empty, 1-2 bases, an
'N', lower case, longer than max_len) against the CPU oracle; and that the
calls after the first on a device leave its free memory unchanged.  They
live in a file of their own that pytest collects last, and pass both alone
and after the other tests.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

from hpgbwt import lib, synth
from oracle.pyoracle import PortOracle

pytestmark = pytest.mark.gpu

MAX_RESULTS = 16


def _bind(clib):
    clib.bwt_gpu_search1_noalloc.restype = ctypes.c_int
    clib.bwt_gpu_search1_noalloc.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                                             ctypes.c_uint32, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p,
                                             ctypes.c_void_p, ctypes.c_void_p]
    clib.bwt_gpu_noalloc_last_error.restype = ctypes.c_char_p
    clib.bwt_gpu_noalloc_scratch_bytes.restype = ctypes.c_size_t


def _noalloc(torch, g, reads, max_results, max_len=None):
    n = len(reads)
    if max_len is None:
        max_len = int(np.diff(reads.offsets).max())
    d_seq = torch.from_numpy(reads.seq).cuda()
    d_off = torch.from_numpy(reads.offsets.view(np.int64)).cuda()
    # Caller-owned outputs, pre-filled with garbage so unwritten slots would show.
    d_hits = torch.full((2 * n * max_results * 32,), 0xAB, dtype=torch.uint8, device="cuda")
    d_cnt = torch.full((2 * n,), -1, dtype=torch.int32, device="cuda")
    d_trn = torch.full((2 * n,), 7, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    rc = g.lib.bwt_gpu_search1_noalloc(g.handle, d_seq.data_ptr(), d_off.data_ptr(), n, max_len, max_results,
                                       d_hits.data_ptr(), d_cnt.data_ptr(), d_trn.data_ptr(), None)
    assert rc == 0, g.lib.bwt_gpu_noalloc_last_error().decode()
    torch.cuda.synchronize()
    hits = d_hits.cpu().numpy().view(lib.HIT_DTYPE).reshape(2 * n, max_results)
    return hits, d_cnt.cpu().numpy().astype(np.uint32), d_trn.cpu().numpy()


def _check(reference: lib.Result, hits, cnt, trn):
    assert np.array_equal(cnt, reference.rs_count)
    assert np.array_equal(trn, reference.rs_truncated)
    off = np.concatenate([[0], np.cumsum(reference.rs_count.astype(np.int64))])
    for t in np.nonzero(cnt)[0]:
        assert np.array_equal(hits[t, :cnt[t]], reference.hits[off[t]:off[t + 1]]), f"(read, strand) slot {t}"


def test_noalloc_matches_batch_entry_point(case_factory):
    torch = pytest.importorskip("torch")
    c = case_factory("human_like", 200_000, 31, 3)
    batches = [synth.reads(c.genome, 3000, 41, length=(36, 150), edits="mix_30_50_20"),
               synth.reads(c.genome, 2500, 43, length=(20, 120), edits="per_base_capped")]
    with lib.GpuIndex(c.index) as g:
        _bind(g.lib)
        assert g.lib.bwt_gpu_noalloc_scratch_bytes() == 16 << 20
        for reads in batches:  # two calls in a row through the same fixed scratch
            want = g.search(reads, mode=lib.MODE_SEARCH1, form=lib.FORM_PLAIN, max_results=MAX_RESULTS)
            hits, cnt, trn = _noalloc(torch, g, reads, MAX_RESULTS)
            assert cnt.sum() > 0
            _check(want, hits, cnt, trn)


def test_noalloc_rejects_oversized_batch(case_factory):
    torch = pytest.importorskip("torch")
    c = case_factory("human_like", 200_000, 31, 3)
    with lib.GpuIndex(c.index) as g:
        _bind(g.lib)
        d = torch.zeros(16, dtype=torch.uint8, device="cuda")
        rc = g.lib.bwt_gpu_search1_noalloc(g.handle, d.data_ptr(), d.data_ptr(), 100_000, 100, 4, d.data_ptr(),
                                           d.data_ptr(), d.data_ptr(), None)
        assert rc == -1
        assert b"scratch" in g.lib.bwt_gpu_noalloc_last_error()


def test_noalloc_edge_reads_match_oracle(case_factory):
    """Empty, 1-2 base, 'N'-containing and lower-case reads, and reads longer
    than the max_len the caller passes (those get no hits), against the oracle."""
    torch = pytest.importorskip("torch")
    c = case_factory("iid", 50_000, 9, 1)
    g0 = c.genome
    A = np.frombuffer(b"ACGT", dtype=np.uint8)
    seqs = [b"", b"A", b"AC", b"ACG", A[g0[100:105]].tobytes(), b"ACGTN" * 10, b"acgt" * 20,
            A[g0[1000:1100]].tobytes(), A[g0[-80:]].tobytes(), A[g0[:64]].tobytes(), b"T" * 120,
            A[g0[5000:5300]].tobytes(), b"", A[g0[7000:7150]].tobytes()]
    reads = synth.from_strings(seqs)
    max_len = 150  # the 300-base read is longer: it must come back empty
    lens = np.diff(reads.offsets).astype(np.int64)
    want = PortOracle(c.index).search(reads, mode=lib.MODE_SEARCH1, max_results=MAX_RESULTS, threads=1)
    with lib.GpuIndex(c.index) as g:
        _bind(g.lib)
        for _ in range(2):  # two calls in a row
            hits, cnt, trn = _noalloc(torch, g, reads, MAX_RESULTS, max_len=max_len)
            off = np.concatenate([[0], np.cumsum(want.rs_count.astype(np.int64))])
            for t in range(2 * len(reads)):
                if lens[t >> 1] > max_len:
                    assert cnt[t] == 0 and trn[t] == 0, f"over-long read {t >> 1} was searched"
                    continue
                assert cnt[t] == want.rs_count[t], f"(read, strand) slot {t}: count"
                assert trn[t] == want.rs_truncated[t], f"(read, strand) slot {t}: truncation"
                assert np.array_equal(hits[t, :cnt[t]], want.hits[off[t]:off[t + 1]]), f"(read, strand) slot {t}"
    assert want.rs_count[2 * 7] + want.rs_count[2 * 7 + 1] > 0  # the genome's own 100-mer maps


def test_noalloc_calls_after_the_first_allocate_nothing(case_factory):
    """The first call on a device may create the fixed scratch (lazy module
    loading); every call after it leaves the device's free memory as it was."""
    torch = pytest.importorskip("torch")
    c = case_factory("human_like", 200_000, 31, 3)
    reads = synth.reads(c.genome, 2000, 47, length=(36, 150), edits="mix_30_50_20")
    n = len(reads)
    max_len = int(np.diff(reads.offsets).max())
    with lib.GpuIndex(c.index) as g:
        _bind(g.lib)
        d_seq = torch.from_numpy(reads.seq).cuda()
        d_off = torch.from_numpy(reads.offsets.view(np.int64)).cuda()
        d_hits = torch.empty((2 * n * MAX_RESULTS * 32,), dtype=torch.uint8, device="cuda")
        d_cnt = torch.empty((2 * n,), dtype=torch.int32, device="cuda")
        d_trn = torch.empty((2 * n,), dtype=torch.uint8, device="cuda")
        torch.cuda.synchronize()

        def call():
            rc = g.lib.bwt_gpu_search1_noalloc(g.handle, d_seq.data_ptr(), d_off.data_ptr(), n, max_len,
                                               MAX_RESULTS, d_hits.data_ptr(), d_cnt.data_ptr(), d_trn.data_ptr(),
                                               None)
            assert rc == 0, g.lib.bwt_gpu_noalloc_last_error().decode()
            torch.cuda.synchronize()
            return torch.cuda.mem_get_info()[0]

        call()  # may create the scratch
        free = [call() for _ in range(3)]
        assert free[0] == free[1] == free[2], f"free device memory moved between calls: {free}"
        assert int(d_cnt.sum().item()) > 0
