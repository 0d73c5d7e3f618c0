"""The allocation-free BWSearch1 entry point against the regular batch entry point.

bwt_gpu_search1_noalloc serves callers that may not allocate device memory
(a process whose HBM belongs to another allocator, or a latency-critical
thread that cannot afford a cudaMalloc): it keeps its scratch in a fixed
array inside the library.  This test gives it caller-owned device buffers,
calls it twice in a row on different read batches, and checks every
per-strand hit list, count and truncation flag against bwt_gpu_search_batch
on the same reads, bit for bit.  It lives in a file of its own that pytest
collects last, and passes both alone and after the other tests.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

from hpgbwt import lib, synth

pytestmark = pytest.mark.gpu

MAX_RESULTS = 16


def _bind(clib):
    clib.bwt_gpu_search1_noalloc.restype = ctypes.c_int
    clib.bwt_gpu_search1_noalloc.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                                             ctypes.c_uint32, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p,
                                             ctypes.c_void_p, ctypes.c_void_p]
    clib.bwt_gpu_noalloc_last_error.restype = ctypes.c_char_p
    clib.bwt_gpu_noalloc_scratch_bytes.restype = ctypes.c_size_t


def _noalloc(torch, g, reads, max_results):
    n = len(reads)
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
