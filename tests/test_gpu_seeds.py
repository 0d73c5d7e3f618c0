"""Seeds and CALs on the GPU (bwt_map_exact_seeds_seq, bwt_map_exact_seeds_by_region,
bwt_map_exact_seed, bwt_generate_cals, bwt_generate_cals_batch) against the reference's own records
in the golden fixtures: every region, CAL, seed list, duplicate list and
candidate list, in order."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

import seed_lists as sl
from golden_cases import GoldenCase, names
from hpgbwt import lib

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def loaded(tmp_path_factory):
    L = lib.load()
    sl.bind(L)
    out = {}
    for name in names():
        gc = GoldenCase(name)
        out[name] = (gc, gc.build(tmp_path_factory.mktemp("seeds_" + name)))
    return L, out


def _first_diff(a: bytes, b: bytes) -> str:
    la, lb = a.decode().splitlines(), b.decode().splitlines()
    for i, (x, y) in enumerate(zip(la, lb)):
        if x != y:
            return f"line {i}: got {x!r}, reference {y!r}"
    return f"lengths {len(la)} != {len(lb)}"


@pytest.mark.parametrize("name", names())
def test_seeds_and_cals_match_reference(loaded, name):
    L, cases = loaded
    gc, index = cases[name]
    reads = gc.seed_reads()
    nchrom = len(gc.chrom_lengths)
    with lib.GpuIndex(index) as g:
        for run in gc.seed_runs():
            mode, ss, filt, minc, intron = run
            want = gc.seed_expected(*run)
            got = sl.product_seeds_cals(L, g.handle, mode, reads, ss, filt, minc, intron, nchrom)
            assert got == want, f"{run}: {_first_diff(got, want)}"


@pytest.mark.parametrize("name", names())
def test_cal_batch_equals_reference(loaded, name):
    """bwt_generate_cals_batch: every read's CALs as bwt_generate_cals builds them."""
    L, cases = loaded
    gc, index = cases[name]
    reads = gc.seed_reads()
    with lib.GpuIndex(index) as g:
        for run in gc.seed_runs():
            mode, ss, filt, minc, intron = run
            if mode != sl.MODE_CALS:
                continue
            got = sl.product_seeds_cals(L, g.handle, mode, reads, ss, filt, minc, intron, len(gc.chrom_lengths),
                                        batch=True)
            want = gc.seed_expected(*run)
            assert got == want, f"{run}: {_first_diff(got, want)}"


def test_single_seed_entry_point(loaded):
    """bwt_map_exact_seed on codes gives, seed by seed, the regions of the seed plan."""
    L, cases = loaded
    gc, index = cases["repeats_3chr"]
    L.bwt_map_exact_seed.restype = ctypes.c_size_t
    L.bwt_map_exact_seed.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_size_t,
                                     ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
    code = {ord(c): i for i, c in enumerate("ACGT")}
    want_text = gc.seed_expected(0, 16, 300, 0, 0).decode().splitlines()
    reads = gc.seed_reads()[:40]
    with lib.GpuIndex(index) as g:
        opt = L.bwt_optarg_new(1, 1, 200, 300)
        at = 0
        for r in reads:
            ret, n = map(int, want_text[at].split()[1:])
            want = want_text[at + 1:at + 1 + n]
            at += 1 + n
            codes = np.array([code[c] for c in r], dtype=np.uint8)
            L_ = len(r)
            plan = [(8, 23)] + [(o, o + 15) for o in range(0, L_ - L_ % 16, 16)]
            if L_ % 16:
                plan.append((L_ - 16, L_ - 1))
            if L_ % 16 != 8:
                plan.append((L_ - 24, L_ - 9))
            lst = L.array_list_new(16, 1.25, 2)
            total = 0
            for sid, (a, b) in enumerate(plan):
                total += L.bwt_map_exact_seed(codes.ctypes.data, L_, a, b, opt, g.handle, lst, sid)
            out = []
            sl._write(L, sl.MODE_SEEDS, total, lst, out)
            assert [x.rstrip("\n") for x in out[1:]] == want
            assert total == n
        L.bwt_optarg_free(opt)


def test_short_and_odd_reads(loaded):
    """Reads the seed plan reaches past (the reference reads beyond them) and
    reads with other letters map what lies inside them, without faults."""
    L, cases = loaded
    gc, index = cases["iid_1chr"]
    A = np.frombuffer(b"ACGT", dtype=np.uint8)
    g0 = gc.genome
    reads = [b"", b"ACGT", A[g0[100:117]].tobytes(), A[g0[200:230]].tobytes(), b"N" * 50,
             A[g0[300:340]].tobytes() + b"N" + A[g0[341:400]].tobytes()]
    with lib.GpuIndex(index) as g:
        for mode in (sl.MODE_SEEDS, sl.MODE_CALS):
            text = sl.product_seeds_cals(L, g.handle, mode, reads, 16, 300, 20, 500000, 1).decode()
            assert sum(1 for x in text.splitlines() if x.startswith("R ")) == len(reads)
        seeds = sl.product_seeds_cals(L, g.handle, sl.MODE_SEEDS, [A[g0[200:230]].tobytes()], 16, 300, 0, 0, 1)
        # a 30-base read: seeds [8,23], [0,15], [14,29] and [6,21], each once on the '+' strand
        assert seeds.decode().splitlines()[0] == "R 4 4"
        # a 17-base read: [8,23] and [17-16-8, ...] reach past it; [0,15] and [1,16] map
        seeds = sl.product_seeds_cals(L, g.handle, sl.MODE_SEEDS, [A[g0[100:117]].tobytes()], 16, 300, 0, 0, 1)
        assert seeds.decode().splitlines()[0] == "R 2 2"
