"""GPU parity at a benchmark configuration's full size.

The 4 Mbp configuration: a seeded 4 Mbp i.i.d. A/C/G/T genome (one
chromosome) indexed by this library's builder at the reference's ratios (O
table every 64 rows, SA sample every 16 rows), and 200 000 error-free reads of
100 bp drawn from either strand -- the same genome and reads as
``bench.py --workload c1``.  Every (read, strand) hit list, truncation flag and
located row of the plain and the batched form, in exact mode and in BWSearch1
mode, must equal the oracle's on the whole batch.
"""
from __future__ import annotations

import os

import numpy as np
import pytest

from hpgbwt import lib, synth
from oracle.pyoracle import PortOracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def c1_case(tmp_path_factory):
    d = tmp_path_factory.mktemp("c1_full")
    genome = synth.genome("iid", 4_000_000, 1)
    synth.write_fasta(str(d / "genome.fa"), genome)
    lib.build_index(str(d / "genome.fa"), str(d / "index"), 16)
    reads = synth.reads_fast(genome, 200_000, 2, 100, "none")
    return str(d / "index"), reads


@pytest.mark.parametrize("mode", [lib.MODE_EXACT, lib.MODE_SEARCH1])
def test_c1_full_size_matches_oracle(c1_case, mode):
    index, reads = c1_case
    assert len(reads) == 200_000 and np.all(np.diff(reads.offsets) == 100)
    want = PortOracle(index).search(reads, mode=mode, max_results=1024, threads=os.cpu_count() or 1)
    # error-free reads of the genome map on exactly one strand or more
    mapped = (want.rs_count.reshape(-1, 2) > 0).any(axis=1)
    assert mapped.mean() > 0.99
    with lib.GpuIndex(index) as g:
        for form in (lib.FORM_PLAIN, lib.FORM_BATCHED):
            got = g.search(reads, mode=mode, form=form, max_results=1024)
            assert np.array_equal(got.rs_count, want.rs_count), f"form {form}: per-strand hit counts differ"
            assert np.array_equal(got.rs_truncated, want.rs_truncated), f"form {form}: truncation flags differ"
            assert np.array_equal(got.hits, want.hits), f"form {form}: hits differ"
            assert np.array_equal(got.locs, want.locs), f"form {form}: located rows differ"
