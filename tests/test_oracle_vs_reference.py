"""The C restatement against the reference's compiled sources (CPU; only where
the reference tree was present at build time)."""
from __future__ import annotations

import hashlib
from pathlib import Path

import numpy as np
import pytest

from hpgbwt import lib, synth
from oracle.pyoracle import PortOracle, RefOracle, ref_available

pytestmark = pytest.mark.skipif(not ref_available(), reason="reference oracle not built here")


@pytest.mark.parametrize("kind,n,chroms,seed,length,edits,maxr", [
    ("iid", 80_000, 1, 1, 100, "per_base_capped", 1 << 16),
    ("repeats", 150_000, 4, 2, (36, 250), "mix_30_50_20", 1 << 16),
    ("human_like", 60_000, 3, 3, (3, 150), "mix_30_50_20", 5),
    ("human_like", 30_000, 2, 4, (10, 60), "none", 1),
])
def test_port_equals_reference(tmp_path, kind, n, chroms, seed, length, edits, maxr):
    g = synth.genome(kind, n, seed)
    cl = [n // chroms] * (chroms - 1)
    cl.append(n - sum(cl))
    synth.write_fasta(str(tmp_path / "g.fa"), g, cl)
    RefOracle().build_index(str(tmp_path / "g.fa"), str(tmp_path / "ref"), 16)
    reads = synth.reads(g, 1500, seed + 10, length=length, edits=edits)
    ref = RefOracle(str(tmp_path / "ref"))
    port = PortOracle(str(tmp_path / "ref"))
    for mode in (0, 1):
        a = ref.search(reads, mode=mode, max_results=maxr)
        b = port.search(reads, mode=mode, max_results=maxr, threads=4)
        assert a.equal(b), (mode, len(a.hits), len(b.hits))
    a = ref.block_search(reads, max_results=maxr)
    b = port.block_search(reads, max_results=maxr, threads=4)
    assert a.equal(b, truncation=False), (len(a.result.hits), len(b.result.hits))
    ref.close()
    port.close()


@pytest.mark.parametrize("ratio", [1, 8, 10, 32])
def test_builder_equals_reference_builder_at_other_ratios(tmp_path, ratio):
    g = synth.genome("repeats", 40_000, 9)
    synth.write_fasta(str(tmp_path / "g.fa"), g, [30_000, 10_000])
    RefOracle().build_index(str(tmp_path / "g.fa"), str(tmp_path / "ref"), ratio)
    lib.build_index(str(tmp_path / "g.fa"), str(tmp_path / "mine"), ratio)
    for p in sorted((tmp_path / "ref").iterdir()):
        q = tmp_path / "mine" / p.name
        assert hashlib.sha256(p.read_bytes()).digest() == hashlib.sha256(q.read_bytes()).digest(), p.name



def test_seed_fixtures_are_the_reference(tmp_path):
    """The recorded seed and CAL runs are what the compiled reference writes now."""
    from golden_cases import GoldenCase
    gc = GoldenCase("repeats_3chr")
    index = str(tmp_path / "index")
    fa = tmp_path / "genome.fa"
    synth.write_fasta(str(fa), gc.genome, gc.chrom_lengths)
    RefOracle().build_index(str(fa), index, 16)
    ro = RefOracle(index)
    reads = gc.seed_reads()
    for run in gc.seed_runs():
        mode, ss, filt, minc, intron = run
        assert ro.seeds_cals(mode, reads, ss, filt, minc, intron, len(gc.chrom_lengths)) == gc.seed_expected(*run)
    ro.close()
