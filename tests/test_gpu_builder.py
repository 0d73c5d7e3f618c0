"""Index builder with the suffix arrays on the GPU: every file byte-identical to
the reference builder's (SHA-256 recorded in the golden manifest) and to the
host builder's, over genomes with long exact repeats (many doubling rounds),
tiny texts and several sampling ratios."""
from __future__ import annotations

import hashlib
from pathlib import Path

import numpy as np
import pytest

from golden_cases import GoldenCase, names
from hpgbwt import lib, synth

pytestmark = pytest.mark.gpu


def _files(d: Path) -> dict:
    return {p.name: hashlib.sha256(p.read_bytes()).hexdigest() for p in sorted(d.iterdir())}


@pytest.mark.parametrize("name", names())
def test_gpu_builder_matches_reference_files(tmp_path, name):
    gc = GoldenCase(name)
    fa = tmp_path / "g.fa"
    synth.write_fasta(str(fa), gc.genome, gc.chrom_lengths)
    lib.build_index(str(fa), str(tmp_path / "idx"), int(gc.meta["sa_ratio"]), device=0)
    assert _files(tmp_path / "idx") == gc.meta["index_sha256"]


def _genomes():
    rng = np.random.default_rng(4)
    yield "repeats", synth.genome("repeats", 400_000, 11), [150_000, 250_000]
    yield "human_like", synth.genome("human_like", 300_000, 12), [300_000]
    yield "one_letter", np.zeros(40_000, dtype=np.uint8), [40_000]           # LCP up to n: every round
    yield "two_letter", np.tile(np.array([0, 1], np.uint8), 30_000), [30_000, 30_000]
    yield "tiny", rng.integers(0, 4, 7, dtype=np.uint8), [7]
    yield "single", np.array([2], np.uint8), [1]


@pytest.mark.parametrize("ratio", [16, 1, 10, 32])
def test_gpu_builder_matches_host_builder(tmp_path, ratio):
    for label, g, chroms in _genomes():
        d = tmp_path / label
        d.mkdir()
        synth.write_fasta(str(d / "g.fa"), g, chroms)
        lib.build_index(str(d / "g.fa"), str(d / "host"), ratio, device=-1)
        lib.build_index(str(d / "g.fa"), str(d / "gpu"), ratio, device=0)
        host, gpu = _files(d / "host"), _files(d / "gpu")
        assert host == gpu, f"{label}: files differ"


def test_gpu_built_index_maps(tmp_path):
    """A GPU-built index loads and maps like the host-built one."""
    g = synth.genome("repeats", 500_000, 13)
    synth.write_fasta(str(tmp_path / "g.fa"), g, [500_000])
    lib.build_index(str(tmp_path / "g.fa"), str(tmp_path / "gpu"), 16, device=0)
    lib.build_index(str(tmp_path / "g.fa"), str(tmp_path / "host"), 16)
    reads = synth.reads(g, 3000, 14, length=100, edits="mix_30_50_20")
    with lib.GpuIndex(str(tmp_path / "gpu")) as a, lib.GpuIndex(str(tmp_path / "host")) as b:
        assert a.search(reads, form=lib.FORM_BATCHED).equal(b.search(reads, form=lib.FORM_BATCHED))
