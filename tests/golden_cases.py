"""Loader of the committed golden fixtures (tests/golden/, made by make_golden.py)."""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np

from hpgbwt import lib, synth

GOLDEN = Path(__file__).resolve().parent / "golden"


def manifest() -> dict:
    return json.loads((GOLDEN / "manifest.json").read_text())


class GoldenCase:
    def __init__(self, name: str):
        self.name = name
        self.meta = manifest()[name]
        z = np.load(GOLDEN / f"{name}.npz")
        self.arrays = {k: z[k] for k in z.files}
        n = int(self.arrays["genome_len"][0])
        bits = np.unpackbits(self.arrays["genome_2bit"])[: 2 * n].reshape(n, 2)
        self.genome = (bits[:, 0] * 2 + bits[:, 1]).astype(np.uint8)
        self.chrom_lengths = [int(x) for x in self.arrays["chrom_lengths"]]
        self.reads = synth.ReadSet(self.arrays["seq"], self.arrays["offsets"].astype(np.uint64),
                                   np.zeros(1), np.zeros(1), np.zeros(1))

    def tags(self):
        return sorted(k[:-5] for k in self.arrays if k.endswith("_hits"))

    def expected(self, tag: str) -> lib.Result:
        a = self.arrays
        return lib.Result(a[f"{tag}_hits"].view(lib.HIT_DTYPE) if a[f"{tag}_hits"].dtype != lib.HIT_DTYPE
                          else a[f"{tag}_hits"], a[f"{tag}_locs"], a[f"{tag}_count"], a[f"{tag}_trunc"])

    def build(self, tmp: Path) -> str:
        fa = tmp / "genome.fa"
        synth.write_fasta(str(fa), self.genome, self.chrom_lengths)
        lib.build_index(str(fa), str(tmp / "index"), int(self.meta["sa_ratio"]))
        return str(tmp / "index")


def names():
    return sorted(manifest())
