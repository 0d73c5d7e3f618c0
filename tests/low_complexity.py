"""A low-complexity genome and reads whose hit intervals hold thousands of rows."""
from __future__ import annotations

import numpy as np

from hpgbwt import lib, synth


def low_complexity_case(tmp):
    """300 kbp i.i.d. genome with a 1.5 kbp G run, 100 scattered 170 bp G runs and
    (AC)/(AGT) tandem runs: reads drawn from them hit thousands of rows per interval
    and fill the result list (indel variants of one homopolymer interval)."""
    rng = np.random.default_rng(5)
    g = rng.integers(0, 4, size=300_000, dtype=np.uint8)
    g[10_000:11_500] = 2
    g[50_000:52_000] = np.resize(np.array([0, 1], dtype=np.uint8), 2000)
    g[90_000:91_800] = np.resize(np.array([0, 2, 3], dtype=np.uint8), 1800)
    for s in rng.integers(100_000, 290_000, size=100):
        g[s:s + 170] = 2
    fasta = str(tmp / "genome.fa")
    synth.write_fasta(fasta, g, [150_000, 150_000])
    index = str(tmp / "index")
    lib.build_index(fasta, index, 16)
    seqs = [b"G" * 150, b"C" * 150, b"G" * 120, b"G" * 149 + b"A", b"T" + b"G" * 99, b"AC" * 75, b"CA" * 60,
            b"AGT" * 50, b"ACT" * 40, b"G" * 60 + b"T" + b"G" * 60]
    A = np.frombuffer(b"ACGT", dtype=np.uint8)
    for s in rng.integers(0, 299_800, size=100):
        seqs.append(A[g[s:s + 120]].tobytes())
    return index, synth.from_strings(seqs)
