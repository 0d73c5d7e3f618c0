"""TEST INFRASTRUCTURE ONLY: the C restatement's speed against the compiled
reference on the same cores, reads and index (one thread each).

The GPU machine runs the restatement (oracle/fm_oracle.c) as the timed CPU
baseline, because the compiled reference (oracle/_ref/libhpgref.so, built from
the reference's own sources by oracle/ref/Makefile) exists only where those
sources are.  This script measures, where both exist, how the restatement's
search-level rate compares with the reference's own BWExactSearchBackward /
BWSearch1VectorHelper + locate loop, so the baseline's stand-in is a number,
not an assumption.  It also checks that both give the same records.

    python oracle/ref/speed_vs_port.py [reads]
"""
from __future__ import annotations

import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT / "hpg-libs_gb300"))
sys.path.insert(0, str(ROOT))

from hpgbwt import build, lib, synth  # noqa: E402
from oracle.pyoracle import PortOracle, RefOracle, ref_available  # noqa: E402


def main() -> int:
    n_reads = int(sys.argv[1]) if len(sys.argv) > 1 else 20_000
    build.build_oracle()
    build.build_reference_oracle()
    if not ref_available():
        print("the compiled reference is not available (no reference checkout here)")
        return 1
    cases = [("4 Mbp i.i.d. genome, 100 bp error-free reads", "iid", 4_000_000, "none", 100, 0),
             ("20 Mbp repeat-rich genome, 100 bp reads, <=1 edit", "repeats", 20_000_000, "per_base_capped", 100, 1),
             ("20 Mbp repeat-rich genome, 36-250 bp reads, 30/50/20 mix", "repeats", 20_000_000, "mix_30_50_20",
              (36, 250), 1)]
    with tempfile.TemporaryDirectory() as td:
        for label, kind, size, edits, length, mode in cases:
            g = synth.genome(kind, size, 1)
            fa, idx = f"{td}/{kind}{size}.fa", f"{td}/{kind}{size}"
            if not Path(idx).exists():
                synth.write_fasta(fa, g)
                lib.build_index(fa, idx, 16)
            reads = synth.reads(g, n_reads, 2, length=length, edits=edits)
            ref, port = RefOracle(idx), PortOracle(idx)
            for m in ([0, 1] if mode == 0 else [1]):
                t = time.perf_counter()
                a = ref.search(reads, mode=m, max_results=1024)
                tr = time.perf_counter() - t
                t = time.perf_counter()
                b = port.search(reads, mode=m, max_results=1024, threads=1)
                tp = time.perf_counter() - t
                same = a.equal(b)
                print(f"{label}, mode {'exact' if m == 0 else 'BWSearch1'}: reference {n_reads / tr:,.0f} reads/s, "
                      f"restatement {n_reads / tp:,.0f} reads/s (x{tr / tp:.2f}), records equal: {same}")
            ref.close()
            port.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
