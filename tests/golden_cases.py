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

    def block_capacities(self) -> list[int]:
        """Result-list capacities of the recorded k-error block searches."""
        return sorted(int(k[5:-6]) for k in self.arrays if k.startswith("blk_r") and k.endswith("_bhits"))

    def block_expected(self, mr: int) -> lib.BlockResult:
        """The reference's block search (rs_truncated is not recorded: all 0)."""
        a = self.arrays
        hits = a[f"blk_r{mr}_bhits"]
        res = lib.Result(hits.view(lib.HIT_DTYPE) if hits.dtype != lib.HIT_DTYPE else hits, a[f"blk_r{mr}_blocs"],
                         a[f"blk_r{mr}_bcount"], np.zeros_like(a[f"blk_r{mr}_bcount"], dtype=np.uint8))
        anch = a[f"blk_r{mr}_banch"]
        return lib.BlockResult(res, anch.view(lib.ANCHOR_DTYPE) if anch.dtype != lib.ANCHOR_DTYPE else anch,
                               a[f"blk_r{mr}_bnanch"])

    def api_runs(self):
        """(api, filter_read_mappings, flag) of the recorded alignment-list runs."""
        out = []
        for k in self.arrays:
            if k.startswith("api") and "_f" in k:
                a, f, g = k[3:].split("_")
                out.append((int(a), int(f[1:]), int(g[1:])))
        return sorted(out)

    def api_fastq(self):
        import api_lists
        s, o = self.arrays["api_seq"], self.arrays["api_offs"]
        return api_lists.FastqSet([s[o[i]:o[i + 1]].tobytes() for i in range(len(o) - 1)])

    def api_expected(self, api: int, filt: int, flag: int, n_reads: int):
        import api_lists
        return api_lists.parse_blob(api, self.arrays[f"api{api}_f{filt}_g{flag}"].tobytes(), n_reads)

    def seed_runs(self):
        """(mode, seed_size, filter_seed_mappings, min_cal_size, max_intron_size) of the recorded seed/CAL runs."""
        out = []
        for k in self.arrays:
            if k.startswith("seed") and k[4:5].isdigit():
                m, s, f, c, i = k[4:].split("_")
                out.append((int(m), int(s[1:]), int(f[1:]), int(c[1:]), int(i[1:])))
        return sorted(out)

    def seed_reads(self) -> list[bytes]:
        s, o = self.arrays["seed_seq"], self.arrays["seed_offs"]
        return [s[o[i]:o[i + 1]].tobytes() for i in range(len(o) - 1)]

    def seed_expected(self, mode: int, seed_size: int, filt: int, min_cal: int, intron: int) -> bytes:
        return self.arrays[f"seed{mode}_s{seed_size}_f{filt}_c{min_cal}_i{intron}"].tobytes()

    def build(self, tmp: Path) -> str:
        fa = tmp / "genome.fa"
        synth.write_fasta(str(fa), self.genome, self.chrom_lengths)
        lib.build_index(str(fa), str(tmp / "index"), int(self.meta["sa_ratio"]))
        return str(tmp / "index")


def names():
    return sorted(manifest())
