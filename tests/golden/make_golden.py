"""Generate the golden fixtures in tests/golden/ from the reference's own code.

Run in a container that has the read-only reference tree (the fixtures are
committed; the GPU machine and CI only read them):

    python hpg-libs_gb300/hpgbwt/build.py          # builds oracle/_ref/libhpgref.so
    python tests/golden/make_golden.py

For every case it stores the genome (2-bit codes + chromosome lengths), the
SHA-256 of every index file written by the reference builder
(bwt_generate_index_files, bwt.c:744-819, at SA ratio 16), the reads, and the
reference's search outputs (oracle/ref/ref_harness.c: BWExactSearchBackward
on both strands, and the four vector searches + BWSearch1VectorHelper per
strand with the bwt.c:2158-2166 locate; the k-error block search BWSearchCPU
with its anchors) for several result-list capacities, and the alignment lists
of the entry points.
"""
from __future__ import annotations

import hashlib
import json
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT / "hpg-libs_gb300"))
sys.path.insert(0, str(ROOT))

sys.path.insert(0, str(ROOT / "tests"))
from hpgbwt import synth  # noqa: E402
from oracle.pyoracle import RefOracle, ref_available  # noqa: E402
import api_lists  # noqa: E402

# Alignment-list entry points recorded per case: (api, filter_read_mappings, list flag).
API_RUNS = [(api_lists.API_EXACT_READ, 200, 0), (api_lists.API_EXACT_READ, 2, 0),
            (api_lists.API_EXACT_SEQS, 200, 0), (api_lists.API_EXACT_BATCH, 200, 0),
            (api_lists.API_INEXACT_READ, 200, 0), (api_lists.API_INEXACT_READ, 3, 0),
            (api_lists.API_INEXACT_READ, 200, 1), (api_lists.API_INEXACT_READ, 3, 1),
            (api_lists.API_INEXACT_READ, 0, 1),
            (api_lists.API_INEXACT_READ2, 200, 0), (api_lists.API_INEXACT_READ2, 3, 0),
            (api_lists.API_INEXACT_READ2, 200, 1), (api_lists.API_INEXACT_READ2, 3, 1),
            (api_lists.API_INEXACT_READ2, 0, 1)]
API_READS = 400  # first reads of each case taken through the entry points

# Seeds and CALs recorded per case (ref_seeds_cals): (mode 0 bwt_map_exact_seeds_seq /
# 1 bwt_generate_cals / 2 bwt_map_exact_seeds_by_region, seed_size, filter_seed_mappings,
# min_cal_size, max_intron_size); mode 2 reads the last two as the window [a, len - b).
SEED_RUNS = [(0, 16, 300, 0, 0), (0, 20, 4, 0, 0), (1, 16, 300, 20, 500_000), (1, 20, 40, 30, 1_000),
             (1, 8, 300, 60, 200), (2, 16, 300, 5, 3), (2, 20, 40, 0, 7), (2, 8, 300, 11, 0)]
SEED_READS = 300


def seed_read_set(seq: np.ndarray, offs: np.ndarray) -> list[bytes]:
    """Reads the seed entry points are recorded on: upper-case A/C/G/T only and
    at least 40 bases, so that every seed of the reference's plan lies inside
    the read (the plan reaches past shorter reads, which the reference then
    reads beyond their end)."""
    out = []
    for i in range(len(offs) - 1):
        s = seq[offs[i]:offs[i + 1]].tobytes()
        if len(s) >= 40 and not s.strip(b"ACGT"):
            out.append(s)
        if len(out) == SEED_READS:
            break
    return out


def api_read_set(seq: np.ndarray, offs: np.ndarray) -> list[bytes]:
    """Reads the entry points are recorded on: upper-case A/C/G/T only (other
    characters index an uninitialised table in the reference, bwt_commons.c:60-92)
    and at least 4 bases (shorter reads overflow the reference's cigar buffer,
    bwt.c:960-961)."""
    out = []
    for i in range(len(offs) - 1):
        s = seq[offs[i]:offs[i + 1]].tobytes()
        if len(s) >= 4 and not s.strip(b"ACGT"):
            out.append(s)
        if len(out) == API_READS:
            break
    return out


def spliced_reads(g: np.ndarray, n: int, seed: int) -> list[bytes]:
    """Reads joined from two pieces of the genome 30-3000 bases apart (either
    strand), whose seeds fall into two CALs, one often below min_cal_size: they
    exercise the CAL merges and the candidate seed lists."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        L = int(rng.integers(60, 160))
        L1 = int(rng.integers(16, L - 16))
        gap = int(rng.integers(30, 3000))
        a = int(rng.integers(0, len(g) - L - gap - 1))
        s = np.concatenate([g[a:a + L1], g[a + L1 + gap:a + gap + L]])
        if rng.random() < 0.5:
            s = 3 - s[::-1]
        out.append(A[s].tobytes())
    return out

CASES = [
    # name, genome kind, length, seed, chromosome lengths, reads: (n, seed, length, edits), max_results list
    ("iid_1chr", "iid", 30_000, 101, None, (1200, 5, 100, "mix_30_50_20"), [1 << 16, 4]),
    ("repeats_3chr", "repeats", 60_000, 102, [25_000, 20_000, 15_000], (1500, 6, (20, 150), "mix_30_50_20"),
     [1 << 16, 3]),
    ("lowcomplexity_2chr", "human_like", 16_000, 103, [10_000, 6_000], (250, 7, (3, 120), "mix_30_50_20"),
     [1 << 16, 0, 2, 17]),
]

A = np.frombuffer(b"ACGT", dtype=np.uint8)


def edge_reads(g: np.ndarray, chrom_lengths: list[int]) -> list[bytes]:
    """Reads the reference's edge behaviour hinges on."""
    out = [b"", b"A", b"AC", b"ACG", b"ACGT", A[g[10:15]].tobytes(), b"ACGTN" * 8, A[g[100:160]].tobytes().lower(),
           A[g[:50]].tobytes(), A[g[-50:]].tobytes(), b"T" * 200, b"GA" * 60]
    pos = 0
    for cl in chrom_lengths[:-1]:  # reads spanning chromosome junctions (located but invalid)
        pos += cl
        out.append(A[g[pos - 40:pos + 40]].tobytes())
    return out


def sha(path: Path) -> str:
    return hashlib.sha256(path.read_bytes()).hexdigest()


def main() -> int:
    if not ref_available():
        print("oracle/_ref/libhpgref.so is missing: build it where the reference tree exists", file=sys.stderr)
        return 1
    manifest = {}
    for name, kind, n, seed, chroms, rd, maxes in CASES:
        g = synth.genome(kind, n, seed)
        cl = chroms or [n]
        reads = synth.reads(g, rd[0], rd[1], length=rd[2], edits=rd[3])
        extra = synth.from_strings(edge_reads(g, cl))
        seq = np.concatenate([reads.seq, extra.seq])
        offs = np.concatenate([reads.offsets, extra.offsets[1:] + reads.offsets[-1]]).astype(np.uint64)
        with tempfile.TemporaryDirectory() as td:
            fa = Path(td) / "genome.fa"
            synth.write_fasta(str(fa), g, cl)
            ref = RefOracle()
            ref.build_index(str(fa), str(Path(td) / "index"), 16)
            hashes = {p.name: sha(p) for p in sorted((Path(td) / "index").iterdir())}
            ro = RefOracle(str(Path(td) / "index"))

            class RS:
                pass
            rs = RS()
            rs.seq, rs.offsets = seq, offs
            arrays = {"genome_2bit": np.packbits(np.unpackbits(g[:, None], axis=1)[:, 6:].reshape(-1)),
                      "genome_len": np.array([len(g)]), "chrom_lengths": np.array(cl, dtype=np.int64),
                      "seq": seq, "offsets": offs}
            for mode in (0, 1):
                for mr in (maxes if mode == 1 else [1 << 16]):
                    r = ro.search(rs, mode=mode, max_results=mr)
                    tag = f"m{mode}_r{mr}"
                    arrays[f"{tag}_hits"] = r.hits
                    arrays[f"{tag}_locs"] = r.locs
                    arrays[f"{tag}_count"] = r.rs_count
                    arrays[f"{tag}_trunc"] = r.rs_truncated
            for mr in maxes:  # the k-error block search (BWSearchCPU as bwt_map_inexact_read_2 runs it)
                b = ro.block_search(rs, max_results=mr)
                arrays[f"blk_r{mr}_bhits"] = b.result.hits
                arrays[f"blk_r{mr}_blocs"] = b.result.locs
                arrays[f"blk_r{mr}_bcount"] = b.result.rs_count
                arrays[f"blk_r{mr}_banch"] = b.anchors
                arrays[f"blk_r{mr}_bnanch"] = b.n_anchors
            edge = synth.from_strings(edge_reads(g, cl))
            fq = api_lists.FastqSet(api_read_set(seq, offs)[:API_READS - 20] + api_read_set(edge.seq, edge.offsets))
            arrays["api_seq"] = np.frombuffer(b"".join(fq.seqs), dtype=np.uint8)
            arrays["api_offs"] = np.cumsum([0] + [len(x) for x in fq.seqs]).astype(np.uint64)
            for api, filt, flag in API_RUNS:
                arrays[f"api{api}_f{filt}_g{flag}"] = np.frombuffer(ro.map_api(api, fq, filt, flag), dtype=np.uint8)
            sreads = seed_read_set(seq, offs) + spliced_reads(g, 100, seed)
            arrays["seed_seq"] = np.frombuffer(b"".join(sreads), dtype=np.uint8)
            arrays["seed_offs"] = np.cumsum([0] + [len(x) for x in sreads]).astype(np.uint64)
            for mode, ss, filt, minc, intron in SEED_RUNS:
                arrays[f"seed{mode}_s{ss}_f{filt}_c{minc}_i{intron}"] = np.frombuffer(
                    ro.seeds_cals(mode, sreads, ss, filt, minc, intron, len(cl)), dtype=np.uint8)
            ro.close()
        np.savez_compressed(HERE / f"{name}.npz", **arrays)
        manifest[name] = {"kind": kind, "length": n, "seed": seed, "chrom_lengths": cl, "sa_ratio": 16,
                          "index_sha256": hashes, "max_results": maxes, "reads": len(offs) - 1}
        print(name, {k: v.shape for k, v in arrays.items() if k.endswith("_hits")})
    (HERE / "manifest.json").write_text(json.dumps(manifest, indent=1) + "\n")
    return 0


if __name__ == "__main__":
    sys.exit(main())
