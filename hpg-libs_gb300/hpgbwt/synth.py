"""Seeded synthetic genomes and reads with the shapes of the benchmark workloads.

No public dataset is involved: every genome and read set is generated here
from a seed, with the sizes, base composition, repeat structure and error
model of the named workload.  Bases are 2-bit codes in the alphabet order
A=0, C=1, G=2, T=3 (the default ``config.txt`` of the reference builder,
c/src/aligners/bwt/bwt.c:744-757).

Workloads
---------
- ``iid``:      i.i.d. uniform A/C/G/T (4 Mbp exact-search workload).
- ``repeats``:  GC 41 % background plus 5 % of the length as copies of
                300 bp elements at 85-95 % identity (100 Mbp workloads).
- ``human_like``: GC 41 %, 45 % repeats: 300 bp elements (10 %), 6 kbp
                elements (17 %) at 80-98 % identity, the rest (18 %) 1-6 bp
                tandem repeats (3.1 Gbp workloads).
"""
from __future__ import annotations

import numpy as np

ALPHABET = b"ACGT"
_COMP = np.array([3, 2, 1, 0], dtype=np.uint8)
_ASCII = np.frombuffer(ALPHABET, dtype=np.uint8)


def background(n: int, rng: np.random.Generator, gc: float = 0.5) -> np.ndarray:
    p_at = (1.0 - gc) / 2.0
    p_cg = gc / 2.0
    return rng.choice(4, size=n, p=[p_at, p_cg, p_cg, p_at]).astype(np.uint8)


def _mutate(seq: np.ndarray, identity: float, rng: np.random.Generator) -> np.ndarray:
    out = seq.copy()
    m = rng.random(len(out)) > identity
    out[m] = (out[m] + rng.integers(1, 4, size=int(m.sum()), dtype=np.uint8)) % 4
    return out


def _plant_elements(g: np.ndarray, frac: float, elem_len: int, families: int, ident: tuple[float, float],
                    gc: float, rng: np.random.Generator) -> None:
    """Overwrite ~frac*len(g) bases with mutated copies of `families` elements."""
    n = len(g)
    copies = int(frac * n) // elem_len
    if copies == 0:
        return
    elems = [background(elem_len, rng, gc) for _ in range(families)]
    fam = rng.integers(0, families, size=copies)
    starts = rng.integers(0, n - elem_len, size=copies)
    idents = rng.uniform(ident[0], ident[1], size=copies)
    for f, s, idt in zip(fam, starts, idents):
        g[s:s + elem_len] = _mutate(elems[f], idt, rng)


def _plant_tandem(g: np.ndarray, frac: float, rng: np.random.Generator) -> None:
    n = len(g)
    target = int(frac * n)
    done = 0
    while done < target:
        unit = rng.integers(0, 4, size=int(rng.integers(1, 7)), dtype=np.uint8)
        length = int(rng.integers(20, 400))
        s = int(rng.integers(0, n - length))
        g[s:s + length] = np.resize(unit, length)
        done += length


def genome(kind: str, n: int, seed: int) -> np.ndarray:
    """Genome codes (uint8, values 0..3) of length n."""
    rng = np.random.default_rng(seed)
    if kind == "iid":
        return rng.integers(0, 4, size=n, dtype=np.uint8)
    if kind == "repeats":
        g = background(n, rng, 0.41)
        _plant_elements(g, 0.05, 300, 16, (0.85, 0.95), 0.41, rng)
        return g
    if kind == "human_like":
        g = background(n, rng, 0.41)
        _plant_elements(g, 0.10, 300, 64, (0.80, 0.98), 0.41, rng)
        _plant_elements(g, 0.17, 6000, 32, (0.80, 0.98), 0.41, rng)
        _plant_tandem(g, 0.18, rng)
        return g
    raise ValueError(f"unknown genome kind {kind!r}")


def write_fasta(path: str, g: np.ndarray, chrom_lengths: list[int] | None = None, width: int = 80) -> None:
    """Write codes as FASTA; chrom_lengths splits the genome into chromosomes."""
    if chrom_lengths is None:
        chrom_lengths = [len(g)]
    assert sum(chrom_lengths) == len(g)
    with open(path, "wb") as f:
        pos = 0
        for ci, cl in enumerate(chrom_lengths):
            f.write(b">chr%d synthetic\n" % (ci + 1))
            seq = _ASCII[g[pos:pos + cl]]
            pos += cl
            full = (cl // width) * width
            if full:
                block = np.empty((full // width, width + 1), dtype=np.uint8)
                block[:, :width] = seq[:full].reshape(-1, width)
                block[:, width] = ord("\n")
                f.write(block.tobytes())
            if cl > full:
                f.write(seq[full:].tobytes() + b"\n")


def revcomp_codes(codes: np.ndarray) -> np.ndarray:
    return _COMP[codes[::-1]]


class ReadSet:
    """Reads as concatenated ASCII bytes plus offsets (n+1 entries)."""

    def __init__(self, seq: np.ndarray, offsets: np.ndarray, truth_pos: np.ndarray, truth_strand: np.ndarray,
                 edit: np.ndarray):
        self.seq = seq            # uint8 ASCII, concatenated
        self.offsets = offsets    # uint64, n+1
        self.truth_pos = truth_pos
        self.truth_strand = truth_strand
        self.edit = edit          # 0 none, 1 substitution, 2 insertion in read, 3 deletion from read

    def __len__(self) -> int:
        return len(self.offsets) - 1

    def read(self, i: int) -> bytes:
        return self.seq[self.offsets[i]:self.offsets[i + 1]].tobytes()

    def lengths(self) -> np.ndarray:
        return np.diff(self.offsets).astype(np.int64)

    def subset(self, idx) -> "ReadSet":
        idx = np.asarray(idx)
        lens = self.lengths()[idx]
        offs = np.zeros(len(idx) + 1, dtype=np.uint64)
        np.cumsum(lens, out=offs[1:])
        parts = [self.seq[self.offsets[i]:self.offsets[i + 1]] for i in idx]
        seq = np.concatenate(parts) if parts else np.zeros(0, dtype=np.uint8)
        return ReadSet(seq, offs, self.truth_pos[idx], self.truth_strand[idx], self.edit[idx])


def _edit_plan(kind: str, n: int, lens: np.ndarray, rng: np.random.Generator) -> np.ndarray:
    """Per-read edit: 0 none, 1 substitution, 2 insertion, 3 deletion."""
    if kind == "none":
        return np.zeros(n, dtype=np.int8)
    if kind == "per_base_capped":  # 0.5 % subst, 0.02 % ins, 0.02 % del per base, at most one edit
        p_s, p_i, p_d = 0.005, 0.0002, 0.0002
        p_any = 1.0 - (1.0 - p_s - p_i - p_d) ** lens
        has = rng.random(n) < p_any
        which = rng.choice(3, size=n, p=np.array([p_s, p_i, p_d]) / (p_s + p_i + p_d)) + 1
        return np.where(has, which, 0).astype(np.int8)
    if kind == "subst_capped":  # 0.5 % substitution per base, at most one
        has = rng.random(n) < 1.0 - (1.0 - 0.005) ** lens
        return np.where(has, 1, 0).astype(np.int8)
    if kind == "mix_30_50_20":  # 30 % exact, 50 % one substitution, 20 % one indel
        u = rng.random(n)
        e = np.zeros(n, dtype=np.int8)
        e[(u >= 0.30) & (u < 0.80)] = 1
        indel = u >= 0.80
        e[indel] = np.where(rng.random(int(indel.sum())) < 0.5, 2, 3)
        return e
    raise ValueError(kind)


def reads(g: np.ndarray, n: int, seed: int, length: int | tuple[int, int] = 100, edits: str = "none",
          subst_rate: float = 0.0) -> ReadSet:
    """Sample n reads from uniform positions on either strand (50/50).

    `length` is fixed or (lo, hi) uniform inclusive.  `edits` selects the
    capped single-edit models; `subst_rate` adds independent per-base
    substitutions (uncapped) on top.
    """
    rng = np.random.default_rng(seed)
    if isinstance(length, tuple):
        lens = rng.integers(length[0], length[1] + 1, size=n)
    else:
        lens = np.full(n, int(length))
    plan = _edit_plan(edits, n, lens, rng)
    glen = len(g)
    span = lens + 1  # room for one deleted base
    pos = (rng.random(n) * (glen - span)).astype(np.int64)
    strand = (rng.random(n) < 0.5).astype(np.int8)
    out = np.empty(int(lens.sum()), dtype=np.uint8)
    offs = np.zeros(n + 1, dtype=np.uint64)
    np.cumsum(lens, out=offs[1:])
    for i in range(n):
        L = int(lens[i])
        p = int(pos[i])
        e = int(plan[i])
        if e == 3:  # one base of the fragment is left out of the read
            frag = g[p:p + L + 1].copy()
            cut = int(rng.integers(1, L))
            frag = np.delete(frag, cut)
        elif e == 2:  # one extra base inside the read
            frag = g[p:p + L - 1].copy()
            at = int(rng.integers(1, L - 1))
            frag = np.insert(frag, at, np.uint8(rng.integers(0, 4)))
        else:
            frag = g[p:p + L].copy()
            if e == 1:
                at = int(rng.integers(0, L))
                frag[at] = (frag[at] + rng.integers(1, 4)) % 4
        if subst_rate > 0:
            m = rng.random(L) < subst_rate
            frag[m] = (frag[m] + rng.integers(1, 4, size=int(m.sum()), dtype=np.uint8)) % 4
        if strand[i]:
            frag = revcomp_codes(frag)
        out[offs[i]:offs[i + 1]] = _ASCII[frag]
    return ReadSet(out, offs, pos, strand, plan)


def reads_fast(g: np.ndarray, n: int, seed: int, length: int = 100, edits: str = "none",
               subst_rate: float = 0.0) -> ReadSet:
    """Vectorised sampler for fixed-length reads (large read sets)."""
    rng = np.random.default_rng(seed)
    L = int(length)
    lens = np.full(n, L)
    plan = _edit_plan(edits, n, lens, rng)
    glen = len(g)
    pos = (rng.random(n) * (glen - L - 1)).astype(np.int64)
    strand = (rng.random(n) < 0.5).astype(np.int8)
    idx = pos[:, None] + np.arange(L + 1)[None, :]
    frag = g[idx]                                   # n x (L+1)
    # deletions: drop column `cut`, keeping L of the L+1 bases
    cut = rng.integers(1, L, size=n)
    col = np.arange(L)[None, :]
    del_src = np.where(col >= cut[:, None], col + 1, col)
    # insertions: an extra random base at `at`, the rest shifted right
    at = rng.integers(1, L - 1, size=n)
    ins_src = np.where(col > at[:, None], col - 1, col)
    base = frag[:, :L].copy()
    d = plan == 3
    base[d] = np.take_along_axis(frag[d], del_src[d], axis=1)
    ii = plan == 2
    if ii.any():
        shifted = np.take_along_axis(frag[ii], ins_src[ii], axis=1)
        rows = np.nonzero(ii)[0]
        shifted[np.arange(len(rows)), at[ii]] = rng.integers(0, 4, size=len(rows), dtype=np.uint8)
        base[ii] = shifted
    s = plan == 1
    sat = rng.integers(0, L, size=n)
    rows = np.nonzero(s)[0]
    base[rows, sat[s]] = (base[rows, sat[s]] + rng.integers(1, 4, size=len(rows), dtype=np.uint8)) % 4
    if subst_rate > 0:
        m = rng.random((n, L)) < subst_rate
        base[m] = (base[m] + rng.integers(1, 4, size=int(m.sum()), dtype=np.uint8)) % 4
    rc = strand == 1
    base[rc] = _COMP[base[rc][:, ::-1]]
    seq = _ASCII[base].reshape(-1)
    offs = np.arange(n + 1, dtype=np.uint64) * np.uint64(L)
    return ReadSet(seq, offs, pos, strand, plan)


def from_strings(seqs: list[bytes]) -> ReadSet:
    lens = np.array([len(s) for s in seqs], dtype=np.int64)
    offs = np.zeros(len(seqs) + 1, dtype=np.uint64)
    np.cumsum(lens, out=offs[1:])
    seq = np.frombuffer(b"".join(seqs), dtype=np.uint8).copy()
    z = np.zeros(len(seqs), dtype=np.int64)
    return ReadSet(seq, offs, z, z.astype(np.int8), z.astype(np.int8))


def reads_fast_var(g: np.ndarray, n: int, seed: int, lo: int, hi: int, edits: str = "none",
                   chunk: int = 200_000, subst_rate: float = 0.0) -> ReadSet:
    """Vectorised sampler for reads of uniform length in [lo, hi] (large read
    sets): the same models as reads(), drawn row-wise over fixed-width tiles;
    subst_rate adds independent per-base substitutions (uncapped) on top."""
    rng = np.random.default_rng(seed)
    lens = rng.integers(lo, hi + 1, size=n)
    plan = _edit_plan(edits, n, lens, rng)
    pos = (rng.random(n) * (len(g) - lens - 1)).astype(np.int64)
    strand = (rng.random(n) < 0.5).astype(np.int8)
    cut = (rng.random(n) * (lens - 1)).astype(np.int64) + 1          # deletion: in [1, L)
    at = (rng.random(n) * np.maximum(lens - 2, 1)).astype(np.int64) + 1  # insertion: in [1, L-1)
    ins_base = rng.integers(0, 4, size=n, dtype=np.uint8)
    sat = (rng.random(n) * lens).astype(np.int64)                     # substitution: in [0, L)
    sdelta = rng.integers(1, 4, size=n, dtype=np.uint8)
    offs = np.zeros(n + 1, dtype=np.uint64)
    np.cumsum(lens, out=offs[1:])
    out = np.empty(int(offs[-1]), dtype=np.uint8)
    W = hi + 1
    col = np.arange(hi)[None, :]
    for a in range(0, n, chunk):
        b = min(n, a + chunk)
        L = lens[a:b, None]
        frag = g[np.minimum(pos[a:b, None] + np.arange(W)[None, :], len(g) - 1)]  # rows x (hi + 1); past L unused
        src = col.repeat(b - a, axis=0)
        d = np.nonzero(plan[a:b] == 3)[0]
        src[d] = np.where(col >= cut[a:b][d, None], col + 1, col)
        ii = np.nonzero(plan[a:b] == 2)[0]
        src[ii] = np.where(col > at[a:b][ii, None], col - 1, col)
        base = np.take_along_axis(frag, src, axis=1)
        base[ii, at[a:b][ii]] = ins_base[a:b][ii]
        rows = np.nonzero(plan[a:b] == 1)[0]
        base[rows, sat[a:b][rows]] = (base[rows, sat[a:b][rows]] + sdelta[a:b][rows]) % 4
        if subst_rate > 0:
            m = rng.random(base.shape) < subst_rate
            base[m] = (base[m] + rng.integers(1, 4, size=int(m.sum()), dtype=np.uint8)) % 4
        rc = np.nonzero(strand[a:b] == 1)[0]
        if len(rc):
            ridx = np.clip(L[rc] - 1 - col, 0, hi - 1)
            base[rc] = _COMP[np.take_along_axis(base[rc], ridx, axis=1)]
        keep = col < L
        out[offs[a]:offs[b]] = _ASCII[base[keep]]
    return ReadSet(out, offs, pos, strand, plan)


def _skip(rng: np.random.Generator, n: int) -> None:
    """Advance rng past n 64-bit outputs as drawing n doubles would: PCG64's
    advance() drops the buffered half of a 64-bit output that 32-bit draws
    keep, and drawing doubles leaves it in place, so it is put back."""
    before = rng.bit_generator.state
    rng.bit_generator.advance(n)
    after = rng.bit_generator.state
    after["has_uint32"], after["uinteger"] = before["has_uint32"], before["uinteger"]
    rng.bit_generator.state = after


def _uniform_threads(rng: np.random.Generator, shape, chunk: int = 1 << 22) -> np.ndarray:
    """rng.random(shape), the same doubles (one 64-bit PCG64 output each), filled
    by host threads from copies of the generator advanced to their slice."""
    import concurrent.futures as cf
    import os
    out = np.empty(shape, dtype=np.float64)
    flat = out.reshape(-1)
    state = rng.bit_generator.state

    def fill(a: int) -> None:
        bg = np.random.PCG64()
        bg.state = state
        bg.advance(a)
        np.random.Generator(bg).random(out=flat[a:a + chunk])

    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 1)) as ex:
        list(ex.map(fill, range(0, flat.size, chunk)))
    _skip(rng, flat.size)
    return out


def _background_draws(g: np.ndarray, rng: np.random.Generator, cum: np.ndarray, chunk: int) -> None:
    """g[i] = number of thresholds in cum that are <= the i-th uniform double of
    rng's stream (one 64-bit PCG64 output per double), filled by host threads
    from copies of the generator advanced to their slice of the stream; rng
    ends advanced past all len(g) draws, as if it had drawn them in order."""
    import concurrent.futures as cf
    import os
    n = len(g)
    state = rng.bit_generator.state

    def fill(a: int) -> None:
        bg = np.random.PCG64()
        bg.state = state
        bg.advance(a)
        u = np.random.Generator(bg).random(min(chunk, n - a))
        v = g[a:a + len(u)]
        np.greater_equal(u, cum[0], out=v.view(bool))
        for c in cum[1:]:
            v += u >= c

    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 1)) as ex:
        list(ex.map(fill, range(0, n, chunk)))
    _skip(rng, n)


def genome_large(n: int, seed: int, chunk: int = 1 << 22) -> np.ndarray:
    """Human-like genome of n bases built in bounded memory (about 1.2 n bytes
    at peak): GC 41 % background, 10 % copies of 300 bp elements and 17 % of
    6 kbp elements at 80-98 % identity, 18 % tandem repeats of 1-6 bp units
    (perfect runs of 20-149 bp, each closed at both ends by a base that breaks
    its period, so that no two runs of one unit merge into a stretch as long as
    a 150 bp read: a read lying inside a longer run of a 1-6 bp unit matches
    every window of every such run with up to max_results indel variants of
    that interval, millions of rows per read at 3.1 Gbp).
    Deterministic for (n, seed); meant for the 3.1 Gbp shapes, where genome()
    would need tens of GB of temporaries."""
    rng = np.random.default_rng(seed)
    g = np.empty(n, dtype=np.uint8)
    _background_draws(g, rng, np.cumsum([0.295, 0.205, 0.205]), chunk)
    for frac, L, fams, batch in ((0.10, 300, 64, 100_000), (0.17, 6000, 32, 5_000)):
        elems = np.stack([background(L, rng, 0.41) for _ in range(fams)])
        copies = int(frac * n) // L
        col = np.arange(L)
        for b0 in range(0, copies, batch):
            b = min(batch, copies - b0)
            fam = rng.integers(0, fams, size=b)
            starts = rng.integers(0, n - L, size=b)
            ident = rng.uniform(0.80, 0.98, size=b)
            mat = elems[fam]
            m = _uniform_threads(rng, (b, L)) > ident[:, None]
            mat[m] = (mat[m] + rng.integers(1, 4, size=int(m.sum()), dtype=np.uint8)) % 4
            g[starts[:, None] + col[None, :]] = mat
    # tandem runs: parameters drawn in order (the two breakers of a run are its
    # two flips, the one before the run first), positions and bases built by host
    # threads, written in draw order so that later runs overwrite earlier ones
    target, done = int(0.18 * n), 0
    j = np.arange(-1, 151)  # run bases 0..rlen-1, breakers at -1 and rlen
    runs = []
    while done < target:
        b = 200_000
        units = rng.integers(0, 4, size=(b, 6), dtype=np.uint8)
        ulen = rng.integers(1, 7, size=b)
        rlen = rng.integers(20, 150, size=b)
        starts = rng.integers(1, n - 151, size=b)
        flips = rng.integers(1, 4, size=2 * b, dtype=np.uint8)
        runs.append((units, ulen, rlen, starts, flips))
        done += int(rlen.sum())

    def tandem(run):
        units, ulen, rlen, starts, flips = run
        keep = j[None, :] <= rlen[:, None]
        vals = np.take_along_axis(units, (j[None, :] % ulen[:, None]), axis=1)
        r = np.arange(len(rlen))
        vals[r, 0] = (vals[r, 0] + flips[0::2]) % 4
        vals[r, rlen + 1] = (vals[r, rlen + 1] + flips[1::2]) % 4
        return (starts[:, None] + j[None, :])[keep], vals[keep]

    import concurrent.futures as cf
    import os
    w = min(8, os.cpu_count() or 1)
    with cf.ThreadPoolExecutor(max_workers=w) as ex:
        for a in range(0, len(runs), w):
            for at, vals in ex.map(tandem, runs[a:a + w]):
                g[at] = vals
    return g


def reads_large(g: np.ndarray, n: int, seed: int, length: int, subst_rate: float, chunk: int = 1_000_000) -> ReadSet:
    """n reads of `length` bases from uniform positions on either strand with
    independent per-base substitutions at subst_rate (uncapped), generated in
    chunks so that memory stays near the output size."""
    rng = np.random.default_rng(seed)
    L = int(length)
    offs = np.arange(n + 1, dtype=np.uint64) * np.uint64(L)
    out = np.empty(n * L, dtype=np.uint8)
    pos_all = np.empty(n, dtype=np.int64)
    strand_all = np.empty(n, dtype=np.int8)
    col = np.arange(L)
    for a in range(0, n, chunk):
        b = min(n, a + chunk)
        pos = (rng.random(b - a) * (len(g) - L)).astype(np.int64)
        strand = (rng.random(b - a) < 0.5).astype(np.int8)
        frag = g[pos[:, None] + col[None, :]]
        m = rng.random(frag.shape) < subst_rate
        frag[m] = (frag[m] + rng.integers(1, 4, size=int(m.sum()), dtype=np.uint8)) % 4
        rc = np.nonzero(strand)[0]
        frag[rc] = _COMP[frag[rc][:, ::-1]]
        out[a * L:b * L] = _ASCII[frag].reshape(-1)
        pos_all[a:b] = pos
        strand_all[a:b] = strand
    return ReadSet(out, offs, pos_all, strand_all, np.zeros(n, dtype=np.int8))
