"""Seeded generators (CPU): deterministic, with the configured shapes and error models."""
from __future__ import annotations

import numpy as np

from hpgbwt import synth


def test_genomes_are_seeded():
    for kind in ("iid", "repeats", "human_like"):
        a = synth.genome(kind, 50_000, 7)
        b = synth.genome(kind, 50_000, 7)
        assert np.array_equal(a, b) and a.max() <= 3
    g = synth.genome("repeats", 200_000, 1)
    gc = np.isin(g, [1, 2]).mean()
    assert 0.38 < gc < 0.44


def test_reads_shapes_and_edits():
    g = synth.genome("iid", 100_000, 1)
    r = synth.reads(g, 2000, 3, length=(36, 250), edits="mix_30_50_20")
    L = r.lengths()
    assert L.min() >= 36 and L.max() <= 250
    frac = np.bincount(r.edit, minlength=4) / len(r)
    assert abs(frac[0] - 0.3) < 0.05 and abs(frac[1] - 0.5) < 0.05 and abs(frac[2] + frac[3] - 0.2) < 0.05
    f = synth.reads_fast(g, 20000, 4, 100, "per_base_capped")
    assert np.all(f.lengths() == 100)
    assert 0.35 < (f.edit > 0).mean() < 0.48  # 1 - (1 - 0.0054)^100 ~ 0.42


def test_error_free_reads_come_from_the_genome():
    g = synth.genome("iid", 20_000, 5)
    r = synth.reads_fast(g, 200, 6, 50, "none")
    A = np.frombuffer(b"ACGT", dtype=np.uint8)
    text = A[g].tobytes()
    rc = A[synth.revcomp_codes(g)].tobytes()
    for i in range(len(r)):
        s = r.read(i)
        assert s in text or s in rc


def test_reads_fast_var_models():
    """The vectorised variable-length sampler draws the same edit models as reads()."""
    g = synth.genome("iid", 50_000, 3)
    for edits in ("none", "mix_30_50_20", "subst_capped"):
        rs = synth.reads_fast_var(g, 3000, 11, 50, 300, edits)
        lens = np.diff(rs.offsets.astype(np.int64))
        assert lens.min() >= 50 and lens.max() <= 300 and len(rs.seq) == lens.sum()
        comp = {ord("A"): 3, ord("C"): 2, ord("G"): 1, ord("T"): 0}
        code = {ord("A"): 0, ord("C"): 1, ord("G"): 2, ord("T"): 3}
        for i in range(0, 3000, 7):
            r = rs.seq[rs.offsets[i]:rs.offsets[i + 1]]
            c = np.array([comp[x] for x in r[::-1]] if rs.truth_strand[i] else [code[x] for x in r], np.uint8)
            p, L, e = int(rs.truth_pos[i]), len(c), int(rs.edit[i])
            if e == 0:
                assert np.array_equal(c, g[p:p + L])
            elif e == 1:
                assert int((c != g[p:p + L]).sum()) == 1
            elif e == 3:  # one genome base left out
                f = g[p:p + L + 1]
                assert any(np.array_equal(c, np.delete(f, k)) for k in range(1, L))
            else:  # one base inserted
                f = g[p:p + L - 1]
                k = next(k for k in range(L) if k >= L - 1 or c[k] != f[k])
                assert np.array_equal(np.delete(c, k), f) or any(
                    np.array_equal(np.delete(c, j), f) for j in range(1, L - 1))


def test_threaded_draws_equal_sequential_ones():
    """genome_large's background and element copies draw doubles from copies of
    the generator advanced to their slice: the same numbers, and the generator
    left where drawing them in order would leave it (the 32-bit half a bounded
    integer draw buffered included)."""
    rng_a, rng_b = np.random.default_rng(11), np.random.default_rng(11)
    rng_a.integers(0, 4, size=5)  # leaves a buffered half in both
    rng_b.integers(0, 4, size=5)
    want = rng_a.random((37, 1001))
    got = synth._uniform_threads(rng_b, (37, 1001), chunk=4096)
    assert np.array_equal(want, got)
    assert np.array_equal(rng_a.integers(0, 4, size=9, dtype=np.uint8), rng_b.integers(0, 4, size=9, dtype=np.uint8))
    assert rng_a.random() == rng_b.random()
    cum = np.cumsum([0.295, 0.205, 0.205])
    rng_a, rng_b = np.random.default_rng(12), np.random.default_rng(12)
    want = np.searchsorted(cum, rng_a.random(100_003), side="right").astype(np.uint8)
    got = np.empty(100_003, dtype=np.uint8)
    synth._background_draws(got, rng_b, cum, 8192)
    assert np.array_equal(want, got) and rng_a.random() == rng_b.random()


def test_large_genome_is_seeded():
    a = synth.genome_large(3_000_000, 4)
    assert np.array_equal(a, synth.genome_large(3_000_000, 4)) and a.max() <= 3
    assert not np.array_equal(a, synth.genome_large(3_000_000, 5))
