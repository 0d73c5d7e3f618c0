"""Golden pins (CPU): the product's index builder and the CPU oracle against
outputs of the reference's own code, committed in tests/golden/."""
from __future__ import annotations

import hashlib
from pathlib import Path

import numpy as np
import pytest

from golden_cases import GoldenCase, names
from oracle.pyoracle import PortOracle


@pytest.fixture(scope="module", params=names())
def built_case(request, tmp_path_factory):
    c = GoldenCase(request.param)
    return c, c.build(tmp_path_factory.mktemp(request.param))


def test_builder_writes_reference_index_files(built_case):
    c, index = built_case
    want = c.meta["index_sha256"]
    got = {p.name: hashlib.sha256(p.read_bytes()).hexdigest() for p in Path(index).iterdir()}
    assert sorted(got) == sorted(want)
    for f in want:
        assert got[f] == want[f], f"{f} differs from the reference builder's file"


def test_oracle_matches_reference_outputs(built_case):
    c, index = built_case
    ora = PortOracle(index)
    for tag in c.tags():
        mode = int(tag[1])
        mr = int(tag.split("_r")[1])
        got = ora.search(c.reads, mode=mode, max_results=mr, threads=2)
        want = c.expected(tag)
        assert np.array_equal(got.rs_count, want.rs_count), tag
        assert np.array_equal(got.rs_truncated, want.rs_truncated), tag
        assert np.array_equal(got.hits, want.hits), tag
        assert np.array_equal(got.locs, want.locs), tag
    ora.close()


def test_oracle_block_search_matches_reference_outputs(built_case):
    """The k-error block search (BWSearchCPU as bwt_map_inexact_read_2 runs it): results,
    located rows and anchors equal the reference's at every recorded list capacity."""
    c, index = built_case
    ora = PortOracle(index)
    caps = c.block_capacities()
    assert caps
    for mr in caps:
        got = ora.block_search(c.reads, max_results=mr, threads=2)
        assert got.equal(c.block_expected(mr), truncation=False), mr
        assert not (got.result.rs_truncated & 2).any()
    ora.close()


def test_block_fixtures_exercise_edges():
    """Exact and one-error results of every kind on both halves, multi-row intervals,
    lists cut by their capacity (fewer results than without a cap), empty anchors."""
    kinds, dirs, multi, cut = set(), set(), False, False
    for name in names():
        c = GoldenCase(name)
        caps = c.block_capacities()
        full = c.block_expected(max(caps))
        h = full.result.hits
        kinds |= set(int(x) for x in h["err_kind"][h["nm"] == 1])
        dirs |= set(int(x) for x in h["dir"])
        multi |= bool(((h["l"] - h["k"]) > 0).any())
        for mr in caps:
            if mr < max(caps):
                cut |= len(c.block_expected(mr).result.hits) < len(h)
        assert (h["nm"] == 0).any()
    assert kinds == {1, 2, 3} and dirs == {0, 1} and multi and cut


def test_golden_cases_exercise_edges():
    seen_trunc = seen_invalid = seen_quirk = seen_multi = False
    for name in names():
        c = GoldenCase(name)
        for tag in c.tags():
            e = c.expected(tag)
            seen_trunc |= bool(e.rs_truncated.any())
            seen_invalid |= bool(len(e.locs) and (e.locs["valid"] == 0).any())
            seen_quirk |= bool(((e.hits["err_kind"] == 3) & (e.hits["err_base"] == 3) & (e.hits["dir"] == 0)).any())
            seen_multi |= bool(((e.hits["l"] - e.hits["k"]) > 0).any())
    assert seen_trunc and seen_invalid and seen_quirk and seen_multi


def test_oracle_locate_limit(tmp_path):
    """The oracle's locate limit: hits, counts and overflow bits unchanged; lists
    whose kept hits cover more rows than the limit lose exactly their located rows
    and get truncation bit 1."""
    from low_complexity import low_complexity_case
    index, reads = low_complexity_case(tmp_path)
    ora = PortOracle(index)
    full = ora.search(reads, mode=1, max_results=100, threads=4)
    lim = ora.search(reads, mode=1, max_results=100, threads=4, locate_limit=5000)
    assert np.array_equal(full.hits, lim.hits) and np.array_equal(full.rs_count, lim.rs_count)
    assert np.array_equal(full.rs_truncated, lim.rs_truncated & 1)
    sz = np.maximum(full.hits["l"] - full.hits["k"] + 1, 0).astype(np.int64)
    lst = 2 * full.hits["read"].astype(np.int64) + full.hits["strand"]
    rows = np.bincount(lst, weights=sz, minlength=2 * len(reads.offsets) - 2)
    over = rows > 5000
    assert over.any() and not over.all()
    assert np.array_equal((lim.rs_truncated & 2) != 0, over)
    keep = ~over[lst[full.locs["hit"]]]
    assert np.array_equal(lim.locs, full.locs[keep])
