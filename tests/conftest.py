"""Shared fixtures: built libraries, seeded genomes and indexes built by the product builder."""
from __future__ import annotations

import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT / "hpg-libs_gb300"))
sys.path.insert(0, str(ROOT))

from hpgbwt import build as hbuild  # noqa: E402
from hpgbwt import synth  # noqa: E402


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GB300 device (runs through the C ABI)")


@pytest.fixture(scope="session", autouse=True)
def built():
    hbuild.build_all()
    return True


def has_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


class Case:
    """A seeded genome written as FASTA plus its index directory."""

    def __init__(self, tmp: Path, kind: str, n: int, seed: int, chroms: int = 1):
        self.dir = tmp
        self.genome = synth.genome(kind, n, seed)
        cl = [n // chroms] * (chroms - 1)
        cl.append(n - sum(cl))
        self.chrom_lengths = cl
        self.fasta = str(tmp / "genome.fa")
        synth.write_fasta(self.fasta, self.genome, cl)
        self.index = str(tmp / "index")
        from hpgbwt import lib
        lib.build_index(self.fasta, self.index, 16)


_cases: dict = {}


@pytest.fixture(scope="session")
def case_factory(tmp_path_factory):
    def make(kind: str, n: int, seed: int, chroms: int = 1) -> Case:
        key = (kind, n, seed, chroms)
        if key not in _cases:
            _cases[key] = Case(tmp_path_factory.mktemp(f"{kind}_{n}_{seed}_{chroms}"), kind, n, seed, chroms)
        return _cases[key]
    return make
