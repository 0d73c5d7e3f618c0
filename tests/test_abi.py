"""The C ABI library (CPU): it loads, exports every function the public headers
declare, and fails loudly (no CPU fallback) where no GPU is present."""
from __future__ import annotations

import ctypes
import re
import subprocess
from pathlib import Path

import pytest

from conftest import has_gpu
from hpgbwt import lib, synth

INCLUDE = Path(__file__).resolve().parent.parent / "include"


def declared_functions() -> set[str]:
    names = set()
    for h in INCLUDE.glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w\s\*]*?\b([a-z_][a-z0-9_]*)\s*\(", text, flags=re.M):
            if not m.group(0).lstrip().startswith(("typedef", "#", "return")):
                names.add(m.group(1))
    return names


def test_header_declares_the_reference_entry_points():
    fns = declared_functions()
    for f in ["bwt_index_new", "bwt_index_free", "bwt_optarg_new", "bwt_optarg_free", "bwt_generate_index_files",
              "bwt_gpu_search_batch", "bwt_gpu_search_device", "bwt_gpu_search1_noalloc"]:
        assert f in fns


def test_library_exports_every_declared_function():
    lib.load()
    out = subprocess.run(["nm", "-D", "--defined-only", str(lib.LIB_PATH)], capture_output=True, text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    missing = sorted(declared_functions() - exported)
    assert not missing, f"declared but not exported: {missing}"


def test_builder_rejects_bad_input(tmp_path):
    (tmp_path / "bad.fa").write_text(">c1\nACGTNACGT\n")
    with pytest.raises(RuntimeError, match="outside the index alphabet"):
        lib.build_index(str(tmp_path / "bad.fa"), str(tmp_path / "idx"))
    (tmp_path / "empty.fa").write_text("")
    with pytest.raises(RuntimeError, match="no sequence"):
        lib.build_index(str(tmp_path / "empty.fa"), str(tmp_path / "idx2"))
    with pytest.raises(RuntimeError, match="Error opening"):
        lib.build_index(str(tmp_path / "missing.fa"), str(tmp_path / "idx3"))


@pytest.mark.skipif(has_gpu(), reason="checks the no-GPU failure path")
def test_open_without_gpu_fails_loudly(tmp_path):
    g = synth.genome("iid", 5000, 1)
    synth.write_fasta(str(tmp_path / "g.fa"), g)
    lib.build_index(str(tmp_path / "g.fa"), str(tmp_path / "idx"))
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        lib.GpuIndex(str(tmp_path / "idx"))


def test_open_reports_missing_index(tmp_path):
    with pytest.raises(RuntimeError, match="Error opening file"):
        lib.GpuIndex(str(tmp_path / "nope"))


def test_karyotype_and_config_files(tmp_path):
    g = synth.genome("iid", 3000, 2)
    synth.write_fasta(str(tmp_path / "g.fa"), g, [1000, 1500, 500])
    lib.build_index(str(tmp_path / "g.fa"), str(tmp_path / "idx"))
    assert (tmp_path / "idx" / "index").read_text() == ">chr1 0 999\n>chr2 0 1499\n>chr3 0 499\n"
    assert (tmp_path / "idx" / "config.txt").read_text() == "ACGT\n0\n"
