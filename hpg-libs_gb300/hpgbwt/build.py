"""Build the in-tree shared libraries.

- ``hpg-libs_gb300/libhpgbwt.so``: CUDA kernels for sm_103a + the C ABI
  (nvcc for .cu, g++ for .cpp, compiled in parallel, linked by nvcc with the
  static CUDA runtime).
- ``oracle/liboracle.so``: the CPU oracle (test infrastructure).
- ``oracle/_ref/libhpgref.so``: the reference's own sources, only where the
  reference tree is present (never on the GPU machine).

Objects go to ``hpg-libs_gb300/_build``; sources are rebuilt when newer than
their object.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent.parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
BUILD = PKG / "_build"
LIB = PKG / "libhpgbwt.so"
ORACLE_SRC = ROOT / "oracle" / "fm_oracle.c"
ORACLE_LIB = ROOT / "oracle" / "liboracle.so"
# The reference checkout the oracle library is compiled from: HPG_REFERENCE_DIR,
# else a checkout named "reference" beside this repository's directory.
REF_DIR = Path(os.environ.get("HPG_REFERENCE_DIR") or (ROOT.parent / "reference"))
REF_LIB = ROOT / "oracle" / "_ref" / "libhpgref.so"

ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return cand


def _cuda_include() -> str:
    return str(Path(_nvcc()).resolve().parent.parent / "include")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _stale(src: Path, obj: Path, deps: list[Path]) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return src.stat().st_mtime > t or any(d.stat().st_mtime > t for d in deps)


def build_lib(verbose: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.h*")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))
    jobs = []
    objs = []
    for src in sorted(CSRC.glob("*.cu")):
        obj = BUILD / (src.name + ".o")
        objs.append(obj)
        if _stale(src, obj, headers):
            jobs.append([_nvcc(), ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-fopenmp",
                         f"-I{INCLUDE}", f"-I{CSRC}", "-c", str(src), "-o", str(obj)])
    for src in sorted(CSRC.glob("*.cpp")):
        obj = BUILD / (src.name + ".o")
        objs.append(obj)
        if _stale(src, obj, headers):
            jobs.append(["g++", "-O3", "-std=c++17", "-fPIC", "-fopenmp", "-Wall", "-Wno-unused-function",
                         f"-I{INCLUDE}", f"-I{CSRC}", f"-I{_cuda_include()}", "-c", str(src), "-o", str(obj)])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for f in [ex.submit(_run, j) for j in jobs]:
            f.result()
    if jobs or not LIB.exists():
        tmp = LIB.with_suffix(".so.tmp")
        _run([_nvcc(), ARCH, "-shared", "-o", str(tmp)] + [str(o) for o in objs] +
             ["-Xcompiler", "-fopenmp", "-lgomp"])
        os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}")
    return LIB


def build_oracle() -> Path:
    if not ORACLE_LIB.exists() or ORACLE_SRC.stat().st_mtime > ORACLE_LIB.stat().st_mtime or \
            (INCLUDE / "hpg_bwt_records.h").stat().st_mtime > ORACLE_LIB.stat().st_mtime:
        tmp = ORACLE_LIB.with_suffix(".so.tmp")
        _run(["gcc", "-O2", "-std=gnu11", "-fopenmp", "-fPIC", "-shared", str(ORACLE_SRC), "-o", str(tmp)])
        os.replace(tmp, ORACLE_LIB)
    return ORACLE_LIB


def build_reference_oracle() -> Path | None:
    """Compile the reference's sources where they lie (only in the build container)."""
    if not (REF_DIR / "c" / "src" / "aligners" / "bwt" / "bwt.c").exists():
        return None
    jobs = str(os.cpu_count() or 4)
    _run(["make", "-s", "-C", str(ROOT / "oracle" / "ref"), f"REF={REF_DIR}", "-j", jobs])
    return REF_LIB


def build_all(verbose: bool = False) -> None:
    with cf.ThreadPoolExecutor(max_workers=3) as ex:
        futs = [ex.submit(build_lib, verbose), ex.submit(build_oracle), ex.submit(build_reference_oracle)]
        for f in futs:
            f.result()


if __name__ == "__main__":
    build_all(verbose=True)
    sys.exit(0)
