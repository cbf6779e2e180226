"""Build the native parts in-tree: the CUDA step library for sm_103a, the
C oracle (test infrastructure) and the reference's own step as the oracle's
pin (oracle/_ref), from the reference tree where it is present or from the
snapshot of its files that oracle/Makefile keeps in oracle/_ref/src.

    python -m spacelab_gb300.build            # everything
    python -m spacelab_gb300.build --lib      # only libspacelab_gb300.so

No cmake: nvcc and g++ are invoked directly, translation units in parallel.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = ROOT / "_build"
LIB = PKG / "libspacelab_gb300.so"
ORACLE_DIR = ROOT / "oracle"
ORACLE_LIB = ORACLE_DIR / "liboracle.so"
# Root of the reference tree: SPACELAB_REF_ROOT, else oracle/Makefile's
# default (REF).  Where neither holds the reference, the snapshot in
# oracle/_ref/src (made by an earlier build) is compiled instead.
REF_ENV = "SPACELAB_REF_ROOT"
REF_SNAPSHOT = ORACLE_DIR / "_ref" / "src"
REF_LIBS = (ORACLE_DIR / "_ref" / "libslref.so", ORACLE_DIR / "_ref" / "libslref_native.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                      "-I", str(ROOT / "include")]
# Per-file arithmetic contract: the exact step must not contract a*b+c.
NVCC_FILE_FLAGS = {
    "sl_step.cu": ["--fmad=false"],
    "sl_rowsum_tma.cu": ["--fmad=false"],
    "sl_capi.cu": ["--fmad=false"],
    "sl_static.cu": ["--fmad=false"],
    "sl_batch.cu": ["--fmad=false"],
    "sl_batch_capi.cu": ["--fmad=false"],
    "sl_diag.cu": ["--fmad=false"],
}
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-I", str(ROOT / "include")]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build spacelab_gb300")


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"build step failed ({proc.returncode}): {' '.join(cmd)}\n{proc.stdout}")


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build_lib(force: bool = False) -> Path:
    nvcc = _nvcc()
    BUILD.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list((ROOT / "include").glob("*.h"))
    jobs = []
    objs = []
    for cu in sorted(CSRC.glob("*.cu")):
        obj = BUILD / (cu.stem + ".o")
        objs.append(obj)
        if force or _stale(obj, [cu] + headers):
            jobs.append([nvcc, *NVCC_COMMON, *NVCC_FILE_FLAGS.get(cu.name, []), "-c", str(cu), "-o", str(obj)])
    for cpp in sorted((CSRC / "host").glob("*.cpp")):
        obj = BUILD / ("host_" + cpp.stem + ".o")
        objs.append(obj)
        if force or _stale(obj, [cpp] + headers):
            jobs.append(["g++", *CXX_FLAGS, "-c", str(cpp), "-o", str(obj)])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        list(ex.map(_run, jobs))
    if force or jobs or not LIB.exists():
        tmp = LIB.with_suffix(".so.tmp")
        _run([nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lpthread"])
        os.replace(tmp, LIB)
    return LIB


def build_oracle(force: bool = False) -> Path:
    src = ORACLE_DIR / "sl_oracle.c"
    if force or _stale(ORACLE_LIB, [src, ORACLE_DIR / "sl_oracle.h"]):
        tmp = ORACLE_LIB.with_suffix(".so.tmp")
        _run(["gcc", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared", "-o", str(tmp), str(src), "-lm"])
        os.replace(tmp, ORACLE_LIB)
    return ORACLE_LIB


def build_reference_pin(force: bool = False) -> Path | None:
    """oracle/_ref/libslref.so (and the -O3 native timing build) from the
    reference's own sources; None where neither the reference tree nor a
    snapshot of it is at hand."""
    make = ["make", "-s", "-C", str(ORACLE_DIR)]
    if os.environ.get(REF_ENV):
        make.append(f"REF={os.environ[REF_ENV]}")
    # refresh the snapshot where the tree is present; where it is not, make
    # fails here and an existing snapshot is used as it is
    subprocess.run(make + ["snapshot"], stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    if not (REF_SNAPSHOT / "ColliderSingleCore" / "ColliderSingleCore.cpp").exists():
        return None
    _run(make + (["-B"] if force else []) + ["all"])
    return REF_LIBS[0]


def build_all(force: bool = False) -> None:
    with cf.ThreadPoolExecutor(max_workers=3) as ex:
        futs = [ex.submit(build_lib, force), ex.submit(build_oracle, force), ex.submit(build_reference_pin, force)]
        for f in futs:
            f.result()


def main(argv: list[str] | None = None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--lib", action="store_true", help="only the CUDA library")
    ap.add_argument("--force", action="store_true")
    args = ap.parse_args(argv)
    if args.lib:
        build_lib(args.force)
    else:
        build_all(args.force)
    return 0


if __name__ == "__main__":
    sys.exit(main())
