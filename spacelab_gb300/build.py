"""Build the native parts in-tree: the CUDA step library for sm_103a, the
C oracle (test infrastructure) and, where the reference tree is present,
the reference's own step as the oracle's pin (oracle/_ref).

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
REF_ROOT = Path("/root/reference")

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
    """oracle/_ref/libslref.so from the reference sources, where present."""
    if not (REF_ROOT / "ColliderSingleCore" / "ColliderSingleCore.cpp").exists():
        return None
    out = ORACLE_DIR / "_ref" / "libslref.so"
    if force or _stale(out, [ORACLE_DIR / "ref_harness.cpp", ORACLE_DIR / "Makefile"]):
        _run(["make", "-s", "-C", str(ORACLE_DIR), f"REF={REF_ROOT}", "-B" if force else "all"])
    return out


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
