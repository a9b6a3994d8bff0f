"""In-tree build of the fitter library (libgb300kf.so) for sm_103a.

The CUDA translation units are compiled with nvcc for
``-gencode arch=compute_103a,code=sm_103a``; the host generator with g++.
Everything lands in ``gpukalmanfitter_gb300/_lib/``.  Rebuilds only when a
source is newer than the library.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
LIBDIR = PKG / "_lib"
LIB = LIBDIR / "libgb300kf.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["kf_capi.cu", "kf_fit_fp64.cu", "kf_fit_mixed.cu", "kf_fit_fp64_mat.cu",
              "kf_fit_mixed_mat.cu", "kf_batch.cu", "kf_diag.cu",
              "kf_noalloc.cu", "kf_adjoint.cu", "kf_sim.cu"] + [f"kf_tune_{p}_{m}.cu" for p in ("fp64", "mixed")
                                                     for m in ("2", "3", "5", "64x4", "64x8", "256x1", "256x2")]
CXX_SOURCES = ["synth.cpp", "kf_io.cpp", "kf_fieldmap.cpp"]
# The simulation kernel runs the host generator's per-track code; without
# contraction into FMA on either side the two differ only by the math
# library's rounding (the host side is built with -ffp-contract=off).
CU_EXTRA_FLAGS = {"kf_sim.cu": ["-fmad=false"]}


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libgb300kf")


def _sources() -> list[Path]:
    deps = [CSRC / s for s in CU_SOURCES + CXX_SOURCES]
    deps += sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + sorted(INCLUDE.glob("*.h"))
    return deps


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps if d.exists())


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile libgb300kf.so if needed and return its path."""
    deps = _sources()
    if not force and not _stale(LIB, deps):
        return LIB
    LIBDIR.mkdir(parents=True, exist_ok=True)
    obj = LIBDIR / "obj"
    obj.mkdir(exist_ok=True)
    nvcc = _nvcc()
    cu_flags = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                       "-I", str(INCLUDE)]
    cxx_flags = ["-O2", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off", "-I", str(INCLUDE)]
    jobs = []
    objs = []
    for s in CU_SOURCES:
        o = obj / (Path(s).stem + ".o")
        objs.append(o)
        jobs.append([nvcc, *cu_flags, *CU_EXTRA_FLAGS.get(s, []), "-c", str(CSRC / s), "-o",
                     str(o)])
    for s in CXX_SOURCES:
        o = obj / (Path(s).stem + ".o")
        objs.append(o)
        jobs.append(["g++", *cxx_flags, "-c", str(CSRC / s), "-o", str(o)])
    with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
        for cmd, _ in zip(jobs, ex.map(_run, jobs)):
            if verbose:
                print(" ".join(cmd))
    tmp = LIB.with_suffix(".so.tmp")
    _run([nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-Xcompiler", "-fopenmp",
          "-lgomp"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
