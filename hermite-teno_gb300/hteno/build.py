"""Build recipe of the CUDA library libhteno.so (sm_103a) and of the CPU oracle.

The library is compiled in-tree: objects go to hermite-teno_gb300/build/, the shared object to
hermite-teno_gb300/lib/libhteno.so.  Translation units compile in parallel; the whole build
takes well under a minute on one host.  Nothing here needs a GPU.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent.parent          # hermite-teno_gb300/
REPO_DIR = PKG_DIR.parent
CSRC = PKG_DIR / "csrc"
BUILD = PKG_DIR / "build"
LIB_DIR = PKG_DIR / "lib"
LIB = LIB_DIR / "libhteno.so"
ORACLE_DIR = REPO_DIR / "oracle"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr"]
# Units compiled without implicit fused multiply-adds: the bit-reproducible FP64 units, and the
# fused mixed-precision units, whose tile-shape candidates must give the same bits (with implicit
# contraction the compiler fused different float expressions in different instantiations).
NO_FMAD = {"fv2d_fp64.cu", "fv1d.cu", "pointwise.cu", "hermite2d_fp64.cu", "hermite1d.cu",
           "fv2d_fused.cu", "fv2d_batch.cu", "mlp.cu"}


def _cuda_home() -> Path:
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and (Path(cand) / "bin" / "nvcc").exists():
            return Path(cand)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    raise RuntimeError("nvcc not found: set CUDA_HOME")


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"command failed ({proc.returncode}): {' '.join(cmd)}\n"
                           f"{proc.stdout}\n{proc.stderr}")


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build_library(force: bool = False, jobs: int | None = None, verbose: bool = False) -> Path:
    """Compile every CUDA translation unit for sm_103a and link libhteno.so."""
    cuda = _cuda_home()
    nvcc = str(cuda / "bin" / "nvcc")
    BUILD.mkdir(parents=True, exist_ok=True)
    LIB_DIR.mkdir(parents=True, exist_ok=True)
    headers = sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + \
        [REPO_DIR / "include" / "hteno.h"]
    units = sorted(CSRC.glob("*.cu"))
    host_units = sorted(CSRC.glob("*.cpp"))
    jobs_todo = []
    objs = []
    for u in units:
        o = BUILD / (u.stem + ".o")
        objs.append(o)
        if force or _stale(o, [u] + headers):
            extra = ["--fmad=false"] if u.name in NO_FMAD else []
            jobs_todo.append([nvcc, *ARCH, *NVCC_FLAGS, *extra, "-I", str(REPO_DIR / "include"),
                              "-c", str(u), "-o", str(o)])
    for u in host_units:
        o = BUILD / (u.stem + ".host.o")
        objs.append(o)
        if force or _stale(o, [u] + headers):
            jobs_todo.append(["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off",
                              "-I", str(cuda / "include"), "-c", str(u), "-o", str(o)])
    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        for fut in [ex.submit(_run, c) for c in jobs_todo]:
            fut.result()
    if force or jobs_todo or _stale(LIB, objs):
        _run([nvcc, *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-lcudart"])
    if verbose:
        print(f"built {LIB} ({len(jobs_todo)} units recompiled)")
    return LIB


def build_oracle(with_reference: bool | None = None) -> Path:
    """Compile the CPU oracle (test infrastructure) and, where the reference sources are present,
    the reference itself against the project's Eigen-subset header (oracle/_ref)."""
    _run(["make", "-s", "-C", str(ORACLE_DIR), "oracle"])
    # the reference tree: HTENO_REFERENCE_DIR, else a "reference" directory beside the repository
    ref_src = os.environ.get("HTENO_REFERENCE_DIR") or str(REPO_DIR.parent / "reference")
    if with_reference is None:
        with_reference = Path(ref_src, "FV_System2D.cpp").exists()
    if with_reference:
        _run(["make", "-s", "-j8", "-C", str(ORACLE_DIR), "ref", f"REF={ref_src}"])
    return ORACLE_DIR / "build" / "liboracle.so"


if __name__ == "__main__":
    build_library(force="--force" in sys.argv, verbose=True)
    print(build_oracle())
