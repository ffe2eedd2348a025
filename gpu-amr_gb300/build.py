"""Build recipe for the GB300 AMR library (in-tree, sm_103a only).

    python gpu-amr_gb300/build.py          # -> gpu-amr_gb300/lib/libamr_gb300.so

Each CUDA translation unit compiles in parallel with
`nvcc -gencode arch=compute_103a,code=sm_103a`; the shared library links the
CUDA runtime dynamically.  Works on x86_64 (cross-compiles, no GPU needed) and
on the aarch64 GPU host alike.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
REPO = PKG.parent
CSRC = PKG / "csrc"
LIBDIR = PKG / "lib"
BUILD = PKG / "_build"
LIB = LIBDIR / "libamr_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-lineinfo", "-std=c++20", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
           "-I", str(REPO / "include"), "-I", str(CSRC), "-I", str(PKG / "host")]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


# Translation units whose arithmetic must match the reference's CPU code
# operation for operation: no multiply-add contraction.
NO_CONTRACTION = {"amr_euler.cu", "amr_ssprk.cu", "amr_dg.cu"}


def sources():
    return sorted(CSRC.glob("*.cu"))


def flags_for(src: Path):
    return ["-fmad=false"] if src.name in NO_CONTRACTION else []


def _stale(out: Path, deps) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def build(verbose: bool = False, extra=None) -> Path:
    BUILD.mkdir(exist_ok=True)
    LIBDIR.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + list((REPO / "include").glob("*.h")) + list((PKG / "host").rglob("*.hpp"))
    nv = nvcc()
    jobs = []
    for src in sources():
        obj = BUILD / (src.stem + ".o")
        if _stale(obj, [src, *headers, Path(__file__)]):
            jobs.append([nv, *ARCH, *NVFLAGS, *flags_for(src), *(extra or []), "-c", str(src), "-o", str(obj)])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return r.stderr

    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
        for log in ex.map(run, jobs):
            if verbose and log:
                print(log)
    objs = [BUILD / (s.stem + ".o") for s in sources()]
    if jobs or _stale(LIB, objs):
        run([nv, *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-lcudart"])
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
