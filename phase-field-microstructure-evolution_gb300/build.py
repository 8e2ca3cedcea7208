"""Build recipe of libpfgpu.so (sm_103a).

Compiles every translation unit under ``csrc/`` with nvcc in parallel
(one ``-gencode arch=compute_103a,code=sm_103a``) and links the shared library
into ``_build/libpfgpu.so`` next to this file.  Rebuilds only what changed.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
OUT = HERE / "_build"
INCLUDE = HERE.parent / "include"
LIB = OUT / "libpfgpu.so"
DRIVERS = HERE / "driver"
EXE = OUT / "pf_var_diff"          # the var_diff.x drop-in
PARAVIEW_EXE = OUT / "pf_paraview"  # the paraview.x drop-in
SWEEP_EXE = OUT / "pf_sweep"        # many var_diff.x cases in one process

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-std=c++17", "-lineinfo", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
           "-Xcompiler", "-Wall", "-diag-suppress", "550"]


def cuda_home() -> Path:
    for cand in (os.environ.get("CUDA_HOME"), os.environ.get("CUDA_PATH"), "/usr/local/cuda"):
        if cand and (Path(cand) / "bin" / "nvcc").exists():
            return Path(cand)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    raise RuntimeError("nvcc not found: set CUDA_HOME")


def _sources():
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))


def _headers():
    return list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list(INCLUDE.glob("*.h"))


def _compile(nvcc: Path, src: Path, obj: Path, verbose: bool):
    cmd = [str(nvcc)] + ARCH + NVFLAGS + ["-I", str(INCLUDE), "-c", str(src), "-o", str(obj)]
    if src.suffix == ".cpp":
        cmd = [str(nvcc), "-O2", "-std=c++17", "-Xcompiler", "-fPIC", "-I", str(INCLUDE), "-c", str(src), "-o", str(obj)]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compiling {src.name} failed:\n{r.stdout}\n{r.stderr}")
    return obj


def build(force: bool = False, verbose: bool = False, jobs: int | None = None) -> Path:
    """Compile and link ``libpfgpu.so``; return its path."""
    home = cuda_home()
    nvcc = home / "bin" / "nvcc"
    OUT.mkdir(exist_ok=True)
    hdr_mtime = max(p.stat().st_mtime for p in _headers())
    todo = []
    objs = []
    for src in _sources():
        obj = OUT / (src.stem + ".o")
        objs.append(obj)
        if force or not obj.exists() or obj.stat().st_mtime < max(src.stat().st_mtime, hdr_mtime):
            todo.append((src, obj))
    if todo:
        n = jobs or min(len(todo), os.cpu_count() or 4)
        with cf.ThreadPoolExecutor(max_workers=n) as ex:
            list(ex.map(lambda so: _compile(nvcc, so[0], so[1], verbose), todo))
    if todo or not LIB.exists() or force:
        libdir = home / "lib64"
        if not libdir.exists():
            libdir = home / "lib"
        cmd = [str(nvcc)] + ARCH + ["-shared", "-o", str(LIB)] + [str(o) for o in objs] + [
            "-L", str(libdir), "-lcufft", "-Xlinker", f"-rpath={libdir}"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"linking libpfgpu.so failed:\n{r.stdout}\n{r.stderr}")
    build_driver(nvcc, force, verbose)
    return LIB


def build_driver(nvcc: Path, force: bool = False, verbose: bool = False):
    """Link the executables of ``driver/`` (the var_diff.x and paraview.x
    drop-ins) against the library."""
    hdr = max(p.stat().st_mtime for p in list(INCLUDE.glob("*.h")) + list(DRIVERS.glob("*.h")))
    cxx = shutil.which("g++") or str(nvcc)
    for src in sorted(DRIVERS.glob("*.cpp")):
        exe = OUT / src.stem
        if not force and exe.exists() and exe.stat().st_mtime >= max(src.stat().st_mtime, LIB.stat().st_mtime, hdr):
            continue
        rpath = ["-Wl,-rpath,$ORIGIN"] if cxx != str(nvcc) else ["-Xlinker", "-rpath=$ORIGIN"]
        cmd = [cxx, "-O2", "-std=c++17", "-I", str(INCLUDE), str(src), "-o", str(exe),
               "-L", str(OUT), "-lpfgpu"] + rpath
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"linking {exe.name} failed:\n{r.stdout}\n{r.stderr}")


if __name__ == "__main__":
    p = build(force="--force" in sys.argv, verbose=True)
    print(p)
