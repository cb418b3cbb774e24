"""Build libhcgpu.so in-tree with nvcc for sm_103a (two translation units compiled in
parallel, then linked). Output: homotopycontinuation.jl_gb300/_build/libhcgpu.so."""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(PKG_ROOT, "csrc")
BUILD = os.path.join(PKG_ROOT, "_build")
LIB = os.path.join(BUILD, "libhcgpu.so")
SOURCES = ["hc_kernels.cu", "hc_capi.cu", "hc_peak.cu", "hc_mlp.cu", "hc_certify.cu", "hc_mixed.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-diag-suppress", "39"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libhcgpu.so")


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(PKG_ROOT, "..", "include", "hcgpu.h"))
    return [f for f in files if os.path.isfile(f)]


def up_to_date(lib: str = LIB) -> bool:
    if not os.path.exists(lib):
        return False
    t = os.path.getmtime(lib)
    return all(os.path.getmtime(f) <= t for f in _deps())


def build(force: bool = False, verbose: bool = False, defines=(), build_dir: str = BUILD) -> str:
    """Compile and link; ``defines`` (e.g. ("HC_PHASE_CLOCKS",) for a phase-profiling
    library) go to nvcc as -D flags, ``build_dir`` receives the objects and the library."""
    lib = os.path.join(build_dir, "libhcgpu.so")
    if not force and up_to_date(lib):
        return lib
    os.makedirs(build_dir, exist_ok=True)
    cc = nvcc()
    dflags = [f"-D{d}" for d in defines]

    def compile_one(src):
        obj = os.path.join(build_dir, src.replace(".cu", ".o"))
        cmd = [cc, *ARCH, *FLAGS, *dflags, "-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        if verbose:
            print(r.stdout + r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = lib + ".tmp"
    r = subprocess.run([cc, *ARCH, "-shared", "-o", tmp, *objs], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib)
    return lib
