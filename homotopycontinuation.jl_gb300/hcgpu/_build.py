"""Build libhcgpu.so in-tree with nvcc for sm_103a (translation units compiled in parallel,
then linked against NVRTC). Output: homotopycontinuation.jl_gb300/_build/libhcgpu.so.

The device headers the run-time compiler needs for per-system kernels (hc_slp.cu) are embedded
in the library: the build writes them as string literals into _build/hc_jit_headers.inc."""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(PKG_ROOT, "csrc")
BUILD = os.path.join(PKG_ROOT, "_build")
LIB = os.path.join(BUILD, "libhcgpu.so")
SOURCES = ["hc_kernels.cu", "hc_capi.cu", "hc_peak.cu", "hc_mlp.cu", "hc_certify.cu", "hc_mixed.cu", "hc_slp.cu"]
# headers of the NVRTC translation unit, under the names its #include lines use
JIT_HEADERS = [("hc_rtc.h", "hc_rtc.h"), ("hc_types.cuh", "hc_types.cuh"), ("hc_dev.h", "hc_dev.h"),
               ("../../include/hcgpu.h", os.path.join("..", "..", "include", "hcgpu.h")),
               ("hc_track.cuh", "hc_track.cuh"), ("hc_track_kernel.cuh", "hc_track_kernel.cuh"),
               ("hc_slp_ops.cuh", "hc_slp_ops.cuh")]
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


def write_jit_headers(build_dir: str) -> str:
    """_build/hc_jit_headers.inc: kJitHeaderCount, kJitHeaderNames, kJitHeaderSources."""
    out = os.path.join(build_dir, "hc_jit_headers.inc")
    lines = ["// generated by hcgpu/_build.py from csrc/ and include/: do not edit",
             f"static const int kJitHeaderCount = {len(JIT_HEADERS)};",
             "static const char* const kJitHeaderNames[] = {" + ", ".join(f'"{n}"' for n, _ in JIT_HEADERS) + "};",
             "static const char* const kJitHeaderSources[] = {"]
    for _, rel in JIT_HEADERS:
        text = open(os.path.join(CSRC, rel)).read()
        if ')HCJIT"' in text:
            raise RuntimeError(f"{rel} contains the raw-string delimiter")
        # long texts go in as concatenated raw literals of at most 16 KB each
        chunks = [text[i:i + 16000] for i in range(0, len(text), 16000)] or [""]
        lines.append("    " + "\n    ".join(f'R"HCJIT({c})HCJIT"' for c in chunks) + ",")
    lines.append("};")
    body = "\n".join(lines) + "\n"
    if not (os.path.exists(out) and open(out).read() == body):
        with open(out, "w") as f:
            f.write(body)
    return out


def toolkit_lib_dir(cc: str) -> str:
    root = os.path.dirname(os.path.dirname(os.path.realpath(cc)))
    for cand in ("lib64", "lib", os.path.join("targets", "sbsa-linux", "lib"), os.path.join("targets", "x86_64-linux", "lib")):
        d = os.path.join(root, cand)
        if os.path.exists(os.path.join(d, "libnvrtc.so")):
            return d
    return os.path.join(root, "lib64")


def build(force: bool = False, verbose: bool = False, defines=(), build_dir: str = BUILD) -> str:
    """Compile and link; ``defines`` (e.g. ("HC_PHASE_CLOCKS",) for a phase-profiling
    library) go to nvcc as -D flags, ``build_dir`` receives the objects and the library."""
    lib = os.path.join(build_dir, "libhcgpu.so")
    if not force and up_to_date(lib):
        return lib
    os.makedirs(build_dir, exist_ok=True)
    cc = nvcc()
    dflags = [f"-D{d}" for d in defines] + ["-I", build_dir]
    write_jit_headers(build_dir)

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
    libdir = toolkit_lib_dir(cc)
    r = subprocess.run([cc, *ARCH, "-shared", "-o", tmp, *objs, "-L", libdir, "-lnvrtc",
                        "-Xlinker", "-rpath", "-Xlinker", libdir], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib)
    return lib
