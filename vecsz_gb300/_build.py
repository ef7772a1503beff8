"""Builds libvecsz_gb300.so (every translation unit of vecsz_gb300/csrc) for sm_103a.

nvcc compiles the .cu and .cpp files in parallel into vecsz_gb300/_build/, then links the shared library
into vecsz_gb300/_lib/.  Rebuilds only when a source or header is newer than the library.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIBDIR, "libvecsz_gb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
CLI_SRC = os.path.join(HERE, "cli", "vecsz_cli.cpp")
CLI = os.path.join(LIBDIR, "vecsz")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -fmad=false: no contraction -- every FP step must round like the reference's separate operations.
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-fmad=false", "-Xcompiler", "-fPIC,-O3",
              f"-I{INCLUDE}", "-Xptxas", "-warn-spills"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build vecsz_gb300")


def cuda_lib_dir(nv: str) -> str:
    root = os.path.dirname(os.path.dirname(os.path.realpath(nv)))
    for sub in ("lib64", "lib", "targets/sbsa-linux/lib", "targets/x86_64-linux/lib"):
        p = os.path.join(root, sub)
        if os.path.exists(os.path.join(p, "libcudart.so")):
            return p
    return os.path.join(root, "lib64")


def sources() -> list[str]:
    # .cu: device code and the C ABI; .cpp: host-only code (nvcc hands it to the host compiler)
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = sources() + glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(INCLUDE, "*.h")) + [__file__]
    return any(os.path.getmtime(d) > t for d in deps)


def build_cli(force: bool = False) -> str:
    """The `vecsz` command line (host C++ over the library's C ABI), linked next to the library."""
    deps = [CLI_SRC, LIB] + glob.glob(os.path.join(INCLUDE, "*.h"))
    if not force and os.path.exists(CLI) and all(os.path.getmtime(d) <= os.path.getmtime(CLI) for d in deps):
        return CLI
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        raise RuntimeError("g++ not found: needed for the vecsz command line")
    tmp = CLI + ".tmp"
    cmd = [cxx, "-std=c++17", "-O2", "-Wall", f"-I{INCLUDE}", CLI_SRC, "-o", tmp, f"-L{LIBDIR}", "-lvecsz_gb300",
           "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"vecsz command line failed to build:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, CLI)
    return CLI


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not _stale():
        build_cli()
        return LIB
    nv = nvcc()
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)

    def compile_one(src: str) -> str:
        obj = os.path.join(OBJ, os.path.splitext(os.path.basename(src))[0] + ".o")
        cmd = [nv, *ARCH, *NVCC_FLAGS, "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and r.stderr.strip():
            print(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, sources()))
    libdir = cuda_lib_dir(nv)
    tmp = LIB + ".tmp"
    cmd = [nv, *ARCH, "-shared", "-o", tmp, *objs, "-cudart", "shared", f"-L{libdir}",
           "-Xlinker", f"-rpath,{libdir}", "-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    build_cli(force=True)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
