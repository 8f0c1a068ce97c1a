"""In-tree build of libsimpois_gpu.so (sm_103a) and of the simpois CLI.

Every CUDA translation unit is compiled in parallel with
``nvcc -gencode arch=compute_103a,code=sm_103a``; the shared library links the
CUDA runtime statically, so it depends on the driver only.  The CLI is plain
C linked against the library.  Outputs go to ``imscript_gb300/_build/``.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
CLI = os.path.join(PKG, "cli")
OUT = os.path.join(PKG, "_build")
INCLUDE = os.path.join(ROOT, "include")
LIB = os.path.join(OUT, "libsimpois_gpu.so")
CLI_BIN = os.path.join(OUT, "simpois")
AMLE_BIN = os.path.join(OUT, "amle")

CU_SOURCES = ["abi.cu", "ref_schedule.cu", "mg_solver.cu", "noalloc.cu", "amle.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2", "--expt-relaxed-constexpr"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise FileNotFoundError("nvcc not found")


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs.append(os.path.join(INCLUDE, "simpois_gpu.h"))
    return hs


def build_library(verbose=False, force=False) -> str:
    os.makedirs(OUT, exist_ok=True)
    nv = nvcc()
    hdrs = _headers()
    objs = []
    jobs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + hdrs):
            jobs.append([nv, *ARCH, *NVCC_FLAGS, "-I", INCLUDE, "-c", s, "-o", o])

    def run(cmd):
        if verbose:
            print(" ".join(cmd))
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return r.stderr

    with ThreadPoolExecutor(max_workers=len(jobs) or 1) as ex:
        list(ex.map(run, jobs))
    if force or jobs or _stale(LIB, objs):
        run([nv, *ARCH, "-shared", "-o", LIB, *objs])
    return LIB


# the commands: each main source linked with the image I/O and the library
COMMANDS = {"simpois": "simpois_main.c", "amle": "amle_main.c"}


def build_cli(verbose=False, force=False) -> str:
    hdrs = [os.path.join(CLI, f) for f in os.listdir(CLI) if f.endswith(".h")]
    io = os.path.join(CLI, "imageio.c")
    for name, main in COMMANDS.items():
        srcs = [os.path.join(CLI, main), io]
        binary = os.path.join(OUT, name)
        if force or _stale(binary, srcs + hdrs + [LIB, os.path.join(INCLUDE, "simpois_gpu.h")]):
            cc = os.environ.get("CC", "gcc")
            cmd = [cc, "-O2", "-std=gnu99", "-Wall", "-I", INCLUDE, *srcs, "-o", binary,
                   "-L", OUT, "-lsimpois_gpu", "-Wl,-rpath,$ORIGIN", "-lm"]
            if verbose:
                print(" ".join(cmd))
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"cc failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return CLI_BIN


def build(verbose=False, force=False):
    lib = build_library(verbose, force)
    cli = build_cli(verbose, force)
    return lib, cli


if __name__ == "__main__":
    import sys
    print(build(verbose=True, force="-f" in sys.argv))
