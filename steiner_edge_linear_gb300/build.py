"""In-tree build of the native parts of the EMV solver.

Products (under ``steiner_edge_linear_gb300/lib/``, git-ignored):
  * ``libemv.so``      -- the C-ABI library of ``include/emv.h``: host code
    (STP reader, CSR, generator, server) and the sm_103a CUDA kernels;
  * ``reader-el-gpu``  -- the command-line front end with the flags and output
    lines of the reference's ``reader-el``;
  * ``emv-gen``        -- the instance generator as a stand-alone executable
    (host sources only, no CUDA, no libemv.so), for processes that must not
    load the solver.

Every CUDA translation unit is compiled for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``).  Host code is compiled with
``-ffp-contract=off`` and no machine-specific flags so that x86-64 and
aarch64 builds compute the same generator output.
"""
from __future__ import annotations

import concurrent.futures
import os
import shutil
import subprocess
import sys

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
ROOT_DIR = os.path.dirname(PKG_DIR)
CSRC = os.path.join(PKG_DIR, "csrc")
INCLUDE = os.path.join(ROOT_DIR, "include")
LIB_DIR = os.path.join(PKG_DIR, "lib")
OBJ_DIR = os.path.join(LIB_DIR, "obj")
LIB_PATH = os.path.join(LIB_DIR, "libemv.so")
CLI_PATH = os.path.join(LIB_DIR, "reader-el-gpu")
GEN_PATH = os.path.join(LIB_DIR, "emv-gen")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = [
    "emv_host.cpp",
    "emv_device.cu",
    "emv_batch.cu",
    "emv_server.cpp",
    "emv_noalloc.cu",
    "emv_bin.cpp",
    "emv_plan.cpp",
]
CLI_SOURCES = ["cli.cpp"]
GEN_SOURCES = ["gen_main.cpp", "emv_host.cpp"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found; the EMV solver needs the CUDA toolkit to build")


def _flags() -> list[str]:
    return ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off,-Wall",
            "-I", INCLUDE, "-I", CSRC] + ARCH


def _headers() -> list[str]:
    hs = [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    hs += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    return hs


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if proc.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + proc.stdout)


def build(force: bool = False, verbose: bool = False) -> str:
    """Compiles libemv.so, reader-el-gpu and emv-gen if any source changed; returns the library path."""
    os.makedirs(OBJ_DIR, exist_ok=True)
    nvcc = _nvcc()
    headers = _headers()
    jobs = []
    objs = []
    for src in SOURCES:
        path = os.path.join(CSRC, src)
        if not os.path.exists(path):
            continue
        obj = os.path.join(OBJ_DIR, src + ".o")
        objs.append(obj)
        if force or _stale(obj, [path] + headers):
            jobs.append([nvcc] + _flags() + ["-c", path, "-o", obj])
    if jobs:
        with concurrent.futures.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 1)) as ex:
            for fut in [ex.submit(_run, j) for j in jobs]:
                fut.result()
    if force or jobs or _stale(LIB_PATH, objs):
        _run([nvcc] + ARCH + ["-shared", "-o", LIB_PATH] + objs + ["-lpthread"])
    cli_srcs = [os.path.join(CSRC, s) for s in CLI_SOURCES]
    if force or _stale(CLI_PATH, cli_srcs + headers + [LIB_PATH]):
        _run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-Wall", "-I", INCLUDE, "-I", CSRC, "-o", CLI_PATH]
             + cli_srcs + ["-L", LIB_DIR, "-lemv", "-Wl,-rpath,$ORIGIN"])
    gen_srcs = [os.path.join(CSRC, s) for s in GEN_SOURCES]
    if force or _stale(GEN_PATH, gen_srcs + headers):
        _run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-Wall", "-I", INCLUDE, "-I", CSRC, "-o", GEN_PATH]
             + gen_srcs + ["-static-libstdc++", "-static-libgcc"])
    if verbose:
        print(f"built {LIB_PATH} ({len(jobs)} units recompiled)", file=sys.stderr)
    return LIB_PATH


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
