"""Build libimagew_gb300.so in-tree: host C++ with g++, device code with nvcc
for sm_103a, linked with nvcc into one shared library.

    python -m imageworsener_gb300.build          # build if out of date
    python -m imageworsener_gb300.build --force  # rebuild everything

Objects go to imageworsener_gb300/_build/, the library to
imageworsener_gb300/libimagew_gb300.so and the command-line tool to
imageworsener_gb300/imagew_gb300 (all git-ignored).  Sources compile
in parallel; a file is recompiled only when it, or a header, changed.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libimagew_gb300.so")

HOST_SRCS = ["api.cpp", "plan.cpp", "weights.cpp", "tables.cpp", "optimize.cpp", "server.cpp"]
DEVICE_SRCS = ["pipeline.cu", "fastpath.cu", "fastbatch.cu", "noalloc.cu", "tcvert.cu"]
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    return hs + [os.path.join(INCLUDE, "imagew.h"), os.path.join(INCLUDE, "imagew_gb300.h")]


def _stale(obj: str, src: str, deps: list[str]) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.exists(d) and os.path.getmtime(d) > t for d in [src, *deps])


def _cmd_host(src: str, obj: str) -> list[str]:
    # -ffp-contract=off: host tables must be computed with separately rounded
    # multiplies and adds, like the reference (aarch64 gcc fuses by default).
    return ["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-Wall",
            "-Wno-unused-function", f"-I{INCLUDE}", f"-I{CSRC}", "-c", src, "-o", obj]


def _cmd_dev(src: str, obj: str) -> list[str]:
    # -fmad=false: the exact form must not fuse multiply-adds; the fast form
    # requests its fused operations explicitly.
    return [_nvcc(), ARCH, "-std=c++17", "-O3", "-lineinfo", "-fmad=false", "-Xcompiler", "-fPIC",
            "-Xptxas", "-warn-spills", f"-I{INCLUDE}", f"-I{CSRC}", "-c", src, "-o", obj]


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile and link; returns the library path.  Raises on failure."""
    os.makedirs(BUILD, exist_ok=True)
    deps = _headers()
    jobs = []
    objs = []
    for f in HOST_SRCS + DEVICE_SRCS:
        src = os.path.join(CSRC, f)
        obj = os.path.join(BUILD, f + ".o")
        objs.append(obj)
        if force or _stale(obj, src, deps):
            jobs.append(_cmd_host(src, obj) if f.endswith(".cpp") else _cmd_dev(src, obj))
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
            results = list(ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs))
        for cmd, r in zip(jobs, results):
            if verbose or r.returncode:
                sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
            if r.returncode:
                raise RuntimeError(f"compile failed: {cmd[-3]}")
    if force or jobs or not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [_nvcc(), ARCH, "-shared", "-o", LIB, *objs, "-Xcompiler", "-fPIC", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose or r.returncode:
            sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        if r.returncode:
            raise RuntimeError("link failed")
    build_cli(force)
    return LIB


CLI_DIR = os.path.join(PKG, "cli")
CLI = os.path.join(PKG, "imagew_gb300")


def build_cli(force: bool = False) -> str:
    """The imagew_gb300 command-line tool (cli/*.c), linked against the
    library next to it."""
    srcs = [os.path.join(CLI_DIR, f) for f in ("imagew_cli.c", "pnm.c")]
    deps = srcs + [os.path.join(CLI_DIR, "pnm.h"), os.path.join(INCLUDE, "imagew.h"), LIB]
    if force or not os.path.exists(CLI) or any(os.path.getmtime(d) > os.path.getmtime(CLI) for d in deps):
        cmd = ["gcc", "-std=gnu99", "-O2", "-Wall", f"-I{INCLUDE}", f"-I{CLI_DIR}", "-o", CLI, *srcs,
               f"-L{PKG}", "-limagew_gb300", "-Wl,-rpath,$ORIGIN", "-lm"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
            raise RuntimeError("CLI build failed")
    return CLI


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(LIB)
