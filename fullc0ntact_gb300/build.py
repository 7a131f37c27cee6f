"""Builds libfcdem.so in-tree for sm_103a with nvcc (no CMake, no torch
extension machinery): each translation unit is compiled in parallel, then
linked with nvcc -shared.  Output: fullc0ntact_gb300/_lib/libfcdem.so."""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libfcdem.so")

SOURCES = [
    "fcdem_context.cu",
    "fcdem_stages.cu",
    "fcdem_sort.cu",
    "fcdem_collide.cu",
    "fcdem_count.cu",
    "fcdem_distmap.cu",
    "fcdem_batch.cu",
    "fcdem_sdf.cu",
    "fcdem_host.cpp",
    "fcdem_scenes.cpp",
    "fcdem_i3d.cu",
    "fcdem_i3d_integrate.cpp",
]
# per-file host-compiler flags (the scene generators round every a*b+c
# twice, as the reference arm's build of the same file does)
EXTRA = {"fcdem_scenes.cpp": ["-Xcompiler", "-ffp-contract=off"]}

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = [
    "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
    "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills",
]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA 13 toolkit is required to build libfcdem")


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    inc = os.path.join(os.path.dirname(HERE), "include")
    hs += [os.path.join(inc, f) for f in os.listdir(inc) if f.endswith(".h")]
    return hs


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    headers = _headers()
    jobs = []
    objs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o").replace(".cpp", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + headers):
            cmd = [cc] + ARCH + NVFLAGS + EXTRA.get(src, []) + ["-c", s, "-o", o]
            jobs.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for cmd, r in ex.map(run, jobs):
                if verbose or r.returncode != 0:
                    sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
                if r.returncode != 0:
                    raise RuntimeError(f"nvcc failed on {cmd[-3]}")
    if force or jobs or _stale(LIB, objs):
        cmd = [cc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose or r.returncode != 0:
            sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        if r.returncode != 0:
            raise RuntimeError("linking libfcdem.so failed")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
