"""Build the CUDA library libmpmc_gb300_flash.so in-tree for sm_103a.

Each kernel translation unit is compiled once per component capacity
(-DMPMC_NM=4, 8, 12, 16, 20) in parallel, then everything is linked into one
shared library with the C ABI of include/mpmc_gb300_flash.h.  Objects are
rebuilt only when a source or header is newer.
"""

from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "_lib")
LIB = os.path.join(LIBDIR, "libmpmc_gb300_flash.so")
PROBE_LIB = os.path.join(LIBDIR, "libmpmc_gb300_probe.so")

CAPACITIES = (4, 8, 12, 16, 20)
# translation units compiled once per capacity
PER_CAPACITY = ("flash_plain.cu", "sensitivity.cu", "flash_batched.cu", "flash_max3.cu", "chart.cu")
# extra nvcc flags per translation unit (none: every unit at -O3; the
# max-3-phase unit keeps its large FP64 routines out of line, which keeps its
# -O3 build near 20 s)
EXTRA_FLAGS: dict[str, list[str]] = {}
# translation units compiled once
SINGLE = ("capi.cu", "server.cu", "peak_probe.cu")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                     "-I" + os.path.join(ROOT, "include")]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _deps() -> float:
    files = glob.glob(os.path.join(CSRC, "*")) + glob.glob(os.path.join(ROOT, "include", "*.h")) + [__file__]
    return max(os.path.getmtime(f) for f in files)


def _compile(src: str, obj: str, extra: list[str], newest: float, verbose: bool) -> str:
    if os.path.exists(obj) and os.path.getmtime(obj) >= newest:
        return obj
    cmd = [_nvcc()] + NVCC_FLAGS + extra + ["-c", os.path.join(CSRC, src), "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src} {extra}:\n{res.stdout}\n{res.stderr}")
    return obj


def build(verbose: bool = False, jobs: int | None = None) -> str:
    """Compile and link; returns the library path."""
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    newest = _deps()
    tasks = []
    for src in PER_CAPACITY:
        stem = os.path.splitext(src)[0]
        for nm in CAPACITIES:
            tasks.append((src, os.path.join(BUILD, f"{stem}_nm{nm}.o"), [f"-DMPMC_NM={nm}"] + EXTRA_FLAGS.get(src, [])))
    for src in SINGLE:
        tasks.append((src, os.path.join(BUILD, os.path.splitext(src)[0] + ".o"), []))
    jobs = jobs or min(len(tasks), max(1, os.cpu_count() or 1))
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(lambda a: _compile(*a, newest, verbose), tasks))
    probe_obj = os.path.join(BUILD, "peak_probe.o")
    flash_objs = [o for o in objs if o != probe_obj]
    for lib, parts in ((LIB, flash_objs), (PROBE_LIB, [probe_obj])):
        if not os.path.exists(lib) or any(os.path.getmtime(o) > os.path.getmtime(lib) for o in parts):
            cmd = [_nvcc()] + ARCH + ["-shared", "-o", lib] + parts + ["-lpthread"]
            if verbose:
                print(" ".join(cmd), flush=True)
            subprocess.check_call(cmd)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
