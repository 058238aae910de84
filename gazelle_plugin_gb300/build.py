"""In-tree build of libgzsplit.so (sm_103a CUDA kernels + host C++ + C ABI) with nvcc.

Translation units are compiled in parallel, then linked into
gazelle_plugin_gb300/libgzsplit.so.  No cmake; one -gencode.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
ROOT = os.path.dirname(HERE)
BUILD_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libgzsplit.so")
TASK_LIB = os.path.join(HERE, "libgztask.so")  # simulated map tasks calling the C ABI

SOURCES = ["kernels.cu", "splitter.cc", "splitter_nested.cc", "ipc.cc", "schema_ipc.cc", "capi.cc", "host_util.cc",
           "hash_static.cu", "serve.cc", "tune.cc", "reader.cc", "read_kernels.cu", "lz4_kernels.cu"]
NOT_IN_LIB = {"task_driver.cc"}  # built into libgztask.so
GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _compile(src: str, verbose: bool) -> str:
    obj = os.path.join(BUILD_DIR, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), *GENCODE, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
           "-I", os.path.join(ROOT, "include"), "-c", os.path.join(CSRC, src), "-o", obj]
    if src.endswith(".cu"):
        cmd[1:1] = ["-Xptxas", "-v"] if verbose else []
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    if verbose and (r.stdout or r.stderr):
        sys.stderr.write(r.stdout + r.stderr)
    return obj


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f not in NOT_IN_LIB] + [
        os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include")) if f != "gz_task.h"]
    return any(os.path.getmtime(d) > t for d in deps)


def build_task_driver(force: bool = False) -> str:
    """libgztask.so: the map-task driver (csrc/task_driver.cc), linked against libgzsplit.so and
    calling only its C ABI."""
    src = os.path.join(CSRC, "task_driver.cc")
    deps = [src, LIB] + [os.path.join(ROOT, "include", f) for f in ("gz_split.h", "gz_task.h")]
    if not force and os.path.exists(TASK_LIB) and all(os.path.getmtime(d) <= os.path.getmtime(TASK_LIB) for d in deps):
        return TASK_LIB
    tmp = TASK_LIB + ".tmp"
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-I", os.path.join(ROOT, "include"), src,
           "-o", tmp, "-L", HERE, "-lgzsplit", "-Wl,-rpath,$ORIGIN", "-pthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"task driver build failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, TASK_LIB)
    return TASK_LIB


def build_library(force: bool = False, verbose: bool = False) -> str:
    if not force and not _stale():
        build_task_driver()
        return LIB
    os.makedirs(BUILD_DIR, exist_ok=True)
    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    tmp = LIB + ".tmp"
    cmd = [nvcc(), *GENCODE, "-shared", "-o", tmp, *objs, "-lcuda"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    build_task_driver(force=True)
    return LIB


if __name__ == "__main__":
    print(build_library(force="--force" in sys.argv, verbose="-v" in sys.argv))
