"""Build libbgk2d_gb300.so in-tree with nvcc for sm_103a.

Each .cu translation unit compiles in its own process (in parallel); the FP32/FP64 kernels are
compiled with -fmad=false so every reference operation is one IEEE operation, host code with
-ffp-contract=off for the same reason; the 16-bit storage kernels keep FMA contraction.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB_NAME = "libbgk2d_gb300.so"
LIB_PATH = os.path.join(OUT_DIR, LIB_NAME)
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

SOURCES = {
    "bgk_api.cu": ["-fmad=false"],
    "bgk_batch.cu": ["-fmad=false"],
    "bgk_noalloc.cu": ["-fmad=false"],
    "bgk_peaks.cu": ["-fmad=false"],
    "bgk_inst_f32_f32.cu": ["-fmad=false"],
    "bgk_inst_f32_f64.cu": ["-fmad=false"],
    "bgk_inst_f64_f64.cu": ["-fmad=false"],
    "bgk_inst_f16_f32.cu": ["-fmad=true"],
    "bgk_inst_bf16_f32.cu": ["-fmad=true"],
}
HOST_SOURCES = ["bgk_serve.cpp"]
DRIVER = "bgk2d_main.cpp"          # host driver executable linked against the library
EXE_PATH = os.path.join(OUT_DIR, "bgk2d_gb300")


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libbgk2d_gb300.so")


def _flags(extra):
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
                   "-I", os.path.join(HERE, "..", "include")] + extra


def _compile(src, extra, obj, verbose):
    cmd = [nvcc()] + _flags(extra) + ["-c", os.path.join(CSRC, src), "-o", obj]
    if verbose:
        cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return r.stderr


def _stale(obj, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False, jobs: int | None = None) -> str:
    """Compile every translation unit and link the shared library; returns its path."""
    os.makedirs(OUT_DIR, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(HERE, "..", "include", "bgk2d_gb300.h"))
    objs, todo = [], []
    for src, extra in SOURCES.items():
        if not os.path.exists(os.path.join(CSRC, src)):
            continue
        obj = os.path.join(OUT_DIR, src.replace(".cu", ".o"))
        objs.append(obj)
        if force or _stale(obj, [os.path.join(CSRC, src)] + headers):
            todo.append((src, extra, obj))
    for src in HOST_SOURCES:
        if not os.path.exists(os.path.join(CSRC, src)):
            continue
        obj = os.path.join(OUT_DIR, src.replace(".cpp", ".o"))
        objs.append(obj)
        if force or _stale(obj, [os.path.join(CSRC, src)] + headers):
            todo.append((src, [], obj))
    logs = {}
    if todo:
        with cf.ThreadPoolExecutor(max_workers=jobs or min(len(todo), os.cpu_count() or 4)) as ex:
            futs = {ex.submit(_compile, s, e, o, verbose): s for s, e, o in todo}
            for f in cf.as_completed(futs):
                logs[futs[f]] = f.result()
    if todo or not os.path.exists(LIB_PATH):
        tmp = LIB_PATH + ".tmp"
        cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB_PATH)
    drv = os.path.join(CSRC, DRIVER)
    if os.path.exists(drv) and (force or _stale(EXE_PATH, [drv, LIB_PATH])):
        cxx = shutil.which("g++") or "g++"
        cmd = [cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I", os.path.join(HERE, "..", "include"), drv,
               "-L", OUT_DIR, "-lbgk2d_gb300", "-Wl,-rpath,$ORIGIN", "-o", EXE_PATH]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"driver build failed:\n{r.stdout}\n{r.stderr}")
    if verbose:
        for k, v in logs.items():
            sys.stdout.write(f"== {k}\n{v}\n")
    return LIB_PATH


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
