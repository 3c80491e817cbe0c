"""Builds libfastedm_gb300.so in place (sm_103a only).

CUDA sources go through nvcc with one -gencode for sm_103a; the exact-FP64
kernels are compiled with --fmad=false so no multiply-add is fused.  Host C++
is compiled with -ffp-contract=off so that Arm and x86 hosts build
bit-identical manifolds.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
SRC = PKG / "csrc"
OUT = PKG / "_build"
LIB = PKG / "libfastedm_gb300.so"
CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
NVCC = str(CUDA_HOME / "bin" / "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_FLAGS = {
    "kernels_exact.cu": ["--fmad=false"],
    "kernels_util.cu": [],
    "kernels_mixed.cu": [],
    "kernels_wide.cu": [],
    "kernels_one16.cu": [],
    "kernels_pen.cu": [],
    "kernels_manifold.cu": ["--fmad=false"],
    "kernels_split.cu": [],
    "kernels_gram_tc.cu": [],
    "static_entry.cu": [],
    "kernels_adjoint.cu": [],
}
CPP = ["host.cpp", "engine.cpp", "capi.cpp"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r.stdout + r.stderr


def _stale(obj, deps):
    return not obj.exists() or any(d.stat().st_mtime > obj.stat().st_mtime for d in deps)


def build(verbose=False, ptxas_info=False):
    OUT.mkdir(exist_ok=True)
    headers = list(SRC.glob("*.h")) + list(SRC.glob("*.cuh")) + [PKG.parent / "include" / "fastedm_gb300.h"]
    jobs, objs = [], []
    for name, extra in CU_FLAGS.items():
        src = SRC / name
        if not src.exists():
            continue
        obj = OUT / (name + ".o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            cmd = [NVCC, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                   *extra, "-c", str(src), "-o", str(obj)]
            if ptxas_info:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    for name in CPP:
        src = SRC / name
        obj = OUT / (name + ".o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            jobs.append(["g++", "-O3", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-sign-compare",
                         f"-I{CUDA_HOME / 'include'}", "-c", str(src), "-o", str(obj)])
    with ThreadPoolExecutor(max_workers=max(1, min(8, os.cpu_count() or 1))) as ex:
        logs = list(ex.map(_run, jobs))
    if verbose:
        for cmd, log in zip(jobs, logs):
            print(" ".join(cmd))
            if log.strip():
                print(log)
    if jobs or not LIB.exists():
        tmp = LIB.with_suffix(".so.tmp")
        _run(["g++", "-shared", "-o", str(tmp), *map(str, objs), f"-L{CUDA_HOME / 'lib64'}", "-lcudart",
              "-lpthread", f"-Wl,-rpath,{CUDA_HOME / 'lib64'}"])
        shutil.move(str(tmp), str(LIB))
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, ptxas_info="--ptxas" in sys.argv))
