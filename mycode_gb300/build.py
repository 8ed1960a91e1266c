"""Build libcfdgpu.so in-tree (mycode_gb300/_lib/) for sm_103a.

Translation units and their floating-point contracts:
  kern_f64.cu  nvcc --fmad=false  (FP64 residual/Krylov kernels match the CPU reference)
  kern_f32.cu  nvcc --prec-div=false --prec-sqrt=false  (FP32 residual and mixed-precision
               vectors: FP32 divides and square roots to ~2 ulp; FP64 untouched)
  kern_jv.cu   nvcc --prec-div=false --prec-sqrt=false  (dual-number exact J v, same)
  solver.cu    nvcc               (host driver and C ABI; host code without contraction)
  noalloc.cu   nvcc --fmad=false  (residual norm with static scratch, no allocation)
  kern_adj.cu  nvcc               (adjoint / VJP of the FP64 residual)
  kern_qoi.cu  nvcc --fmad=false  (wall distance, Cp/Cf, drag, entropy error)
  mesh_gpu.cu  nvcc --fmad=false  (mesh connectivity, geometry and renumbering on the GPU)
  mesh.cpp     g++ -ffp-contract=off (host geometry bit-exact on x86 and Arm)
Compiles in parallel, links with nvcc (static cudart).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT, "libcfdgpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU = {
    "kern_f64.cu": ["--fmad=false"],
    "kern_f32.cu": ["--prec-div=false", "--prec-sqrt=false"],
    "kern_jv.cu": ["--prec-div=false", "--prec-sqrt=false"],
    "solver.cu": [],
    "noalloc.cu": ["--fmad=false"],
    "kern_adj.cu": [],
    "kern_qoi.cu": ["--fmad=false"],
    "mesh_gpu.cu": ["--fmad=false"],
}
CPP = ["mesh.cpp"]


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _cuda_home(nvcc: str) -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def _sources():
    return [os.path.join(SRC, f) for f in os.listdir(SRC)] + [os.path.join(HERE, "..", "include", "cfdg.h")]


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(p) <= t for p in _sources())


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and up_to_date():
        return LIB
    nvcc = _nvcc()
    inc = os.path.join(_cuda_home(nvcc), "include")
    obj = os.path.join(OUT, "obj")
    os.makedirs(obj, exist_ok=True)
    jobs = []
    for f, extra in CU.items():
        o = os.path.join(obj, f + ".o")
        cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", *extra,
               "-Xcompiler", "-fPIC,-ffp-contract=off", "-c", os.path.join(SRC, f), "-o", o]
        jobs.append((f, cmd, o))
    for f in CPP:
        o = os.path.join(obj, f + ".o")
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", f"-I{inc}", "-c",
               os.path.join(SRC, f), "-o", o]
        jobs.append((f, cmd, o))
    procs = [(f, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True), o)
             for f, cmd, o in jobs]
    errs = []
    for f, p, o in procs:
        out, _ = p.communicate()
        if verbose and out:
            print(out)
        if p.returncode != 0:
            errs.append(f"{f}:\n{out}")
    if errs:
        raise RuntimeError("libcfdgpu build failed:\n" + "\n".join(errs))
    tmp = LIB + f".tmp{os.getpid()}"
    link = [nvcc, *ARCH, "-shared", "-o", tmp] + [o for _, _, o in jobs]
    r = subprocess.run(link, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("libcfdgpu link failed:\n" + r.stdout)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
