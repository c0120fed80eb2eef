"""Build recipe of libllfem_gb300.so: every CUDA translation unit compiled for
sm_103a in parallel with nvcc, host C++ with the same no-contraction flag
(the FP64 contract forbids compiler-introduced fused multiply-adds on the
host as on the device), linked into one in-tree shared library."""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libllfem_gb300.so")

CU_SOURCES = ["abi.cu", "scan.cu", "pattern.cu", "assemble.cu", "assemble_fp32.cu", "solve.cu", "ic0.cu", "tl.cu", "field.cu", "autotune.cu"]
CXX_SOURCES = ["tables.cpp", "serve.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def build_library(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(HERE, "..", "include", "llfem_gb300.h"))
    jobs, objs = [], []
    NV = nvcc()
    for src in CU_SOURCES:
        path = os.path.join(CSRC, src)
        if not os.path.exists(path):
            continue
        obj = os.path.join(BUILD, src + ".o")
        objs.append(obj)
        if not force and _newer(obj, [path] + headers):
            continue
        cmd = [NV, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
               "-Xcompiler", "-ffp-contract=off", "--fmad=false", "-c", path, "-o", obj]
        jobs.append((cmd, src))
    for src in CXX_SOURCES:
        path = os.path.join(CSRC, src)
        obj = os.path.join(BUILD, src + ".o")
        objs.append(obj)
        if not force and _newer(obj, [path] + headers):
            continue
        cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-pthread", "-ffp-contract=off", "-c", path, "-o", obj]
        jobs.append((cmd, src))
    procs = [(subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT), src)
             for cmd, src in jobs]
    failed = []
    for p, src in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((src, out.decode(errors="replace")))
        elif verbose and out:
            sys.stdout.write(out.decode(errors="replace"))
    if failed:
        msg = "\n".join(f"--- {s}\n{o}" for s, o in failed)
        raise RuntimeError(f"nvcc failed:\n{msg}")
    if force or jobs or not os.path.exists(LIB):
        tmp = LIB + ".tmp"
        subprocess.check_call([NV, *ARCH, "-shared", "-o", tmp, *objs])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build_library(verbose=True, force="--force" in sys.argv))
