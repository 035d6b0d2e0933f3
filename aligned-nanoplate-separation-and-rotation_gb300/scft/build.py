"""Builds libscft.so (CUDA kernels + C ABI) and the scft_run driver for sm_103a.

    python -m scft.build            (from the package directory)

Every .cu under csrc/ is compiled in parallel with
    nvcc -gencode arch=compute_103a,code=sm_103a -O3 -lineinfo -std=c++17
and linked into build/libscft.so; host/*.cpp is linked against it into
build/scft_run.  Nothing is installed outside the package directory.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(PKG, "host")
BUILD = os.path.join(PKG, "build")
LIB = os.path.join(BUILD, "libscft.so")
DRIVER = os.path.join(BUILD, "scft_run")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    p = shutil.which("nvcc")
    if p:
        return p
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise FileNotFoundError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _stale(target: str, sources) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build(verbose: bool = False, ptxas_info: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(ROOT, "include", "scft.h"))
    cus = sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))
    objs = []
    jobs = []
    flags = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I" + CSRC,
                    "-I" + os.path.join(ROOT, "include")]
    if ptxas_info:
        flags += ["-Xptxas", "-v"]
    for cu in cus:
        obj = os.path.join(BUILD, os.path.basename(cu)[:-3] + ".o")
        objs.append(obj)
        if ptxas_info or _stale(obj, [cu] + headers):
            jobs.append([nvcc()] + flags + ["-c", cu, "-o", obj])
    logs = []
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        for out in ex.map(_run, jobs):
            logs.append(out)
    if jobs or _stale(LIB, objs):
        _run([nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"])
    hosts = sorted(os.path.join(HOST, f) for f in os.listdir(HOST) if f.endswith(".cpp")) if os.path.isdir(HOST) else []
    if hosts and _stale(DRIVER, hosts + [LIB] + headers):
        _run(["g++", "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "include"), "-o", DRIVER] + hosts
             + ["-L" + BUILD, "-lscft", "-Wl,-rpath,$ORIGIN"])
    if verbose or ptxas_info:
        print("\n".join(l for l in logs if l.strip()))
    return LIB


if __name__ == "__main__":
    build(verbose=True, ptxas_info="-v" in sys.argv)
    print(LIB)
