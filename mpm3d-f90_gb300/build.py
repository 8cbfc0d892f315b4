"""Build recipe for libmpm3d_gpu (sm_103a) and the CPU oracle.

Outputs (all git-ignored, built in-tree so that they travel with the tree):
  mpm3d-f90_gb300/_build/libmpm3d_gpu.so   -- the C-ABI library (CUDA + C)
  mpm3d-f90_gb300/_build/mpm3d_gpu         -- command-line driver (MPM3D.f90 loop)
  oracle/_build/libmpm_oracle.so           -- CPU oracle (test infrastructure)
  oracle/_build/mpm3d_oracle               -- oracle command-line driver

Translation units are compiled in parallel; the FP64 step is compiled with
--fmad=false (no fused multiply-add contraction) and the host C code (the
oracle included, which is also the timed CPU baseline) with -O3
-ffp-contract=off, so that both sides round every product and sum.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INC = os.path.join(ROOT, "include")
BUILD = os.path.join(HERE, "_build")
ORACLE = os.path.join(ROOT, "oracle")
ORACLE_BUILD = os.path.join(ORACLE, "_build")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
                      "-Xcompiler", "-ffp-contract=off", "-I" + INC, "-I" + CSRC]
CC_COMMON = ["-O3", "-fPIC", "-std=c11", "-ffp-contract=off", "-D_POSIX_C_SOURCE=200809L",
             "-Wall", "-I" + INC, "-I" + CSRC]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _newer(target: str, sources: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def _headers() -> list[str]:
    out = []
    for d in (CSRC, INC):
        for f in os.listdir(d):
            if f.endswith((".h", ".cuh")):
                out.append(os.path.join(d, f))
    return out


def build_library(force: bool = False) -> str:
    """Compile libmpm3d_gpu.so for sm_103a; returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    hdr = _headers()
    units = [
        ("mpm_fp64.cu", ["--fmad=false"]),
        ("mpm_gpu.cu", []),
        ("mpm_noalloc.cu", ["--fmad=false"]),
        ("mpm_setup.cu", []),
        ("mpm_batch.cu", []),
        ("mpm_serve.cu", []),
        ("mpm_probe.cu", []),
    ]
    jobs = []
    objs = []
    for src, extra in units:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _newer(o, [s] + hdr):
            jobs.append([nvcc] + NVCC_COMMON + extra + ["-c", s, "-o", o])
    for csrc in ("mpm_deck.c", "mpm_output.c"):
        c_src = os.path.join(CSRC, csrc)
        c_obj = os.path.join(BUILD, csrc.replace(".c", ".o"))
        objs.append(c_obj)
        if force or _newer(c_obj, [c_src] + hdr):
            jobs.append(["gcc"] + CC_COMMON + ["-c", c_src, "-o", c_obj])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
        for f in [ex.submit(_run, j) for j in jobs]:
            f.result()
    lib = os.path.join(BUILD, "libmpm3d_gpu.so")
    if force or jobs or not os.path.exists(lib):
        _run([nvcc] + ARCH + ["-shared", "-o", lib] + objs + ["-lcudart"])
    drv_src = os.path.join(HERE, "host", "mpm3d_gpu_main.c")
    drv = os.path.join(BUILD, "mpm3d_gpu")
    if os.path.exists(drv_src) and (force or _newer(drv, [drv_src, lib])):
        _run(["gcc"] + CC_COMMON + [drv_src, "-o", drv, "-L" + BUILD, "-lmpm3d_gpu",
                                    "-Wl,-rpath," + BUILD, "-lm"])
    return lib


def build_oracle(force: bool = False) -> str:
    """Compile the CPU oracle (test infrastructure) as a shared library + CLI."""
    os.makedirs(ORACLE_BUILD, exist_ok=True)
    srcs = [os.path.join(ORACLE, "mpm_oracle.c"), os.path.join(CSRC, "mpm_deck.c")]
    hdr = _headers() + [os.path.join(ORACLE, "mpm_oracle.h")]
    lib = os.path.join(ORACLE_BUILD, "libmpm_oracle.so")
    cli = os.path.join(ORACLE_BUILD, "mpm3d_oracle")
    inc = ["-I" + ORACLE]
    jobs = []
    if force or _newer(lib, srcs + hdr):
        jobs.append(["gcc"] + CC_COMMON + inc + ["-shared", "-o", lib] + srcs + ["-lm"])
    main = os.path.join(ORACLE, "oracle_main.c")
    if force or _newer(cli, srcs + hdr + [main]):
        jobs.append(["gcc"] + CC_COMMON + inc + ["-o", cli, main] + srcs + ["-lm"])
    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        for f in [ex.submit(_run, j) for j in jobs]:
            f.result()
    return lib


def build_all(force: bool = False) -> None:
    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        a = ex.submit(build_library, force)
        b = ex.submit(build_oracle, force)
        a.result()
        b.result()


if __name__ == "__main__":
    build_all(force="--force" in sys.argv)
    print("built", BUILD, ORACLE_BUILD)
