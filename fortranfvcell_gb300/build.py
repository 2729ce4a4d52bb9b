"""Build recipe for libfvcgpu.so (sm_103a), in-tree.

Compiles every translation unit under ``csrc/`` with nvcc in parallel and
links ``fortranfvcell_gb300/lib/libfvcgpu.so``.  No cmake, one -gencode, so
the same recipe runs on the x86_64 build host and on the aarch64 GPU host.
"""
from __future__ import annotations

import concurrent.futures as cf
import fcntl
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "lib")
# FVC_CHECK=1 in the environment selects the check variant: every
# translation unit compiled with -DFVC_CHECK (device bounds checks that
# record a code and redirect the access, see csrc/fvc_device.cuh) into
# lib/libfvcgpu_check.so, which the package then loads instead.
CHECK = os.environ.get("FVC_CHECK", "0") not in ("", "0")
BUILD = os.path.join(HERE, "_build_check" if CHECK else "_build")
LIB = os.path.join(LIBDIR, "libfvcgpu_check.so" if CHECK else "libfvcgpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["fvc_krylov.cu", "fvc_cluster.cu", "fvc_mixed.cu", "fvc_gather.cu", "fvc_assembly.cu",
           "fvc_noalloc.cu", "fvc_simple.cu", "fvc_simple_driver.cu", "fvc_api.cpp",
           "fvc_mesh.cpp"]
# files whose kernels reproduce the reference's rounding: no FMA contraction
NO_FMAD = {"fvc_simple.cu"}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _compile(src: str, verbose_ptxas: bool) -> str:
    path = os.path.join(CSRC, src)
    obj = os.path.join(BUILD, src + ".o")
    cmd = [nvcc(), "-c", path, "-o", obj, "-O3", "-std=c++17", "-lineinfo",
           "-Xcompiler", "-fPIC,-O3,-Wall", *ARCH]
    if CHECK:
        cmd.append("-DFVC_CHECK")
    if src.endswith(".cu"):
        cmd += ["--expt-relaxed-constexpr"]
        if src in NO_FMAD:
            cmd += ["--fmad=false"]
        if verbose_ptxas:
            cmd += ["-Xptxas", "-v"]
    else:
        cmd = [c for c in cmd if c not in ("-lineinfo",)]
        cmd[cmd.index(path)] = path
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{res.stdout}\n{res.stderr}")
    if verbose_ptxas and res.stderr:
        with open(os.path.join(BUILD, src + ".ptxas.txt"), "w") as f:
            f.write(res.stderr)
    return obj


def sources() -> list[str]:
    return [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]


def needs_build() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(HERE, "..", "include", "fvcgpu.h"))
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force: bool = False, verbose_ptxas: bool = False) -> str:
    if not force and not needs_build():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    # one build at a time: processes started together wait for the first
    with open(os.path.join(BUILD, ".lock"), "w") as lock:
        fcntl.flock(lock, fcntl.LOCK_EX)
        if not force and not needs_build():
            return LIB
        with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 2)) as ex:
            objs = list(ex.map(lambda s: _compile(s, verbose_ptxas), sources()))
        tmp = f"{LIB}.{os.getpid()}.tmp"
        cmd = [nvcc(), "-shared", "-o", tmp, *objs, *ARCH, "-Xcompiler", "-fPIC"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv))
