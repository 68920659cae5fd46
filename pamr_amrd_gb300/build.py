"""Builds libpamr_gb300.so in place: CUDA kernels for sm_103a (nvcc) and the
C host driver (gcc), linked against the CUDA runtime.

The FP64 kernels are compiled with -fmad=false so that their arithmetic
rounds like the reference's CPU code; host C is compiled with
-ffp-contract=off for the same reason.
"""
from __future__ import annotations

import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libpamr_gb300.so")
LIB_F77 = os.path.join(os.path.dirname(LIB), "libpamr_gb300_f77.so")
# the drop-in multigrid module (amrd/mg.c's entry points over libpamr_gb300):
# a shared library and a static archive (AMRD applications link static libs)
LIB_AMRD_MG = os.path.join(HERE, "libamrd_mg_gb300.so")
LIB_AMRD_MG_A = os.path.join(HERE, "libamrd_mg_gb300.a")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"

CU_SOURCES = {"pgb_kernels64.cu": ["-fmad=false"], "pgb_noalloc.cu": ["-fmad=false"],
              "pgb_mutil_ex.cu": ["-fmad=false"], "pgb_bo.cu": ["-fmad=false"], "pgb_diss.cu": ["-fmad=false"], "pgb_linbnd.cu": ["-fmad=false"], "pgb_kernels32.cu": [],
              "pgb_net.cu": []}
C_SOURCES = ["pgb_plan.c", "pgb_solver.c", "pgb_op.c"]


def cuda_home() -> str:
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found")


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    cuda = cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(OBJ, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(ROOT, "include", "pamr_gb300.h"))
    jobs, objs = [], []
    for src, extra in CU_SOURCES.items():
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            cmd = [nvcc, ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                   "-I" + CSRC, "-I" + os.path.join(ROOT, "include")] + extra + ["-c", s, "-o", o]
            jobs.append(cmd)
    for src in C_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            cmd = ["gcc", "-std=gnu11", "-O2", "-fPIC", "-ffp-contract=off", "-fno-fast-math",
                   "-Wall", "-I" + CSRC, "-I" + os.path.join(ROOT, "include"),
                   "-I" + os.path.join(cuda, "include"), "-c", s, "-o", o]
            jobs.append(cmd)
    procs = [(c, subprocess.Popen(c, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True))
             for c in jobs]
    for c, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError("build failed: " + " ".join(c) + "\n" + out)
        if verbose and out:
            print(out)
    if force or _stale(LIB, objs):
        libdir = os.path.join(cuda, "lib64")
        cmd = [nvcc, ARCH, "-shared", "-o", LIB] + objs + ["-L" + libdir, "-lcudart",
                                                           "-Xlinker", "-rpath",
                                                           "-Xlinker", libdir]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed: " + r.stdout + r.stderr)
    # the Fortran-ABI drop-in (m_util_r8.h symbols on host arrays) over LIB
    fsrc = os.path.join(CSRC, "pgb_f77.c")
    if force or _stale(LIB_F77, [fsrc, LIB] + headers):
        libdir = os.path.join(cuda, "lib64")
        cmd = ["gcc", "-std=gnu11", "-O2", "-fPIC", "-shared", "-Wall",
               "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(cuda, "include"),
               fsrc, "-o", LIB_F77, "-L" + os.path.dirname(LIB), "-lpamr_gb300",
               "-L" + libdir, "-lcudart", "-Wl,-rpath,$ORIGIN", "-Wl,-rpath," + libdir]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed: " + r.stdout + r.stderr)
    # the drop-in multigrid module: PAMR_* / AMRD_* stay undefined here and
    # resolve against the application's libpamr / libamrd when it links
    msrc = os.path.join(CSRC, "amrd_mg_gb300.c")
    mobj = os.path.join(OBJ, "amrd_mg_gb300.c.o")
    mdeps = [msrc, os.path.join(CSRC, "amrd_abi.h"), os.path.join(ROOT, "include", "amrd_mg_gb300.h")] + headers
    if force or _stale(mobj, mdeps):
        cmd = ["gcc", "-std=gnu11", "-O2", "-fPIC", "-Wall", "-I" + CSRC, "-I" + os.path.join(ROOT, "include"),
               "-c", msrc, "-o", mobj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("build failed: " + r.stdout + r.stderr)
    if force or _stale(LIB_AMRD_MG, [mobj, LIB]):
        libdir = os.path.join(cuda, "lib64")
        cmd = ["gcc", "-shared", "-o", LIB_AMRD_MG, mobj, "-L" + HERE, "-lpamr_gb300", "-L" + libdir, "-lcudart",
               "-lm", "-Wl,-rpath,$ORIGIN", "-Wl,-rpath," + libdir]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed: " + r.stdout + r.stderr)
    if force or _stale(LIB_AMRD_MG_A, [mobj]):
        if os.path.exists(LIB_AMRD_MG_A):
            os.remove(LIB_AMRD_MG_A)
        r = subprocess.run(["ar", "rcs", LIB_AMRD_MG_A, mobj], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("ar failed: " + r.stdout + r.stderr)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
