"""
Build libfsgpu.so (the CUDA kernels and the C-ABI of include/fsgpu.h) for
sm_103a with nvcc, and libfsghost.so (the arbitrary-precision host side of
include/fsghost.h, g++ against the system MPFR / MPC / GMP), in-tree: objects
in fractalshades_gb300/_build/, the shared libraries in fractalshades_gb300/_lib/.

The translation units that reproduce the reference's rounding are compiled
with -fmad=false (no contraction of a*b+c into an FMA); the FP32 fast kernel
and the host-side ABI keep the default.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
ROOT = os.path.dirname(PKG)
BUILD = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "_lib")
LIB = os.path.join(LIBDIR, "libfsgpu.so")
HOST_LIB = os.path.join(LIBDIR, "libfsghost.so")
HOST_SRC = os.path.join(HERE, "host", "fsg_host.cpp")
HOST_DEPS = [HOST_SRC, os.path.join(HERE, "host", "fsg_mp.h"),
             os.path.join(ROOT, "include", "fsghost.h")]
# runtime sonames of the libraries the reference's Cython module links
# (FP_loop.pyx); no development headers are needed (host/fsg_mp.h)
HOST_LIBS = ["-l:libmpc.so.3", "-l:libmpfr.so.6", "-l:libgmp.so.10"]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
          "-I", os.path.join(ROOT, "include")]
SOURCES = {
    "fsg_std.cu": ["-fmad=false"],
    "fsg_perturb.cu": ["-fmad=false"],
    "fsg_ref.cu": ["-fmad=false"],
    "fsg_perturb_fe32.cu": [],
    "fsg_perturb_bs32.cu": [],
    "fsg_peak.cu": [],
    "fsg_noalloc.cu": [],
    "fsg_lpt.cu": [],
    "fsg_postproc.cu": ["-fmad=false"],
    "fsg_abi.cu": [],
}
HEADERS = ["fsg_num.cuh", "fsg_internal.cuh", "fsg_bs.cuh", "fsg_mn.cuh"]


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libfsgpu.so")
    return exe


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build_host(verbose=False):
    """libfsghost.so: g++ -O2, no architecture-specific flags (x86_64 and
    aarch64 give the same results: MPFR's arithmetic is exact-rounded)."""
    os.makedirs(LIBDIR, exist_ok=True)
    if not _stale(HOST_LIB, HOST_DEPS):
        return HOST_LIB
    cxx = shutil.which("g++") or "g++"
    cmd = [cxx, "-O2", "-std=c++17", "-fPIC", "-shared", "-Wall", "-o", HOST_LIB, HOST_SRC,
           "-Wl,--no-undefined"] + HOST_LIBS
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("g++ failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    if verbose and (r.stdout or r.stderr):
        print(r.stdout + r.stderr)
    return HOST_LIB


def build(verbose=False, ptxas_info=False):
    build_host(verbose)
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    hdrs = [os.path.join(HERE, h) for h in HEADERS] + [os.path.join(ROOT, "include", "fsgpu.h")]
    jobs = []
    objs = []
    for src, flags in SOURCES.items():
        sp = os.path.join(HERE, src)
        obj = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(obj)
        if _stale(obj, [sp] + hdrs) or ptxas_info:
            cmd = [nvcc()] + ARCH + COMMON + flags + ["-c", sp, "-o", obj]
            if ptxas_info:
                cmd += ["-Xptxas", "-v"]
            jobs.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        return r.stdout + r.stderr

    logs = []
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        for out in ex.map(run, jobs):
            logs.append(out)
    if jobs or not os.path.exists(LIB) or _stale(LIB, objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
        logs.append(run(cmd))
    if verbose:
        print("\n".join(l for l in logs if l))
    return LIB


if __name__ == "__main__":
    build(verbose=True, ptxas_info="-v" in sys.argv)
