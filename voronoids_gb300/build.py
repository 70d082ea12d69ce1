"""Build the CUDA library ``libvoronoids_gpu.so`` in-tree for sm_103a.

Each ``csrc/*.cu`` file is compiled by nvcc in parallel, then linked into
``voronoids_gb300/libvoronoids_gpu.so``.  Host code is compiled with
``-ffp-contract=off`` so the restated reference arithmetic (bounding sphere,
super simplex) rounds exactly as the reference does.

A host-only build of the predicate header (``libvd_pred_host.so``, plain g++)
is produced as well; the CPU test suite uses it to check the exact predicate
tiers without a GPU.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libvoronoids_gpu.so")
HOSTLIB = os.path.join(HERE, "libvd_pred_host.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["vd_build.cu", "vd_edges.cu", "vd_check.cu", "vd_size.cu", "vd_locate.cu", "vd_noalloc.cu", "vd_capi.cu",
           "vd_server.cu", "vd_dual.cu"]
HEADERS = ["vd_common.cuh", "vd_predicates.cuh"]


def _nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def nvcc_flags(extra=()):
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                   "--expt-relaxed-constexpr", "-I", os.path.join(HERE, "..", "include")] + list(extra)


def build(force=False, verbose=False, ptxas_info=False):
    """Compile and link the device library; returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [
        os.path.join(HERE, "..", "include", "voronoids_gpu.h")]
    objs = []
    jobs = []
    for s in SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, s.replace(".cu", ".o"))
        objs.append(obj)
        if force or _stale(obj, [src] + hdrs):
            extra = ["-Xptxas", "-v"] if ptxas_info else []
            jobs.append([nvcc] + nvcc_flags(extra) + ["-c", src, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for cmd, r in ex.map(run, jobs):
                if verbose or ptxas_info:
                    sys.stderr.write(r.stderr)
                if r.returncode != 0:
                    sys.stderr.write(r.stdout + r.stderr)
                    raise RuntimeError("nvcc failed: " + " ".join(cmd))
    if force or jobs or _stale(LIB, objs):
        tmp = LIB + f".tmp{os.getpid()}"
        cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link failed")
        os.replace(tmp, LIB)
    return LIB


def build_host(force=False):
    """Host-only build of the predicate tiers (for CPU tests)."""
    src = os.path.join(CSRC, "vd_pred_host.cpp")
    deps = [src, os.path.join(CSRC, "vd_predicates.cuh")]
    if force or _stale(HOSTLIB, deps):
        tmp = HOSTLIB + f".tmp{os.getpid()}"
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-o", tmp, src]
        subprocess.run(cmd, check=True)
        os.replace(tmp, HOSTLIB)
    return HOSTLIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True, ptxas_info="--ptxas" in sys.argv))
    print(build_host(force="--force" in sys.argv))
