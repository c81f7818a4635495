"""Build libcpmgpu.so (the C-ABI + sm_103a kernels) in-tree with nvcc.

Each translation unit compiles in parallel; the setup units (tube, opset) are
built with -fmad=false so grid coordinates, base points and tricubic weights
round exactly like the reference's host code.  Host code is compiled with
-ffp-contract=off for the same reason on Arm hosts.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libcpmgpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off", "--expt-relaxed-constexpr"]
UNITS = {
    "capi.cu": [],
    "tube.cu": ["-fmad=false"],
    "opset.cu": ["-fmad=false"],
    "solver.cu": [],
    "geodesic.cu": [],
}


def nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _deps_newer(obj, src):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    if os.path.getmtime(src) > t or os.path.getmtime(__file__) > t:
        return True
    for h in os.listdir(CSRC):
        if h.endswith((".h", ".cuh")) and os.path.getmtime(os.path.join(CSRC, h)) > t:
            return True
    hdr = os.path.join(HERE, "..", "include", "cpm_gpu.h")
    return os.path.getmtime(hdr) > t


def build(verbose=False, extra=()):
    os.makedirs(BUILD, exist_ok=True)
    nv = nvcc()
    jobs = []
    for unit, flags in UNITS.items():
        src = os.path.join(CSRC, unit)
        obj = os.path.join(BUILD, unit.replace(".cu", ".o"))
        if _deps_newer(obj, src):
            jobs.append([nv, *ARCH, *COMMON, *flags, *extra, "-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        for cmd, res in zip(jobs, ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs)):
            if res.returncode != 0:
                sys.stderr.write(res.stdout + res.stderr)
                raise RuntimeError("nvcc failed: " + " ".join(cmd))
            if verbose and (res.stdout or res.stderr):
                sys.stderr.write(res.stdout + res.stderr)
    objs = [os.path.join(BUILD, u.replace(".cu", ".o")) for u in UNITS]
    if not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [nv, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            sys.stderr.write(res.stdout + res.stderr)
            raise RuntimeError("link failed")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, extra=["-Xptxas", "-v"] if "--ptxas" in sys.argv else []))
