"""Compile libnsem_gpu.so (sm_103a) in-tree with nvcc.

Each translation unit is compiled in parallel, then linked into
nebulasem_gb300/_lib/libnsem_gpu.so.  The plain-form kernels and the host
side are built without floating-point contraction (--fmad=false,
-ffp-contract=off) so their arithmetic matches the reference's operation by
operation; the precision-form kernels may contract.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT, "libnsem_gpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
                 "-I" + CSRC, "-I" + os.path.join(ROOT, "include")]
EXACT = ["--fmad=false", "-Xcompiler", "-ffp-contract=off"]

UNITS = [
    ("nsem_api.cpp", EXACT),
    ("nsem_fp64.cu", EXACT),
    ("nsem_aux.cu", EXACT),
    ("nsem_mixed.cu", []),
    ("nsem_mixed_stage.cu", []),
    ("nsem_mixed_gen.cu", []),
    ("nsem_mixed_adj.cu", []),
    ("nsem_mixed_adj_gen.cu", []),
    ("nsem_noalloc.cu", EXACT),
    ("nsem_seg.cu", EXACT),
    ("nsem_adjoint.cu", []),
]


def nvcc():
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libnsem_gpu")
    return path


def _stale(obj, src):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    deps = [src] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    deps.append(os.path.join(ROOT, "include", "nsem.h"))
    deps.append(__file__)
    return any(os.path.getmtime(d) > t for d in deps)


DRIVER = os.path.join(HERE, "driver")
DRIVER_EXE = os.path.join(OUT, "nsem_euler")


def build_driver(verbose=False, force=False):
    """The host driver nsem_euler (C++17, links libnsem_gpu.so through the C ABI)."""
    srcs = sorted(os.path.join(DRIVER, f) for f in os.listdir(DRIVER) if f.endswith(".cpp"))
    deps = srcs + [os.path.join(DRIVER, f) for f in os.listdir(DRIVER) if f.endswith(".h")]
    deps += [LIB, os.path.join(ROOT, "include", "nsem.h"), __file__]
    if not force and os.path.exists(DRIVER_EXE):
        t = os.path.getmtime(DRIVER_EXE)
        if all(os.path.getmtime(d) <= t for d in deps):
            return DRIVER_EXE
    cxx = shutil.which("g++") or "g++"
    # no contraction: the mesh geometry follows the reference operation by operation
    cmd = [cxx, "-O2", "-std=c++17", "-Wall", "-ffp-contract=off",
           "-I" + os.path.join(ROOT, "include"), "-I" + DRIVER]
    cmd += srcs + ["-L" + OUT, "-lnsem_gpu", "-Wl,-rpath,$ORIGIN", "-o", DRIVER_EXE]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"g++ failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose and (r.stdout or r.stderr):
        print(r.stdout, r.stderr, file=sys.stderr)
    return DRIVER_EXE


def build(verbose=False, force=False):
    os.makedirs(OUT, exist_ok=True)
    cc = nvcc()
    jobs = []
    for name, extra in UNITS:
        src = os.path.join(CSRC, name)
        obj = os.path.join(OUT, name + ".o")
        if force or _stale(obj, src):
            lang = ["-x", "cu"] if name.endswith(".cu") else []
            jobs.append([cc] + COMMON + extra + lang + ["-c", src, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr, file=sys.stderr)

    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        list(ex.map(run, jobs))
    objs = [os.path.join(OUT, n + ".o") for n, _ in UNITS]
    if jobs or not os.path.exists(LIB):
        run([cc] + ARCH + ["-shared", "-o", LIB] + objs)
    build_driver(verbose, force)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
