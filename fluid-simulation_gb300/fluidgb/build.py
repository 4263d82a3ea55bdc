"""Build libfluidgb.so in-tree from csrc/ with nvcc for sm_103a.

Each translation unit is compiled in parallel, then linked into one shared
library with the CUDA runtime linked statically, so the C ABI has no
dependency beyond the driver.  Output: fluidgb/_lib/libfluidgb.so
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG_DIR)               # fluid-simulation_gb300/
REPO = os.path.dirname(ROOT)
CSRC = os.path.join(ROOT, "csrc")
INCLUDE = os.path.join(REPO, "include")
OUT_DIR = os.path.join(PKG_DIR, "_lib")
OBJ_DIR = os.path.join(OUT_DIR, "obj")
LIB_NAME = "libfluidgb.so"
LIB_PATH = os.path.join(OUT_DIR, LIB_NAME)

SOURCES = ["fl_bin.cu", "fl_grid.cu", "fl_cg.cu", "fl_g2p.cu", "fl_adjoint.cu", "fl_host.cpp", "fl_noalloc.cu",
           "fl_timestep.cpp", "fl_slice.cu", "fl_scene.cu", "fl_mg.cu", "fl_relax.cu"]
HEADERS = ["fl_device.cuh"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# --fmad=false: no a*b+c contraction anywhere in device code; the parity-critical
# arithmetic is also written with explicit _rn intrinsics.  The host side is
# compiled -ffp-contract=off for the same reason (aarch64 GCC contracts by default).
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--fmad=false", "-Xcompiler", "-fPIC,-ffp-contract=off",
              "-I" + INCLUDE, "-I" + CSRC]


def nvcc():
    exe = shutil.which("nvcc")
    if exe:
        return exe
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found; the CUDA toolkit is required to build libfluidgb")


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src, verbose):
    obj = os.path.join(OBJ_DIR, os.path.basename(src) + ".o")
    deps = [src] + [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(INCLUDE, "fluidgb.h"), __file__]
    if not _stale(obj, deps):
        return obj, ""
    cmd = [nvcc()] + ARCH + NVCC_FLAGS + ["-c", src, "-o", obj + ".tmp"]
    if verbose:
        cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
    os.replace(obj + ".tmp", obj)
    return obj, r.stderr


def build(force=False, verbose=False):
    os.makedirs(OBJ_DIR, exist_ok=True)
    srcs = [os.path.join(CSRC, s) for s in SOURCES]
    if force:
        for s in srcs:
            o = os.path.join(OBJ_DIR, os.path.basename(s) + ".o")
            if os.path.exists(o):
                os.remove(o)
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose), srcs))
    objs = [o for o, _ in results]
    if verbose:
        for _, log in results:
            if log:
                sys.stderr.write(log)
    if _stale(LIB_PATH, objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-cudart", "static", "-o", LIB_PATH + ".tmp"] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
        os.replace(LIB_PATH + ".tmp", LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
