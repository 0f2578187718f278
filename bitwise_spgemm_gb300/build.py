"""Build the CUDA library ``libbsp.so`` (sm_103a) in-tree.

Every ``csrc/*.cu`` is compiled by nvcc in parallel into ``_build/`` and
linked into ``bitwise_spgemm_gb300/libbsp.so`` (CUDA runtime linked
statically), then the C++ harness ``harness/bsp_harness`` is linked against
it, and cuSPARSE's CSR SpMM (the reference's library baseline, timing only)
is built into its own ``libbsp_cusparse.so``.  No cmake, one ``-gencode``; rebuilds only changed sources.
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OBJ = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libbsp.so")
INCLUDE = os.path.join(ROOT, "include")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
              "--expt-relaxed-constexpr", "-I", INCLUDE, "-I", CSRC]


def nvcc():
    exe = shutil.which("nvcc")
    if exe is None and os.path.exists("/usr/local/cuda/bin/nvcc"):
        exe = "/usr/local/cuda/bin/nvcc"
    if exe is None:
        raise RuntimeError("nvcc not found: the bitmap-SpMM library needs the CUDA toolkit")
    return exe


def _deps():
    return (glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h"))
            + glob.glob(os.path.join(INCLUDE, "*.h")))


def _compile(src, force):
    obj = os.path.join(OBJ, os.path.basename(src)[:-3] + ".o")
    newest = max([os.path.getmtime(src)] + [os.path.getmtime(d) for d in _deps()])
    if not force and os.path.exists(obj) and os.path.getmtime(obj) >= newest:
        return obj
    tmp = obj + ".tmp%d" % os.getpid()
    subprocess.check_call([nvcc()] + ARCH + NVCC_FLAGS + ["-c", src, "-o", tmp])
    os.replace(tmp, obj)
    return obj


HARNESS_SRC = os.path.join(PKG, "harness", "bsp_harness.cpp")
HARNESS = os.path.join(PKG, "harness", "bsp_harness")


def build_harness(force=False):
    """The C++ harness (replaces the reference's main(); C ABI only),
    linked against the in-tree libbsp.so through an $ORIGIN rpath."""
    newest = max(os.path.getmtime(p) for p in [HARNESS_SRC, LIB] + glob.glob(os.path.join(INCLUDE, "*.h")))
    if not force and os.path.exists(HARNESS) and os.path.getmtime(HARNESS) >= newest:
        return HARNESS
    tmp = HARNESS + ".tmp%d" % os.getpid()
    subprocess.check_call([nvcc(), "-O2", "-std=c++17", "-I", INCLUDE, HARNESS_SRC, "-o", tmp, "-L", PKG, "-lbsp",
                           "-Xlinker", "-rpath,$ORIGIN/.."])
    os.replace(tmp, HARNESS)
    return HARNESS


E2E_SRC = os.path.join(PKG, "harness", "bsp_e2e.cpp")
E2E = os.path.join(PKG, "harness", "bsp_e2e")


def build_e2e(force=False):
    """The C++ end-to-end serving loop (C ABI only), linked like the harness."""
    newest = max(os.path.getmtime(p) for p in [E2E_SRC, LIB] + glob.glob(os.path.join(INCLUDE, "*.h")))
    if not force and os.path.exists(E2E) and os.path.getmtime(E2E) >= newest:
        return E2E
    tmp = E2E + ".tmp%d" % os.getpid()
    subprocess.check_call([nvcc(), "-O2", "-std=c++17", "-I", INCLUDE, E2E_SRC, "-o", tmp, "-L", PKG, "-lbsp",
                           "-Xlinker", "-rpath,$ORIGIN/.."])
    os.replace(tmp, E2E)
    return E2E


CUSPARSE_SRC = os.path.join(PKG, "baselines", "cusparse_spmm.cpp")
CUSPARSE_LIB = os.path.join(PKG, "libbsp_cusparse.so")


def build_cusparse_baseline(force=False):
    """cuSPARSE's CSR SpMM, the reference's library baseline (timing and
    cross-checks only), as its own libbsp_cusparse.so next to libbsp.so.
    Returns None, with the reason printed, when the toolkit cannot link it:
    the bitmap library does not depend on it."""
    newest = max(os.path.getmtime(p) for p in [CUSPARSE_SRC] + glob.glob(os.path.join(INCLUDE, "*.h")))
    if not force and os.path.exists(CUSPARSE_LIB) and os.path.getmtime(CUSPARSE_LIB) >= newest:
        return CUSPARSE_LIB
    libdir = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc()))), "lib64")
    tmp = CUSPARSE_LIB + ".tmp%d" % os.getpid()
    try:
        subprocess.check_call([nvcc(), "-O2", "-std=c++17", "-shared", "-Xcompiler", "-fPIC", "-I", INCLUDE,
                               CUSPARSE_SRC, "-o", tmp, "-lcusparse", "-Xlinker", "-rpath," + libdir])
    except (subprocess.CalledProcessError, OSError) as exc:
        print("cuSPARSE baseline not built: %s" % exc)
        return None
    os.replace(tmp, CUSPARSE_LIB)
    return CUSPARSE_LIB


def build(force=False, jobs=None):
    os.makedirs(OBJ, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    jobs = jobs or min(len(srcs), max(1, os.cpu_count() or 1))
    with cf.ThreadPoolExecutor(jobs) as ex:
        objs = list(ex.map(lambda s: _compile(s, force), srcs))
    if (force or not os.path.exists(LIB)
            or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs)):
        tmp = LIB + ".tmp%d" % os.getpid()
        subprocess.check_call([nvcc()] + ARCH + ["-shared", "-o", tmp] + objs)
        os.replace(tmp, LIB)
    build_harness(force)
    build_e2e(force)
    build_cusparse_baseline(force)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
