"""Recipe that builds the reference's own code for this path into oracle/_ref/.

TEST INFRASTRUCTURE ONLY.  Reads the reference checkout (default
/root/reference, override with BSP_REFERENCE_DIR); writes only into
oracle/_ref/ (git-ignored).  Nothing is copied into the repository.

Two artefacts:

* ``libref_check.so`` — backup/bit_wise_gemm.cu compiled as-is by nvcc
  (its ``main`` renamed so the file links as a library).  Exports the
  reference's CPU path ``check()`` (bit_wise_gemm.cu:13-32), a C++ symbol.
* ``libref_emu.so`` — the reference kernels listed in ref_emu.cpp, extracted
  by line range from source/src/main.cu and backup/layout_trans.cu into
  oracle/_ref/*.inc and compiled for the host against ref_shim.h, which
  emulates threadIdx/__syncthreads/atomics with serialised fibers.

The reference's main.cu as a whole does not compile here (it needs
cusparseLt and a CUDA-13-incompatible cusp), so whole-program builds are not
attempted.  Returns the list of built files; missing reference = nothing.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
REF = os.environ.get("BSP_REFERENCE_DIR", "/root/reference")

# (output .inc, reference file, first line, last line, text expected on first/last line)
EXTRACTS = [
    ("ref_generate_groups_large.inc", "source/src/main.cu", 50, 247,
     "template <typename BitMaskType", "}"),
    ("ref_dense2bitmask.inc", "source/src/main.cu", 591, 628,
     "template <typename BitMaskType", "}"),
    ("ref_group2dense.inc", "source/src/main.cu", 829, 850,
     "template <typename OutputType", "}"),
    ("ref_layout_trans.inc", "backup/layout_trans.cu", 75, 97,
     "__global__ void layout_trans", "}"),
    ("ref_uint8_spmm.inc", "backup/layout_trans.cu", 158, 171,
     "__global__ void uint8_spmm_2d_1d", "}"),
]


def _extract(name, rel, a, b, first, last):
    with open(os.path.join(REF, rel), "r", encoding="utf-8", errors="replace") as f:
        lines = f.read().split("\n")
    chunk = lines[a - 1:b]
    if not chunk[0].startswith(first) or chunk[-1].strip() != last:
        raise RuntimeError("reference %s:%d-%d does not hold the expected function" % (rel, a, b))
    with open(os.path.join(OUT, name), "w") as f:
        f.write("#line %d \"%s\"\n" % (a, rel))
        f.write("\n".join(chunk) + "\n")


def available():
    return os.path.isdir(os.path.join(REF, "source", "src"))


def build(force=False, quiet=True):
    if not available():
        return []
    os.makedirs(OUT, exist_ok=True)
    built = []
    emu = os.path.join(OUT, "libref_emu.so")
    if force or not os.path.exists(emu):
        for e in EXTRACTS:
            _extract(*e)
        cmd = ["g++", "-O0", "-g0", "-w", "-fPIC", "-shared", "-std=c++17",
               "-I", OUT, "-I", HERE, "-o", emu, os.path.join(HERE, "ref_emu.cpp")]
        subprocess.check_call(cmd)
    built.append(emu)
    chk = os.path.join(OUT, "libref_check.so")
    if force or not os.path.exists(chk):
        cmd = ["nvcc", "-shared", "-Xcompiler", "-fPIC", "-w", "-Dmain=bsp_ref_unused_main",
               "-o", chk, os.path.join(REF, "backup", "bit_wise_gemm.cu")]
        try:
            subprocess.check_call(cmd, stdout=subprocess.DEVNULL if quiet else None)
        except (OSError, subprocess.CalledProcessError) as exc:  # nvcc absent or failed
            print("oracle/_ref: libref_check.so not built: %s" % exc, file=sys.stderr)
            return built
    built.append(chk)
    return built


if __name__ == "__main__":
    print("\n".join(build(force=True, quiet=False)))
