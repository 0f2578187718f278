"""Recipe that builds the reference's own code for this path into oracle/_ref/.

TEST INFRASTRUCTURE ONLY.  Reads the reference checkout named by
BSP_REFERENCE_DIR or, without it, by "reference_path" in the repository's
the benchmark spec; writes only into oracle/_ref/ (git-ignored).  Nothing is
copied into the repository.

Two artefacts:

* ``libref_check.so`` — backup/bit_wise_gemm.cu compiled as-is by nvcc
  (its ``main`` renamed so the file links as a library).  Exports the
  reference's CPU path ``check()`` (bit_wise_gemm.cu:13-32), a C++ symbol.
* ``libref_emu.so`` — the reference kernels listed in ref_emu.cpp and
  ref_emu_out.cpp, extracted by line range from source/src/main.cu,
  source/src/transform.cuh and backup/layout_trans.cu into oracle/_ref/*.inc
  and compiled for the host against ref_shim.h, which emulates
  threadIdx/__syncthreads/atomics with serialised fibers; and the Thrust
  pipeline of ref_emu_tiles.cpp (source/src/main.cu, source/src/mm.h),
  compiled against the CUDA toolkit's Thrust on its sequential back end.

The reference's main.cu as a whole does not compile here (it needs
cusparseLt and a CUDA-13-incompatible cusp), so whole-program builds are not
attempted.  Returns the list of built files; missing reference = nothing.
"""
import json
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")


def _reference_dir():
    env = os.environ.get("BSP_REFERENCE_DIR")
    if env:
        return env
    try:
        with open(os.path.join(os.path.dirname(HERE), "BASELINE.json")) as f:
            return json.load(f).get("reference_path", "")
    except (OSError, ValueError):
        return ""


REF = _reference_dir()

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
    ("ref_csr2tiledcsr.inc", "source/src/main.cu", 499, 588,
     "template <typename InitValueType", "}"),
    ("ref_pre_spgemm.inc", "source/src/transform.cuh", 984, 1157,
     "template <typename BitMaskType>", "}"),
    ("ref_coo2bmp.inc", "source/src/main.cu", 692, 779,
     "template <typename ValueType>", "}"),
    ("ref_find_tile_index.inc", "source/src/mm.h", 83, 104,
     "struct find_tile_index", "};"),
    ("ref_absolute2relative.inc", "source/src/mm.h", 106, 121,
     "struct absolute2relative", "};"),
    ("ref_bmp_popcount_d.inc", "source/src/mm.h", 134, 144,
     "struct bmp_popcount_d", "};"),
]
SOURCES = ["ref_emu.cpp", "ref_emu_out.cpp", "ref_emu_tiles.cpp"]


def _cuda_include():
    nvcc = shutil.which("nvcc")
    base = os.path.dirname(os.path.dirname(nvcc)) if nvcc else "/usr/local/cuda"
    return [os.path.join(base, "include"), os.path.join(base, "include", "cccl")]


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
    return bool(REF) and os.path.isdir(os.path.join(REF, "source", "src"))


def build(force=False, quiet=True):
    if not available():
        return []
    os.makedirs(OUT, exist_ok=True)
    built = []
    emu = os.path.join(OUT, "libref_emu.so")
    if force or not os.path.exists(emu):
        for e in EXTRACTS:
            _extract(*e)
        inc = []
        for d in _cuda_include():
            inc += ["-I", d]
        cmd = (["g++", "-O0", "-g0", "-w", "-fPIC", "-shared", "-std=c++17",
                "-I", OUT, "-I", HERE] + inc + ["-o", emu]
               + [os.path.join(HERE, s) for s in SOURCES])
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
