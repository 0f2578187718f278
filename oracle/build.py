"""Build the C oracle (``bsp_oracle.c``) into ``oracle/_build/liboracle.so``.

Test infrastructure: the library never links this.  Plain gcc, no
architecture flags, so the same source builds on x86-64 and Arm hosts.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "bsp_oracle.c")
    hdr = os.path.join(HERE, "bsp_oracle.h")
    os.makedirs(OUT_DIR, exist_ok=True)
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(src), os.path.getmtime(hdr))):
        return LIB
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O3", "-std=c99", "-fPIC", "-shared", "-Wall", "-Wextra",
           "-fno-fast-math", "-ffp-contract=off", "-o", tmp, src, "-lpthread", "-lm"]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
