"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle/ms_oracle.c into oracle/_build/libtsoracle.so with gcc.
Float contraction is off so that every multiply and add rounds separately,
as the restated Rust code does.

The reference itself (Rust) cannot be compiled on this machine: there is no
Rust toolchain and none of its crates; oracle/_ref/ therefore stays empty.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libtsoracle.so")
SRC = os.path.join(HERE, "ms_oracle.c")
HDR = os.path.join(os.path.dirname(HERE), "include", "tsgpu.h")  # TS_MAX_SAMPLE_DRAWS

CFLAGS = ["-O2", "-std=gnu11", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math", "-pthread"]


def build(force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    newest = max(os.path.getmtime(SRC), os.path.getmtime(HDR))
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["gcc", *CFLAGS, "-o", tmp, SRC, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
