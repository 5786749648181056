"""Build recipe for the FP64 oracle (test infrastructure only).

Compiles oracle/tp_oracle.c into oracle/_build/libtp_oracle.so.  The flags
pin the arithmetic: -ffp-contract=off keeps gcc from fusing a*b+c on
aarch64/x86_64 so the oracle returns the same doubles on x86 and Arm.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libtp_oracle.so")
SRC = os.path.join(HERE, "tp_oracle.c")
HDR = os.path.join(HERE, "tp_oracle.h")


def build(force=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(SRC), os.path.getmtime(HDR))):
        return LIB
    tmp = LIB + ".tmp.%d" % os.getpid()
    cmd = ["gcc", "-O2", "-std=gnu11", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
           "-pthread", "-Wall", "-o", tmp, SRC, "-lm"]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
