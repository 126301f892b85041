"""Build recipe of the oracle's C restatement (FP64 elastic FD forward/adjoint):
gcc on oracle/fwi_oracle.c into oracle/_lib/libfwi_oracle.so.  Test
infrastructure only."""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT_DIR, "libfwi_oracle.so")


def build(force=False):
    src = os.path.join(HERE, "fwi_oracle.c")
    os.makedirs(OUT_DIR, exist_ok=True)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(src):
        subprocess.run(["gcc", "-O2", "-std=c99", "-fPIC", "-shared", "-o", LIB, src, "-lm"], check=True)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
