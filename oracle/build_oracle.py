"""Build recipe for the CPU oracle (test infrastructure, see sw_oracle.cpp).

    python oracle/build_oracle.py          # -> oracle/_build/libsw_oracle.so

-ffp-contract=off keeps every float expression in source order on both x86-64
and aarch64 (gcc contracts a*b+c into FMA by default on aarch64), so the
oracle's float32 fields are identical across the two machines and match the
golden fixtures bit for bit.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libsw_oracle.so")
SRC = os.path.join(HERE, "sw_oracle.cpp")


def build(force=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-fno-fast-math", SRC, "-o", LIB + ".tmp"]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
