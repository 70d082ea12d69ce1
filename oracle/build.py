"""Build recipe for the CPU oracle (test infrastructure only).

Compiles ``vd_oracle.cpp`` into ``oracle/_build/libvd_oracle.so`` with the
host compiler.  ``-ffp-contract=off`` keeps every floating-point operation
individually rounded, which the bit-exact restatement of the reference's
bounding sphere and super simplex relies on (Rust never fuses operations).
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libvd_oracle.so")
SRC = os.path.join(HERE, "vd_oracle.cpp")


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off",
           "-fno-fast-math", "-o", tmp, SRC]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
