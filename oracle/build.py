"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle/oracle.cpp into oracle/liborc.so with OpenMP and with FMA
contraction disabled, so that the f64 histogram rule and the float32 volume
generators evaluate in exactly the written order on x86-64 and AArch64 alike.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liborc.so")


def build(force=False):
    src = os.path.join(HERE, "oracle.cpp")
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(src):
        return LIB
    cmd = ["g++", "-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
           src, "-o", LIB + ".tmp"]
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
