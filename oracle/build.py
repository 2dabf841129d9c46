"""Build recipe for the CPU oracle (test infrastructure).

Compiles oracle/stafft.c and oracle/ps3d_oracle.c into
oracle/_build/libps3d_oracle.so with gcc/OpenMP.  FP contraction is disabled
so the oracle gives the same FP64 results on x86-64 and aarch64 hosts.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libps3d_oracle.so")
SOURCES = ["stafft.c", "ps3d_oracle.c"]


def build(force: bool = False) -> str:
    srcs = [os.path.join(HERE, s) for s in SOURCES] + [os.path.join(HERE, "ps3d_oracle.h")]
    if not force and os.path.exists(LIB):
        lib_t = os.path.getmtime(LIB)
        if all(os.path.getmtime(s) <= lib_t for s in srcs):
            return LIB
    os.makedirs(BUILD, exist_ok=True)
    cmd = ["gcc", "-O2", "-std=c11", "-fopenmp", "-fPIC", "-ffp-contract=off",
           "-Wall", "-Wextra", "-shared", "-o", LIB + ".tmp"]
    cmd += [os.path.join(HERE, s) for s in SOURCES] + ["-lm"]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
