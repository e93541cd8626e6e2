"""Build recipe of the CPU oracle (test infrastructure only).

Compiles oracle/sdnn_oracle.c into oracle/_build/libsdnn_oracle.so with gcc.
`-ffp-contract=off` keeps a*b + c as two roundings on every host (x86 and
Arm), so the FP32 port gives the same bits on both machines.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libsdnn_oracle.so")


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "sdnn_oracle.c")
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(src):
        return LIB
    tmp = LIB + ".tmp"
    cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-pthread", "-ffp-contract=off",
           src, "-o", tmp, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
