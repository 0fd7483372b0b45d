"""Build recipe for the C oracle (test infrastructure only).

Compiles ``oracle/dto_oracle.c`` into ``oracle/_build/liboracle_dto.so`` with
``-ffp-contract=off`` so that every fused multiply-add in the FP64 tail
specification is an explicit ``fma()`` call, on x86-64 and on aarch64 alike.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle_dto.so")
SRC = os.path.join(HERE, "dto_oracle.c")


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O2", "-std=c11", "-ffp-contract=off", "-fno-fast-math", "-fPIC",
           "-shared", "-pthread", "-fvisibility=hidden", SRC, "-o", tmp, "-lm"]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
