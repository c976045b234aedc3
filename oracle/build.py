"""Build recipe for the oracle's C restatement (test infrastructure only).

Compiles ``oracle/scalit_oracle.c`` into ``oracle/_build/liborc.so`` with gcc,
OpenMP and no host-specific flags, so the same source builds on x86-64 and
aarch64 hosts.
"""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "scalit_oracle.c")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liborc.so")


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= os.path.getmtime(SRC)):
        return LIB
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = ["gcc", "-O3", "-fopenmp", "-fPIC", "-shared", "-fno-fast-math",
           "-ffp-contract=off", "-Wall", "-o", tmp, SRC, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
