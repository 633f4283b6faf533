"""Build recipe of the C oracle (oracle/csrc/*.c -> oracle/_build/liboracle.so, gcc, OpenMP).
TEST INFRASTRUCTURE ONLY: the oracle is the checker and the CPU baseline, never the product.
The reference (igmhub/SaclayMocks) is pure Python, so there is no reference C code to build
into oracle/_ref."""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")


def build(force: bool = False) -> str:
    srcs = sorted(os.path.join(HERE, "csrc", f) for f in os.listdir(os.path.join(HERE, "csrc"))
                  if f.endswith(".c"))
    os.makedirs(BUILD, exist_ok=True)
    newest = max(os.path.getmtime(s) for s in srcs)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    tmp = LIB + ".tmp"
    cmd = ["gcc", "-O3", "-fPIC", "-shared", "-fopenmp", "-o", tmp, *srcs, "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("gcc failed on the C oracle:\n" + r.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
