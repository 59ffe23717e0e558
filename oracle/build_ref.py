"""Build the oracle's compiled checker (TEST INFRASTRUCTURE ONLY).

    python oracle/build_ref.py

Compiles ``oracle/sv_ref.cpp`` (the complex128 CPU state-vector simulator
with the adjoint gradient) with g++ into ``oracle/_build/libsv_ref.so``.  The
reference itself is pure Python, so nothing of it is compiled here.  Plain
portable flags (x86-64 and aarch64 hosts alike).
"""

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libsv_ref.so")


def build():
    os.makedirs(OUT_DIR, exist_ok=True)
    src = os.path.join(HERE, "sv_ref.cpp")
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(src):
        return LIB
    tmp = LIB + ".tmp"
    cmd = ["g++", "-O3", "-std=c++17", "-shared", "-fPIC", "-pthread", "-Wall", src, "-o", tmp]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build())
    sys.exit(0)
