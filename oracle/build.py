"""Build recipe of the C oracle (test infrastructure only).

``python oracle/build.py`` compiles ``oracle/abm_oracle.c`` with gcc into
``oracle/_build/liboracle.so``.  ``-ffp-contract=off`` keeps float32 multiplies and adds
separately rounded (gcc fuses them into FMAs on aarch64 by default).
"""

import ctypes
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRCS = sorted(os.path.join(HERE, f) for f in os.listdir(HERE) if f.endswith(".c"))
HDRS = sorted(os.path.join(HERE, f) for f in os.listdir(HERE) if f.endswith(".h"))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")
FLAGS = ["-O2", "-std=gnu11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
         "-fno-fast-math"]


def build(force=False):
    newest = max(os.path.getmtime(p) for p in SRCS + HDRS + [__file__])
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = LIB + ".tmp"
    cmd = ["gcc"] + FLAGS + SRCS + ["-o", tmp, "-lm"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + res.stderr)
    os.replace(tmp, LIB)
    return LIB


_lib = None


def load():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
    return _lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
