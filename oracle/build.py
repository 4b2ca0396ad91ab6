"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle_capi.cpp into oracle/_build/liboracle.so with g++.  FP contraction
is disabled so that the restated algorithms round like the reference's Julia code
(which does not fuse multiply-adds unless asked to).
"""
import glob
import os
import platform
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")
SOURCES = ["oracle_capi.cpp"]
HEADERS = sorted(os.path.basename(h) for h in glob.glob(os.path.join(HERE, "*.hpp")))


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    for f in SOURCES + HEADERS + ["build.py"]:
        if os.path.getmtime(os.path.join(HERE, f)) > t:
            return True
    return False


def build(force=False):
    """Compile the oracle shared library if it is missing or stale; return its path."""
    if not force and not _stale():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    cmd = ["g++", "-O2", "-std=gnu++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-o", LIB + ".tmp"] + [os.path.join(HERE, s) for s in SOURCES]
    if platform.machine() in ("x86_64", "AMD64", "i686"):
        cmd.append("-lquadmath")
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
