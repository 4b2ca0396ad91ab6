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


MP_LIB = os.path.join(OUT_DIR, "liboracle_mpfr.so")
MP_SOURCES = ["oracle_mpfr.cpp"]
MP_HEADERS = ["scalar.hpp", "mp256.hpp", "gschur_oracle.hpp"]


def build_mpfr(force=False):
    """The 256-bit (BigFloat-precision) instance of the Schur restatement, linked against
    libmpfr.so.6.  Optional: it only generates the committed high-precision fixtures, so a
    machine without MPFR skips it.  Returns the library path or None."""
    if not force and os.path.exists(MP_LIB) and all(
            os.path.getmtime(os.path.join(HERE, f)) <= os.path.getmtime(MP_LIB)
            for f in MP_SOURCES + MP_HEADERS + ["build.py"]):
        return MP_LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    cmd = ["g++", "-O2", "-std=gnu++17", "-fPIC", "-shared", "-ffp-contract=off", "-o", MP_LIB + ".tmp"] + \
        [os.path.join(HERE, s) for s in MP_SOURCES] + ["-l:libmpfr.so.6"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return None
    os.replace(MP_LIB + ".tmp", MP_LIB)
    return MP_LIB


def build(force=False):
    """Compile the oracle shared library if it is missing or stale; return its path."""
    build_mpfr(force)
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
