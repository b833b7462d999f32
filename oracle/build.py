"""ORACLE build recipe -- test infrastructure only.

Compiles the CPU restatement (oracle_core.hpp, oracle_pt.hpp, oracle_api.cpp) into
oracle/liboracle.so.  Strict IEEE single precision (no contraction into FMAs, no fast-math) so
that the FP32 instantiation follows the reference's scalar arithmetic.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
SOURCES = ["oracle_api.cpp"]
HEADERS = ["oracle_core.hpp", "oracle_pt.hpp"]


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(os.path.join(HERE, f)) > t for f in SOURCES + HEADERS + ["build.py"])


def build_oracle(force=False, verbose=False):
    if not force and not _stale():
        return LIB
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-pthread", "-ffp-contract=off", "-fno-fast-math",
           "-o", LIB + ".tmp"] + [os.path.join(HERE, s) for s in SOURCES]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    build_oracle(force="--force" in sys.argv, verbose=True)
