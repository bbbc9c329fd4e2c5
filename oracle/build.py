"""Builds the oracle loops (oracle/oracle.cpp) into oracle/_build/liboracle.so.

Test infrastructure only. Plain g++, no architecture-specific flags, so the
same recipe works on x86_64 and aarch64 hosts.
"""

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")
SRC = os.path.join(HERE, "oracle.cpp")


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    tmp = LIB + f".tmp{os.getpid()}"
    subprocess.check_call(["g++", "-O3", "-std=c++17", "-shared", "-fPIC", "-o", tmp, SRC])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
