"""Builds the oracle loops (oracle/oracle.cpp) into oracle/_build/liboracle.so.

Test infrastructure only. Plain g++ at -O3, tuned for the host it is built on
(-march=native on x86_64, -mcpu=native on aarch64), since the timed CPU
baseline runs it; integer arithmetic gives the same results either way.
"""

import os
import platform
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
    arch = ["-mcpu=native"] if platform.machine() in ("aarch64", "arm64") else ["-march=native"]
    subprocess.check_call(["g++", "-O3"] + arch + ["-std=c++17", "-shared", "-fPIC", "-pthread", "-o", tmp, SRC])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
