"""Build recipe for the oracle restatement (``oracle/od_oracle.cpp``).

Produces ``oracle/_build/libodoracle.so`` (test infrastructure only).
``-ffp-contract=off`` keeps x86-64 and aarch64 builds bit-identical.
"""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libodoracle.so")


def build() -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    src = os.path.join(HERE, "od_oracle.cpp")
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off",
                           "-Wall", "-Wno-unused-function", src, "-o", LIB])
    return LIB


if __name__ == "__main__":
    print(build())
