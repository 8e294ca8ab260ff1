"""Compiles the oracle's CPU restatement (oracle/muon_oracle.cc) into
oracle/lib/libmuon_oracle.so. Test infrastructure only."""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "muon_oracle.cc")
OUT = os.path.join(HERE, "lib", "libmuon_oracle.so")


def build() -> str:
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    if not os.path.exists(OUT) or os.path.getmtime(OUT) < os.path.getmtime(SRC):
        subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-pthread", SRC,
                        "-o", OUT], check=True)
    return OUT


if __name__ == "__main__":
    print(build())
