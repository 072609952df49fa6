"""Builds libgraspsynth.so (host C++) in-tree into inputs/_build/."""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build")
SOURCES = [os.path.join(HERE, "csrc", "synth.cpp")]
HEADER = os.path.join(HERE, "grasp_synth.h")
LIB_SYNTH = os.path.join(OUT, "libgraspsynth.so")


def build(force: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    deps = SOURCES + [HEADER]
    if force or not os.path.exists(LIB_SYNTH) or any(os.path.getmtime(d) > os.path.getmtime(LIB_SYNTH)
                                                      for d in deps):
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-I" + HERE, "-o", LIB_SYNTH] + SOURCES + ["-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return LIB_SYNTH


if __name__ == "__main__":
    print(build(force=True))
