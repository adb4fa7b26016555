"""Build recipe for the oracle (test infrastructure only).

Compiles the f64 C++ restatement of the reference's lifting-line path into
oracle/_build/libsb_oracle.so. Flags: -O3 for the timed CPU baseline, OpenMP for the
per-target parallel loop the reference runs with rayon, and -ffp-contract=off so the
compiler fuses no multiply-add (the Rust reference does not either).
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libsb_oracle.so")
SOURCES = [os.path.join(HERE, "sb_oracle_capi.cpp")]
DEPS = SOURCES + [
    os.path.join(HERE, "sb_oracle.hpp"),
    os.path.join(HERE, "sb_oracle_wind.hpp"),
    os.path.join(HERE, "sb_oracle_controller.hpp"),
    os.path.join(HERE, "..", "stormbird_gb300", "csrc", "sb_controller_setup.hpp"),
    os.path.join(HERE, "..", "stormbird_gb300", "csrc", "sb_wind_setup.hpp"),
    os.path.join(HERE, "..", "stormbird_gb300", "csrc", "sb_setup.hpp"),
    os.path.join(HERE, "..", "stormbird_gb300", "csrc", "json_min.hpp"),
    os.path.join(HERE, "..", "include", "stormbird_gb300.h"),
]


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(d) > t for d in DEPS)


def build(force: bool = False, verbose: bool = False) -> str:
    """Builds the oracle library if missing or out of date; returns its path."""
    if not force and not _stale():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = ["g++", "-std=c++17", "-O3", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared",
           "-Wall", "-Wextra", "-Wno-unused-parameter", "-o", tmp] + SOURCES
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
