"""Build recipe for the FP64 CPU oracle (TEST INFRASTRUCTURE ONLY).

Compiles ``oracle.cpp`` into ``oracle/liboracle.so`` with strict IEEE double
semantics (``-ffp-contract=off``: JS numbers never fuse a multiply-add, and
aarch64 GCC would otherwise emit ``fmadd``).  The GPU library never links it.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
SRC = [os.path.join(HERE, f) for f in ("oracle.cpp", "oracle_collide.h", "oracle_math.h", "oracle_joints.h",
                                              "oracle_joint_types.h", "oracle_frozen.h")]


def build(force: bool = False) -> str:
    if not force and os.path.exists(LIB):
        t = os.path.getmtime(LIB)
        if all(os.path.getmtime(p) < t for p in SRC + [__file__]):
            return LIB
    cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
           "-o", LIB, os.path.join(HERE, "oracle.cpp")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
