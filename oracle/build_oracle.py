"""Build recipe of the CPU oracle (test infrastructure only).

Compiles oracle/*.cpp into oracle/build/liboracle.so with g++ -O2 -fopenmp
-ffp-contract=off (no fused multiply-add, matching the GPU parity build).
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "build")
LIB = os.path.join(OUT_DIR, "liboracle.so")
SOURCES = ["oracle_mg.cpp", "oracle_transport.cpp"]


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    srcs = [os.path.join(HERE, s) for s in SOURCES if os.path.exists(os.path.join(HERE, s))]
    deps = srcs + [os.path.join(HERE, "oracle_common.h"),
                   os.path.join(HERE, "..", "include", "afivo_gpu.h"),
                   os.path.join(HERE, "..", "afivo-streamer_gb300", "csrc", "afg_math.h"),
                   os.path.join(HERE, "..", "afivo-streamer_gb300", "csrc", "afg_lsf.h")]
    if not force and os.path.exists(LIB):
        t = os.path.getmtime(LIB)
        if all(os.path.getmtime(d) <= t for d in deps if os.path.exists(d)):
            return LIB
    cmd = ["g++", "-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC",
           "-shared", "-o", LIB] + srcs
    subprocess.run(cmd, check=True)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
