"""Builds the CPU oracle (oracle/pamo_oracle.cpp: stage 2, oracle/stage3_oracle.cpp: stage 3,
oracle/mesh_check.cpp: exact self-intersection check and Hausdorff distance, oracle/cpu_qem.cpp: the sequential
QEM baseline, oracle/cost_fp64.cpp: the float64 edge cost of the precision figures) into oracle/build/libpamo_oracle.so.

Test infrastructure: the oracle is the checker of the CUDA path, loaded only by tests/, the smoke check of
__graft_entry__ and the CPU-baseline leg of bench.py. -ffp-contract=off keeps every float product and sum
rounded separately, as nvcc --fmad=false does for the reference.
"""

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRCS = [os.path.join(HERE, n) for n in ("pamo_oracle.cpp", "stage3_oracle.cpp", "mesh_check.cpp", "cpu_qem.cpp",
                                        "cost_fp64.cpp")]
OUT = os.path.join(HERE, "build", "libpamo_oracle.so")


def build(force: bool = False) -> str:
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    if force or not os.path.exists(OUT) or any(os.path.getmtime(s) > os.path.getmtime(OUT) for s in SRCS):
        cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC", "-shared",
               "-o", OUT, *SRCS]
        subprocess.run(cmd, check=True)
    return OUT


if __name__ == "__main__":
    print(build())
