"""Generates tests/golden/thrust_shuffle.npz: the permutations thrust::shuffle(first, last,
thrust::default_random_engine()) applies, taken from the CCCL headers of the installed CUDA toolkit.

Built from tests/golden/thrust_shuffle_golden.cpp with g++ and the CPP device system. Small sizes are
stored in full, large ones (the face counts of the level-5 and level-9 icospheres) as SHA-256 digests of
the int32 permutation.

    python tests/golden/make_shuffle_golden.py
"""

import hashlib
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
FULL = [1, 2, 3, 5, 16, 17, 40, 1000, 4097, 20480]
HASHED = [65537, 1310720, 5242880]


def main():
    cccl = "/usr/local/cuda/include/cccl"
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "tsg")
        subprocess.run(["g++", "-O2", "-std=c++17", f"-I{cccl}", "-I/usr/local/cuda/include",
                        "-DTHRUST_DEVICE_SYSTEM=THRUST_DEVICE_SYSTEM_CPP", "-o", exe,
                        os.path.join(HERE, "thrust_shuffle_golden.cpp")], check=True)
        out = {}
        for m in FULL + HASHED:
            line = subprocess.run([exe, str(m)], check=True, capture_output=True, text=True).stdout.split()
            perm = np.array(line[1:], dtype=np.int32)
            assert int(line[0]) == m and perm.size == m
            if m in FULL:
                out[f"perm_{m}"] = perm
            else:
                out[f"sha256_{m}"] = np.frombuffer(hashlib.sha256(perm.tobytes()).digest(), dtype=np.uint8)
    with open(os.path.join(cccl, "thrust", "version.h")) as f:
        ver = [l for l in f if l.startswith("#define THRUST_VERSION ")][0].split()[2]
    out["thrust_version"] = np.array(int(ver))
    np.savez_compressed(os.path.join(HERE, "thrust_shuffle.npz"), **out)


if __name__ == "__main__":
    main()
