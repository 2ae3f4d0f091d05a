"""Compiles the reference's host-callable tri-tri code (simp_cuda/src/bvh under /root/reference) with the
harness oracle/ref_tritri.cu into oracle/_ref/ref_tritri. Test infrastructure: run where the reference
sources are present (this container); the GPU machine has no reference tree and uses the committed fixtures.
"""

import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REF_SRC = "/root/reference/simp_cuda/src"
OUT = os.path.join(HERE, "_ref", "ref_tritri")


def available() -> bool:
    return os.path.isdir(os.path.join(REF_SRC, "bvh")) and shutil.which("nvcc") is not None


def build(force: bool = False) -> str:
    if not available():
        raise RuntimeError("reference sources or nvcc not available")
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    src = os.path.join(HERE, "ref_tritri.cu")
    if force or not os.path.exists(OUT) or os.path.getmtime(src) > os.path.getmtime(OUT):
        cmd = ["nvcc", "-O2", "--fmad=false", "-std=c++17", "--extended-lambda", "--expt-relaxed-constexpr",
               "-Xcompiler", "-ffp-contract=off", f"-I{REF_SRC}", "-I/usr/local/cuda/include/cccl", "-o", OUT, src]
        subprocess.run(cmd, check=True, capture_output=True)
    return OUT


if __name__ == "__main__":
    print(build(force=True))
