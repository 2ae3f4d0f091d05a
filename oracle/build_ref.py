"""Builds the reference's own code, from the reference checkout, into oracle/_ref/ as pins of the oracle.

* oracle/_ref/ref_tritri: the reference's host-callable tri-tri functions (simp_cuda/src/bvh/tri_tri_3d.cuh,
  self_intersect.cuh) behind the harness oracle/ref_tritri.cu (nvcc, host code only).
* oracle/_ref/libref_round_emu.so: the reference's whole stage-2 round (simp_cuda/src/cusimp_free.cu with
  simp_cuda/src/bvh/*.cuh) and its legacy round without rollback (simp_cuda/src/cusimp.cu), compiled by g++ for
  the host under the CUDA-runtime emulation of oracle/ref_emu and exported by oracle/ref_round_emu.cpp and
  oracle/ref_legacy_emu.cpp. g++ cannot parse the launch syntax K<<<G, B>>>(args), so the recipe writes the files of
  the rounds into oracle/_ref/emu_src/ with each launch rewritten as EMU_LAUNCH(K, G, B)(args) and the kernels'
  float->uint32 cost conversions (cusimp_free.cu:584, cusimp.cu:470) as the device's saturating conversion; every
  other line is the reference's. oracle/_ref/ is a git-ignored build folder: nothing of the reference is committed.

The reference checkout is taken from $PAMO_REFERENCE_ROOT (default /root/reference, where this container has it).
Test infrastructure: run where the reference sources are present; the GPU machine has no reference tree and uses the
committed fixtures under tests/golden/.
"""

import os
import re
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REF_ROOT = os.environ.get("PAMO_REFERENCE_ROOT", "/root/reference")
REF_SRC = os.path.join(REF_ROOT, "simp_cuda", "src")
OUT_DIR = os.path.join(HERE, "_ref")
OUT = os.path.join(OUT_DIR, "ref_tritri")
EMU_SRC = os.path.join(OUT_DIR, "emu_src")
EMU_LIB = os.path.join(OUT_DIR, "libref_round_emu.so")
CCCL = "/usr/local/cuda/include/cccl"

# the files of the round, relative to simp_cuda/src
ROUND_FILES = ["cusimp_free.cu", "cusimp_free.h", "cusimp.cu", "cusimp.h"] + [
    os.path.join("bvh", n) for n in ("aabb.cuh", "bvh.cuh", "math.cuh", "morton_code.cuh", "predicator.cuh",
                                     "query.cuh", "self_intersect.cuh", "tri_tri_2d.cuh", "tri_tri_3d.cuh",
                                     "types.cuh", "utility.cuh")]
LAUNCH = re.compile(r"([A-Za-z_][\w:]*)\s*<<<(.+?)>>>\s*\(")
COST_CVT = "sp.edge_cost[edge_index] = uint32_t("
EXPECTED_LAUNCHES = {"cusimp_free.cu": 16, "cusimp.cu": 8, os.path.join("bvh", "self_intersect.cuh"): 2,
                     os.path.join("bvh", "bvh.cuh"): 1}
# the kernels' float->uint32 cost conversions, one per round file (cusimp_free.cu:584, cusimp.cu:470)
COST_FILES = ("cusimp_free.cu", "cusimp.cu")


def available() -> bool:
    return os.path.isdir(os.path.join(REF_SRC, "bvh")) and shutil.which("nvcc") is not None


def build(force: bool = False) -> str:
    if not available():
        raise RuntimeError("reference sources or nvcc not available (set PAMO_REFERENCE_ROOT)")
    os.makedirs(OUT_DIR, exist_ok=True)
    src = os.path.join(HERE, "ref_tritri.cu")
    if force or not os.path.exists(OUT) or os.path.getmtime(src) > os.path.getmtime(OUT):
        cmd = ["nvcc", "-O2", "--fmad=false", "-std=c++17", "--extended-lambda", "--expt-relaxed-constexpr",
               "-Xcompiler", "-ffp-contract=off", f"-I{REF_SRC}", f"-I{CCCL}", "-o", OUT, src]
        subprocess.run(cmd, check=True, capture_output=True)
    return OUT


def _rewrite(rel: str, text: str) -> str:
    n = len(LAUNCH.findall(text))
    if n != EXPECTED_LAUNCHES.get(rel, 0):
        raise RuntimeError(f"{rel}: {n} launches, expected {EXPECTED_LAUNCHES.get(rel, 0)}")
    text = LAUNCH.sub(lambda m: f"EMU_LAUNCH({m.group(1)}, {m.group(2)})(", text)
    if rel in COST_FILES:
        if text.count(COST_CVT) != 1:
            raise RuntimeError(f"{rel}: the edge-cost conversion was not found once")
        text = text.replace(COST_CVT, "sp.edge_cost[edge_index] = ::emu::device_f2u32(")
    return text


def build_round_emu(force: bool = False) -> str:
    """The reference's stage-2 round for the host (see the module docstring); returns the library path."""
    if not os.path.isdir(os.path.join(REF_SRC, "bvh")):
        raise RuntimeError("reference sources not available (set PAMO_REFERENCE_ROOT)")
    srcs = [os.path.join(HERE, "ref_round_emu.cpp"), os.path.join(HERE, "ref_legacy_emu.cpp")]
    deps = srcs + [os.path.join(HERE, "build_ref.py")] + [
        os.path.join(HERE, "ref_emu", n) for n in os.listdir(os.path.join(HERE, "ref_emu"))]
    if not force and os.path.exists(EMU_LIB) and all(os.path.getmtime(d) <= os.path.getmtime(EMU_LIB) for d in deps):
        return EMU_LIB
    for rel in ROUND_FILES:
        with open(os.path.join(REF_SRC, rel)) as f:
            text = _rewrite(rel, f.read())
        dst = os.path.join(EMU_SRC, rel)
        os.makedirs(os.path.dirname(dst), exist_ok=True)
        with open(dst, "w") as f:
            f.write(text)
    cmd = ["g++", "-O1", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-w",
           "-DTHRUST_DEVICE_SYSTEM=THRUST_DEVICE_SYSTEM_CPP", "-DTHRUST_HOST_SYSTEM=THRUST_HOST_SYSTEM_CPP",
           f"-I{os.path.join(HERE, 'ref_emu')}", f"-I{EMU_SRC}", f"-I{CCCL}", "-o", EMU_LIB, *srcs]
    subprocess.run(cmd, check=True)
    return EMU_LIB


if __name__ == "__main__":
    print(build(force=True))
    print(build_round_emu(force=True))
