"""Pins of two device behaviours that the oracle and the host-compiled reference round take as given.

* thrust::shuffle on the CUDA backend (the reference's call, simp_cuda/src/cusimp_free.cu:937-941) gives the same
  permutations as tests/golden/thrust_shuffle.npz, which was made with Thrust's CPP device system: the generator
  tests/golden/thrust_shuffle_golden.cpp is compiled here as CUDA and run on the GPU.
* the device's pow(float, 2) (the reference's skinny term, cusimp_free.cu:533,573) differs from x * x only by one
  ulp, on a few floats in a million; the oracle and, by default, the CUDA path square by multiplication, and the
  CUDA path gives the same rounds with the device function (option skinny_pow) on the test meshes and the
  20,480-face workload.

Both programs are compiled with nvcc for sm_103a at test time.
"""

import hashlib
import os
import shutil
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.join(os.path.dirname(__file__), "golden")
CCCL = "/usr/local/cuda/include/cccl"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    n = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    assert os.path.exists(n), "nvcc is required"
    return n


def test_thrust_shuffle_cuda_backend_matches_golden(tmp_path):
    exe = str(tmp_path / "tsg_cuda")
    subprocess.run([_nvcc(), *ARCH, "-O2", "-std=c++17", "-x", "cu", f"-I{CCCL}", "-o", exe,
                    os.path.join(HERE, "thrust_shuffle_golden.cpp")], check=True, capture_output=True)
    g = np.load(os.path.join(HERE, "thrust_shuffle.npz"))
    sizes = [int(k.split("_")[1]) for k in g.files if k.startswith(("perm_", "sha256_"))]
    out = subprocess.run([exe, *map(str, sizes)], check=True, capture_output=True, text=True, timeout=600).stdout
    for line in out.strip().splitlines():
        vals = line.split()
        m = int(vals[0])
        perm = np.array(vals[1:], dtype=np.int32)
        assert perm.size == m
        if f"perm_{m}" in g.files:
            assert np.array_equal(perm, g[f"perm_{m}"]), m
        else:
            assert hashlib.sha256(perm.tobytes()).digest() == g[f"sha256_{m}"].tobytes(), m


def test_device_pow_float_int_2_is_within_one_ulp_of_square(tmp_path):
    exe = str(tmp_path / "powcheck")
    subprocess.run([_nvcc(), *ARCH, "--fmad=false", "-O3", "-o", exe, os.path.join(HERE, "device_pow_check.cu")],
                   check=True, capture_output=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True, timeout=300).stdout
    lines = out.strip().splitlines()
    tested, bad = (int(x) for x in lines[-1].split())
    assert tested == 1 << 22
    assert bad <= tested // 100000, out  # a few in a million
    for line in lines[:-1]:  # the first mismatches: one ulp apart
        _, x, p, m = line.split()
        a, b = float.fromhex(p.split("=")[1]), float.fromhex(m.split("=")[1])
        assert abs(np.float32(a).view(np.int32) - np.float32(b).view(np.int32)) == 1, line


@pytest.mark.parametrize("name", ["plain_small", "tangled", "sphere12_rough", "high_threshold"])
def test_skinny_pow_and_square_give_the_same_rounds(name):
    import torch

    import pamo_gb300
    from tests.golden import make_ref_round_golden as gen

    v, f, ratio, tol, thr, iters = gen.cases()[name]
    out = []
    for pw in (1, 0):
        ctx = pamo_gb300.Context("cuda:0")
        ctx.set_option("skinny_pow", pw)
        V, F, rounds = pamo_gb300.simplify(torch.from_numpy(v).cuda(), torch.from_numpy(f).cuda(), ratio, tol, thr,
                                           iters, 0, ctx=ctx)
        out.append((V.cpu().numpy(), F.cpu().numpy(), rounds))
    assert out[0][2] == out[1][2]
    assert np.array_equal(out[0][1], out[1][1]) and np.array_equal(out[0][0], out[1][0])
