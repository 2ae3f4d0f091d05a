"""pamo_self_intersect_noalloc, the allocation-free variant of the self-intersection check.

It exists for callers that must not allocate device memory (a host that owns a fixed memory budget and
forbids plug-ins from calling cudaMalloc/cudaFree, or code that cannot afford the device synchronisation an
allocation may cause). Its scratch is one fixed device array inside the library, limited to meshes of at
most 65536 points and 65536 triangles. The tests call it through the C ABI twice in a row, on two different
meshes, and check both results bit-for-bit against pamo_self_intersect (the context-based entry point); that
an oversized mesh is rejected; that a call on a non-default stream leaves the device's allocated and free
memory unchanged; and, in a fresh process without torch, that the scratch address is looked up again after
the device's primary context is reset (a context keeps its own address for the array). This file sorts last
so that a run stopping at the first failure has run every other test before it.
"""

import ctypes
import json
import os
import subprocess
import sys

import numpy as np
import pytest
import torch

from tests import meshes

pytestmark = pytest.mark.gpu


def _call_noalloc(lib, v, f):
    pts = torch.from_numpy(v).cuda()
    tri = torch.from_numpy(f).cuda()
    out = torch.full((len(f),), 7, dtype=torch.uint8, device="cuda")
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = lib.pamo_self_intersect_noalloc(ctypes.c_void_p(pts.data_ptr()), ctypes.c_void_p(tri.data_ptr()), len(v),
                                         len(f), ctypes.c_void_p(out.data_ptr()), st)
    return rc, out.cpu().numpy()


def test_noalloc_matches_context_entry_point_twice():
    import pamo_gb300
    from pamo_gb300 import _native

    lib = _native.load()
    cases = [meshes.tangled(10, seed=10, amp=0.4), meshes.tangled(12, seed=9, amp=0.25)]
    for v, f in cases:  # two calls in a row; the second must not see the first one's state
        ref = pamo_gb300.self_intersect(torch.from_numpy(v).cuda(), torch.from_numpy(f).cuda()).cpu().numpy()
        assert ref.sum() > 0
        rc, got = _call_noalloc(lib, v, f)
        assert rc == 0, _native.STATUS_NAMES.get(rc, rc)
        assert np.array_equal(got, ref)


def test_noalloc_rejects_oversized_mesh():
    from pamo_gb300 import _native

    lib = _native.load()
    v, f = meshes.sphere(60)  # 72000 faces > 65536
    rc, _ = _call_noalloc(lib, v, f)
    assert rc == 3  # PAMO_ERR_CAPACITY


def test_noalloc_allocates_no_device_memory():
    import pamo_gb300
    from pamo_gb300 import _native

    lib = _native.load()
    v1, f1 = meshes.tangled(10, seed=10, amp=0.4)
    v2, f2 = meshes.tangled(12, seed=9, amp=0.25)
    rc, _ = _call_noalloc(lib, v1, f1)  # warm-up: kernels loaded, scratch address looked up
    assert rc == 0
    ref = pamo_gb300.self_intersect(torch.from_numpy(v2).cuda(), torch.from_numpy(f2).cuda()).cpu().numpy()
    side = torch.cuda.Stream()
    pts, tri = torch.from_numpy(v2).cuda(), torch.from_numpy(f2).cuda()
    out = torch.full((len(f2),), 7, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    allocated, free = torch.cuda.memory_allocated(), torch.cuda.mem_get_info()[0]
    rc = lib.pamo_self_intersect_noalloc(ctypes.c_void_p(pts.data_ptr()), ctypes.c_void_p(tri.data_ptr()), len(v2),
                                         len(f2), ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(side.cuda_stream))
    assert rc == 0, _native.STATUS_NAMES.get(rc, rc)
    torch.cuda.synchronize()
    assert torch.cuda.memory_allocated() == allocated
    assert torch.cuda.mem_get_info()[0] == free
    assert np.array_equal(out.cpu().numpy(), ref)


_RESET_CHILD = r"""
import ctypes, json, sys
import numpy as np
lib = ctypes.CDLL(sys.argv[1])
rt = ctypes.CDLL("libcudart.so.13")
P = ctypes.c_void_p
lib.pamo_self_intersect_noalloc.argtypes = [P, P, ctypes.c_int32, ctypes.c_int32, P, P]
rt.cudaMalloc.argtypes = [ctypes.POINTER(P), ctypes.c_size_t]
rt.cudaMemcpy.argtypes = [P, P, ctypes.c_size_t, ctypes.c_int]
rt.cudaFree.argtypes = [P]
data = np.load(sys.argv[2])
v, f = np.ascontiguousarray(data["v"], np.float32), np.ascontiguousarray(data["f"], np.int32)

def dev(nbytes):
    p = P()
    assert rt.cudaMalloc(ctypes.byref(p), nbytes) == 0
    return p

def call():
    dp, dt, do = dev(v.nbytes), dev(f.nbytes), dev(len(f))
    assert rt.cudaMemcpy(dp, v.ctypes.data, v.nbytes, 1) == 0
    assert rt.cudaMemcpy(dt, f.ctypes.data, f.nbytes, 1) == 0
    rc = lib.pamo_self_intersect_noalloc(dp, dt, len(v), len(f), do, None)
    out = np.zeros(len(f), np.uint8)
    assert rt.cudaMemcpy(out.ctypes.data, do, len(f), 2) == 0
    for p in (dp, dt, do):
        rt.cudaFree(p)
    return rc, out

rc1, a = call()
assert rt.cudaDeviceReset() == 0
rc2, b = call()
print(json.dumps({"rc": [rc1, rc2], "a": a.tolist(), "b": b.tolist()}))
"""


def test_noalloc_after_primary_context_reset(tmp_path):
    import pamo_gb300
    from pamo_gb300 import _native

    v, f = meshes.tangled(10, seed=10, amp=0.4)
    ref = pamo_gb300.self_intersect(torch.from_numpy(v).cuda(), torch.from_numpy(f).cuda()).cpu().numpy()
    np.savez(tmp_path / "mesh.npz", v=v, f=f)
    r = subprocess.run([sys.executable, "-c", _RESET_CHILD, _native.lib_path(), str(tmp_path / "mesh.npz")],
                       capture_output=True, text=True, timeout=300, env=dict(os.environ))
    assert r.returncode == 0, r.stderr[-2000:]
    res = json.loads(r.stdout.strip().splitlines()[-1])
    assert res["rc"] == [0, 0]
    assert np.array_equal(np.array(res["a"], np.uint8), ref)
    assert np.array_equal(np.array(res["b"], np.uint8), ref)
