"""pamo_self_intersect_noalloc, the allocation-free variant of the self-intersection check.

It exists for callers that must not allocate device memory (a host that owns a fixed memory budget and
forbids plug-ins from calling cudaMalloc/cudaFree, or code that cannot afford the device synchronisation an
allocation may cause). Its scratch is one fixed device array inside the library, limited to meshes of at
most 65536 points and 65536 triangles. The test calls it through the C ABI twice in a row, on two different
meshes, and checks both results bit-for-bit against pamo_self_intersect (the context-based entry point);
it also checks that an oversized mesh is rejected. This file sorts last so that a run stopping at the first
failure has run every other test before it.
"""

import ctypes

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
