"""The PyTorch extension module pamo_gb300._C (the reference's pamo._C, simp_cuda/src/pybind.cpp:16-197) builds,
loads, and checks its inputs like the reference's CHECK_INPUT / TORCH_INTERNAL_ASSERT (no GPU calls)."""

import pytest
import torch


def test_module_exposes_the_reference_classes(torch_ext):
    assert hasattr(torch_ext, "CUDSP_Free") and hasattr(torch_ext, "CUDSP")
    doc = torch_ext.CUDSP_Free.forward.__doc__
    for arg in ("points", "triangles", "verts_undo", "n_verts_undo", "scale", "threshold", "is_stuck", "init"):
        assert arg in doc
    for arg in ("points", "triangles", "scale", "threshold", "init"):
        assert arg in torch_ext.CUDSP.forward.__doc__


def test_cpu_tensors_are_rejected(torch_ext):
    p = torch.zeros(3, 3)
    t = torch.zeros(1, 3, dtype=torch.int32)
    u = torch.zeros(0, dtype=torch.int32)
    with pytest.raises(RuntimeError, match="CUDA"):
        torch_ext.CUDSP_Free().forward(p, t, u, 0, 1.0, 1e-3, False, True)
    with pytest.raises(RuntimeError, match="CUDA"):
        torch_ext.CUDSP().forward(p, t, 1.0, 1e-3, True)
