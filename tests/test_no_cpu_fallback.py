"""The product path has no CPU fallback: host tensors and host-only machines get an error, never a CPU result.
(These run without a GPU; on a machine with one, the CPU-tensor checks still hold.)"""

import numpy as np
import pytest
import torch

from tests import meshes


def _mesh():
    V, F = meshes.octahedron()
    return torch.from_numpy(np.asarray(V, np.float32)), torch.from_numpy(np.asarray(F, np.int32))


def test_simplify_rejects_host_tensors():
    import pamo_gb300

    V, F = _mesh()
    with pytest.raises(RuntimeError, match="CUDA"):
        pamo_gb300.simplify(V, F, 0.5)


def test_stage3_rejects_a_host_device():
    from pamo_gb300 import safe_project

    with pytest.raises(ValueError):
        safe_project.Stage3System(safe_project.Stage3Config(), "cpu")


@pytest.mark.skipif(torch.cuda.is_available(), reason="checks the behaviour of a machine without a GPU")
def test_pamo_run_without_a_gpu_raises():
    import pamo_gb300

    V, F = _mesh()
    model = pamo_gb300.PaMO((V.numpy().astype(np.float64), F.numpy()), use_stage1=False, use_stage3=False)
    with pytest.raises(RuntimeError):
        model.run(V, F, ratio=0.5, min_verts=0)
