"""pamo_gb300 — GB300-native (sm_103a) PaMO: stage 2 (parallel QEM edge collapse with LBVH self-intersection
rollback) behind the reference's ``CUDSP_Free`` operator and ``PaMO.run`` API, the legacy simplifier without
rollback (``CUDSP``, ``PaSP``), and stage 3 (barrier/CCD
Newton-CG safe projection, ``pamo_gb300.safe_project``).

The compute path is the CUDA library ``_lib/libpamo_gb300.so`` reached through its C ABI
(include/pamo_gb300.h); build it with ``pamo_gb300._build.build()``.
"""

from .api import (  # noqa: F401
    CUDSP,
    Context,
    CUDSP_Free,
    PaMO,
    PaSP,
    Remesher,
    cost_probe,
    launch_count,
    pamo_simplify,
    round_faces,
    self_intersect,
    simplify,
    simplify_to_target,
    tris_mean,
)
from ._native import PamoError  # noqa: F401

__all__ = ["Context", "CUDSP", "CUDSP_Free", "PaMO", "PaSP", "PamoError", "simplify", "pamo_simplify", "round_faces", "launch_count",
           "self_intersect", "tris_mean", "Remesher",
           "simplify_to_target"]
