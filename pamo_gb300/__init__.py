"""pamo_gb300 — GB300-native (sm_103a) PaMO stage-2 simplification: parallel QEM edge collapse with LBVH
self-intersection rollback, behind the reference's ``CUDSP_Free`` operator and ``PaMO.run`` API.

The compute path is the CUDA library ``_lib/libpamo_gb300.so`` reached through its C ABI
(include/pamo_gb300.h); build it with ``pamo_gb300._build.build()``.
"""

from .api import Context, CUDSP_Free, PaMO, launch_count, round_faces, self_intersect, simplify  # noqa: F401
from ._native import PamoError  # noqa: F401

__all__ = ["Context", "CUDSP_Free", "PaMO", "PamoError", "simplify", "round_faces", "launch_count", "self_intersect"]
