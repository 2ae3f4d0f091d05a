"""Stage 3 of PaMO (safe projection) over the C ABI — mirror of the reference package ``pamo_safe_project``.

``process(gt_V, gt_F, stage2_V, stage2_F, n_iters, system=None, config=None)`` follows
simp_cuda/safe_project/src/pamo_safe_project/processing.py:23-106; ``Stage3Config`` holds the defaults of
config.py:6-73 that the default energy set reads; ``Stage3System`` (system.py:28-110) owns the device buffers
and is reused across calls. All arithmetic runs in ``libpamo_gb300.so`` (``pamo_safe_project``); there is no
CPU path.

``mesh_process`` restates what ``trimesh.Trimesh(vertices, faces)`` does to the stage-2 output before the
reference hands it to stage 3 (simp_cuda/pamo/__init__.py:166-172, trimesh 4.4.0 as pinned in env.yaml):
drop faces that touch non-finite vertices, then merge vertices whose coordinates agree after rounding to
8 decimals, keeping referenced vertices only, in order of first occurrence.
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass, fields

import numpy as np
import torch

from . import _native


@dataclass
class Stage3Config:
    """Stage3Config defaults used by the default energy set (config.py:6-73)."""

    n_newton_iters: int = 10
    n_cg_iters: int = 40
    n_line_search_iters: int = 10
    d_hat: float = 1e-3
    coll_stiffness: float = 1e2
    contact_detection_radius: float = 1e-2
    ee_classify_thres: float = 1e-3
    ccd_slackness: float = 0.7
    ccd_thickness: float = 1e-6
    ccd_max_iters: int = 100
    spd_max_iters: int = 3
    elas_young_modulus: float = 1e-1
    elas_poisson_ratio: float = 0.0
    hinge_stiffness: float = 1e-2
    mesh2gt_dist_stiffness: float = 1e3
    min_angle_thres: float = 0.0
    max_blocks: int = 1 << 25
    # this build's precision mode for the CCD step: 2 double-float (hi + lo float pairs, the default), 1 (or True)
    # float64, 0 (or False) float32 as Warp's kernels compute it
    ccd_fp64: int = 2


class Stage3System:
    """Device state of stage 3 (system.py:28-110); one per device, reused by ``process``."""

    def __init__(self, config: Stage3Config | None = None, device="cuda:0"):
        self.config = config or Stage3Config()
        self.device = torch.device(device)
        if self.device.type != "cuda":
            raise ValueError("Stage3System needs a CUDA device")
        lib = _native.load()
        h = ctypes.c_void_p()
        index = self.device.index if self.device.index is not None else torch.cuda.current_device()
        st = lib.pamo_stage3_create(ctypes.byref(h), index)
        if st != _native.PAMO_OK:
            raise _native.PamoError(st, f"pamo_stage3_create on cuda:{index}")
        self._lib = lib
        self._h = h
        self._applied = None
        from .autotune import best_cg_mode

        lib.pamo_stage3_set_param(h, b"cg_mode", float(best_cg_mode()))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                self._lib.pamo_stage3_destroy(h)
            except Exception:  # interpreter shutdown
                pass
            self._h = None

    def clear(self):
        """Kept for the reference's API (system.clear()); buffers are reused as they are."""

    def set(self, name: str, value) -> None:
        """An execution knob of the solver that keeps the method (pamo_stage3_set_param): use_cuda_graph, ccd_fp64,
        cg_mode (PCG launch shape), ls_mode (line search launch shape)."""
        self._check(self._lib.pamo_stage3_set_param(self._h, name.encode(), float(value)), f"set {name}")

    def _apply_config(self):
        cfg = tuple((f.name, getattr(self.config, f.name)) for f in fields(self.config))
        if cfg == self._applied:
            return
        for name, value in cfg:
            st = self._lib.pamo_stage3_set_param(self._h, name.encode(), float(value))
            self._check(st, f"set {name}")
        self._applied = cfg

    def _check(self, status: int, what: str):
        if status != _native.PAMO_OK:
            msg = self._lib.pamo_stage3_last_error(self._h)
            raise _native.PamoError(status, f"{what}: {msg.decode() if msg else ''}")

    def stats(self) -> dict:
        out = (ctypes.c_double * len(_native.STAGE3_STATS))()
        self._lib.pamo_stage3_stats(self._h, out, len(out))
        return dict(zip(_native.STAGE3_STATS, list(out)))

    def project(self, gt_V, gt_F, V, F, n_iters: int, stream=None) -> torch.Tensor:
        """Device-level call: tensors on this system's device (float64 points, int32 faces); returns the
        projected float64 points as a device tensor."""
        self._apply_config()
        gt_V = _dev(gt_V, torch.float64, self.device)
        gt_F = _dev(gt_F, torch.int32, self.device)
        V = _dev(V, torch.float64, self.device)
        F = _dev(F, torch.int32, self.device)
        for name, t in (("gt_V", gt_V), ("gt_F", gt_F), ("V", V), ("F", F)):
            if t.dim() != 2 or t.shape[1] != 3:
                raise ValueError(f"{name} must have shape [n, 3]")
        out = torch.empty_like(V)
        if stream is None:
            stream = torch.cuda.current_stream(self.device)
        st = self._lib.pamo_safe_project(
            self._h, gt_V.data_ptr(), gt_F.data_ptr(), gt_V.shape[0], gt_F.shape[0], V.data_ptr(), F.data_ptr(),
            V.shape[0], F.shape[0], int(n_iters), out.data_ptr(), ctypes.c_void_p(stream.cuda_stream))
        self._check(st, "pamo_safe_project")
        return out


def _dev(x, dtype, device) -> torch.Tensor:
    if isinstance(x, torch.Tensor):
        return x.to(device=device, dtype=dtype).contiguous()
    return torch.as_tensor(np.ascontiguousarray(x), dtype=dtype, device=device)


_SYSTEMS: dict = {}


def process(gt_V, gt_F, stage2_V, stage2_F, n_iters, system: Stage3System | None = None,
            config: Stage3Config | None = None):
    """Safe projection (processing.py:23-106). Returns ``(V, F)``: the projected vertices as a float64
    NumPy array in the input frame, and ``stage2_F`` unchanged."""
    if system is None:
        dev = torch.device("cuda", torch.cuda.current_device())
        if config is not None:
            system = Stage3System(config, dev)
        else:
            system = _SYSTEMS.get(dev.index)
            if system is None:
                system = _SYSTEMS[dev.index] = Stage3System(None, dev)
    out = system.project(gt_V, gt_F, stage2_V, stage2_F, n_iters)
    return out.cpu().numpy(), stage2_F


def mesh_process(V, F):
    """``trimesh.Trimesh(V, F)`` with its default processing (see the module docstring). Returns
    ``(V float64, F int64)``."""
    V = np.asarray(V, dtype=np.float64)
    F = np.asarray(F, dtype=np.int64).reshape(-1, 3)
    if len(V) == 0 or len(F) == 0:
        return V.reshape(-1, 3), F
    finite = np.isfinite(V).all(axis=1)
    if not finite.all():
        keep_f = finite[F].all(axis=1)
        F = F[keep_f]
        remap = np.cumsum(finite) - 1
        V = V[finite]
        F = remap[F]
    referenced = np.zeros(len(V), dtype=bool)
    referenced[F] = True
    stacked = np.round(V * (10 ** 8)).astype(np.int64)
    ref_idx = np.nonzero(referenced)[0]
    rows = stacked[referenced]
    _, first, inverse = np.unique(rows, axis=0, return_index=True, return_inverse=True)
    order = np.argsort(first, kind="stable")  # unique rows in order of first occurrence
    rank = np.empty_like(order)
    rank[order] = np.arange(len(order))
    inv_full = np.zeros(len(V), dtype=np.int64)
    inv_full[referenced] = rank[inverse.reshape(-1)]
    mask = ref_idx[first[order]]
    return V[mask], inv_full[F]
