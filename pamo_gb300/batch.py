"""Many meshes on one GPU: batched simplification and a request server over the C ABI.

``CsrBatch`` runs all meshes of a CSR batch through the PaMO.run stage-2 loop together, every round one pass of the
round's kernels over all live meshes (``pamo_csr_*``). ``Batch`` and ``Server`` run the whole loop per mesh on a pool
of worker contexts (one CUDA stream and host thread each). Every mesh starts from the state of a new context, so a
mesh's result is the same alone, in a batch, or among other requests.
"""

from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _native


def _err(lib_fn, handle) -> str:
    raw = lib_fn(handle)
    return raw.decode() if raw else ""


class Batch:
    """A worker pool for batches of meshes in CSR form (``pamo_batch_*``)."""

    def __init__(self, device=None, workers: int | None = None):
        self.device = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
        if workers is None:
            from .autotune import best_workers

            workers = best_workers()
        lib = _native.load()
        h = ctypes.c_void_p()
        st = lib.pamo_batch_create(ctypes.byref(h), self.device.index or 0, int(workers))
        if st != _native.PAMO_OK:
            raise _native.PamoError(st, "pamo_batch_create")
        self._lib, self._h, self.workers = lib, h, workers

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                self._lib.pamo_batch_destroy(h)
            except Exception:  # interpreter shutdown
                pass
            self._h = None

    def simplify_csr(self, points: torch.Tensor, triangles: torch.Tensor, vert_offsets, face_offsets, ratios,
                     tolerance: int = 4, threshold: float = 1e-3, iter: int = 1000000, min_verts: int = 0):
        """points float32 [V,3] and triangles int32 [F,3] (CUDA, triangle indices local to each mesh), offsets
        of n+1 entries. Returns (points, triangles, vert_offsets, face_offsets) of the results, packed."""
        n = len(vert_offsets) - 1
        voff = np.ascontiguousarray(vert_offsets, dtype=np.int64)
        foff = np.ascontiguousarray(face_offsets, dtype=np.int64)
        rat = np.ascontiguousarray(np.broadcast_to(np.asarray(ratios, dtype=np.float64), (n,)))
        pts = points.to(self.device, torch.float32).contiguous()
        tri = triangles.to(self.device, torch.int32).contiguous()
        out_p = torch.empty_like(pts)
        out_t = torch.empty_like(tri)
        ovoff = np.zeros(n + 1, np.int64)
        ofoff = np.zeros(n + 1, np.int64)
        stream = torch.cuda.current_stream(self.device).cuda_stream
        st = self._lib.pamo_batch_simplify(self._h, pts.data_ptr(), tri.data_ptr(), voff.ctypes.data, foff.ctypes.data,
                                           n, rat.ctypes.data, int(tolerance), ctypes.c_float(threshold), int(iter),
                                           int(min_verts), out_p.data_ptr(), out_t.data_ptr(), ovoff.ctypes.data,
                                           ofoff.ctypes.data, ctypes.c_void_p(stream))
        if st != _native.PAMO_OK:
            raise _native.PamoError(st, _err(self._lib.pamo_batch_last_error, self._h))
        return out_p[: ovoff[-1]], out_t[: ofoff[-1]], ovoff, ofoff

    def rounds(self, n: int) -> np.ndarray:
        out = np.zeros(n, np.int32)
        k = self._lib.pamo_batch_rounds(self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), n)
        return out[:k]


class CsrBatch:
    """Batched rounds (``pamo_csr_*``): all meshes of a CSR batch run the PaMO.run loop together on one stream,
    every round one pass of the round's kernels over all live meshes; each result equals the mesh's result alone."""

    def __init__(self, device=None):
        self.device = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
        lib = _native.load()
        h = ctypes.c_void_p()
        st = lib.pamo_csr_create(ctypes.byref(h), self.device.index or 0)
        if st != _native.PAMO_OK:
            raise _native.PamoError(st, "pamo_csr_create")
        self._lib, self._h = lib, h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                self._lib.pamo_csr_destroy(h)
            except Exception:  # interpreter shutdown
                pass
            self._h = None

    def set_option(self, name: str, value: int):
        st = self._lib.pamo_csr_set_option(self._h, name.encode(), int(value))
        if st != _native.PAMO_OK:
            raise _native.PamoError(st, _err(self._lib.pamo_csr_last_error, self._h))

    def simplify_csr(self, points: torch.Tensor, triangles: torch.Tensor, vert_offsets, face_offsets, ratios,
                     tolerance: int = 4, threshold: float = 1e-3, iter: int = 1000000, min_verts: int = 0):
        """The contract of Batch.simplify_csr."""
        n = len(vert_offsets) - 1
        voff = np.ascontiguousarray(vert_offsets, dtype=np.int64)
        foff = np.ascontiguousarray(face_offsets, dtype=np.int64)
        rat = np.ascontiguousarray(np.broadcast_to(np.asarray(ratios, dtype=np.float64), (n,)))
        pts = points.to(self.device, torch.float32).contiguous()
        tri = triangles.to(self.device, torch.int32).contiguous()
        out_p = torch.empty_like(pts)
        out_t = torch.empty_like(tri)
        ovoff = np.zeros(n + 1, np.int64)
        ofoff = np.zeros(n + 1, np.int64)
        stream = torch.cuda.current_stream(self.device).cuda_stream
        st = self._lib.pamo_csr_simplify(self._h, pts.data_ptr(), tri.data_ptr(), voff.ctypes.data, foff.ctypes.data,
                                         n, rat.ctypes.data, int(tolerance), ctypes.c_float(threshold), int(iter),
                                         int(min_verts), out_p.data_ptr(), out_t.data_ptr(), ovoff.ctypes.data,
                                         ofoff.ctypes.data, ctypes.c_void_p(stream))
        if st != _native.PAMO_OK:
            raise _native.PamoError(st, _err(self._lib.pamo_csr_last_error, self._h))
        return out_p[: ovoff[-1]], out_t[: ofoff[-1]], ovoff, ofoff

    def rounds(self, n: int) -> np.ndarray:
        out = np.zeros(n, np.int32)
        k = self._lib.pamo_csr_rounds(self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), n)
        return out[:k]


def pack(meshes):
    """[(V [n,3], F [m,3]), ...] -> (points, triangles, vert_offsets, face_offsets) NumPy CSR form."""
    voff = np.zeros(len(meshes) + 1, np.int64)
    foff = np.zeros(len(meshes) + 1, np.int64)
    for i, (v, f) in enumerate(meshes):
        voff[i + 1] = voff[i] + len(v)
        foff[i + 1] = foff[i] + len(f)
    P = np.concatenate([np.asarray(v, np.float32).reshape(-1, 3) for v, _ in meshes])
    T = np.concatenate([np.asarray(f, np.int32).reshape(-1, 3) for _, f in meshes])
    return P, T, voff, foff


def unpack(points, triangles, voff, foff):
    P = points.cpu().numpy() if isinstance(points, torch.Tensor) else np.asarray(points)
    T = triangles.cpu().numpy() if isinstance(triangles, torch.Tensor) else np.asarray(triangles)
    return [(P[voff[i]:voff[i + 1]], T[foff[i]:foff[i + 1]]) for i in range(len(voff) - 1)]


def simplify_batch(meshes, ratios, tolerance: int = 4, threshold: float = 1e-3, iter: int = 1000000,
                   min_verts: int = 0, workers: int | None = None, batch=None):
    """Simplify a list of (V, F) meshes; returns a list of (V float32, F int32) NumPy results. Batched rounds
    (CsrBatch) unless a worker count or a Batch is given."""
    batch = batch or (Batch(workers=workers) if workers is not None else CsrBatch())
    P, T, voff, foff = pack(meshes)
    out = batch.simplify_csr(torch.from_numpy(P).to(batch.device), torch.from_numpy(T).to(batch.device), voff, foff,
                             ratios, tolerance, threshold, iter, min_verts)
    return unpack(*out)


class Server:
    """A request loop (``pamo_server_*``): requests are admitted in arrival order while their estimated device
    bytes fit ``hbm_budget_bytes``, then run on the next free worker."""

    def __init__(self, device=None, workers: int | None = None, hbm_budget_bytes: int = 80 << 30):
        self.device = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
        if workers is None:
            from .autotune import best_workers

            workers = best_workers()
        lib = _native.load()
        h = ctypes.c_void_p()
        st = lib.pamo_server_create(ctypes.byref(h), self.device.index or 0, int(workers), int(hbm_budget_bytes))
        if st != _native.PAMO_OK:
            raise _native.PamoError(st, "pamo_server_create")
        self._lib, self._h = lib, h

    def close(self):
        if self._h is not None and self._h.value:
            self._lib.pamo_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # interpreter shutdown
            pass

    def submit(self, verts, tris, ratio: float, tolerance: int = 4, threshold: float = 1e-3,
               stage3: bool = False) -> int:
        """Queue one PaMO.run job; with stage3 the result is also projected onto the request's own input mesh
        (PaMO(use_stage3=True)), with float64 positions."""
        v = np.ascontiguousarray(verts, np.float32).reshape(-1, 3)
        t = np.ascontiguousarray(tris, np.int32).reshape(-1, 3)
        rid = ctypes.c_int64()
        st = self._lib.pamo_server_submit_ex(self._h, v.ctypes.data, t.ctypes.data, len(v), len(t), float(ratio),
                                             int(tolerance), ctypes.c_float(threshold), int(bool(stage3)),
                                             ctypes.byref(rid))
        if st != _native.PAMO_OK:
            raise _native.PamoError(st, _err(self._lib.pamo_server_last_error, self._h))
        return rid.value

    def wait(self, timeout_ms: int = 1000):
        """(request id, status, n_points, n_triangles, (queued ms, run ms, total ms)) or None on time-out."""
        rid, st, npt, ntr = ctypes.c_int64(), ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        times = (ctypes.c_double * 3)()
        got = self._lib.pamo_server_wait(self._h, int(timeout_ms), ctypes.byref(rid), ctypes.byref(st), ctypes.byref(npt),
                                         ctypes.byref(ntr), times)
        if got != 1:
            return None
        return rid.value, st.value, npt.value, ntr.value, tuple(times)

    def fetch(self, request_id: int, n_points: int, n_triangles: int, float64: bool = False):
        v = np.zeros((n_points, 3), np.float64 if float64 else np.float32)
        t = np.zeros((n_triangles, 3), np.int32)
        fn = self._lib.pamo_server_fetch_f64 if float64 else self._lib.pamo_server_fetch
        st = fn(self._h, int(request_id), v.ctypes.data, t.ctypes.data)
        if st != _native.PAMO_OK:
            raise _native.PamoError(st, _err(self._lib.pamo_server_last_error, self._h))
        return v, t

    def stats(self) -> dict:
        out = (ctypes.c_int64 * 7)()
        self._lib.pamo_server_stats(self._h, out, 7)
        return dict(zip(["in_use", "max_in_use", "admitted", "finished", "queued", "budget", "stage3_reruns"], list(out)))

    @staticmethod
    def job_bytes(n_points: int, n_triangles: int) -> int:
        return int(_native.load().pamo_server_job_bytes(int(n_points), int(n_triangles)))
