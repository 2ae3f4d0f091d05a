"""The reference's evaluation metrics (simp_cuda/safe_project/src/pamo_safe_project/metrics.py:7-107) with the
distance and angle computations on the GPU (``pamo_point_mesh_sqdist``, ``pamo_face_min_angles``).

* ``sample_surface`` restates trimesh 4.4.0's ``trimesh.sample.sample_surface``: faces drawn in proportion to
  their areas by searching uniform numbers times the total area in the cumulative areas, then two uniform
  numbers per sample folded back into the triangle (u + v > 1 maps to 1 - u, 1 - v). It is not pinned against
  trimesh here (trimesh is not installed), so sampled metrics may differ from the reference's by sampling.
* ``compute_trimesh_CD_HD`` / ``compute_igl_CD_HD``: Chamfer distance as the sum of the two mean squared
  sample-to-surface distances; Hausdorff distance as the largest sample-to-surface distance both ways
  (trimesh variant) or igl's vertex-to-surface distance from the ground truth to the generated mesh.
* ``compute_min_angle_VF`` and ``compute_bad_tri_ratio`` from per-face minimum angles.
"""

from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _native


def _dev(device):
    return torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)


def point_mesh_sqdist(points, vertices, faces, device=None):
    """(squared distances float64 [n], closest face int32 [n]) from points to the mesh (float64 math)."""
    dev = _dev(device)
    P = torch.as_tensor(np.ascontiguousarray(points, np.float64).reshape(-1, 3), device=dev)
    V = torch.as_tensor(np.ascontiguousarray(vertices, np.float64).reshape(-1, 3), device=dev)
    F = torch.as_tensor(np.ascontiguousarray(faces, np.int32).reshape(-1, 3), device=dev)
    d2 = torch.empty(P.shape[0], dtype=torch.float64, device=dev)
    fi = torch.empty(P.shape[0], dtype=torch.int32, device=dev)
    with torch.cuda.device(dev):
        st = _native.load().pamo_point_mesh_sqdist(
            ctypes.c_void_p(P.data_ptr()), int(P.shape[0]), ctypes.c_void_p(V.data_ptr()), int(V.shape[0]),
            ctypes.c_void_p(F.data_ptr()), int(F.shape[0]), ctypes.c_void_p(d2.data_ptr()),
            ctypes.c_void_p(fi.data_ptr()), ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream))
    if st != _native.PAMO_OK:
        raise _native.PamoError(st, "pamo_point_mesh_sqdist")
    return d2.cpu().numpy(), fi.cpu().numpy()


def face_min_angles(vertices, faces, device=None):
    """(edge-vector form, igl form) per-face minimum angles in radians; NaN for index-degenerate faces."""
    dev = _dev(device)
    V = torch.as_tensor(np.ascontiguousarray(vertices, np.float64).reshape(-1, 3), device=dev)
    F = torch.as_tensor(np.ascontiguousarray(faces, np.int32).reshape(-1, 3), device=dev)
    a = torch.empty(F.shape[0], dtype=torch.float64, device=dev)
    b = torch.empty(F.shape[0], dtype=torch.float64, device=dev)
    with torch.cuda.device(dev):
        st = _native.load().pamo_face_min_angles(
            ctypes.c_void_p(V.data_ptr()), ctypes.c_void_p(F.data_ptr()), int(F.shape[0]), ctypes.c_void_p(a.data_ptr()),
            ctypes.c_void_p(b.data_ptr()), ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream))
    if st != _native.PAMO_OK:
        raise _native.PamoError(st, "pamo_face_min_angles")
    return a.cpu().numpy(), b.cpu().numpy()


def face_areas(vertices, faces) -> np.ndarray:
    V = np.asarray(vertices, np.float64)
    F = np.asarray(faces, np.int64)
    return 0.5 * np.linalg.norm(np.cross(V[F[:, 1]] - V[F[:, 0]], V[F[:, 2]] - V[F[:, 0]]), axis=1)


def sample_surface(vertices, faces, count: int, seed=None) -> np.ndarray:
    """``count`` points on the surface, area-weighted (trimesh 4.4.0's sample_surface without face weights)."""
    V = np.asarray(vertices, np.float64)
    F = np.asarray(faces, np.int64)
    area = face_areas(V, F)
    cum = np.cumsum(area)
    rng = np.random.default_rng(seed)
    pick = np.searchsorted(cum, rng.random(count) * cum[-1])
    tri = V[F[pick]]
    origins = tri[:, 0]
    vectors = tri[:, 1:] - origins[:, None, :]
    lengths = rng.random((len(vectors), 2, 1))
    fold = lengths.sum(axis=1).reshape(-1) > 1.0
    lengths[fold] -= 1.0
    lengths = np.abs(lengths)
    return (vectors * lengths).sum(axis=1) + origins


def compute_trimesh_CD_HD(gt_V, gt_F, gen_V, gen_F, num_mesh_samples=5000, seed=42):
    """metrics.py:7-29: (Chamfer, Hausdorff) from surface samples of both meshes."""
    gen_s = sample_surface(gen_V, gen_F, num_mesh_samples, seed)
    gt_s = sample_surface(gt_V, gt_F, num_mesh_samples, seed)
    d_gt_gen = np.sqrt(point_mesh_sqdist(gen_s, gt_V, gt_F)[0])
    d_gen_gt = np.sqrt(point_mesh_sqdist(gt_s, gen_V, gen_F)[0])
    chamfer = np.mean(np.square(d_gt_gen)) + np.mean(np.square(d_gen_gt))
    return float(chamfer), float(max(d_gt_gen.max(), d_gen_gt.max()))


def hausdorff_vertices(a_V, a_F, b_V, b_F) -> float:
    """igl.hausdorff: the largest distance from a vertex of either mesh to the other mesh."""
    ab = point_mesh_sqdist(a_V, b_V, b_F)[0].max()
    ba = point_mesh_sqdist(b_V, a_V, a_F)[0].max()
    return float(np.sqrt(max(ab, ba)))


def compute_igl_CD_HD(gt_V, gt_F, gen_V, gen_F, num_mesh_samples=5000, seed=42):
    """metrics.py:32-52: (Chamfer from surface samples, igl Hausdorff between the meshes)."""
    gt_s = sample_surface(gt_V, gt_F, num_mesh_samples, seed)
    gen_s = sample_surface(gen_V, gen_F, num_mesh_samples, seed)
    chamfer = point_mesh_sqdist(gt_s, gen_V, gen_F)[0].mean() + point_mesh_sqdist(gen_s, gt_V, gt_F)[0].mean()
    return float(chamfer), hausdorff_vertices(gt_V, gt_F, gen_V, gen_F)


def compute_min_angle_VF(V, F) -> float:
    """metrics.py:78-96: the smallest corner angle (radians) over faces without a repeated index."""
    edge_form, _ = face_min_angles(V, F)
    edge_form = edge_form[~np.isnan(edge_form)]
    return float(edge_form.min()) if edge_form.size else float("nan")


def compute_bad_tri_ratio(V, F, thresholds=(1, 5, 10)) -> np.ndarray:
    """metrics.py:99-104: the fraction of faces whose smallest angle (degrees) is below each threshold."""
    _, igl_form = face_min_angles(V, F)
    deg = igl_form * 180.0 / np.pi
    t = np.asarray(thresholds, np.float64)
    return np.sum(deg[:, None] < t[None, :], axis=0) / max(1, len(F))
