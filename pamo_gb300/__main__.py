"""Command line equivalent of the reference's example.py: simplify an OBJ mesh with PaMO and write the result.

    python -m pamo_gb300 -i input.obj -o output.obj -r 0.1 [-mv 0] --disable_stage1 [--disable_stage3] [--metrics]

Same flags as example.py (example.py:14-21); stage 1 runs the GPU remesher (``pamo_gb300.Remesher``) unless
``--disable_stage1`` is given. ``--metrics`` adds the reference's evaluation (metrics.py): Chamfer and
Hausdorff distances to the input, the smallest angle and the bad-triangle ratios of the output, and the
reference's self-intersection check of the output.
"""

from __future__ import annotations

import argparse
import sys
import time

import numpy as np
import torch


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(prog="python -m pamo_gb300")
    ap.add_argument("-i", "--input", type=str, required=True)
    ap.add_argument("-o", "--output", type=str, required=True)
    ap.add_argument("-r", "--ratio", type=float, default=0.1)
    ap.add_argument("-mv", "--min-vertex", type=int, default=0)
    ap.add_argument("--disable_stage1", action="store_true", help="Disable remeshing")
    ap.add_argument("--disable_stage3", action="store_true", help="Disable safe projection")
    ap.add_argument("--metrics", action="store_true", help="Report the reference's evaluation metrics")
    args = ap.parse_args(argv)
    import pamo_gb300
    from pamo_gb300 import mesh_io, metrics

    V, F = mesh_io.load_obj(args.input)
    print(f"# of input verts : {len(V)}")
    print(f"# of input faces : {len(F)}")
    model = pamo_gb300.PaMO((V, F), use_stage1=not args.disable_stage1, use_stage3=not args.disable_stage3)
    pts = torch.from_numpy(V).float().cuda()
    tri = torch.from_numpy(F).int().cuda()
    torch.cuda.synchronize()
    start = time.time()
    verts, faces = model.run(pts, tri, min_verts=args.min_vertex, ratio=args.ratio)
    torch.cuda.synchronize()
    print("Total time: ", time.time() - start)
    verts = np.asarray(verts, np.float64)
    faces = np.asarray(faces, np.int32)
    print(f"# of output verts : {len(verts)}")
    print(f"# of output faces : {len(faces)}")
    mesh_io.save_obj(args.output, verts, faces)
    if args.metrics:
        cd, hd = metrics.compute_trimesh_CD_HD(V, F, verts, faces)
        _, hd_v = metrics.compute_igl_CD_HD(V, F, verts, faces)
        hits = pamo_gb300.self_intersect(torch.from_numpy(verts).float().cuda(), torch.from_numpy(faces).int().cuda())
        print(f"Chamfer distance (5000 samples each way): {cd:.6e}")
        print(f"Hausdorff distance (samples / vertices): {hd:.6e} / {hd_v:.6e}")
        print(f"Min angle (degrees): {np.degrees(metrics.compute_min_angle_VF(verts, faces)):.4f}")
        print("Bad triangle ratio (<1, <5, <10 degrees):", metrics.compute_bad_tri_ratio(verts, faces).tolist())
        print(f"Faces in self-intersecting pairs: {int(hits.sum())}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
