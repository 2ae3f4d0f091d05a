"""Measured choice of the launch-shape knobs that are set at run time, cached per GPU model.

* ``tune_batch``: the number of worker contexts (one CUDA stream and host thread each) of ``Batch`` and
  ``Server``: too few leave the GPU idle between the small kernels of late rounds, too many split it into
  slices that each run slower. Each candidate simplifies the same sample of meshes; the fastest wins.
* ``tune_stage3``: the thread-block size of the cooperative PCG of stage 3 (128, 256 or 512 threads, the
  ``cg_mode`` option) on a sample projection.

Results are stored in a JSON file (``$PAMO_GB300_TUNE`` or ``~/.cache/pamo_gb300/autotune.json``) under the
device name, and ``best_workers`` returns the stored choice (or the default when nothing was tuned).
"""

from __future__ import annotations

import json
import os
import time

import numpy as np
import torch

DEFAULT_WORKERS = 16


def _cache_path() -> str:
    return os.environ.get("PAMO_GB300_TUNE") or os.path.join(os.path.expanduser("~"), ".cache", "pamo_gb300",
                                                              "autotune.json")


def _load() -> dict:
    try:
        with open(_cache_path()) as fh:
            return json.load(fh)
    except (OSError, ValueError):
        return {}


def _store(key: str, value) -> None:
    data = _load()
    data.setdefault(torch.cuda.get_device_name(), {})[key] = value
    path = _cache_path()
    os.makedirs(os.path.dirname(path), exist_ok=True)
    with open(path, "w") as fh:
        json.dump(data, fh, indent=1)


def best_workers(default: int = DEFAULT_WORKERS) -> int:
    entry = _load().get(torch.cuda.get_device_name() if torch.cuda.is_available() else "", {})
    return int(entry.get("batch_workers", default))


def tune_batch(meshes, ratios, candidates=(4, 8, 12, 16, 24, 32), repeats: int = 2, store: bool = True) -> dict:
    """Time ``Batch.simplify_csr`` on ``meshes`` for each worker count; returns {workers: faces/s, "best": n}."""
    from .batch import Batch, pack

    dev = torch.device("cuda", torch.cuda.current_device())
    P, T, voff, foff = pack(meshes)
    Pd, Td = torch.from_numpy(P).to(dev), torch.from_numpy(T).to(dev)
    faces = int(foff[-1])
    result = {}
    for w in candidates:
        b = Batch(dev, workers=int(w))
        b.simplify_csr(Pd, Td, voff, foff, ratios)  # warm-up: buffers and graphs
        best = np.inf
        for _ in range(repeats):
            torch.cuda.synchronize(dev)
            t0 = time.perf_counter()
            b.simplify_csr(Pd, Td, voff, foff, ratios)
            torch.cuda.synchronize(dev)
            best = min(best, time.perf_counter() - t0)
        result[int(w)] = faces / best
        del b
    result["best"] = max((k for k in result if isinstance(k, int)), key=lambda k: result[k])
    if store:
        _store("batch_workers", result["best"])
    return result


def tune_stage3(gt_V, gt_F, V, F, n_iters: int = 5, store: bool = True, modes=(0, 3, 4)) -> dict:
    """Time stage 3 with the 128-, 256- and 512-thread cooperative PCG (cg_mode 0, 3, 4); returns
    {cg_mode: seconds, "best": mode}."""
    from . import safe_project

    dev = torch.device("cuda", torch.cuda.current_device())
    result = {}
    for mode in modes:
        s = safe_project.Stage3System(None, dev)
        s._lib.pamo_stage3_set_param(s._h, b"cg_mode", float(mode))
        s.project(gt_V, gt_F, V, F, n_iters)  # warm-up
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        s.project(gt_V, gt_F, V, F, n_iters)
        torch.cuda.synchronize(dev)
        result[mode] = time.perf_counter() - t0
    result["best"] = min((k for k in result if isinstance(k, int)), key=lambda k: result[k])
    if store:
        _store("stage3_cg_mode", result["best"])
    return result


def best_cg_mode(default: int = 0) -> int:
    entry = _load().get(torch.cuda.get_device_name() if torch.cuda.is_available() else "", {})
    return int(entry.get("stage3_cg_mode", default))
