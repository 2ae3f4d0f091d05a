import numpy as np

from pamo_gb300 import synth
from tests import meshes


def test_icosphere_counts_and_manifold():
    for n in (1, 2, 5, 32):
        v, f = synth.icosphere(n)
        assert len(v) == 10 * n * n + 2 and len(f) == 20 * n * n
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
        assert len(np.unique(e, axis=0)) == len(e)  # every directed edge once: closed, oriented
        assert meshes.euler(f) == 2


def test_config_small_matches_spec():
    v, f = synth.config_mesh("plain_small", seed=0)
    assert v.dtype == np.float32 and f.dtype == np.int32
    assert v.shape == (10242, 3) and f.shape == (20480, 3)
    assert synth.is_star_shaped(v, f)
    r = np.linalg.norm(v.astype(np.float64), axis=1)
    assert r.min() >= 0.2


def test_sh_orthonormal():
    N = 100000
    i = np.arange(N) + 0.5
    z = 1 - 2 * i / N
    th = np.pi * (1 + 5 ** 0.5) * i
    d = np.stack([np.sqrt(1 - z * z) * np.cos(th), np.sqrt(1 - z * z) * np.sin(th), z], 1)
    for lm in [(1, 0), (2, 1), (5, -3), (16, 16)]:
        y = synth.sh_radius(d, {lm: 1.0}) - 1
        assert abs((y * y).mean() * 4 * np.pi - 1) < 1e-3
    a = synth.sh_radius(d, {(2, 1): 1.0}) - 1
    b = synth.sh_radius(d, {(3, 1): 1.0}) - 1
    assert abs((a * b).mean() * 4 * np.pi) < 1e-3


def test_seeded():
    a = synth.star_mesh(4, 3, lambda l: 0.05, 7)
    b = synth.star_mesh(4, 3, lambda l: 0.05, 7)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
