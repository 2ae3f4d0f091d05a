"""The oracle's stage-2 restatement against the reference's own round.

tests/golden/ref_rounds.npz holds the rounds of the reference's CUSimp_Free::forward (simp_cuda/src/cusimp_free.cu
with its LBVH, compiled for the host by oracle/build_ref.py) driven through PaMO.run's stage-2 loop on 12 meshes:
the level-5 icosphere workload (20480 faces, 84 rounds), small spheres, an open patch, an index-degenerate face, a
zero-length edge, folded meshes whose rounds take undo passes, and stuck rounds (quirks Q1-Q3). Every round's
five operator outputs must have the same digests from the oracle, and the oracle's own whole loop (oracle_run, the
loop the CUDA path follows) must end on the reference loop's final mesh bit for bit. The same holds for the legacy
round without rollback (simp_cuda/src/cusimp.cu) driven through PaSP.run on 6 meshes.
"""

import os

import numpy as np
import pytest

from oracle import oracle as orc
from tests.golden import make_ref_round_golden as gen

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "ref_rounds.npz")


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN)


def _names(g):
    return sorted({k.split(".")[0] for k in g.files})


def test_fixture_covers_the_cases(golden):
    names = [n for n in _names(golden) if not n.startswith("legacy_")]
    assert set(names) == set(gen.cases())
    assert {n for n in _names(golden) if n.startswith("legacy_")} == set(gen.legacy_cases())
    counts = np.concatenate([golden[f"{n}.counts"] for n in names])
    assert counts[:, 5].sum() >= 6, "stuck rounds are covered"
    assert (counts[:, 2] > 0).sum() >= 50, "rounds that carry undo vertices are covered"
    assert golden["plain_small.counts"].shape[0] == 84


@pytest.mark.parametrize("name", sorted(gen.cases()))
def test_oracle_rounds_equal_reference_rounds(golden, name):
    v, f, ratio, tol, thr, iters = gen.cases()[name]
    assert np.array_equal(golden[f"{name}.input"],
                          np.concatenate([gen.digest(np.ascontiguousarray(v, np.float32)),
                                          gen.digest(np.ascontiguousarray(f, np.int32))])), "input mesh changed"
    counts, digests, V, F = gen.record(gen._OracleOp(orc.Oracle()), v, f, ratio, tol, thr, iters)
    ref_counts, ref_digests = golden[f"{name}.counts"], golden[f"{name}.digests"]
    assert counts.shape == ref_counts.shape, (counts.shape, ref_counts.shape)
    for r in range(len(counts)):
        assert np.array_equal(counts[r], ref_counts[r]), (r, counts[r], ref_counts[r])
        for k, out in enumerate(gen.OUTPUT_NAMES):
            assert np.array_equal(digests[r, k], ref_digests[r, k]), f"round {r}: {out} differs"
    assert np.array_equal(V, golden[f"{name}.final_verts"])
    assert np.array_equal(F, golden[f"{name}.final_faces"])


@pytest.mark.parametrize("name", ["plain_small", "tangled", "tangled_strong", "open_patch"])
def test_oracle_loop_equals_reference_loop(golden, name):
    v, f, ratio, tol, thr, iters = gen.cases()[name]
    V, F, fpr = orc.Oracle().run(v, f, ratio, tolerance=tol, threshold=thr, iters=iters, min_verts=0)
    assert np.array_equal(fpr, golden[f"{name}.counts"][:, 4])
    assert np.array_equal(F, golden[f"{name}.final_faces"])
    assert np.array_equal(V, golden[f"{name}.final_verts"])


@pytest.mark.parametrize("name", sorted(gen.legacy_cases()))
def test_oracle_legacy_rounds_equal_reference_rounds(golden, name):
    v, f, thr, iters = gen.legacy_cases()[name]
    counts, digests, V, F = gen.record_legacy(orc.Oracle(), v, f, thr, iters)
    assert np.array_equal(counts, golden[f"{name}.counts"])
    assert np.array_equal(digests, golden[f"{name}.digests"])
    assert np.array_equal(V, golden[f"{name}.final_verts"])
    assert np.array_equal(F, golden[f"{name}.final_faces"])
    Vr, Fr, rounds = orc.Oracle().run_legacy(v, f, thr, iters)
    assert rounds == len(counts)
    assert np.array_equal(Fr, golden[f"{name}.final_faces"]) and np.array_equal(Vr, golden[f"{name}.final_verts"])
