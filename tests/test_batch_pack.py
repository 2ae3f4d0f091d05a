"""CSR packing of a batch on CPU: per-mesh local indices kept, offsets cumulative, unpack the inverse of pack."""

import numpy as np

from tests import meshes


def test_pack_unpack_round_trip():
    from pamo_gb300.batch import pack, unpack

    batch = [meshes.octahedron(), meshes.sphere(2), meshes.octahedron()]
    P, T, voff, foff = pack(batch)
    assert P.dtype == np.float32 and T.dtype == np.int32
    assert voff.tolist() == [0, 6, 6 + len(batch[1][0]), 12 + len(batch[1][0])]
    assert foff[-1] == sum(len(f) for _, f in batch) == len(T)
    # face indices stay local to their mesh (the batch entry points take per-mesh offsets)
    for i in range(len(batch)):
        assert T[foff[i]:foff[i + 1]].max() < voff[i + 1] - voff[i]
    for (v0, f0), (v1, f1) in zip(batch, unpack(P, T, voff, foff)):
        assert np.array_equal(np.asarray(v0, np.float32), v1) and np.array_equal(f0, f1)
