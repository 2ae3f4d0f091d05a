"""The whole-mesh self-intersection check (pamo_self_intersect) against the oracle's global check."""

import numpy as np
import pytest
import torch

from oracle import oracle as orc
from tests import meshes

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed,amp", [(9, 0.25), (10, 0.4), (11, 0.1)])
def test_flags_match_oracle(seed, amp):
    import pamo_gb300

    v, f = meshes.tangled(10, seed=seed, amp=amp)
    ref, nhits = orc.Oracle().self_intersect(v, f)
    assert nhits > 0
    got = pamo_gb300.self_intersect(torch.from_numpy(v).cuda(), torch.from_numpy(f).cuda()).cpu().numpy()
    assert np.array_equal(got, ref)


def test_star_shaped_input_is_clean():
    import pamo_gb300
    from pamo_gb300 import synth

    v, f = synth.config_mesh("plain_small", seed=0)
    got = pamo_gb300.self_intersect(torch.from_numpy(v).cuda(), torch.from_numpy(f).cuda()).cpu().numpy()
    assert got.sum() == 0
