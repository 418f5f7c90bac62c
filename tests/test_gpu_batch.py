"""Batches: shots with different windows run concurrently give, shot for
shot, the result they give alone (the same kernels on the same inputs; the
comparison is exact up to floating-point reassociation, tolerance 1e-6)."""
import numpy as np
import pytest

import oracle as O
import qpstd
import workloads as W
from cases import rel_l2

pytestmark = pytest.mark.gpu


def _shots(kind, n=3):
    out = []
    for i in range(n):
        out.append(W.make_shot(kind, 50 + 17 * i, 36, 10, 150, 0.001, 25.0, seed=40 + i, snaps=5))
    return out


@pytest.mark.parametrize("kind", [qpstd.ARTM, qpstd.QRTM])
def test_batch_equals_alone(kind):
    shots = _shots(kind)
    mkind = qpstd.APS if kind == qpstd.ARTM else qpstd.VAPS
    obs = [qpstd.model_shot(dict(d, kind=mkind)) for d in shots]
    alone = [qpstd.rtm_shot(d, o) for d, o in zip(shots, obs)]
    imgs, ssgs = qpstd.rtm_batch(shots, obs)
    for (ia, sa), ib, sb in zip(alone, imgs, ssgs):
        assert rel_l2(ib, ia) < 1e-6
        assert rel_l2(sb, sa) < 1e-6


def test_batch_matches_oracle():
    shots = _shots(qpstd.QRTM, n=2)
    obs = [O.OracleShot(dict(d, kind=O.VAPS)).model() for d in shots]
    imgs, ssgs = qpstd.rtm_batch(shots, obs)
    for d, o, img in zip(shots, obs, imgs):
        ref_img, _, _ = O.OracleShot(d).rtm(o)
        assert rel_l2(img, ref_img) < 1e-4
