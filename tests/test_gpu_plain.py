"""Parity of the plain form (cuFFT 2-D C2C + elementwise kernels, the
reference's own step order) against the FP64 oracle, and of the fused form
against the plain form on the same shot.  Tolerance: relative L2 <= 1e-4."""
import numpy as np
import pytest

import oracle as O
import qpstd
from cases import rel_l2, small_shot

pytestmark = pytest.mark.gpu
TOL = 1e-4


@pytest.fixture(scope="module", autouse=True)
def _lib():
    qpstd.lib()


@pytest.mark.parametrize("kind", [qpstd.APS, qpstd.VAPS])
def test_plain_modeling_matches_oracle(kind):
    d = small_shot(kind, nx=57, nz=33, nt=250)
    ref_g, ref_st = O.OracleShot(d).model(want_state=True)
    g, st = qpstd.model_shot(d, method=qpstd.PLAIN, want_state=True)
    assert rel_l2(g, ref_g) < TOL
    for f in range(8 if kind == qpstd.VAPS else 7):
        assert rel_l2(st[f], ref_st[f]) < TOL, f


@pytest.mark.parametrize("kind", [qpstd.ARTM, qpstd.QRTM])
def test_plain_rtm_matches_oracle(kind):
    d = small_shot(kind, nt=160, snaps=5)
    obs = O.OracleShot(dict(d, kind=O.APS if kind == qpstd.ARTM else O.VAPS)).model()
    ref_img, ref_ssg, _ = O.OracleShot(d).rtm(obs)
    img, ssg = qpstd.rtm_shot(d, obs, method=qpstd.PLAIN)
    assert rel_l2(ssg, ref_ssg) < TOL
    assert rel_l2(img, ref_img) < TOL


@pytest.mark.parametrize("kind", [qpstd.APS, qpstd.VAPS])
def test_fused_matches_plain(kind):
    d = small_shot(kind, nx=101, nz=64, nt=300, seed=21)
    g_f = qpstd.model_shot(d, method=qpstd.FUSED)
    g_p = qpstd.model_shot(d, method=qpstd.PLAIN)
    assert rel_l2(g_f, g_p) < TOL
