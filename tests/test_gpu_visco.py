"""Parity of the fused constant-Q CUDA path (vaps, qrtm) against the FP64 oracle.

Tolerance: relative L2 <= 1e-4 against FP64 (gathers, states, images).
"""
import numpy as np
import pytest

import oracle as O
import qpstd
from cases import grid439_shot, rel_l2, small_shot

pytestmark = pytest.mark.gpu
TOL = 1e-4


@pytest.fixture(scope="module", autouse=True)
def _lib():
    qpstd.lib()


@pytest.mark.parametrize("nx,nz", [(60, 40), (57, 33), (90, 51), (83, 37)])  # 83+20 = 103: prime width
def test_vaps_steps_from_random_state(nx, nz):
    d = small_shot(qpstd.VAPS, nx=nx, nz=nz, nt=8)
    rng = np.random.default_rng(nx + nz)
    st0 = rng.standard_normal((8, d["nxx"], d["nzz"]))
    st0 *= np.array([1.0, 1e-3, 1e-3, 1e-4, 1e-4, 1e-4, 1e-4, 1e-2])[:, None, None]
    ref_st, ref_g = O.OracleShot(d).steps(st0, 0, 5)
    sh = qpstd.Shot(d)
    sh.set_state(st0.astype(np.float32))
    g = sh.advance(0, 5)
    st = sh.get_state()
    for f in range(8):
        assert rel_l2(st[f], ref_st[f]) < TOL, (f, rel_l2(st[f], ref_st[f]))
    assert rel_l2(g, ref_g) < TOL


def test_vaps_small_shot_gather():
    d = small_shot(qpstd.VAPS, nt=300)
    ref_g, ref_st = O.OracleShot(d).model(want_state=True)
    g, st = qpstd.model_shot(d, want_state=True)
    assert rel_l2(g, ref_g) < TOL
    for f in range(8):
        assert rel_l2(st[f], ref_st[f]) < TOL, f


def test_vaps_439x200_grid_gather():
    """The 160 x 398 model geometry (439 prime x 200 padded grid), shortened to 300 steps."""
    d = grid439_shot(qpstd.VAPS, nt=300)
    ref_g = O.OracleShot(d).model()
    g = qpstd.model_shot(d)
    assert rel_l2(g, ref_g) < TOL


def test_qrtm_small_shot_image():
    d = small_shot(qpstd.QRTM, nt=200, snaps=6)
    obs = O.OracleShot(dict(d, kind=O.VAPS)).model()
    ref_img, ref_ssg, nfwd = O.OracleShot(d).rtm(obs)
    img, ssg = qpstd.rtm_shot(d, obs)
    assert rel_l2(ssg, ref_ssg) < TOL
    assert rel_l2(img, ref_img) < TOL


def test_qrtm_stabilised_filter_regime():
    """Large eta so the stabilised symbol departs from k^1.01 within the run."""
    d = small_shot(qpstd.QRTM, nt=200, snaps=5)
    d = dict(d, etas=1e4, etar=1e4)
    obs = O.OracleShot(dict(d, kind=O.VAPS)).model()
    ref_img, ref_ssg, _ = O.OracleShot(d).rtm(obs)
    img, ssg = qpstd.rtm_shot(d, obs)
    assert rel_l2(ssg, ref_ssg) < TOL
    assert rel_l2(img, ref_img) < TOL


def test_qrtm_prime_width_image():
    """Padded width 103 (prime): exact x transforms need Bluestein, so the
    stationary symbols run as per-kz convolutions on the smooth length."""
    d = small_shot(qpstd.QRTM, nx=83, nt=200, snaps=6)
    obs = O.OracleShot(dict(d, kind=O.VAPS)).model()
    ref_img, ref_ssg, _ = O.OracleShot(d).rtm(obs)
    img, ssg = qpstd.rtm_shot(d, obs)
    assert rel_l2(ssg, ref_ssg) < TOL
    assert rel_l2(img, ref_img) < TOL


def test_qrtm_prime_width_stabilised_filter():
    """Prime width with a large eta: the filter departs from k^1.01, so the
    aux pass keeps the exact transforms beside the convolution passes."""
    d = small_shot(qpstd.QRTM, nx=83, nt=160, snaps=5)
    d = dict(d, etas=1e4, etar=1e4)
    obs = O.OracleShot(dict(d, kind=O.VAPS)).model()
    ref_img, ref_ssg, _ = O.OracleShot(d).rtm(obs)
    img, ssg = qpstd.rtm_shot(d, obs)
    assert rel_l2(ssg, ref_ssg) < TOL
    assert rel_l2(img, ref_img) < TOL
