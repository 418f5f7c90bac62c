"""The low-rank form of the constant-Q step against the FP64 oracle (GPU).

qpstd_shot_set_lowrank switches a constant-Q shot to the pressure update
p += rho vp^2 dt W{div} -/+ dt tau aux, W{div} = sum_a U[x][a] sum_b A[a][b]
Re F^-1[Vt_b F div] / N (the reference's dormant low-rank operator,
sgpstd-qmodeling/acsglw.cu:1375-1497, fed as its dormant addsa_b_kernel feeds
it, :1542-1571).  The oracle runs the same update in FP64 with the same
factors (decomposed once on the host), so the comparison isolates the device
step.  Tolerance: relative L2 <= 1e-4 against FP64.
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


def _factors(d, rank):
    return qpstd.lowrank_decompose(d["nxx"], d["nzz"], d["dx"], d["dz"], d["dt"], d["vp"], d["tao"], d["gam"],
                                   rank, rank)


@pytest.mark.parametrize("nx,nz,rank", [(60, 40, 4), (83, 37, 3), (57, 50, 5)])  # 83+20 = 103: prime width
def test_lowrank_steps_from_random_state(nx, nz, rank):
    d = small_shot(qpstd.VAPS, nx=nx, nz=nz, nt=8)
    f = _factors(d, rank)
    rng = np.random.default_rng(nx * nz + rank)
    st0 = rng.standard_normal((8, d["nxx"], d["nzz"]))
    st0 *= np.array([1.0, 1e-3, 1e-3, 1e-4, 1e-4, 1e-4, 1e-4, 1e-2])[:, None, None]
    ref_st, ref_g = O.OracleShot(dict(d, lowrank=f)).steps(st0, 0, 5)
    sh = qpstd.Shot(d)
    sh.set_lowrank(f)
    sh.set_state(st0.astype(np.float32))
    g = sh.advance(0, 5)
    st = sh.get_state()
    sh.close()
    for k in range(8):
        assert rel_l2(st[k], ref_st[k]) < TOL, (k, rel_l2(st[k], ref_st[k]))
    assert rel_l2(g, ref_g) < TOL


def test_lowrank_439x200_grid_gather():
    """The 439 x 200 padded grid of the 160 x 398 model at rank 4, shortened to 200 steps."""
    d = grid439_shot(qpstd.VAPS, nt=200)
    f = _factors(d, 4)
    ref_g = O.OracleShot(dict(d, lowrank=f)).model()
    sh = qpstd.Shot(d)
    sh.set_lowrank(f)
    g = sh.advance(0, 200)
    sh.close()
    assert rel_l2(g, ref_g) < TOL, rel_l2(g, ref_g)


def test_lowrank_qrtm_image():
    """Revolve-driven Q-RTM in the low-rank form (source and receiver sides)."""
    d = small_shot(qpstd.QRTM, nt=160, snaps=5)
    f = _factors(d, 4)
    obs = O.OracleShot(dict(d, kind=O.VAPS)).model()
    ref_img, ref_ssg, _ = O.OracleShot(dict(d, lowrank=f)).rtm(obs)
    sh = qpstd.Shot(d)
    sh.set_lowrank(f)
    sh.set_obs(obs)
    sh.rtm_device()
    img, ssg = sh.get_image()
    sh.close()
    assert rel_l2(ssg, ref_ssg) < TOL, rel_l2(ssg, ref_ssg)
    assert rel_l2(img, ref_img) < TOL, rel_l2(img, ref_img)


def test_lowrank_rejects_acoustic_shots():
    d = small_shot(qpstd.APS, nt=8)
    sh = qpstd.Shot(d)
    with pytest.raises(qpstd.QpstdError):
        sh.set_lowrank({"U": np.zeros((d["nxx"] * d["nzz"], 2)), "V": np.zeros((2, 10)), "A": np.zeros((2, 2))})
    sh.close()
