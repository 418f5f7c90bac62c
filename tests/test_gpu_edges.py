"""Edge cases of the fused path against the FP64 oracle (GPU): receivers on the
padded grid's corners and repeated at one point, shots without receivers, and a
source inside the CPML corner, on odd grids (the last z and x line pairs hold one
line).  Tolerance: relative L2 <= 1e-4 against FP64, as for the other parity tests.
The shots run 300 steps, as the other state comparisons do: the CPML memory
fields are compared once the wavefield has filled the CPML (at its first arrival
they are small, and the FP32 rounding of the leading edge weighs more in their
norm: fipx measured 1.4e-4 after 160 steps on the 57 x 33 model).
"""
import numpy as np
import pytest

import oracle as O
import qpstd
import workloads as W
from cases import rel_l2, small_shot

pytestmark = pytest.mark.gpu
TOL = 1e-4


@pytest.fixture(scope="module", autouse=True)
def _lib():
    qpstd.lib()


def _nfields(kind):
    """State fields compared: p, vx, vz, fipx, fipz, fivxx, fivzz, plus the
    auxiliary field that only the viscoacoustic kinds use."""
    return 8 if kind == qpstd.VAPS else 7


def _corner_receivers(d):
    nxx, nzz = d["nxx"], d["nzz"]
    # four corners, two receivers at one interior point, one interior receiver
    gx = [0, nxx - 1, 0, nxx - 1, nxx // 2 + 5, nxx // 2 + 5, nxx // 2]
    gz = [0, 0, nzz - 1, nzz - 1, d["zsg"], d["zsg"], d["zsg"]]
    return dict(d, gxg=np.array(gx, dtype=np.int32), gzg=np.array(gz, dtype=np.int32))


@pytest.mark.parametrize("kind", [qpstd.APS, qpstd.VAPS])
def test_receivers_on_corners_and_repeated(kind):
    d = _corner_receivers(small_shot(kind, nx=57, nz=33, nt=300))
    ref_g, ref_st = O.OracleShot(d).model(want_state=True)
    g, st = qpstd.model_shot(d, want_state=True)
    assert g.shape == (300, 7)
    # a repeated receiver records the same trace twice, bit for bit
    assert np.array_equal(g[:, 4], g[:, 5])
    # corner traces are small (inside the CPML): compare the whole gather, and
    # the interior trace on its own
    assert rel_l2(g, ref_g) < TOL
    assert rel_l2(g[:, 6], ref_g[:, 6]) < TOL
    for f in range(_nfields(kind)):
        assert rel_l2(st[f], ref_st[f]) < TOL, f


@pytest.mark.parametrize("kind", [qpstd.APS, qpstd.VAPS])
def test_shot_without_receivers(kind):
    d = small_shot(kind, nx=57, nz=33, nt=300)
    d = dict(d, gxg=np.zeros(0, dtype=np.int32), gzg=np.zeros(0, dtype=np.int32))
    ref_g, ref_st = O.OracleShot(d).model(want_state=True)
    g, st = qpstd.model_shot(d, want_state=True)
    assert g.shape == (300, 0)
    for f in range(_nfields(kind)):
        assert rel_l2(st[f], ref_st[f]) < TOL, f


def test_source_in_the_cpml_corner():
    d = small_shot(qpstd.APS, nx=57, nz=33, nt=300)
    d = dict(d, xsg=2, zsg=d["nzz"] - 3)
    ref_g, ref_st = O.OracleShot(d).model(want_state=True)
    g, st = qpstd.model_shot(d, want_state=True)
    assert rel_l2(g, ref_g) < TOL
    for f in range(_nfields(qpstd.APS)):
        assert rel_l2(st[f], ref_st[f]) < TOL, f


@pytest.mark.parametrize("kind,fwd", [(qpstd.ARTM, O.APS), (qpstd.QRTM, O.VAPS)])
def test_rtm_with_corner_and_repeated_receivers(kind, fwd):
    """The receiver side sets p to the observed trace at each receiver cell; the
    corner receivers sit inside the CPML, and of two receivers in one cell the
    higher index wins (the reference keeps one receiver index per cell)."""
    d = _corner_receivers(small_shot(kind, nx=57, nz=33, nt=200, snaps=6))
    obs = O.OracleShot(dict(d, kind=fwd)).model()
    ref_img, ref_ssg, _ = O.OracleShot(d).rtm(obs)
    img, ssg = qpstd.rtm_shot(d, obs)
    assert rel_l2(ssg, ref_ssg) < TOL
    assert rel_l2(img, ref_img) < TOL
    # receiver 4 shares its cell with receiver 5: its trace has no effect ...
    obs4 = obs.copy()
    obs4[:, 4] = 0.0
    img4, _ = qpstd.rtm_shot(d, obs4)
    assert np.array_equal(img4, img)
    # ... while receiver 5's trace does
    obs5 = obs.copy()
    obs5[:, 5] = 0.0
    ref_img5, _, _ = O.OracleShot(d).rtm(obs5)
    assert rel_l2(ref_img5, ref_img) > 10 * TOL


@pytest.mark.parametrize("bad,msg", [("source", "shot grid index"), ("receiver", "receiver grid index"),
                                     ("snaps", "snaps"), ("width", None)])
def test_bad_shots_return_a_status(bad, msg):
    """Where the reference prints and exits, the library returns a status (the
    Python binding raises), launches nothing, and stays usable."""
    d = small_shot(qpstd.APS, nx=57, nz=33, nt=20)
    if bad == "source":
        d = dict(d, xsg=d["nxx"])
    elif bad == "receiver":
        d = dict(d, gzg=np.full_like(d["gzg"], -1))
    elif bad == "snaps":
        d = dict(small_shot(qpstd.ARTM, nx=57, nz=33, nt=20), snaps=65)
    else:  # padded width 6021: beyond the longest line the fused form plans
        d = W.make_shot(qpstd.APS, 6000, 24, 10, 20, 0.0005, 25.0, seed=9)
    with pytest.raises(qpstd.QpstdError, match=msg):
        if bad == "snaps":
            qpstd.rtm_shot(d, np.zeros((20, d["gxg"].size), dtype=np.float32))
        else:
            qpstd.model_shot(d)
    good = small_shot(qpstd.APS, nx=57, nz=33, nt=40)
    assert rel_l2(qpstd.model_shot(good), O.OracleShot(good).model()) < TOL
