"""Low-rank form of the constant-Q mixed-domain symbol (sgpstd-qmodeling/sglowrank.c).

Host tests (no GPU): the library's FP64 decomposition against the oracle
restatement (same seeded draws, so the same selected wavenumbers and points),
exactness on piecewise-constant models, the half-grid wavenumbers against the
reference's cal_k2dh, argument checks.  GPU tests: the fused device operator
against the FP64 oracle apply with the same factors (relative L2 <= 1e-4), on
smooth, prime and odd grids, and against the mixed-domain operator itself when
the decomposition is exact.
"""
import numpy as np
import pytest

import lowrank as LR
import qpstd
from cases import rel_l2

GOLD = np.load(__import__("os").path.join(__import__("os").path.dirname(__file__), "golden", "reference_host.npz"))
TOL = 1e-4
DT = 0.001


def smooth_model(nxx, nzz, seed):
    rng = np.random.default_rng(seed)
    x, z = np.meshgrid(np.linspace(0, 1, nxx), np.linspace(0, 1, nzz), indexing="ij")
    a, b, c = rng.uniform(0.5, 2.0, 3)
    vp = 2000.0 + 800.0 * np.sin(a * 3 * x + b * 2 * z) + 300.0 * z
    q = 60.0 + 40.0 * np.cos(c * 4 * x * z)
    gam = np.arctan(1.0 / (np.pi * q)) / np.pi
    tao = 1.0 / (np.pi * 30.0 * q) * 1e-3
    return vp.astype(np.float32).ravel(), tao.astype(np.float32).ravel(), gam.astype(np.float32).ravel()


def layered_model(nxx, nzz, nmat, seed):
    rng = np.random.default_rng(seed)
    vps = rng.uniform(1500.0, 4500.0, nmat)
    qs = rng.uniform(20.0, 200.0, nmat)
    lay = np.minimum((np.arange(nzz) * nmat) // nzz, nmat - 1)
    vp = np.repeat(vps[lay][None, :], nxx, axis=0)
    q = np.repeat(qs[lay][None, :], nxx, axis=0)
    gam = np.arctan(1.0 / (np.pi * q)) / np.pi
    tao = 1e-4 * gam
    return vp.astype(np.float32).ravel(), tao.astype(np.float32).ravel(), gam.astype(np.float32).ravel()


@pytest.mark.parametrize("g", [0, 2, 3])
def test_k2dh_pinned(g):
    pml, fd, nxx, nzz, dx, dz, dt = GOLD[f"g{g}_grid"]
    mine = LR.khalf(int(nxx), int(nzz), dx, dz)
    ref = GOLD[f"g{g}_k2dh"]
    assert np.max(np.abs(mine - ref) / np.maximum(np.abs(ref), 1e-6)) < 2e-6


@pytest.mark.parametrize("nxx,nzz,row,col", [(36, 28, 4, 4), (41, 33, 5, 5), (30, 24, 3, 5)])
def test_decompose_matches_oracle(nxx, nzz, row, col):
    vp, tao, gam = smooth_model(nxx, nzz, nxx)
    f = qpstd.lowrank_decompose(nxx, nzz, 10.0, 10.0, DT, vp, tao, gam, row, col, seed=5)
    o = LR.decompose(nxx, nzz, 10.0, 10.0, DT, vp, tao, gam, row, col, seed=5)
    assert list(f["jrr"]) == list(o["jrr"])
    assert list(f["irr"]) == list(o["irr"])
    assert rel_l2(f["U"], o["U"]) < 1e-6
    assert rel_l2(f["V"], o["V"]) < 1e-6
    assert rel_l2(f["A"], o["A"]) < 1e-6


def test_piecewise_constant_model_is_exact():
    """A model with 3 materials has a symbol of rank 3: row = col = 3 reproduces it."""
    nxx, nzz = 32, 30
    vp, tao, gam = layered_model(nxx, nzz, 3, 9)
    f = qpstd.lowrank_decompose(nxx, nzz, 10.0, 10.0, DT, vp, tao, gam, 3, 3, seed=2)
    for pt in (0, 5 * nzz + 3, nxx * nzz - 1, 17 * nzz + 20):
        We, Wa = qpstd.lowrank_check(f, 10.0, 10.0, DT, vp, tao, gam, pt)
        assert np.max(np.abs(We - Wa)) < 1e-5 * np.max(np.abs(We))


def test_check_matches_oracle_and_smooth_error_is_small():
    nxx, nzz = 40, 32
    vp, tao, gam = smooth_model(nxx, nzz, 3)
    f = qpstd.lowrank_decompose(nxx, nzz, 10.0, 10.0, DT, vp, tao, gam, 5, 5, seed=3)
    pt = 20 * nzz + 16
    We, Wa = qpstd.lowrank_check(f, 10.0, 10.0, DT, vp, tao, gam, pt)
    oWe, oWa = LR.check(f["U"], f["V"], f["A"], vp, tao, gam, DT, 10.0, 10.0, nxx, nzz, pt)
    assert rel_l2(We, oWe) < 1e-6 and rel_l2(Wa, oWa) < 1e-5
    assert rel_l2(Wa, We) < 1e-2


def test_oracle_apply_equals_mixed_domain_operator_when_exact():
    """Pins the oracle's apply (mirroring, normalisation, factor order) against
    the mixed-domain operator evaluated point by point."""
    nxx, nzz = 22, 17
    vp, tao, gam = layered_model(nxx, nzz, 2, 8)
    o = LR.decompose(nxx, nzz, 10.0, 10.0, DT, vp, tao, gam, 2, 2, seed=4)
    field = np.random.default_rng(2).standard_normal((nxx, nzz))
    got = LR.apply(o["U"], o["V"], o["A"], field, nxx, nzz)
    exact = LR.apply_exact(vp, tao, gam, DT, 10.0, 10.0, field, nxx, nzz)
    assert rel_l2(got, exact) < 1e-9


def test_decompose_rejects_bad_arguments():
    vp, tao, gam = smooth_model(8, 8, 1)
    with pytest.raises(qpstd.QpstdError):
        qpstd.lowrank_decompose(8, 8, 10.0, 10.0, DT, vp, tao, gam, 0, 3)
    with pytest.raises(qpstd.QpstdError):
        qpstd.lowrank_decompose(1, 8, 10.0, 10.0, DT, vp, tao, gam, 3, 3)


@pytest.mark.gpu
@pytest.mark.parametrize("nxx,nzz,row,col", [(64, 48, 4, 4), (103, 57, 5, 5), (97, 73, 2, 3)])
def test_device_apply_matches_oracle(nxx, nzz, row, col):
    vp, tao, gam = smooth_model(nxx, nzz, nzz)
    f = qpstd.lowrank_decompose(nxx, nzz, 10.0, 10.0, DT, vp, tao, gam, row, col, seed=11)
    rng = np.random.default_rng(nxx)
    field = rng.standard_normal((nxx, nzz)).astype(np.float32)
    op = qpstd.LowRank(f)
    out = op.apply(field)
    out2 = op.apply(field)
    op.close()
    ref = LR.apply(f["U"], f["V"], f["A"], field, nxx, nzz)
    assert rel_l2(out, ref) < TOL
    assert np.array_equal(out, out2)


@pytest.mark.gpu
def test_device_apply_equals_mixed_domain_operator_when_exact():
    nxx, nzz = 30, 26
    vp, tao, gam = layered_model(nxx, nzz, 3, 4)
    f = qpstd.lowrank_decompose(nxx, nzz, 10.0, 10.0, DT, vp, tao, gam, 3, 3, seed=7)
    field = np.random.default_rng(1).standard_normal((nxx, nzz)).astype(np.float32)
    op = qpstd.LowRank(f)
    out = op.apply(field)
    op.close()
    exact = LR.apply_exact(vp, tao, gam, DT, 10.0, 10.0, field, nxx, nzz)
    assert rel_l2(out, exact) < TOL
