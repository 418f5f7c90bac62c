"""Known answers of the wave physics, on the GPU path (the parity tests pin
the kernels to the FP64 oracle; these pin what both compute to the physics
the reference's equations describe).

* CPML: a trace near the absorbing boundary of a small homogeneous grid equals
  the same trace on a grid large enough that no boundary is reached, to 1 %.
* Constant Q: in a homogeneous medium the spectral ratio of a trace with
  quality factor Q to the same trace with Q -> infinity decays as
  exp(-pi f t / Q), t the travel time (Zhu-Harris fractional-Laplacian model,
  the reference's vaps equations).
* Reciprocity: swapping source and receiver in a layered medium leaves the
  trace unchanged (pressure source, pressure receiver), to 1 %.
"""
import numpy as np
import pytest

import qpstd
import workloads as W
from cases import rel_l2

pytestmark = pytest.mark.gpu
DX, DT, FD = 10.0, 0.001, 20.0


def shot(kind, vp, qp, pml, nt, src, recs, rho=None):
    """A shot on the padded grid of (nx, nz) interior models; src, recs in interior cells."""
    nx, nz = vp.shape
    rho = W.gardner(vp) if rho is None else rho
    models = {"vp": vp, "rho": rho}
    models["bbx"], models["bbz"] = W.bbx_bbz(rho)
    if kind in (qpstd.VAPS, qpstd.QRTM):
        models["gam"], models["lam"], models["vwd"], models["tao"] = W.transfermodel(FD, FD, vp, qp)
    d = dict(kind=kind, nxx=nx + 2 * pml, nzz=nz + 2 * pml, pml=pml, dx=DX, dz=DX, dt=DT, fd=FD, nt=nt,
             rik=W.ricker(nt, DT, FD, 2), xsg=src[0] + pml, zsg=src[1] + pml,
             gxg=np.array([r[0] + pml for r in recs], dtype=np.int32),
             gzg=np.array([r[1] + pml for r in recs], dtype=np.int32), snaps=10, etas=1e-20, etar=1e-20, taoc=0.0)
    for k, a in models.items():
        d[k] = W.expand_pml_areas(np.pad(a, pml), pml).ravel()
    return d


def test_cpml_absorbs():
    v = np.full((120, 120), 2000.0)
    small = qpstd.model_shot(shot(qpstd.APS, v, None, 20, 450, (60, 60), [(8, 60), (60, 8), (8, 8)]))
    vb = np.full((420, 420), 2000.0)
    big = qpstd.model_shot(shot(qpstd.APS, vb, None, 20, 450, (210, 210), [(158, 210), (210, 158), (158, 158)]))
    for j in range(3):
        assert rel_l2(small[:, j], big[:, j]) < 0.01, j


def test_constant_q_amplitude_decay():
    nx, nz, nt = 160, 60, 700
    v = np.full((nx, nz), 2000.0)
    r = 60                                     # cells between source and receiver
    rec = [(20 + r, 30)]
    q = 40.0
    lossy = qpstd.model_shot(shot(qpstd.VAPS, v, np.full((nx, nz), q), 30, nt, (20, 30), rec))[:, 0]
    clear = qpstd.model_shot(shot(qpstd.VAPS, v, np.full((nx, nz), 1e7), 30, nt, (20, 30), rec))[:, 0]
    f = np.fft.rfftfreq(nt, DT)
    band = (f > 12.0) & (f < 30.0)
    ratio = np.abs(np.fft.rfft(lossy))[band] / np.abs(np.fft.rfft(clear))[band]
    t = r * DX / 2000.0
    expect = np.exp(-np.pi * f[band] * t / q)
    assert np.max(np.abs(np.log(ratio) - np.log(expect))) < 0.15 * np.max(np.abs(np.log(expect)))


def test_reciprocity():
    # source and receiver in one homogeneous top layer (equal rho vp^2 at both:
    # the source is added to p, so unequal moduli would scale the two traces),
    # two layers and an off-centre anomaly below
    nx, nz = 150, 80
    z = np.arange(nz)[None, :]
    vp = np.where(z < 30, 2000.0, np.where(z < 55, 3000.0, 2500.0)) * np.ones((nx, 1))
    X, Z = np.meshgrid(np.arange(nx), np.arange(nz), indexing="ij")
    vp = vp + 400.0 * np.exp(-((X - 100) ** 2 + (Z - 66) ** 2) / (2 * 8.0 ** 2)) * (Z >= 55)
    a, b = (30, 10), (118, 20)
    ab = qpstd.model_shot(shot(qpstd.APS, vp, None, 20, 600, a, [b]))[:, 0]
    ba = qpstd.model_shot(shot(qpstd.APS, vp, None, 20, 600, b, [a]))[:, 0]
    assert rel_l2(ab, ba) < 0.02
