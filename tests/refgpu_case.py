"""The shot on which the reference's own cuFFT programs pin the oracle.

TEST INFRASTRUCTURE.  One shot of the 160 x 398 model geometry:
a seeded 398 (x) x 160 (z) layered model (5 layers, one anomaly, Gardner
density, Q per layer in 20..200), dx = dz = 10 m, the source at x = 1990 m,
z = 20 m, 398 receivers at z = 20 m from x = 0 to 3970 m, a 20 Hz Ricker
wavelet, dt = 1 ms, reference frequency 20 Hz.  The reference's window of
that geometry is 399 columns; its programs, as shipped, pad 10 CPML cells
(419 x 180).

`write_tree` lays out the files the reference's mains read (input/*.txt,
geometry/*.bin, output/*.bin, the programs run from run/); `shot_desc`
computes, from the same numbers, the shot the library and the oracle take: the
window, buoyancy, Q transform and wavelet in the reference's float arithmetic
(libqpstd_host, pinned bit for bit to the reference's host C).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

import workloads as W

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "constant-q-pstd_gb300")
NXT, NZT, DX, FD, FO, SEED = 398, 160, 10.0, 20.0, 20.0, 1001
XS, ZS, RDEP, TRDX = 1990.0, 20.0, 20.0, 10.0
APS, VAPS = 0, 1
fp = C.POINTER(C.c_float)


def pf(a):
    return a.ctypes.data_as(fp)


def models():
    """float32 x-major (NXT, NZT) vp, rho, Q."""
    vp, qp = W.layered_model(NXT, NZT, 5, 1, SEED)
    vp = vp.astype(np.float32)
    return vp, W.gardner(vp).astype(np.float32), qp.astype(np.float32)


def geometry():
    """Receiver x / z positions as geometry2d writes them for this shot
    (offset 1990 m, trace interval 10 m: xlp = 0, xrp = 3970, nr = 398)."""
    xlp, xrp = np.float32(0.0), np.float32(3970.0)
    nr = int((xrp - xlp) / np.float32(TRDX)) + 1
    gx = (xlp + np.arange(nr, dtype=np.float32) * np.float32(TRDX)).astype(np.float32)
    gz = np.full(nr, RDEP, dtype=np.float32)
    return gx, gz


def _params(path, fields):
    with open(path, "w") as f:
        for k, v in enumerate(fields):
            f.write(f"--value {k}\n  {v}\n")


def write_tree(d: str, nt: int) -> None:
    """The reference project layout under d, for one shot of nt steps."""
    for sub in ("input", "geometry", "output", "obsdata", "run"):
        os.makedirs(os.path.join(d, sub), exist_ok=True)
    vp, rho, qp = models()
    for name, a in (("vp", vp), ("rho", rho), ("qp", qp)):
        np.ascontiguousarray(a).tofile(os.path.join(d, "output", name + ".bin"))
    gx, gz = geometry()
    g = os.path.join(d, "geometry")
    np.array([gx.size], dtype=np.int32).tofile(os.path.join(g, "tracenum.bin"))
    np.array([XS], dtype=np.float32).tofile(os.path.join(g, "shotxp.bin"))
    np.array([ZS], dtype=np.float32).tofile(os.path.join(g, "shotzp.bin"))
    gx.tofile(os.path.join(g, "gxp0.bin"))
    gz.tofile(os.path.join(g, "gzp0.bin"))
    names = ["../geometry/tracenum.bin", "../geometry/shotxp.bin", "../geometry/shotzp.bin", "../geometry/gxp",
             "../geometry/gzp"]
    head = [1, nt, 1.0, FD]
    grid = [NXT, NZT, DX, DX, 0.0]
    _params(os.path.join(d, "input", "ac2drealmodeling.txt"),
            head + grid + names + ["../output/vp.bin", "../output/rho.bin", 0, 2])
    _params(os.path.join(d, "input", "visac2drealmodeling.txt"),
            head + [FO] + grid + names + ["../output/vp.bin", "../output/rho.bin", "../output/qp.bin", 0, 2])


def _host():
    L = C.CDLL(os.path.join(PKG, "libqpstd_host.so"))
    L.qpcli_cal_bbx_bbz.argtypes = [C.c_int, C.c_int, fp, fp, fp]
    L.qpcli_rik_cal.argtypes = [C.c_int, C.c_float, C.c_float, C.c_int, fp]
    L.qpcli_transfermodel.argtypes = [C.c_int, C.c_float, C.c_float] + [fp] * 6
    return L


def shot_desc(kind: int, nt: int, pml: int) -> dict:
    """The shot as the reference's acforward sets it up (window, CPML padding,
    source and receiver indices), in the library's / oracle's dict form."""
    L = _host()
    vp, rho, qp = models()
    n = NXT * NZT
    bbx, bbz = np.zeros(n, np.float32), np.zeros(n, np.float32)
    L.qpcli_cal_bbx_bbz(NXT, NZT, pf(rho), pf(bbx), pf(bbz))
    full = {"vp": vp, "rho": rho, "bbx": bbx, "bbz": bbz}
    if kind == VAPS:
        out = [np.zeros(n, np.float32) for _ in range(4)]
        L.qpcli_transfermodel(n, FD, FO, pf(vp), pf(np.ascontiguousarray(qp)), *[pf(a) for a in out])
        full.update(zip(["gam", "lam", "vwd", "tao"], out))
    full = {k: np.asarray(v, np.float64).reshape(NXT, NZT) for k, v in full.items()}
    dt = float(np.float32(1.0 / 1000.0))
    rik = np.zeros(nt, np.float32)
    L.qpcli_rik_cal(nt, dt, FD, 2, pf(rik))
    gx, gz = geometry()
    sroffmx = float(max(abs(gx.max() - np.float32(XS)), abs(np.float32(XS) - gx.min())))
    win, nx, nz, xsg, zsg, gxg, gzg = W.window_shot(full, XS, ZS, gx, gz, pml, DX, DX, sroffmx)
    d = dict(kind=kind, nxx=nx + 2 * pml, nzz=nz + 2 * pml, pml=pml, dx=DX, dz=DX, dt=dt, fd=FD, nt=nt, rik=rik,
             xsg=xsg, zsg=zsg, gxg=gxg, gzg=gzg, snaps=4, etas=1e-20, etar=1e-20, taoc=0.0)
    for k, v in win.items():
        d[k] = v.ravel()
    return d
