"""Reference-signature acforward shims (constant-q-pstd_gb300/shims/).

A C harness (tests/shims/harness.c) stands in for each program's main: it
fills the shot table of struct MultiGPU, passes full models, geometry files and
coefficient tables exactly as the reference's mains do, and calls the shim's
acforward; the program's host helpers come from the oracle's restatement
(oracle/host_helpers.c, pinned to the reference).  The outputs -- gather files
in ../obsdata for aps / vaps, the summed projected image and illumination for
artm / qrtm -- are compared with the same shots run through the C ABI directly,
windowed by workloads.window_shot.  The shim recovers the CPML frequency from
the tables, so the tolerance is relative L2 1e-5.
"""
import ctypes as C
import os
import shutil
import subprocess
import tempfile

import numpy as np
import pytest

import oracle as O
import qpstd
import workloads as W
from cases import rel_l2

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "constant-q-pstd_gb300")
TOL = 1e-5
NXT, NZT, PML, DX, DT, FD, TMAX, SROFF = 150, 40, 10, 10.0, 0.001, 25.0, 180, 200.0
SHOTS = [(0, 500.0, 20.0), (3, 1100.0, 20.0), (5, 1400.0, 20.0)]   # the last window runs off the model


def _harness(prog, out):
    obj = os.path.join(out, f"h_{prog}.o")
    exe = os.path.join(out, f"h_{prog}")
    subprocess.run(["gcc", "-O1", "-std=gnu11", "-c", f"-DPROG_{prog.upper()}",
                    os.path.join(ROOT, "tests", "shims", "harness.c"), "-o", obj], check=True)
    subprocess.run(["g++", obj, os.path.join(PKG, "_build", f"acforward_{prog}.o"), "-o", exe,
                    "-L" + PKG, "-lqpstd", "-L" + os.path.join(ROOT, "oracle"), "-loracle", "-lm",
                    "-Wl,-rpath," + PKG, "-Wl,-rpath," + os.path.join(ROOT, "oracle")], check=True)
    return exe


def _setup(kind):
    d = tempfile.mkdtemp(prefix="qs", dir="/tmp")   # short: the programs' file names are char[40]
    for sub in ("in", "out", "run", "obsdata"):
        os.makedirs(os.path.join(d, sub))
    models = {k: np.asarray(v, dtype=np.float32) for k, v in W.parent_model(NXT, NZT, 77, nlayers=4, nanom=1).items()}
    nx = int(2.0 * SROFF / DX + 1.5)
    nxx, nzz = nx + 2 * PML, NZT + 2 * PML
    nr = nx
    rik = W.ricker(TMAX, DT, FD, 2).astype(np.float32)
    wr = lambda name, a: np.ascontiguousarray(a).tofile(os.path.join(d, "in", name))
    for k in ("vp", "rho", "bbx", "bbz", "gam", "lam", "vwd", "tao"):
        wr(k + ".bin", models[k])
    wr("rik.bin", rik)
    wr("shots.bin", np.array([[s, x, z] for s, x, z in SHOTS], dtype=np.float32))
    tr = np.zeros(64, dtype=np.int32)
    geo = {}
    for sid, xs, zs in SHOTS:
        gx = (xs - SROFF + DX * np.arange(nr)).astype(np.float32)
        gz = np.full(nr, 2 * DX, dtype=np.float32)
        wr(f"gxp{sid}.bin", gx)
        wr(f"gzp{sid}.bin", gz)
        tr[sid] = nr
        geo[sid] = (gx, gz)
    wr("tracenum.bin", tr)
    params = [TMAX, DT, len(SHOTS), nr, nx, NZT, nxx, nzz, PML, DX, DX, SROFF, 0.0, NXT, NZT, FD, 6, 25.0, 1500.0,
              1e4, 1e4, 0]
    with open(os.path.join(d, "in", "params.txt"), "w") as f:
        f.write(" ".join(str(p) for p in params) + "\n")
    return d, models, geo, rik, nx, nxx, nzz


def _desc(kind, models, geo, sid, xs, zs, rik):
    keys = ("vp", "rho", "bbx", "bbz") + (("gam", "lam", "vwd", "tao") if kind in (qpstd.VAPS, qpstd.QRTM) else ())
    full = {k: models[k].reshape(NXT, NZT).astype(np.float64) for k in keys}
    gx, gz = geo[sid]
    win, nx, nz, xsg, zsg, gxg, gzg = W.window_shot(full, xs, zs, gx, gz, PML, DX, DX, SROFF)
    d = dict(kind=kind, nxx=nx + 2 * PML, nzz=nz + 2 * PML, pml=PML, dx=DX, dz=DX, dt=DT, fd=FD, nt=TMAX, rik=rik,
             xsg=xsg, zsg=zsg, gxg=gxg, gzg=gzg, snaps=6, etas=1e4, etar=1e4, taoc=0.0)
    for k, v in win.items():
        d[k] = v.ravel()
    if kind == qpstd.QRTM:
        d["taoc"] = float(np.float32(win["tao"]).max())
    return d


@pytest.fixture(scope="module")
def exes():
    out = tempfile.mkdtemp(prefix="qh", dir="/tmp")
    yield {p: _harness(p, out) for p in ("aps", "vaps", "artm", "qrtm")}
    shutil.rmtree(out, ignore_errors=True)


@pytest.mark.parametrize("prog,kind,pre", [("aps", qpstd.APS, "reca"), ("vaps", qpstd.VAPS, "recva")])
def test_modeling_shim_writes_the_gathers(exes, prog, kind, pre):
    d, models, geo, rik, nx, nxx, nzz = _setup(kind)
    try:
        subprocess.run([exes[prog], d], cwd=os.path.join(d, "run"), check=True, capture_output=True)
        for sid, xs, zs in SHOTS:
            got = np.fromfile(os.path.join(d, "obsdata", f"{pre}{sid}_{nx}.bin"), dtype=np.float32)
            ref = qpstd.model_shot(_desc(kind, models, geo, sid, xs, zs, rik)).ravel()
            assert got.size == ref.size and rel_l2(got, ref) < TOL, sid
    finally:
        shutil.rmtree(d, ignore_errors=True)


@pytest.mark.parametrize("prog,kind,mkind", [("artm", qpstd.ARTM, qpstd.APS), ("qrtm", qpstd.QRTM, qpstd.VAPS)])
def test_rtm_shim_sums_the_projected_images(exes, prog, kind, mkind):
    d, models, geo, rik, nx, nxx, nzz = _setup(kind)
    L = O.lib()
    fp = C.POINTER(C.c_float)
    L.removedirect.argtypes = [C.c_int, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, C.c_float, fp, fp,
                               C.c_float, fp]
    L.projectomodel.argtypes = [C.c_int, C.c_float, C.c_float] + [C.c_int] * 6 + [fp, fp]
    pf = lambda a: a.ctypes.data_as(fp)
    try:
        img_sp = np.zeros(NXT * NZT, dtype=np.float32)
        ssg_sp = np.zeros(NXT * NZT, dtype=np.float32)
        for sid, xs, zs in SHOTS:
            desc = _desc(kind, models, geo, sid, xs, zs, rik)
            obs = qpstd.model_shot(dict(desc, kind=mkind)).astype(np.float32)
            obs.tofile(os.path.join(d, "in", f"obs{sid}_{nx}.bin"))
            o = np.ascontiguousarray(obs.ravel())
            gx, gz = geo[sid]
            L.removedirect(nx, TMAX, nx, DT, 25.0, xs, zs, pf(gx), pf(gz), 1500.0, pf(o))
            img, ssg = qpstd.rtm_shot(desc, o.reshape(TMAX, nx))
            imgf = qpstd.filter_image(img, DX, DX)
            lg, rg = int(desc["gxg"].min()) - PML, int(desc["gxg"].max()) - PML
            imgf[:max(lg, 0), :] = 0.0
            imgf[max(rg, 0):, :] = 0.0
            for src, acc in ((imgf, img_sp), (ssg, ssg_sp)):
                pj = np.zeros(NXT * NZT, dtype=np.float32)
                s = np.ascontiguousarray(src.ravel(), dtype=np.float32)
                L.projectomodel(PML, xs - SROFF, DX, NXT, NZT, nx, NZT, nxx, nzz, pf(pj), pf(s))
                acc += pj
        subprocess.run([exes[prog], d], cwd=os.path.join(d, "run"), check=True, capture_output=True)
        got_img = np.fromfile(os.path.join(d, "out", "img.bin"), dtype=np.float32)
        got_ssg = np.fromfile(os.path.join(d, "out", "ssg.bin"), dtype=np.float32)
        assert rel_l2(got_ssg, ssg_sp) < TOL
        assert rel_l2(got_img, img_sp) < TOL
    finally:
        shutil.rmtree(d, ignore_errors=True)
