"""The native programs end to end on the GPU (constant-q-pstd_gb300/cli/).

A project tree laid out as the reference's (input/, geometry/, output/,
obsdata/, and the programs run from a sibling directory) is generated with
the `geometry` program and seeded layered models; then

* aps / vaps write one gather per shot; each equals the same shot run through
  the C ABI with the window, source wavelet and buoyancy computed in Python
  from the same files (relative L2 1e-6), one aps shot is checked against the
  FP64 oracle (1e-4), and the serial, server and snapshot paths agree;
* artm reads the aps gathers as observed data and its RTM.BIN equals the
  per-shot pipeline (direct wave removed, RTM, filter, aperture mute,
  projection, sum) done in Python (1e-5);
* qrtm split over two processes and summed with `qpstd sum` equals one
  process (1e-6).
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
BIN = os.path.join(PKG, "bin")
NXT, NZT, DX, PML, TMAX, FD, FO = 150, 40, 10.0, 10, 180, 25.0, 200.0
GEOM = (3, 300.0, 400.0, 20.0, 20.0, 200.0, 10.0, DX, DX, NXT, NZT)  # shots 300, 700, 1100 m
fp = C.POINTER(C.c_float)


def pf(a):
    return a.ctypes.data_as(fp)


def host():
    L = C.CDLL(os.path.join(PKG, "libqpstd_host.so"))
    L.qpcli_cal_bbx_bbz.argtypes = [C.c_int, C.c_int, fp, fp, fp]
    L.qpcli_rik_cal.argtypes = [C.c_int, C.c_float, C.c_float, C.c_int, fp]
    L.qpcli_transfermodel.argtypes = [C.c_int, C.c_float, C.c_float] + [fp] * 6
    L.removedirect.argtypes = [C.c_int, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, C.c_float, fp, fp,
                               C.c_float, fp]
    L.projectomodel.argtypes = [C.c_int, C.c_float, C.c_float] + [C.c_int] * 6 + [fp, fp]
    return L


def _params(path, fields):
    with open(path, "w") as f:
        for k, v in enumerate(fields):
            f.write(f"--value {k}\n  {v}\n")


@pytest.fixture(scope="module")
def tree():
    d = tempfile.mkdtemp(prefix="qp", dir="/tmp")
    for sub in ("input", "geometry", "output", "obsdata", "run"):
        os.makedirs(os.path.join(d, sub))
    vp, qp = W.layered_model(NXT, NZT, 4, 1, 91)
    vp, qp = vp.astype(np.float32), qp.astype(np.float32)
    rho = W.gardner(vp).astype(np.float32)
    vpm = W.smooth(vp, 4.0).astype(np.float32)
    for name, a in (("vp", vp), ("vpm", vpm), ("rho", rho), ("qp", qp)):
        np.ascontiguousarray(a).tofile(os.path.join(d, "output", name + ".bin"))
    labels = ["shots", "first x", "interval", "shot depth", "receiver depth", "offset", "trace interval", "dx",
              "dz", "nx", "nz"]
    with open(os.path.join(d, "geometry", "parameters.txt"), "w") as f:
        for lab, v in zip(labels, GEOM):
            f.write(f"-- {lab}\n   {v}\n")
    subprocess.run([os.path.join(BIN, "geometry")], cwd=os.path.join(d, "geometry"), check=True,
                   capture_output=True)
    g = ["../geometry/tracenum.bin", "../geometry/shotxp.bin", "../geometry/shotzp.bin", "../geometry/gxp",
         "../geometry/gzp"]
    head = [GEOM[0], TMAX, 1.0, FD]
    grid = [NXT, NZT, DX, DX, 0.0]
    _params(os.path.join(d, "input", "ac2drealmodeling.txt"), head + grid + g + ["../output/vp.bin",
                                                                                  "../output/rho.bin", 0, 2])
    _params(os.path.join(d, "input", "visac2drealmodeling.txt"),
            head + [FO] + grid + g + ["../output/vp.bin", "../output/rho.bin", "../output/qp.bin", 0, 2])
    _params(os.path.join(d, "input", "ac2drtm.txt"),
            head + grid + [1500.0] + g + ["../output/vpm.bin", "../output/rho.bin", "../obsdata/reca", 2, 6])
    _params(os.path.join(d, "input", "visac2drtm.txt"),
            head + [FO] + grid + [1500.0, 1e4, 1e4] + g + ["../output/vpm.bin", "../output/rho.bin",
                                                           "../output/qp.bin", "../obsdata/recva", 2, 6])
    yield dict(dir=d, vp=vp, vpm=vpm, rho=rho, qp=qp)
    shutil.rmtree(d, ignore_errors=True)


def run(t, prog, *args):
    """Runs a program by its link name (aps, ..., geometry) or a qpstd subcommand (sum)."""
    cmd = [os.path.join(BIN, prog)] if os.path.exists(os.path.join(BIN, prog)) else [os.path.join(PKG, "qpstd"), prog]
    r = subprocess.run(cmd + list(args), cwd=os.path.join(t["dir"], "run"), capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    return r.stdout


def geometry(t, sid):
    rd = lambda n, ty: np.fromfile(os.path.join(t["dir"], "geometry", n), dtype=ty)
    return (rd("shotxp.bin", np.float32)[sid], rd("shotzp.bin", np.float32)[sid], rd(f"gxp{sid}.bin", np.float32),
            rd(f"gzp{sid}.bin", np.float32))


def full_models(t, kind, vp):
    L = host()
    n = NXT * NZT
    bbx, bbz = np.zeros(n, np.float32), np.zeros(n, np.float32)
    L.qpcli_cal_bbx_bbz(NXT, NZT, pf(t["rho"]), pf(bbx), pf(bbz))
    m = {"vp": vp, "rho": t["rho"], "bbx": bbx, "bbz": bbz}
    if kind in (qpstd.VAPS, qpstd.QRTM):
        out = [np.zeros(n, np.float32) for _ in range(4)]
        L.qpcli_transfermodel(n, FD, FO, pf(vp), pf(t["qp"]), *[pf(a) for a in out])
        m.update(zip(["gam", "lam", "vwd", "tao"], out))
    return {k: np.asarray(v, np.float64).reshape(NXT, NZT) for k, v in m.items()}


def desc(t, kind, sid, vp):
    L = host()
    dt = float(np.float32(1.0 / 1000.0))
    rik = np.zeros(TMAX, np.float32)
    L.qpcli_rik_cal(TMAX, dt, FD, 2, pf(rik))
    xs, zs, gx, gz = geometry(t, sid)
    win, nx, nz, xsg, zsg, gxg, gzg = W.window_shot(full_models(t, kind, vp), float(xs), float(zs), gx, gz, PML,
                                                    DX, DX, GEOM[5])
    d = dict(kind=kind, nxx=nx + 2 * PML, nzz=nz + 2 * PML, pml=PML, dx=DX, dz=DX, dt=dt, fd=FD, nt=TMAX, rik=rik,
             xsg=xsg, zsg=zsg, gxg=gxg, gzg=gzg, snaps=6, etas=1e4, etar=1e4, taoc=0.0)
    for k, v in win.items():
        d[k] = v.ravel()
    if kind == qpstd.QRTM:
        d["taoc"] = float(np.float32(win["tao"]).max())
    return d, nx


def gather(t, pre, sid, nr):
    return np.fromfile(os.path.join(t["dir"], "obsdata", f"{pre}{sid}_{nr}.bin"), dtype=np.float32)


@pytest.mark.parametrize("prog,kind,pre", [("aps", qpstd.APS, "reca"), ("vaps", qpstd.VAPS, "recva")])
def test_modeling_program_writes_the_c_abi_gathers(tree, prog, kind, pre):
    run(tree, prog, "--serial")
    serial = {s: gather(tree, pre, s, 41).copy() for s in range(GEOM[0])}
    out = run(tree, prog)
    assert "The cost of the run time is" in out
    for sid in range(GEOM[0]):
        got = gather(tree, pre, sid, 41)
        d, nx = desc(tree, kind, sid, tree["vp"])
        assert nx == 41
        ref = qpstd.model_shot(d).ravel()
        assert got.size == ref.size == TMAX * 41
        assert rel_l2(got, ref) < 1e-6, sid
        assert rel_l2(serial[sid], got) < 1e-6, sid
        if kind == qpstd.APS and sid == 1:
            assert rel_l2(got, O.OracleShot(d).model().ravel()) < 1e-4


@pytest.mark.parametrize("extra", [["--plain"], ["--plain", "--serial"]])
def test_plain_form_through_the_programs(tree, extra):
    """The cuFFT plain form (--plain) on both program paths matches the fused gathers."""
    run(tree, "aps")
    fused = {s: gather(tree, "reca", s, 41).copy() for s in range(GEOM[0])}
    run(tree, "aps", *extra)
    for sid in range(GEOM[0]):
        assert rel_l2(gather(tree, "reca", sid, 41), fused[sid]) < 1e-5, sid


def test_snapshot_output_every_tenth_step(tree):
    d = tree["dir"]
    path = os.path.join(d, "input", "ac2drealmodeling.txt")
    txt = open(path).read()
    try:
        open(path, "w").write(txt.replace("--value 16\n  0\n", "--value 16\n  1\n"))
        run(tree, "aps")
    finally:
        open(path, "w").write(txt)
    nsnap = (TMAX - 1) // 10 + 1
    for sid in range(GEOM[0]):
        snap = np.fromfile(os.path.join(d, "obsdata", f"snapa{sid}_{NZT}_41.bin"), dtype=np.float32)
        assert snap.size == nsnap * 41 * NZT
        assert np.isfinite(snap).all() and np.abs(snap[-41 * NZT:]).max() > 0
        dd, _ = desc(tree, qpstd.APS, sid, tree["vp"])
        assert rel_l2(gather(tree, "reca", sid, 41), qpstd.model_shot(dd).ravel()) < 1e-6


def test_rtm_program_sums_the_shot_images(tree):
    run(tree, "aps")
    run(tree, "artm")
    got = np.fromfile(os.path.join(tree["dir"], "run", "RTM.BIN"), dtype=np.float32)
    L = host()
    img_sp = np.zeros(NXT * NZT, np.float32)
    ssg_sp = np.zeros(NXT * NZT, np.float32)
    for sid in range(GEOM[0]):
        xs, zs, gx, gz = geometry(tree, sid)
        d, nx = desc(tree, qpstd.ARTM, sid, tree["vpm"])
        obs = gather(tree, "reca", sid, nx).copy()
        L.removedirect(nx, TMAX, nx, d["dt"], FD, xs, zs, pf(gx), pf(gz), 1500.0, pf(obs))
        img, ssg = qpstd.rtm_shot(d, obs.reshape(TMAX, nx))
        imgf = qpstd.filter_image(img, DX, DX)
        lg, rg = int(d["gxg"].min()) - PML, int(d["gxg"].max()) - PML
        imgf[:max(lg, 0), :] = 0.0
        imgf[max(rg, 0):, :] = 0.0
        for src, acc in ((imgf, img_sp), (ssg, ssg_sp)):
            pj = np.zeros(NXT * NZT, np.float32)
            L.projectomodel(PML, float(xs) - GEOM[5], DX, NXT, NZT, nx, NZT, nx + 2 * PML, NZT + 2 * PML, pf(pj),
                            pf(np.ascontiguousarray(src.ravel(), dtype=np.float32)))
            acc += pj
    assert got.size == 2 * NXT * NZT
    assert np.abs(img_sp).max() > 0
    assert rel_l2(got[:NXT * NZT], img_sp) < 1e-5
    assert rel_l2(got[NXT * NZT:], ssg_sp) < 1e-5


def test_qrtm_over_two_processes_sums_to_one(tree):
    run(tree, "vaps")
    run(tree, "qrtm")
    one = np.fromfile(os.path.join(tree["dir"], "run", "QRTM.BIN"), dtype=np.float32).copy()
    for r in (0, 1):
        run(tree, "qrtm", "--rank", str(r), "--nranks", "2")
    run(tree, "sum", "QRTM2.BIN", "QRTM.BIN.rank0", "QRTM.BIN.rank1")
    two = np.fromfile(os.path.join(tree["dir"], "run", "QRTM2.BIN"), dtype=np.float32)
    assert np.abs(one).max() > 0 and np.isfinite(one).all()
    assert rel_l2(two, one) < 1e-6
