"""ctypes front end of the FP64 oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's cpu_baseline leg import
this module; the product path never does.  It wraps ``oracle/liboracle.so``
(``qpstd_oracle.c``) and the optional reference host objects under
``oracle/_ref/`` that pin the oracle's coefficient setup and revolve schedule.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")

APS, VAPS, ARTM, QRTM = 0, 1, 2, 3
ADVANCE, TAKESHOT, RESTORE, FIRSTURN, YOUTURN, TERMINATE, ERROR = range(7)

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class Shot(C.Structure):
    _fields_ = [
        ("kind", C.c_int), ("nxx", C.c_int), ("nzz", C.c_int), ("pml", C.c_int),
        ("dx", C.c_double), ("dz", C.c_double), ("dt", C.c_double), ("fd", C.c_double),
        ("nt", C.c_int),
        ("vp", _dp), ("rho", _dp), ("bbx", _dp), ("bbz", _dp),
        ("gam", _dp), ("lam", _dp), ("vwd", _dp), ("tao", _dp),
        ("rik", _dp), ("xsg", C.c_int), ("zsg", C.c_int),
        ("nr", C.c_int), ("gxg", _ip), ("gzg", _ip),
        ("etas", C.c_double), ("etar", C.c_double), ("taoc", C.c_double),
        ("snaps", C.c_int),
        ("lr_row", C.c_int), ("lr_col", C.c_int), ("lr_U", _dp), ("lr_Vt", _dp), ("lr_A", _dp),
    ]


def build() -> None:
    subprocess.run(["make", "-s", "-C", HERE], check=True)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        L.orc_fft1d.argtypes = [C.c_int, _dp, C.c_int]
        L.orc_pml_coeffs.argtypes = [C.c_int, C.c_double, C.c_int, C.c_int, C.c_double,
                                     C.c_double, C.c_double] + [_dp] * 8
        L.orc_shift_tables.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double] + [_dp] * 8
        L.orc_k2d.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double] + [_dp] * 4
        L.orc_ricker.argtypes = [C.c_int, C.c_double, C.c_double, C.c_int, _dp]
        L.orc_bbx_bbz.argtypes = [C.c_int, C.c_int, _dp, _dp, _dp]
        L.orc_transfermodel.argtypes = [C.c_int, C.c_double, C.c_double] + [_dp] * 6
        L.orc_numforw.argtypes = [C.c_int, C.c_int]
        L.orc_revolve_trace.argtypes = [C.c_int, C.c_int, _ip, C.c_int]
        L.orc_model_shot.argtypes = [C.POINTER(Shot), _dp, _dp]
        L.orc_model_steps.argtypes = [C.POINTER(Shot), _dp, C.c_int, C.c_int, _dp]
        L.orc_rtm_shot.argtypes = [C.POINTER(Shot), _dp, _dp, _dp]
        L.orc_filter_image.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, _dp, _dp]
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(_dp)


def _i(a):
    return a.ctypes.data_as(_ip)


def fft1d(x: np.ndarray, sign: int = -1) -> np.ndarray:
    buf = np.ascontiguousarray(x, dtype=np.complex128).copy()
    rc = lib().orc_fft1d(buf.size, buf.view(np.float64).ctypes.data_as(_dp), sign)
    assert rc == 0
    return buf


def pml_coeffs(pml, fm, nxx, nzz, dx, dz, dt):
    out = [np.zeros(nxx) if k % 4 < 2 else np.zeros(nzz) for k in range(8)]
    # order: i_ax, i_bx, i_az, i_bz, h_ax, h_bx, h_az, h_bz
    out = [np.zeros(nxx), np.zeros(nxx), np.zeros(nzz), np.zeros(nzz),
           np.zeros(nxx), np.zeros(nxx), np.zeros(nzz), np.zeros(nzz)]
    lib().orc_pml_coeffs(pml, fm, nxx, nzz, dx, dz, dt, *[_d(a) for a in out])
    return dict(zip(["i_ax", "i_bx", "i_az", "i_bz", "h_ax", "h_bx", "h_az", "h_bz"], out))


def shift_tables(nxx, nzz, dx, dz):
    names = ["kxsmr", "kxscr", "kzsmr", "kzscr", "kxsmi", "kxsci", "kzsmi", "kzsci"]
    out = [np.zeros(nxx if n[1] == "x" else nzz) for n in names]
    lib().orc_shift_tables(nxx, nzz, dx, dz, *[_d(a) for a in out])
    return dict(zip(names, out))


def k2d(nxx, nzz, dx, dz):
    out = [np.zeros(nxx * nzz) for _ in range(4)]
    lib().orc_k2d(nxx, nzz, dx, dz, *[_d(a) for a in out])
    return dict(zip(["k2d1", "k2d2", "k2d3", "k2da"], out))


def ricker(nt, dt, fd, flag=2):
    out = np.zeros(nt)
    lib().orc_ricker(nt, dt, fd, flag, _d(out))
    return out


def bbx_bbz(nxx, nzz, rho):
    rho = np.ascontiguousarray(rho, dtype=np.float64).ravel()
    bbx, bbz = np.zeros(nxx * nzz), np.zeros(nxx * nzz)
    lib().orc_bbx_bbz(nxx, nzz, _d(rho), _d(bbx), _d(bbz))
    return bbx, bbz


def transfermodel(fd, fo, vp, qp):
    vp = np.ascontiguousarray(vp, dtype=np.float64).ravel()
    qp = np.ascontiguousarray(qp, dtype=np.float64).ravel()
    n = vp.size
    gam, lam, vwd, tao = (np.zeros(n) for _ in range(4))
    lib().orc_transfermodel(n, fd, fo, _d(vp), _d(qp), _d(gam), _d(lam), _d(vwd), _d(tao))
    return gam, lam, vwd, tao


def numforw(steps, snaps):
    return lib().orc_numforw(steps, snaps)


def revolve_trace(steps, snaps, cap=1 << 20):
    out = np.zeros(3 * cap, dtype=np.int32)
    n = lib().orc_revolve_trace(steps, snaps, _i(out), cap)
    assert n > 0
    return out[: 3 * n].reshape(n, 3)


class OracleShot:
    """Keeps the numpy arrays behind an orc_shot alive."""

    def __init__(self, d: dict):
        self.arrays = {}
        s = Shot()
        for k in ("kind", "nxx", "nzz", "pml", "nt", "xsg", "zsg", "snaps"):
            setattr(s, k, int(d.get(k, 0)))
        for k in ("dx", "dz", "dt", "fd", "etas", "etar", "taoc"):
            setattr(s, k, float(d.get(k, 0.0)))
        for k in ("vp", "rho", "bbx", "bbz", "gam", "lam", "vwd", "tao", "rik"):
            if d.get(k) is not None:
                a = np.ascontiguousarray(d[k], dtype=np.float64).ravel()
                self.arrays[k] = a
                setattr(s, k, _d(a))
        lr = d.get("lowrank")
        if lr is not None:
            # low-rank factors {"U": N x col, "V": row x nxh*nzh, "A": col x row}
            from lowrank import mirror
            U = np.ascontiguousarray(lr["U"], dtype=np.float64)
            A = np.ascontiguousarray(lr["A"], dtype=np.float64)
            Vt = np.ascontiguousarray(mirror(lr["V"], d["nxx"], d["nzz"]).reshape(A.shape[1], -1))
            self.arrays.update(lr_U=U, lr_Vt=Vt, lr_A=A)
            s.lr_row, s.lr_col = A.shape[1], A.shape[0]
            s.lr_U, s.lr_Vt, s.lr_A = _d(U), _d(Vt), _d(A)
        gx = np.ascontiguousarray(d["gxg"], dtype=np.int32)
        gz = np.ascontiguousarray(d["gzg"], dtype=np.int32)
        self.arrays["gxg"], self.arrays["gzg"] = gx, gz
        s.nr, s.gxg, s.gzg = gx.size, _i(gx), _i(gz)
        self.s = s
        self.d = d

    def model(self, want_state=False):
        d = self.d
        g = np.zeros(d["nt"] * self.s.nr)
        st = np.zeros(8 * d["nxx"] * d["nzz"]) if want_state else None
        rc = lib().orc_model_shot(C.byref(self.s), _d(g), _d(st) if st is not None else None)
        assert rc == 0
        g = g.reshape(d["nt"], self.s.nr)
        if want_state:
            return g, st.reshape(8, d["nxx"], d["nzz"])
        return g

    def steps(self, state, t0, nsteps, want_gather=True):
        st = np.ascontiguousarray(state, dtype=np.float64).copy().ravel()
        g = np.zeros(nsteps * self.s.nr) if want_gather else None
        rc = lib().orc_model_steps(C.byref(self.s), _d(st), t0, nsteps,
                                    _d(g) if g is not None else None)
        assert rc == 0
        st = st.reshape(8, self.d["nxx"], self.d["nzz"])
        return (st, g.reshape(nsteps, self.s.nr)) if want_gather else st

    def rtm(self, obs):
        d = self.d
        nx, nz = d["nxx"] - 2 * d["pml"], d["nzz"] - 2 * d["pml"]
        obs = np.ascontiguousarray(obs, dtype=np.float64).ravel()
        img, ssg = np.zeros(nx * nz), np.zeros(nx * nz)
        n = lib().orc_rtm_shot(C.byref(self.s), _d(obs), _d(img), _d(ssg))
        assert n >= 0
        return img.reshape(nx, nz), ssg.reshape(nx, nz), n


def filter_image(img, dx, dz):
    img = np.ascontiguousarray(img, dtype=np.float64)
    nx, nz = img.shape
    out = np.zeros_like(img)
    lib().orc_filter_image(nx, nz, dx, dz, _d(img), _d(out))
    return out


# ---- reference host objects (only where the reference was compiled) --------
def ref_lib(name: str):
    path = os.path.join(REF_DIR, f"libref_{name}.so")
    if not os.path.exists(path):
        return None
    return C.CDLL(path)
