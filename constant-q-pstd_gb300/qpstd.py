"""Python front end of libqpstd (the GB300 Constant-Q-PSTD hot path).

ctypes bindings of ``include/qpstd.h`` plus numpy helpers.  The CUDA library is
the only implementation: if ``libqpstd.so`` is missing or cannot be loaded,
every call raises -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libqpstd.so")

APS, VAPS, ARTM, QRTM = 0, 1, 2, 3
FUSED, PLAIN = 0, 1

_fp = C.POINTER(C.c_float)
_ip = C.POINTER(C.c_int)
_dp = C.POINTER(C.c_double)


class ShotDesc(C.Structure):
    _fields_ = [
        ("kind", C.c_int), ("method", C.c_int),
        ("nxx", C.c_int), ("nzz", C.c_int), ("pml", C.c_int),
        ("dx", C.c_float), ("dz", C.c_float), ("dt", C.c_float), ("fd", C.c_float),
        ("nt", C.c_int),
        ("vp", _fp), ("rho", _fp), ("bbx", _fp), ("bbz", _fp),
        ("gam", _fp), ("lam", _fp), ("vwd", _fp), ("tao", _fp),
        ("rik", _fp), ("xsg", C.c_int), ("zsg", C.c_int),
        ("nr", C.c_int), ("gxg", _ip), ("gzg", _ip),
        ("etas", C.c_float), ("etar", C.c_float), ("taoc", C.c_float),
        ("snaps", C.c_int),
    ]


class QpstdError(RuntimeError):
    pass


def build(verbose: bool = False) -> None:
    """Compile libqpstd.so in-tree for sm_103a (nvcc; no GPU needed)."""
    jobs = str(min(8, os.cpu_count() or 1))
    out = None if verbose else subprocess.DEVNULL
    subprocess.run(["make", "-s", "-j", jobs, "-C", HERE], check=True, stdout=out)


_lib = None

EXPORTS = {
    "qpstd_last_error": (C.c_char_p, []),
    "qpstd_version": (C.c_int, []),
    "qpstd_model_shot": (C.c_int, [C.POINTER(ShotDesc), _fp, _fp]),
    "qpstd_rtm_shot": (C.c_int, [C.POINTER(ShotDesc), _fp, _fp, _fp]),
    "qpstd_filter_image": (C.c_int, [C.c_int, C.c_int, C.c_float, C.c_float, _fp, _fp]),
    "qpstd_normalize_image": (C.c_int, [C.c_int, C.c_int, C.c_float, _fp, _fp, _fp]),
    "qpstd_shot_create": (C.c_int, [C.POINTER(ShotDesc), C.POINTER(C.c_void_p)]),
    "qpstd_shot_destroy": (C.c_int, [C.c_void_p]),
    "qpstd_shot_set_state": (C.c_int, [C.c_void_p, _fp]),
    "qpstd_shot_get_state": (C.c_int, [C.c_void_p, _fp]),
    "qpstd_shot_advance": (C.c_int, [C.c_void_p, C.c_int, C.c_int, _fp]),
    "qpstd_shot_advance_device": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "qpstd_shot_launch_count": (C.c_longlong, [C.c_void_p]),
    "qpstd_shot_set_obs": (C.c_int, [C.c_void_p, _fp]),
    "qpstd_shot_rtm_device": (C.c_int, [C.c_void_p]),
    "qpstd_shot_get_image": (C.c_int, [C.c_void_p, _fp, _fp]),
    "qpstd_shot_forward_steps": (C.c_longlong, [C.c_void_p]),
    "qpstd_shot_sync": (C.c_int, [C.c_void_p]),
    "qpstd_shot_stream": (C.c_void_p, [C.c_void_p]),
    "qpstd_shot_pipeline_begin": (C.c_int, [C.c_void_p]),
    "qpstd_shot_pipeline_step": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "qpstd_shot_pipeline_end": (C.c_int, [C.c_void_p]),
    "qpstd_shot_set_profiling": (C.c_int, [C.c_void_p, C.c_int]),
    "qpstd_shot_profile_read": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_longlong)]),
    "qpstd_shot_info": (C.c_longlong, [C.c_void_p, C.c_int]),
    "qpstd_shot_set_lowrank": (C.c_int, [C.c_void_p, C.c_int, C.c_int, _fp, _fp, _dp]),
    "qpstd_pml_profiles": (C.c_int, [C.c_int, C.c_float, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, _fp]),
    "qpstd_batch_create": (C.c_int, [C.POINTER(ShotDesc), C.c_int, C.POINTER(C.c_void_p)]),
    "qpstd_batch_destroy": (C.c_int, [C.c_void_p]),
    "qpstd_batch_size": (C.c_int, [C.c_void_p]),
    "qpstd_batch_shot": (C.c_void_p, [C.c_void_p, C.c_int]),
    "qpstd_batch_sync": (C.c_int, [C.c_void_p]),
    "qpstd_batch_rtm_device": (C.c_int, [C.c_void_p, C.c_int]),
    "qpstd_batch_pipeline_begin": (C.c_int, [C.c_void_p]),
    "qpstd_batch_pipeline_step": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "qpstd_batch_pipeline_end": (C.c_int, [C.c_void_p]),
    "qpstd_rtm_batch": (C.c_int, [C.POINTER(ShotDesc), C.c_int, C.POINTER(_fp), C.POINTER(_fp), C.POINTER(_fp)]),
    "qpstd_ac_advance_noalloc": (C.c_int, [C.POINTER(ShotDesc)] + [C.c_void_p] * 5
                                 + [C.c_int, C.c_int, C.c_void_p, C.c_void_p]),
    "qpstd_lowrank_decompose": (C.c_int, [C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, _fp, _fp, _fp,
                                          C.c_int, C.c_int, C.c_ulonglong, _fp, _fp, _dp, _ip, _ip]),
    "qpstd_lowrank_check": (C.c_int, [C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, C.c_int, C.c_int,
                                      _fp, _dp, _fp, _fp, _fp, _fp, C.c_int, _fp, _fp]),
    "qpstd_lowrank_create": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, _fp, _fp, _dp, C.POINTER(C.c_void_p)]),
    "qpstd_lowrank_destroy": (C.c_int, [C.c_void_p]),
    "qpstd_lowrank_apply": (C.c_int, [C.c_void_p, _fp, _fp]),
    "qpstd_lowrank_apply_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "qpstd_shot_bytes": (C.c_longlong, [C.POINTER(ShotDesc)]),
    "qpstd_server_create": (C.c_int, [C.c_longlong, C.c_int, C.POINTER(C.c_void_p)]),
    "qpstd_server_destroy": (C.c_int, [C.c_void_p]),
    "qpstd_server_submit": (C.c_longlong, [C.c_void_p, C.POINTER(ShotDesc), _fp, _fp, _fp]),
    "qpstd_server_status": (C.c_int, [C.c_void_p, C.c_longlong, C.POINTER(C.c_double), C.POINTER(C.c_int)]),
    "qpstd_server_wait": (C.c_int, [C.c_void_p, C.c_longlong]),
}
KIND_NAMES = ["xpass", "zpass", "xspec", "other", "plain", "xspec_exact"]
# keys of qpstd_shot_info
INFO_KEYS = ["x_conv_m", "x_conv_maxradix", "x_exact_m", "x_exact_blue", "x_spec_conv", "z_exact_m",
             "z_exact_maxradix", "z_conv_m"]


def lib():
    """Load libqpstd.so (raises if it is absent: the CUDA path is mandatory)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise QpstdError(f"{LIB_PATH} not built; run build() (the CUDA library has no fallback)")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in EXPORTS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _check(rc: int) -> None:
    if rc != 0:
        raise QpstdError(f"libqpstd error {rc}: {lib().qpstd_last_error().decode()}")


def _f(a):
    return a.ctypes.data_as(_fp) if a is not None else None


class Desc:
    """Owns the float32/int32 arrays a qpstd_shot_desc points at."""

    def __init__(self, d: dict, method: int = FUSED):
        self.keep = {}
        s = ShotDesc()
        s.kind = int(d["kind"])
        s.method = int(d.get("method", method))
        for k in ("nxx", "nzz", "pml", "nt", "xsg", "zsg", "snaps"):
            setattr(s, k, int(d.get(k, 0)))
        for k in ("dx", "dz", "dt", "fd", "etas", "etar", "taoc"):
            setattr(s, k, float(d.get(k, 0.0)))
        for k in ("vp", "rho", "bbx", "bbz", "gam", "lam", "vwd", "tao", "rik"):
            if d.get(k) is not None:
                a = np.ascontiguousarray(d[k], dtype=np.float32).ravel()
                self.keep[k] = a
                setattr(s, k, _f(a))
        gx = np.ascontiguousarray(d["gxg"], dtype=np.int32)
        gz = np.ascontiguousarray(d["gzg"], dtype=np.int32)
        self.keep["gx"], self.keep["gz"] = gx, gz
        s.nr = gx.size
        s.gxg = gx.ctypes.data_as(_ip)
        s.gzg = gz.ctypes.data_as(_ip)
        self.s = s
        self.d = d


def model_shot(d: dict, method: int = FUSED, want_state: bool = False):
    D = Desc(d, method)
    g = np.zeros((d["nt"], D.s.nr), dtype=np.float32)
    st = np.zeros((8, d["nxx"], d["nzz"]), dtype=np.float32) if want_state else None
    _check(lib().qpstd_model_shot(C.byref(D.s), _f(g), _f(st)))
    return (g, st) if want_state else g


def rtm_shot(d: dict, obs: np.ndarray, method: int = FUSED):
    D = Desc(d, method)
    nx, nz = d["nxx"] - 2 * d["pml"], d["nzz"] - 2 * d["pml"]
    obs = np.ascontiguousarray(obs, dtype=np.float32)
    img = np.zeros((nx, nz), dtype=np.float32)
    ssg = np.zeros((nx, nz), dtype=np.float32)
    _check(lib().qpstd_rtm_shot(C.byref(D.s), _f(obs), _f(img), _f(ssg)))
    return img, ssg


def filter_image(img: np.ndarray, dx: float, dz: float) -> np.ndarray:
    img = np.ascontiguousarray(img, dtype=np.float32)
    out = np.zeros_like(img)
    _check(lib().qpstd_filter_image(img.shape[0], img.shape[1], dx, dz, _f(img), _f(out)))
    return out


def normalize_image(img: np.ndarray, ssg: np.ndarray, sigma2: float = 1e-26) -> np.ndarray:
    img = np.ascontiguousarray(img, dtype=np.float32)
    ssg = np.ascontiguousarray(ssg, dtype=np.float32)
    out = np.zeros_like(img)
    _check(lib().qpstd_normalize_image(img.shape[0], img.shape[1], sigma2, _f(img), _f(ssg), _f(out)))
    return out


class Shot:
    """Device-resident shot (qpstd_shot handle)."""

    def __init__(self, d: dict, method: int = FUSED):
        self.D = Desc(d, method)
        self.h = C.c_void_p()
        _check(lib().qpstd_shot_create(C.byref(self.D.s), C.byref(self.h)))
        self.d = d

    def close(self):
        if self.h:
            lib().qpstd_shot_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_state(self, st):
        st = np.ascontiguousarray(st, dtype=np.float32)
        _check(lib().qpstd_shot_set_state(self.h, _f(st)))

    def get_state(self):
        st = np.zeros((8, self.d["nxx"], self.d["nzz"]), dtype=np.float32)
        _check(lib().qpstd_shot_get_state(self.h, _f(st)))
        return st

    def advance(self, t0: int, n: int, want_gather: bool = True):
        g = np.zeros((n, self.D.s.nr), dtype=np.float32) if want_gather else None
        _check(lib().qpstd_shot_advance(self.h, t0, n, _f(g)))
        return g

    def advance_device(self, t0: int, n: int):
        _check(lib().qpstd_shot_advance_device(self.h, t0, n))

    def launch_count(self) -> int:
        return int(lib().qpstd_shot_launch_count(self.h))

    def set_obs(self, obs):
        obs = np.ascontiguousarray(obs, dtype=np.float32)
        self._obs = obs
        _check(lib().qpstd_shot_set_obs(self.h, _f(obs)))

    def rtm_device(self):
        _check(lib().qpstd_shot_rtm_device(self.h))

    def get_image(self):
        nx, nz = self.d["nxx"] - 2 * self.d["pml"], self.d["nzz"] - 2 * self.d["pml"]
        img = np.zeros((nx, nz), dtype=np.float32)
        ssg = np.zeros((nx, nz), dtype=np.float32)
        _check(lib().qpstd_shot_get_image(self.h, _f(img), _f(ssg)))
        return img, ssg

    def forward_steps(self) -> int:
        return int(lib().qpstd_shot_forward_steps(self.h))

    def sync(self):
        _check(lib().qpstd_shot_sync(self.h))

    def pipeline_begin(self):
        _check(lib().qpstd_shot_pipeline_begin(self.h))

    def pipeline_step(self, t: int, last: bool = False):
        _check(lib().qpstd_shot_pipeline_step(self.h, t, 1 if last else 0))

    def pipeline_end(self):
        _check(lib().qpstd_shot_pipeline_end(self.h))

    def stream_ptr(self) -> int:
        return int(lib().qpstd_shot_stream(self.h) or 0)

    def set_profiling(self, on: bool):
        _check(lib().qpstd_shot_set_profiling(self.h, 1 if on else 0))

    def profile_read(self):
        n = len(KIND_NAMES)
        ms = (C.c_double * n)()
        cnt = (C.c_longlong * n)()
        _check(lib().qpstd_shot_profile_read(self.h, n, ms, cnt))
        return {KIND_NAMES[k]: (ms[k], cnt[k]) for k in range(n)}

    def set_lowrank(self, f: dict):
        """Low-rank form of the pressure term with factors f = lowrank_decompose(...)."""
        shot_set_lowrank(self.h, f)

    def info(self) -> dict:
        """The transforms this shot runs (qpstd_shot_info)."""
        return {k: int(lib().qpstd_shot_info(self.h, i)) for i, k in enumerate(INFO_KEYS)}


class Batch:
    """Several resident shots advancing together (qpstd_batch handle)."""

    def __init__(self, dicts, method: int = FUSED):
        self.D = [Desc(d, method) for d in dicts]
        arr = (ShotDesc * len(dicts))(*[x.s for x in self.D])
        self._arr = arr
        self.h = C.c_void_p()
        _check(lib().qpstd_batch_create(arr, len(dicts), C.byref(self.h)))
        self.dicts = dicts

    def close(self):
        if self.h:
            lib().qpstd_batch_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def shot(self, i: int):
        return C.c_void_p(lib().qpstd_batch_shot(self.h, i))

    def set_obs(self, i: int, obs):
        obs = np.ascontiguousarray(obs, dtype=np.float32)
        setattr(self, f"_obs{i}", obs)
        _check(lib().qpstd_shot_set_obs(self.shot(i), _f(obs)))

    def rtm_device(self, slice_steps: int = 8):
        _check(lib().qpstd_batch_rtm_device(self.h, slice_steps))

    def get_image(self, i: int):
        d = self.dicts[i]
        nx, nz = d["nxx"] - 2 * d["pml"], d["nzz"] - 2 * d["pml"]
        img = np.zeros((nx, nz), dtype=np.float32)
        ssg = np.zeros((nx, nz), dtype=np.float32)
        _check(lib().qpstd_shot_get_image(self.shot(i), _f(img), _f(ssg)))
        return img, ssg

    def sync(self):
        _check(lib().qpstd_batch_sync(self.h))

    def pipeline_begin(self):
        _check(lib().qpstd_batch_pipeline_begin(self.h))

    def pipeline_step(self, t: int, last: bool = False):
        _check(lib().qpstd_batch_pipeline_step(self.h, t, 1 if last else 0))

    def pipeline_end(self):
        _check(lib().qpstd_batch_pipeline_end(self.h))

    def stream_ptrs(self):
        return [int(lib().qpstd_shot_stream(self.shot(i)) or 0) for i in range(len(self.dicts))]


def rtm_batch(dicts, obs_list, method: int = FUSED):
    """One call with host buffers: concurrent RTM of several shots."""
    D = [Desc(d, method) for d in dicts]
    arr = (ShotDesc * len(dicts))(*[x.s for x in D])
    obs = [np.ascontiguousarray(o, dtype=np.float32) for o in obs_list]
    imgs, ssgs = [], []
    for d in dicts:
        nx, nz = d["nxx"] - 2 * d["pml"], d["nzz"] - 2 * d["pml"]
        imgs.append(np.zeros((nx, nz), dtype=np.float32))
        ssgs.append(np.zeros((nx, nz), dtype=np.float32))
    po = (_fp * len(obs))(*[_f(o) for o in obs])
    pi = (_fp * len(imgs))(*[_f(a) for a in imgs])
    ps = (_fp * len(ssgs))(*[_f(a) for a in ssgs])
    _check(lib().qpstd_rtm_batch(arr, len(dicts), po, pi, ps))
    return imgs, ssgs



# ---- low-rank form of the constant-Q symbol ----------------------------------------
def lowrank_decompose(nxx, nzz, dx, dz, dt, vp, tao, gam, row, col, seed=1):
    """FP64 host decomposition (no GPU): dict with U (N1 x col), V (row x N2),
    A (col x row, float64), jrr, irr."""
    nxh, nzh = nxx // 2 + 1, nzz // 2 + 1
    vp, tao, gam = (np.ascontiguousarray(a, dtype=np.float32).ravel() for a in (vp, tao, gam))
    U = np.zeros((nxx * nzz, col), dtype=np.float32)
    V = np.zeros((row, nxh * nzh), dtype=np.float32)
    A = np.zeros((col, row), dtype=np.float64)
    jrr = np.zeros(col, dtype=np.int32)
    irr = np.zeros(row, dtype=np.int32)
    _check(lib().qpstd_lowrank_decompose(nxx, nzz, dx, dz, dt, _f(vp), _f(tao), _f(gam), row, col, seed,
                                         _f(U), _f(V), A.ctypes.data_as(_dp), jrr.ctypes.data_as(_ip),
                                         irr.ctypes.data_as(_ip)))
    return {"U": U, "V": V, "A": A, "jrr": jrr, "irr": irr, "nxx": nxx, "nzz": nzz, "row": row, "col": col}


def shot_set_lowrank(handle, f: dict) -> None:
    """qpstd_shot_set_lowrank on a shot handle (a Shot's .h or Batch.shot(i))."""
    U = np.ascontiguousarray(f["U"], dtype=np.float32)
    V = np.ascontiguousarray(f["V"], dtype=np.float32)
    A = np.ascontiguousarray(f["A"], dtype=np.float64)
    _check(lib().qpstd_shot_set_lowrank(handle, A.shape[1], A.shape[0], _f(U), _f(V), A.ctypes.data_as(_dp)))


def lowrank_factors(dicts, rank: int, threads: int = 0):
    """lowrank_decompose for each shot window (host FP64; the decompositions run
    concurrently, the library releases the interpreter during each)."""
    from concurrent.futures import ThreadPoolExecutor
    run = lambda d: lowrank_decompose(d["nxx"], d["nzz"], d["dx"], d["dz"], d["dt"], d["vp"], d["tao"], d["gam"],
                                      rank, rank)
    with ThreadPoolExecutor(max_workers=threads or min(16, os.cpu_count() or 1)) as ex:
        return list(ex.map(run, dicts))


def lowrank_check(f, dx, dz, dt, vp, tao, gam, point):
    """Exact and approximated rows W(x_point, k) on the half grid (host only)."""
    n2 = f["V"].shape[1]
    We, Wa = np.zeros(n2, dtype=np.float32), np.zeros(n2, dtype=np.float32)
    vp, tao, gam = (np.ascontiguousarray(a, dtype=np.float32).ravel() for a in (vp, tao, gam))
    _check(lib().qpstd_lowrank_check(f["nxx"], f["nzz"], dx, dz, dt, f["row"], f["col"], _f(f["U"]),
                                     f["A"].ctypes.data_as(_dp), _f(f["V"]), _f(vp), _f(tao), _f(gam), point,
                                     _f(We), _f(Wa)))
    return We, Wa


class LowRank:
    """Device operator out = sum_a U[x,a] sum_b A[a,b] Re F^-1[Vt_b F in] / N."""

    def __init__(self, f: dict):
        self.f = f
        self.h = C.c_void_p()
        _check(lib().qpstd_lowrank_create(f["nxx"], f["nzz"], f["row"], f["col"], _f(f["U"]), _f(f["V"]),
                                          f["A"].ctypes.data_as(_dp), C.byref(self.h)))

    def apply(self, field: np.ndarray) -> np.ndarray:
        a = np.ascontiguousarray(field, dtype=np.float32)
        out = np.zeros_like(a)
        _check(lib().qpstd_lowrank_apply(self.h, _f(a), _f(out)))
        return out

    def apply_device(self, d_in: int, d_out: int, stream: int = 0) -> None:
        """Device pointers (nxx*nzz float32 each), enqueued on the given CUDA stream."""
        _check(lib().qpstd_lowrank_apply_device(self.h, C.c_void_p(d_in), C.c_void_p(d_out), C.c_void_p(stream)))

    def close(self):
        if self.h:
            lib().qpstd_lowrank_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---- serving ----------------------------------------------------------------------
def shot_bytes(d: dict) -> int:
    D = Desc(d)
    return int(lib().qpstd_shot_bytes(C.byref(D.s)))


class Server:
    """Continuous batching of shot requests (qpstd_server).  Keeps every
    request's descriptor arrays and buffers alive until the request is done."""

    def __init__(self, mem_budget: int = 0, max_active: int = 0):
        self.h = C.c_void_p()
        _check(lib().qpstd_server_create(int(mem_budget), int(max_active), C.byref(self.h)))
        self.keep = {}

    def submit(self, d: dict, obs: np.ndarray | None = None) -> int:
        D = Desc(d)
        rtm = d["kind"] in (ARTM, QRTM)
        if rtm:
            nx, nz = d["nxx"] - 2 * d["pml"], d["nzz"] - 2 * d["pml"]
            obs = np.ascontiguousarray(obs, dtype=np.float32)
            out0 = np.zeros((nx, nz), dtype=np.float32)
            out1 = np.zeros((nx, nz), dtype=np.float32)
        else:
            out0 = np.zeros((d["nt"], D.s.nr), dtype=np.float32)
            out1 = None
        rid = int(lib().qpstd_server_submit(self.h, C.byref(D.s), _f(obs), _f(out0), _f(out1)))
        if rid < 0:
            _check(rid)
        self.keep[rid] = (D, obs, out0, out1)
        return rid

    def status(self, rid: int):
        lat = C.c_double()
        sn = C.c_int()
        st = int(lib().qpstd_server_status(self.h, rid, C.byref(lat), C.byref(sn)))
        return st, lat.value, sn.value

    def wait(self, rid: int = -1):
        _check(lib().qpstd_server_wait(self.h, rid))

    def result(self, rid: int):
        """Gather (modeling) or (image, illumination) (RTM) of a finished request."""
        D, obs, out0, out1 = self.keep[rid]
        return out0 if out1 is None else (out0, out1)

    def close(self):
        if self.h:
            lib().qpstd_server_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
