"""Pin the FP64 oracle before trusting it.

* The oracle's FFT against numpy.fft (the cuFFT C2C convention: forward e^{-i},
  inverse e^{+i}, unnormalised) on the awkward lengths the reference windowing
  produces (439 prime, 2461 = 23*107, 860 = 4*5*43, 660 = 4*3*5*11).
* Its coefficient setup and revolve schedule against the reference's own host
  C code, through the committed fixtures in tests/golden/reference_host.npz
  (made by tests/golden/make_golden.py from sgpstd-qmodeling/funca.c, func.c
  and sgpstd-qrtm/src.c), and live against oracle/_ref when it was built.
"""
import os

import numpy as np
import pytest

import oracle as O

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "reference_host.npz"))


@pytest.mark.parametrize("n", [1, 2, 3, 5, 7, 8, 11, 13, 17, 43, 64, 107, 200, 439, 660, 860, 2461])
def test_fft_matches_numpy(n):
    rng = np.random.default_rng(n)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    ref = np.fft.fft(x)
    assert np.abs(O.fft1d(x, -1) - ref).max() <= 1e-12 * np.abs(ref).max() + 1e-14
    refi = np.fft.ifft(x) * n
    assert np.abs(O.fft1d(x, +1) - refi).max() <= 1e-12 * np.abs(refi).max() + 1e-14


def _grids():
    g = 0
    while f"g{g}_grid" in GOLD:
        yield g
        g += 1


def _close(mine, ref, rtol=2e-6, atol=0.0):
    ref = ref.astype(np.float64)
    scale = max(np.abs(ref).max(), 1e-30)
    return np.abs(mine - ref).max() <= rtol * scale + atol


@pytest.mark.parametrize("g", list(_grids()))
def test_pml_coeffs_pinned(g):
    pml, fd, nxx, nzz, dx, dz, dt = GOLD[f"g{g}_grid"]
    mine = O.pml_coeffs(int(pml), fd, int(nxx), int(nzz), dx, dz, dt)
    for k, v in mine.items():
        assert _close(v, GOLD[f"g{g}_{k}"]), k


@pytest.mark.parametrize("g", list(_grids()))
def test_shift_tables_pinned(g):
    pml, fd, nxx, nzz, dx, dz, dt = GOLD[f"g{g}_grid"]
    mine = O.shift_tables(int(nxx), int(nzz), dx, dz)
    for k, v in mine.items():
        assert _close(v, GOLD[f"g{g}_{k}"]), k


@pytest.mark.parametrize("g", [g for g in _grids() if f"g{g}_k2d1" in GOLD])
def test_k2d_pinned(g):
    pml, fd, nxx, nzz, dx, dz, dt = GOLD[f"g{g}_grid"]
    mine = O.k2d(int(nxx), int(nzz), dx, dz)
    for k, v in mine.items():
        assert _close(v, GOLD[f"g{g}_{k}"], rtol=4e-6), k


def test_ricker_bbx_transfermodel_pinned():
    for flag in (1, 2):
        assert _close(O.ricker(3000, 0.0005, 20.0, flag), GOLD[f"rik_flag{flag}"], rtol=1e-6)
    bbx, bbz = O.bbx_bbz(97, 73, GOLD["bb_rho"])
    assert _close(bbx, GOLD["bb_bbx"]) and _close(bbz, GOLD["bb_bbz"])
    gam, lam, vwd, tao = O.transfermodel(30.0, 200.0, GOLD["tm_vp"], GOLD["tm_qp"])
    for k, v in zip(["gam", "lam", "vwd", "tao"], [gam, lam, vwd, tao]):
        assert _close(v, GOLD[f"tm_{k}"]), k


@pytest.mark.parametrize("key", [k for k in GOLD.files if k.startswith("revolve_")])
def test_revolve_schedule_pinned(key):
    _, steps, snaps = key.split("_")
    mine = O.revolve_trace(int(steps), int(snaps))
    ref = GOLD[key]
    assert mine.shape == ref.shape and (mine == ref).all()


def test_numforw_survey_figures():
    assert O.numforw(6000, 40) == 17097
    assert O.numforw(5000, 30) == 14472


def test_live_reference_objects_if_built():
    """Same pins against the freshly compiled reference objects (skip if absent)."""
    import ctypes as C
    lib = O.ref_lib("qr_src")
    if lib is None:
        pytest.skip("oracle/_ref not built here")
    ip = C.POINTER(C.c_int)
    lib.revolve.argtypes = [ip, ip, ip, C.c_int, ip]
    for steps, snaps in [(731, 9), (12, 2), (1000, 64)]:
        check, capo, fine, info = C.c_int(-1), C.c_int(0), C.c_int(steps), C.c_int(0)
        tr = []
        while True:
            a = lib.revolve(C.byref(check), C.byref(capo), C.byref(fine), snaps, C.byref(info))
            tr.append((a, capo.value, check.value))
            if a in (5, 6):
                break
        assert (np.array(tr) == O.revolve_trace(steps, snaps)).all()


def test_host_helpers_pinned():
    """The C restatement of the programs' windowing helpers (oracle/host_helpers.c,
    linked by the acforward shim harness) against the reference's compiled ones."""
    import ctypes as C
    L = O.lib()
    fp = C.POINTER(C.c_float)
    L.select_part_model.argtypes = [C.c_int, C.c_float, C.c_float] + [C.c_int] * 6 + [fp, fp]
    L.expand_pml_areas.argtypes = [C.c_int] * 5 + [fp]
    L.projectomodel.argtypes = [C.c_int, C.c_float, C.c_float] + [C.c_int] * 6 + [fp, fp]
    L.removedirect.argtypes = [C.c_int, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, C.c_float, fp, fp,
                               C.c_float, fp]
    pf = lambda a: a.ctypes.data_as(fp)
    vpt = GOLD["win_vpt"]
    nxt, nzt, pml, dxw = 50, 12, 4, 10.0
    for c in range(4):
        mlx, nx = GOLD[f"win{c}_case"]
        nx = int(nx)
        nxx, nzz = nx + 2 * pml, nzt + 2 * pml
        w = np.zeros(nxx * nzz, dtype=np.float32)
        L.select_part_model(pml, mlx, dxw, nxt, nzt, nx, nzt, nxx, nzz, pf(vpt), pf(w))
        L.expand_pml_areas(nx, nzt, nxx, nzz, pml, pf(w))
        assert np.array_equal(w, GOLD[f"win{c}_model"]), c
        pj = np.zeros(nxt * nzt, dtype=np.float32)
        img = np.ascontiguousarray(GOLD[f"win{c}_img"])
        L.projectomodel(pml, mlx, dxw, nxt, nzt, nx, nzt, nxx, nzz, pf(pj), pf(img))
        assert np.array_equal(pj, GOLD[f"win{c}_pj"]), c
    obs = np.array(GOLD["rd_in"])
    gx = np.linspace(0.0, 600.0, 16).astype(np.float32)
    gz = np.full(16, 20.0, dtype=np.float32)
    L.removedirect(16, 300, 16, 0.001, 25.0, 250.0, 20.0, pf(gx), pf(gz), 1800.0, pf(obs))
    assert np.array_equal(obs, GOLD["rd_out"])
