"""The native programs' host side (constant-q-pstd_gb300/cli/, no GPU needed).

Pinned bit for bit to the reference's own host code through the committed
fixtures in tests/golden/reference_host.npz (made by make_golden.py from
sgpstd-*/func*.c and geometry/geometry2d.c): the parameter readers of the four
programs, the geometry generator, the full-model setup (buoyancy, source
wavelet, constant-Q parameters) and the windowing callbacks.  The `qpstd`
executable's geometry, sum and argument handling run here too.
"""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

import qpstd

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "constant-q-pstd_gb300")
HOST = os.path.join(PKG, "libqpstd_host.so")
EXE = os.path.join(PKG, "qpstd")
GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "reference_host.npz"))
fp = C.POINTER(C.c_float)
PROGS = ["aps", "vaps", "artm", "qrtm"]


@pytest.fixture(scope="module")
def host():
    if not (os.path.exists(HOST) and os.path.exists(EXE)):
        qpstd.build()
    L = C.CDLL(HOST)
    L.qpcli_read_params.argtypes = [C.c_int, C.c_char_p, C.POINTER(C.c_double), C.c_int, C.c_char_p, C.c_int]
    L.qpcli_write_geometry.argtypes = [C.c_char_p, C.c_char_p]
    L.qpcli_last_error.restype = C.c_char_p
    L.qpcli_cal_bbx_bbz.argtypes = [C.c_int, C.c_int, fp, fp, fp]
    L.qpcli_rik_cal.argtypes = [C.c_int, C.c_float, C.c_float, C.c_int, fp]
    L.qpcli_transfermodel.argtypes = [C.c_int, C.c_float, C.c_float] + [fp] * 6
    L.qpcli_get_max_min.argtypes = [C.c_int, fp, fp, fp]
    L.qpcli_cfl_number.argtypes = [C.c_float] * 4
    L.qpcli_cfl_number.restype = C.c_float
    L.qpcli_distribute.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]
    L.qpcli_window_width.argtypes = [C.c_float] * 3
    L.select_part_model.argtypes = [C.c_int, C.c_float, C.c_float] + [C.c_int] * 6 + [fp, fp]
    L.expand_pml_areas.argtypes = [C.c_int] * 5 + [fp]
    L.projectomodel.argtypes = [C.c_int, C.c_float, C.c_float] + [C.c_int] * 6 + [fp, fp]
    L.removedirect.argtypes = [C.c_int, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, C.c_float, fp, fp,
                               C.c_float, fp]
    L.get_max_tao.argtypes = [C.c_int, C.c_int, fp]
    L.get_max_tao.restype = C.c_float
    return L


def pf(a):
    return a.ctypes.data_as(fp)


def test_host_library_exports_every_declared_symbol(host):
    src = re.sub(r"/\*.*?\*/", "", open(os.path.join(ROOT, "include", "qpstd_programs.h")).read(), flags=re.S)
    names = set(re.findall(r"\b(qpcli_\w+)\s*\(", src))
    assert len(names) >= 10
    assert all(hasattr(host, n) for n in names)


@pytest.mark.parametrize("prog", PROGS)
def test_parameter_reader_matches_the_reference(host, prog, tmp_path):
    text = bytes(GOLD[f"par_{prog}_text"])
    path = tmp_path / "params.txt"
    path.write_bytes(text)
    nums = (C.c_double * 64)()
    strs = C.create_string_buffer(4096)
    n = host.qpcli_read_params(PROGS.index(prog), str(path).encode(), nums, 64, strs, 4096)
    ref = GOLD[f"par_{prog}_nums"]
    assert n == ref.size
    assert np.array_equal(np.array(nums[:n]), ref)
    assert strs.value.decode().split("\n")[:-1] == bytes(GOLD[f"par_{prog}_strs"]).decode().split("\n")


def test_parameter_reader_reports_a_short_file(host, tmp_path):
    text = bytes(GOLD["par_qrtm_text"]).decode().split("\n")
    path = tmp_path / "short.txt"
    path.write_text("\n".join(text[:20]) + "\n")
    assert host.qpcli_read_params(3, str(path).encode(), None, 0, None, 0) < 0
    assert b"missing value" in host.qpcli_last_error()
    assert host.qpcli_read_params(0, str(tmp_path / "absent.txt").encode(), None, 0, None, 0) < 0


def _geometry_params(path, g):
    labels = ["shots", "first x", "interval", "shot depth", "receiver depth", "offset", "trace interval", "dx",
              "dz", "nx", "nz"]
    with open(path, "w") as f:
        for lab, v in zip(labels, g):
            f.write(f"-- {lab}\n   {int(v) if lab in ('shots', 'nx', 'nz') else float(v)!r}\n")


def _check_geometry(d, gi):
    g = GOLD[f"geo{gi}_params"]
    rd = lambda n, t: np.fromfile(os.path.join(d, n), dtype=t)
    assert np.array_equal(rd("tracenum.bin", np.int32), GOLD[f"geo{gi}_tracenum"])
    assert np.array_equal(rd("shotxp.bin", np.float32), GOLD[f"geo{gi}_shotxp"])
    assert np.array_equal(rd("shotzp.bin", np.float32), GOLD[f"geo{gi}_shotzp"])
    gx = np.concatenate([rd(f"gxp{i}.bin", np.float32) for i in range(int(g[0]))])
    gz = np.concatenate([rd(f"gzp{i}.bin", np.float32) for i in range(int(g[0]))])
    assert np.array_equal(gx, GOLD[f"geo{gi}_gxp"])
    assert np.array_equal(gz, GOLD[f"geo{gi}_gzp"])


@pytest.mark.parametrize("gi", [0, 1])
def test_geometry_generator_matches_the_reference(host, gi, tmp_path):
    _geometry_params(tmp_path / "parameters.txt", GOLD[f"geo{gi}_params"])
    out = tmp_path / "out"
    out.mkdir()
    assert host.qpcli_write_geometry(str(tmp_path / "parameters.txt").encode(), str(out).encode()) == 0
    _check_geometry(out, gi)


def test_geometry_program_writes_the_same_files(host, tmp_path):
    _geometry_params(tmp_path / "parameters.txt", GOLD["geo1_params"])
    r = subprocess.run([os.path.join(PKG, "bin", "geometry")], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout
    assert r.stdout.count("id=") == int(GOLD["geo1_params"][0])
    _check_geometry(tmp_path, 1)


def test_geometry_rejects_a_shot_outside_the_model(host, tmp_path):
    g = list(GOLD["geo1_params"])
    g[1] = 5000.0   # first shot beyond nx * dx
    _geometry_params(tmp_path / "parameters.txt", g)
    assert host.qpcli_write_geometry(str(tmp_path / "parameters.txt").encode(), str(tmp_path).encode()) < 0
    assert b"exceeds model" in host.qpcli_last_error()


@pytest.mark.parametrize("flag", [1, 2])
def test_source_wavelet_matches_the_reference(host, flag):
    r = np.zeros(3000, dtype=np.float32)
    host.qpcli_rik_cal(3000, 0.0005, 20.0, flag, pf(r))
    assert np.array_equal(r, GOLD[f"rik_flag{flag}"])


def test_buoyancy_matches_the_reference(host):
    rho = GOLD["bb_rho"]
    bbx, bbz = np.zeros_like(rho), np.zeros_like(rho)
    host.qpcli_cal_bbx_bbz(97, 73, pf(rho), pf(bbx), pf(bbz))
    assert np.array_equal(bbx, GOLD["bb_bbx"]) and np.array_equal(bbz, GOLD["bb_bbz"])


def test_constant_q_parameters_match_the_reference(host):
    vp, qp = GOLD["tm_vp"], GOLD["tm_qp"]
    out = [np.zeros_like(vp) for _ in range(4)]
    host.qpcli_transfermodel(vp.size, 30.0, 200.0, pf(vp), pf(qp), *[pf(a) for a in out])
    for k, a in zip(["gam", "lam", "vwd", "tao"], out):
        assert np.array_equal(a, GOLD[f"tm_{k}"]), k


@pytest.mark.parametrize("c", range(4))
def test_windowing_callbacks_match_the_reference(host, c):
    vpt = GOLD["win_vpt"]
    nxt, nzt, pml, dx = 50, 12, 4, 10.0
    mlx, nx = GOLD[f"win{c}_case"]
    nx = int(nx)
    nxx, nzz = nx + 2 * pml, nzt + 2 * pml
    w = np.zeros(nxx * nzz, dtype=np.float32)
    host.select_part_model(pml, mlx, dx, nxt, nzt, nx, nzt, nxx, nzz, pf(vpt), pf(w))
    host.expand_pml_areas(nx, nzt, nxx, nzz, pml, pf(w))
    assert np.array_equal(w, GOLD[f"win{c}_model"])
    img = GOLD[f"win{c}_img"].copy()
    pj = np.zeros(nxt * nzt, dtype=np.float32)
    host.projectomodel(pml, mlx, dx, nxt, nzt, nx, nzt, nxx, nzz, pf(pj), pf(img))
    assert np.array_equal(pj, GOLD[f"win{c}_pj"])


def test_direct_wave_removal_matches_the_reference(host):
    obs = GOLD["rd_in"].copy()
    gx = np.linspace(0.0, 600.0, 16).astype(np.float32)
    gz = np.full(16, 20.0, dtype=np.float32)
    host.removedirect(16, 300, 16, 0.001, 25.0, 250.0, 20.0, pf(gx), pf(gz), 1800.0, pf(obs))
    assert np.array_equal(obs, GOLD["rd_out"])
    tao = np.array([0.0, 3.5, -1.0, 2.0], dtype=np.float32)
    assert host.get_max_tao(2, 2, pf(tao)) == np.float32(3.5)


@pytest.mark.parametrize("shotnum,nranks", [(80, 1), (80, 3), (7, 4), (3, 5), (64, 8)])
def test_shots_are_split_as_the_reference_splits_them(host, shotnum, nranks):
    """acousticsgps4.c:254-270 with one GPU per rank: every shot once, contiguous per rank."""
    seen = []
    for r in range(nranks):
        first, cnt = C.c_int(), C.c_int()
        host.qpcli_distribute(shotnum, nranks, r, C.byref(first), C.byref(cnt))
        rid, ave = shotnum % nranks, shotnum // nranks
        assert cnt.value == ave + (1 if r < rid else 0)
        seen += list(range(first.value, first.value + cnt.value))
    assert seen == list(range(shotnum))


def test_window_width_and_extremes(host):
    for sroff, disx, dx in [(1500.0, 0.0, 10.0), (1999.9, 35.0, 12.5), (333.3, 0.0, 7.5)]:
        simx = np.float32(2.0 * float(np.float32(np.float32(sroff) + np.float32(disx))))
        want = int(float(np.float32(simx / np.float32(dx))) + 1.5)
        assert host.qpcli_window_width(sroff, disx, dx) == want
    a = np.array([3.0, 1.0, 1.00005, 7.0, 6.99995], dtype=np.float32)
    vmax, vmin = C.c_float(), C.c_float()
    host.qpcli_get_max_min(a.size, pf(a), C.byref(vmax), C.byref(vmin))
    assert (vmax.value, vmin.value) == (np.float32(7.0), np.float32(1.00005))  # 1e-4 hysteresis, as the reference
    assert abs(host.qpcli_cfl_number(4500.0, 0.001, 10.0, 10.0) - np.pi * 4500 * 0.001 / 2 * np.sqrt(0.02)) < 1e-4


def test_sum_program_adds_rank_images(host, tmp_path):
    a = np.arange(12, dtype=np.float32)
    b = np.linspace(-1, 1, 12).astype(np.float32)
    a.tofile(tmp_path / "QRTM.BIN.rank0")
    b.tofile(tmp_path / "QRTM.BIN.rank1")
    r = subprocess.run([EXE, "sum", "QRTM.BIN", "QRTM.BIN.rank0", "QRTM.BIN.rank1"], cwd=tmp_path,
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout
    assert np.array_equal(np.fromfile(tmp_path / "QRTM.BIN", dtype=np.float32), a + b)
    np.zeros(5, dtype=np.float32).tofile(tmp_path / "short.bin")
    r = subprocess.run([EXE, "sum", "x.bin", "QRTM.BIN.rank0", "short.bin"], cwd=tmp_path, capture_output=True)
    assert r.returncode != 0


def test_programs_plan_the_shots_without_a_gpu(host, tmp_path):
    """--dry-run reads every file and reports each process's shots and window."""
    for sub in ("input", "geometry", "output", "run"):
        (tmp_path / sub).mkdir()
    _geometry_params(tmp_path / "geometry" / "parameters.txt",
                     (3, 300.0, 400.0, 20.0, 20.0, 200.0, 10.0, 10.0, 10.0, 150, 40))
    assert host.qpcli_write_geometry(str(tmp_path / "geometry" / "parameters.txt").encode(),
                                     str(tmp_path / "geometry").encode()) == 0
    for name in ("vp", "rho", "qp"):
        np.full(150 * 40, 2000.0, dtype=np.float32).tofile(tmp_path / "output" / f"{name}.bin")
    g = ["../geometry/tracenum.bin", "../geometry/shotxp.bin", "../geometry/shotzp.bin", "../geometry/gxp",
         "../geometry/gzp"]
    fields = [3, 100, 1.0, 25.0, 200.0, 150, 40, 10.0, 10.0, 0.0, 1500.0, 1e4, 1e4] + g + \
        ["../output/vp.bin", "../output/rho.bin", "../output/qp.bin", "../obsdata/recva", 2, 6]
    with open(tmp_path / "input" / "visac2drtm.txt", "w") as f:
        for k, v in enumerate(fields):
            f.write(f"--value {k}\n  {v}\n")
    qrtm = os.path.join(PKG, "bin", "qrtm")
    r = subprocess.run([qrtm, "--dry-run"], cwd=tmp_path / "run", capture_output=True, text=True)
    assert r.returncode == 0, r.stdout
    assert "rank 0 of 1: shots 0..2, window nx=41 nz=40, padded 61 x 60, nt=100" in r.stdout
    r = subprocess.run([qrtm, "--dry-run", "--pml", "20", "--rank", "1", "--nranks", "2"], cwd=tmp_path / "run",
                       capture_output=True, text=True)
    assert r.returncode == 0 and "rank 1 of 2: shots 2..2, window nx=41 nz=40, padded 81 x 80" in r.stdout
    r = subprocess.run([qrtm, "--dry-run"], cwd=tmp_path / "run", capture_output=True, text=True,
                       env=dict(os.environ, RANK="0", WORLD_SIZE="3"))
    assert "rank 0 of 3: shots 0..0" in r.stdout
    os.remove(tmp_path / "geometry" / "gxp2.bin")
    r = subprocess.run([qrtm, "--dry-run"], cwd=tmp_path / "run", capture_output=True, text=True)
    assert r.returncode != 0 and "receiver positions" in r.stdout


def test_programs_fail_with_a_status_on_bad_input(host, tmp_path):
    run = tmp_path / "run"
    run.mkdir()
    r = subprocess.run([os.path.join(PKG, "bin", "qrtm")], cwd=run, capture_output=True, text=True)
    assert r.returncode == 1 and "visac2drtm.txt" in r.stdout
    r = subprocess.run([EXE, "aps", "--bogus"], capture_output=True, text=True)
    assert r.returncode == 1 and "usage" in r.stdout
