"""Generate the golden fixtures that pin the oracle to the reference.

The reference has no tests and no golden outputs, and its stepping path runs
only on a GPU through cuFFT.  What does run here is its host C code: the
coefficient setup (sgpstd-qmodeling/funca.c, func.c; sgpstd-qrtm/func.c), the
windowing helpers and the revolve controller (sgpstd-qrtm/src.c).  ``make -C
oracle ref`` compiles those files, where they lie, into ``oracle/_ref/``; this
script calls them on a set of grids and writes their outputs to
``tests/golden/reference_host.npz`` so the pins also run where the reference
sources are absent.

Run:  make -C oracle ref && python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "oracle"))
import oracle as O  # noqa: E402

fp = C.POINTER(C.c_float)
ip = C.POINTER(C.c_int)

GRIDS = [  # (pml, fd, nxx, nzz, dx, dz, dt)
    (20, 20.0, 439, 200, 10.0, 10.0, 0.001),
    (30, 30.0, 2461, 860, 10.0, 10.0, 0.0005),
    (10, 30.0, 64, 48, 10.0, 12.5, 0.001),
    (10, 25.0, 97, 73, 8.0, 10.0, 0.0008),
]
REVOLVE = [(10, 3), (100, 5), (2000, 20), (3000, 20), (6000, 40), (5000, 30), (37, 4), (400, 8)]


def f32(n):
    return np.zeros(n, dtype=np.float32)


def pf(a):
    return a.ctypes.data_as(fp)


# Parameter files of the four programs: (reference library, file name, fields),
# each field (kind, value) with kind i / f / s; values are synthetic.
PARAM_FILES = {
    "aps": ("qm_funca", "ac2drealmodeling.txt",
            [("i", 7), ("i", 1201), ("f", 0.75), ("f", 22.5), ("i", 301), ("i", 97), ("f", 12.5), ("f", 10.0),
             ("f", 35.0), ("s", "../g/tn.bin"), ("s", "../g/sx.bin"), ("s", "../g/sz.bin"), ("s", "../g/gx"),
             ("s", "../g/gz"), ("s", "../m/vp.bin"), ("s", "../m/rho.bin"), ("i", 1), ("i", 1)]),
    "vaps": ("qm_func", "visac2drealmodeling.txt",
             [("i", 9), ("i", 1500), ("f", 0.5), ("f", 25.0), ("f", 150.0), ("i", 256), ("i", 120), ("f", 10.0),
              ("f", 7.5), ("f", 0.0), ("s", "../g/tn.bin"), ("s", "../g/sx.bin"), ("s", "../g/sz.bin"),
              ("s", "../g/gx"), ("s", "../g/gz"), ("s", "../m/vp.bin"), ("s", "../m/rho.bin"),
              ("s", "../m/qp.bin"), ("i", 0), ("i", 2)]),
    "artm": ("qr_funca", "ac2drtm.txt",
             [("i", 12), ("i", 3001), ("f", 0.5), ("f", 18.0), ("i", 800), ("i", 240), ("f", 10.0), ("f", 10.0),
              ("f", 100.0), ("f", 1480.0), ("s", "../g/tn.bin"), ("s", "../g/sx.bin"), ("s", "../g/sz.bin"),
              ("s", "../g/gx"), ("s", "../g/gz"), ("s", "../m/vpm.bin"), ("s", "../m/rho.bin"),
              ("s", "../obs/reca"), ("i", 2), ("i", 25)]),
    "qrtm": ("qr_func", "visac2drtm.txt",
             [("i", 64), ("i", 5000), ("f", 0.5), ("f", 30.0), ("f", 200.0), ("i", 6000), ("i", 600),
              ("f", 10.0), ("f", 10.0), ("f", 0.0), ("f", 1500.0), ("f", 1e-20), ("f", 3e-20),
              ("s", "../g/tn.bin"), ("s", "../g/sx.bin"), ("s", "../g/sz.bin"), ("s", "../g/gx"), ("s", "../g/gz"),
              ("s", "../m/vpm.bin"), ("s", "../m/rho.bin"), ("s", "../m/qp.bin"), ("s", "../obs/recva"),
              ("i", 2), ("i", 30)]),
}
# geometry/parameters.txt variants: shotnum, sx0, sxdx, sdep, rdep, offset, trdx, dx, dz, nx, nz
GEOMETRY = [
    (6, 400.0, 40.0, 0.0, 0.0, 1500.0, 10.0, 10.0, 10.0, 398, 160),
    (5, 15.0, 237.5, 20.0, 12.5, 333.3, 7.5, 12.5, 12.5, 97, 41),
]


def param_text(fields):
    """Label lines and values, with blank lines and trailing blanks the readers skip."""
    lines = []
    for k, (kind, v) in enumerate(fields):
        lines.append(f"--field {k} ({kind})")
        if k % 3 == 1:
            lines.append("")
        lines.append(f"  {v!r}" if kind == "f" else f"  {v}" + ("  " if k % 2 else ""))
    return "\n".join(lines) + "\n"


def program_fixtures(out):
    """The programs' own parameter readers and geometry generator on synthetic files."""
    import subprocess
    import tempfile

    cwd = os.getcwd()
    for prog, (libname, fname, fields) in PARAM_FILES.items():
        lib = O.ref_lib(libname)
        d = tempfile.mkdtemp(prefix="qpar")
        os.makedirs(os.path.join(d, "input"))
        os.makedirs(os.path.join(d, "run"))
        text = param_text(fields)
        with open(os.path.join(d, "input", fname), "w") as f:
            f.write(text)
        args, back = [], []
        for k, (kind, _) in enumerate(fields):
            if kind == "i":
                a = C.c_int(0)
                args.append(C.byref(a))
            elif kind == "f":
                a = C.c_float(0.0)
                args.append(C.byref(a))
            else:
                a = C.create_string_buffer(128)
                args.append(a)
            back.append((kind, a))
        os.chdir(os.path.join(d, "run"))
        try:
            lib.input_ac2d_parameters(*args)
        finally:
            os.chdir(cwd)
        nums = [float(a.value) for kind, a in back if kind != "s"]
        strs = "\n".join(a.value.decode() for kind, a in back if kind == "s")
        out[f"par_{prog}_text"] = np.frombuffer(text.encode(), dtype=np.uint8)
        out[f"par_{prog}_nums"] = np.array(nums, dtype=np.float64)
        out[f"par_{prog}_strs"] = np.frombuffer(strs.encode(), dtype=np.uint8)
    exe = os.path.join(HERE, "..", "..", "oracle", "_ref", "geometry2d")
    for gi, g in enumerate(GEOMETRY):
        d = tempfile.mkdtemp(prefix="qgeo")
        labels = ["shots", "first x", "interval", "shot depth", "receiver depth", "offset", "trace interval",
                  "dx", "dz", "nx", "nz"]
        with open(os.path.join(d, "parameters.txt"), "w") as f:
            for lab, v in zip(labels, g):
                f.write(f"-- {lab}\n   {v}\n")
        subprocess.run([os.path.abspath(exe)], cwd=d, check=True, capture_output=True)
        rd = lambda n, t: np.fromfile(os.path.join(d, n), dtype=t)
        out[f"geo{gi}_params"] = np.array(g, dtype=np.float64)
        out[f"geo{gi}_tracenum"] = rd("tracenum.bin", np.int32)
        out[f"geo{gi}_shotxp"] = rd("shotxp.bin", np.float32)
        out[f"geo{gi}_shotzp"] = rd("shotzp.bin", np.float32)
        out[f"geo{gi}_gxp"] = np.concatenate([rd(f"gxp{i}.bin", np.float32) for i in range(g[0])])
        out[f"geo{gi}_gzp"] = np.concatenate([rd(f"gzp{i}.bin", np.float32) for i in range(g[0])])


def main():
    qm_a = O.ref_lib("qm_funca")
    qm_f = O.ref_lib("qm_func")
    qr_s = O.ref_lib("qr_src")
    if qm_a is None or qm_f is None or qr_s is None:
        raise SystemExit("reference objects missing: run `make -C oracle ref` first")
    qm_a.get_pml_parameters.argtypes = [C.c_int, C.c_float] + [fp] * 8 + [C.c_int, C.c_int, C.c_float, C.c_float, C.c_float]
    qm_a.cal_shift_parameters.argtypes = [fp] * 8 + [C.c_float, C.c_float, C.c_int, C.c_int]
    qm_f.cal_k2d.argtypes = [C.c_float, C.c_float, C.c_int, C.c_int] + [fp] * 4
    qm_f.cal_k2dh.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_float, C.c_float, fp]
    qm_a.rik_cal.argtypes = [C.c_int, C.c_float, C.c_float, fp, C.c_int]
    qm_a.cal_bbx_bbz.argtypes = [C.c_int, C.c_int, fp, fp, fp]
    qm_f.transfermodel.argtypes = [C.c_int, C.c_int, C.c_float, C.c_float] + [fp] * 6
    qr_s.revolve.argtypes = [ip, ip, ip, C.c_int, ip]
    out = {}
    for g, (pml, fd, nxx, nzz, dx, dz, dt) in enumerate(GRIDS):
        pmlt = [f32(nxx), f32(nxx), f32(nzz), f32(nzz), f32(nxx), f32(nxx), f32(nzz), f32(nzz)]
        qm_a.get_pml_parameters(pml, fd, *[pf(a) for a in pmlt], nxx, nzz, dx, dz, dt)
        for k, a in zip(["i_ax", "i_bx", "i_az", "i_bz", "h_ax", "h_bx", "h_az", "h_bz"], pmlt):
            out[f"g{g}_{k}"] = a
        sh = [f32(nxx), f32(nxx), f32(nzz), f32(nzz), f32(nxx), f32(nxx), f32(nzz), f32(nzz)]
        # argument order: kxsmr,kxscr,kzsmr,kzscr,kxsmi,kxsci,kzsmi,kzsci
        names = ["kxsmr", "kxscr", "kzsmr", "kzscr", "kxsmi", "kxsci", "kzsmi", "kzsci"]
        sh = [f32(nxx if n[1] == "x" else nzz) for n in names]
        qm_a.cal_shift_parameters(*[pf(a) for a in sh], dx, dz, nxx, nzz)
        for k, a in zip(names, sh):
            out[f"g{g}_{k}"] = a
        if nxx * nzz <= 100000:  # keep the fixture small: 2-D tables for small grids only
            ks = [f32(nxx * nzz) for _ in range(4)]
            qm_f.cal_k2d(dx, dz, nxx, nzz, *[pf(a) for a in ks])
            for k, a in zip(["k2d1", "k2d2", "k2d3", "k2da"], ks):
                out[f"g{g}_{k}"] = a
            # |k| on the half grid, the wavenumbers of the low-rank form
            nxh, nzh = nxx // 2 + 1, nzz // 2 + 1
            kh = f32(nxh * nzh)
            qm_f.cal_k2dh(nxh, nzh, nxx, nzz, dx, dz, pf(kh))
            out[f"g{g}_k2dh"] = kh
        out[f"g{g}_grid"] = np.array([pml, fd, nxx, nzz, dx, dz, dt], dtype=np.float64)
    for flag in (1, 2):
        r = f32(3000)
        qm_a.rik_cal(3000, 0.0005, 20.0, pf(r), flag)
        out[f"rik_flag{flag}"] = r
    rng = np.random.default_rng(7)
    rho = rng.uniform(1000.0, 2600.0, size=97 * 73).astype(np.float32)
    bbx, bbz = f32(97 * 73), f32(97 * 73)
    qm_a.cal_bbx_bbz(97, 73, pf(rho), pf(bbx), pf(bbz))
    out["bb_rho"], out["bb_bbx"], out["bb_bbz"] = rho, bbx, bbz
    vp = rng.uniform(1500.0, 4500.0, size=500).astype(np.float32)
    qp = rng.uniform(20.0, 200.0, size=500).astype(np.float32)
    tm = [f32(500) for _ in range(4)]
    qm_f.transfermodel(500, 1, 30.0, 200.0, pf(vp), pf(qp), *[pf(a) for a in tm])
    out["tm_vp"], out["tm_qp"] = vp, qp
    for k, a in zip(["gam", "lam", "vwd", "tao"], tm):
        out[f"tm_{k}"] = a
    # windowing helpers of the programs (sgpstd-qrtm/funca.c): select_part_model,
    # expand_pml_areas, projectomodel for windows inside, across the right edge
    # of, and left of the model; removedirect on a small gather
    qr_a = O.ref_lib("qr_funca")
    qr_a.select_part_model.argtypes = [C.c_int, C.c_float, C.c_float] + [C.c_int] * 6 + [fp, fp]
    qr_a.expand_pml_areas.argtypes = [C.c_int] * 5 + [fp]
    qr_a.projectomodel.argtypes = [C.c_int, C.c_float, C.c_float] + [C.c_int] * 6 + [fp, fp]
    qr_a.removedirect.argtypes = [C.c_int, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, C.c_float, fp, fp,
                                  C.c_float, fp]
    nxt, nzt, pml, dxw = 50, 12, 4, 10.0
    vpt = rng.uniform(1500.0, 4500.0, size=nxt * nzt).astype(np.float32)
    for c, (mlx, nx) in enumerate([(55.0, 20), (402.0, 20), (-63.0, 30), (-41.0, 70)]):
        nxx, nzz = nx + 2 * pml, nzt + 2 * pml
        w = f32(nxx * nzz)
        qr_a.select_part_model(pml, mlx, dxw, nxt, nzt, nx, nzt, nxx, nzz, pf(vpt), pf(w))
        qr_a.expand_pml_areas(nx, nzt, nxx, nzz, pml, pf(w))
        img = rng.standard_normal(nx * nzt).astype(np.float32)
        pj = f32(nxt * nzt)
        qr_a.projectomodel(pml, mlx, dxw, nxt, nzt, nx, nzt, nxx, nzz, pf(pj), pf(img))
        out[f"win{c}_case"] = np.array([mlx, nx], dtype=np.float64)
        out[f"win{c}_model"], out[f"win{c}_img"], out[f"win{c}_pj"] = w, img, pj
    out["win_vpt"] = vpt
    obs = rng.standard_normal(300 * 16).astype(np.float32)
    gx = np.linspace(0.0, 600.0, 16).astype(np.float32)
    gz = np.full(16, 20.0, dtype=np.float32)
    out["rd_in"] = obs.copy()
    qr_a.removedirect(16, 300, 16, 0.001, 25.0, 250.0, 20.0, pf(gx), pf(gz), 1800.0, pf(obs))
    out["rd_out"] = obs
    for steps, snaps in REVOLVE:
        check, capo, fine, info = C.c_int(-1), C.c_int(0), C.c_int(steps), C.c_int(0)
        tr = []
        while True:
            a = qr_s.revolve(C.byref(check), C.byref(capo), C.byref(fine), snaps, C.byref(info))
            tr.append((a, capo.value, check.value))
            if a in (5, 6):
                break
        out[f"revolve_{steps}_{snaps}"] = np.array(tr, dtype=np.int32)
    program_fixtures(out)
    path = os.path.join(HERE, "reference_host.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
