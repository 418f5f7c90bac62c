"""Seeded synthetic shots with the shapes of the reference's use cases.

The reference ships only four 160x398 model files and no benchmark data, so the
workloads are generated: layered vp with Gaussian anomalies, Gardner density,
per-layer Q, a Ricker source, a receiver line.  The per-shot preparation then
follows the reference drivers:
  window width      nx = (int)(2*(sroffmx+disx)/dx + 1.5)  (acousticsgps4.c:332)
  window extraction select_part_model  (funca.c:623-733)
  CPML padding      expand_pml_areas   (funca.c:735-770)
  buoyancy          cal_bbx_bbz on the full model (funca.c:169)
  Q transform       transfermodel      (func.c:912)
  source / receiver grid indices       (acps4.cu:384-410)
All of it is host-side input preparation, evaluated in double and handed to
the library as float32.
"""
from __future__ import annotations

import math

import numpy as np

REF_PI = 3.1415926


def layered_model(nx: int, nz: int, nlayers: int, nanom: int, seed: int, dx: float = 10.0,
                  vmin: float = 1500.0, vmax: float = 4500.0, sigma_cells: float = 15.0):
    """x-major vp (nx, nz): flat layers increasing with depth plus anomalies."""
    rng = np.random.default_rng(seed)
    bounds = np.sort(rng.uniform(0, nz, size=nlayers - 1)).astype(int)
    vel = np.sort(rng.uniform(vmin, vmax, size=nlayers))
    z = np.arange(nz)
    layer = np.searchsorted(bounds, z, side="right")
    vp = np.tile(vel[layer][None, :], (nx, 1)).astype(np.float64)
    X, Z = np.meshgrid(np.arange(nx), np.arange(nz), indexing="ij")
    for _ in range(nanom):
        cx, cz = rng.uniform(0.2 * nx, 0.8 * nx), rng.uniform(0.3 * nz, 0.8 * nz)
        amp = rng.choice([-300.0, 300.0])
        vp += amp * np.exp(-((X - cx) ** 2 + (Z - cz) ** 2) / (2 * sigma_cells ** 2))
    layer_q = rng.uniform(20.0, 200.0, size=nlayers)
    qp = np.tile(layer_q[layer][None, :], (nx, 1))
    return vp, qp


def gardner(vp):
    return 310.0 * np.power(vp, 0.25)


def smooth(vp, cells: float):
    """Gaussian blur (migration model), separable, edge-replicated."""
    r = int(3 * cells)
    k = np.exp(-0.5 * (np.arange(-r, r + 1) / cells) ** 2)
    k /= k.sum()
    out = vp.copy()
    for axis in (0, 1):
        pad = [(0, 0), (0, 0)]
        pad[axis] = (r, r)
        a = np.pad(out, pad, mode="edge")
        out = np.apply_along_axis(lambda v: np.convolve(v, k, mode="valid"), axis, a)
    return out


def bbx_bbz(rho):
    """cal_bbx_bbz (funca.c:169-198) on an (nx, nz) x-major array."""
    bbx = np.empty_like(rho)
    bbz = np.empty_like(rho)
    bbx[:-1, :] = 2.0 / (rho[:-1, :] + rho[1:, :])
    bbx[-1, :] = 1.0 / rho[-1, :]
    bbz[:, :-1] = 2.0 / (rho[:, :-1] + rho[:, 1:])
    bbz[:, -1] = 1.0 / rho[:, -1]
    return bbx, bbz


def transfermodel(fd, fo, vp, qp):
    """func.c:912-930."""
    gam = 1.0 / REF_PI / qp
    lam = np.power(fd / fo, 2.0 * gam)
    vwd = np.power(vp / (2 * REF_PI * fd), 1.0 / 16.0)
    tao = lam * vp / qp
    return gam, lam, vwd, tao


def ricker(nt, dt, fd, flag=2):
    """rik_cal (funca.c:201-220)."""
    t = np.arange(nt) * dt - 1.0 / fd
    if flag == 2:
        a = (REF_PI * fd * t) ** 2
        return (1.0 - 2.0 * a) * np.exp(-a)
    a = (2.0 * REF_PI * fd * t) ** 2
    return t * np.exp(-a)


def select_part_model(pml, mlx, dx, full, nx, nz):
    """select_part_model (funca.c:623-733): window nx columns starting at
    model x = mlx into the interior of an (nx+2pml, nz+2pml) array."""
    nxt, nzt = full.shape
    nxx, nzz = nx + 2 * pml, nz + 2 * pml
    out = np.zeros((nxx, nzz))
    if mlx >= 0.0:
        f0 = int(mlx / dx)
        f1 = f0 + nx - 1
        if f1 < nxt:
            out[pml:pml + nx, pml:pml + nzt] = full[f0:f1 + 1, :]
        else:
            out[pml:pml + nxt - f0, pml:pml + nzt] = full[f0:nxt, :]
            for i in range(nxt, f1 + 1):
                out[i - f0 + pml, pml:nzz - pml] = out[nxt - 1 - f0 + pml, pml:nzz - pml]
    else:
        f0 = int(abs(mlx) / dx + 0.5)
        f1 = nx - f0
        if f1 <= nxt:
            out[f0 + pml:f0 + pml + f1, pml:pml + nzt] = full[0:f1, :]
        else:
            out[f0 + pml:f0 + pml + nxt, pml:pml + nzt] = full[:, :]
            for i in range(nxt, f1):
                out[i + f0 + pml, pml:nzz - pml] = out[nxt - 1 + f0 + pml, pml:nzz - pml]
        for i in range(f0):
            out[i + pml, pml:nzz - pml] = out[f0 + pml, pml:nzz - pml]
    return out


def expand_pml_areas(a, pml):
    """expand_pml_areas (funca.c:735-770)."""
    nxx, nzz = a.shape
    a[pml:nxx - pml, :pml] = a[pml:nxx - pml, pml:pml + 1]
    a[pml:nxx - pml, nzz - pml:] = a[pml:nxx - pml, nzz - pml - 1:nzz - pml]
    a[:pml, :] = a[pml:pml + 1, :]
    a[nxx - pml:, :] = a[nxx - pml - 1:nxx - pml, :]
    return a


def window_shot(models: dict, xs, zs, gxp, gzp, pml, dx, dz, sroffmx, disx=0.0):
    """Per-shot window and grid indices as in acforward (acps4.cu:326-426)."""
    nxt, nzt = models["vp"].shape
    nx = int(2.0 * (sroffmx + disx) / dx + 1.5)
    nz = nzt
    mlx = xs - sroffmx - disx
    out = {}
    for k, full in models.items():
        out[k] = expand_pml_areas(select_part_model(pml, mlx, dx, full, nx, nz), pml)
    xsg = int((sroffmx + disx) / dx + 0.5) + pml
    zsg = int(zs / dz + 0.5) + pml
    gzg = (np.floor(np.asarray(gzp) / dz + 0.5)).astype(np.int32) + pml
    gxg = np.where(np.asarray(gxp) >= xs,
                   xsg + np.floor((np.asarray(gxp) - xs) / dx + 0.5),
                   xsg - np.floor((xs - np.asarray(gxp)) / dx + 0.5)).astype(np.int32)
    nxx = nx + 2 * pml
    gxg = np.clip(gxg, pml, nxx - pml - 1).astype(np.int32)
    return out, nx, nz, xsg, zsg, gxg, gzg


def parent_model(nx: int, nz: int, seed: int, nlayers: int = 12, nanom: int = 3, fd: float = 20.0,
                 fo: float = 20.0, dx: float = 10.0):
    """A seeded parent model (vp, rho, Q and the derived fields) for batches."""
    vp, qp = layered_model(nx, nz, nlayers, nanom, seed, dx=dx, sigma_cells=15.0)
    rho = gardner(vp)
    bbx, bbz = bbx_bbz(rho)
    gam, lam, vwd, tao = transfermodel(fd, fo, vp, qp)
    return {"vp": vp, "rho": rho, "bbx": bbx, "bbz": bbz, "gam": gam, "lam": lam, "vwd": vwd, "tao": tao}


def window_of_parent(kind: int, parent: dict, x0: int, nx: int, pml: int, nt: int, dt: float, fd: float,
                     snaps: int, dx: float = 10.0, dz: float = 10.0):
    """One shot whose window is columns [x0, x0+nx) of the parent model: the
    source at the window centre and z = 2 cells, a receiver in every window
    column at z = 2 cells, the window padded by expand_pml_areas."""
    nz = parent["vp"].shape[1]
    nxx, nzz = nx + 2 * pml, nz + 2 * pml
    d = dict(kind=kind, nxx=nxx, nzz=nzz, pml=pml, dx=dx, dz=dz, dt=dt, fd=fd, nt=nt,
             rik=ricker(nt, dt, fd, 2), xsg=pml + nx // 2, zsg=pml + 2,
             gxg=np.arange(pml, pml + nx, dtype=np.int32), gzg=np.full(nx, pml + 2, dtype=np.int32),
             snaps=snaps, etas=1e-20, etar=1e-20)
    for k, full in parent.items():
        a = np.zeros((nxx, nzz))
        a[pml:pml + nx, pml:pml + nz] = full[x0:x0 + nx, :]
        d[k] = expand_pml_areas(a, pml).ravel()
    if "tao" in parent:
        d["taoc"] = float(d["tao"].max())
    return d


def make_shot(kind: int, nx_model: int, nz_model: int, pml: int, nt: int, dt: float, fd: float,
              seed: int, nlayers: int = 5, nanom: int = 1, fo: float = 20.0, snaps: int = 20,
              xs_cells: int | None = None, dx: float = 10.0, dz: float = 10.0,
              receivers: str = "all", smooth_cells: float = 0.0):
    """One seeded shot dict (float64 arrays) ready for libqpstd / the oracle."""
    vp, qp = layered_model(nx_model, nz_model, nlayers, nanom, seed, dx=dx)
    if smooth_cells > 0:
        vp = smooth(vp, smooth_cells)
    rho = gardner(vp)
    bbx, bbz = bbx_bbz(rho)
    models = {"vp": vp, "rho": rho, "bbx": bbx, "bbz": bbz}
    visco = kind in (1, 3)
    if visco:
        gam, lam, vwd, tao = transfermodel(fd, fo, vp, qp)
        models.update(gam=gam, lam=lam, vwd=vwd, tao=tao)
    xs = (nx_model // 2 if xs_cells is None else xs_cells) * dx
    zs = 2 * dz
    gxp = np.arange(nx_model) * dx
    gzp = np.full(nx_model, 2 * dz)
    sroffmx = max(abs(gxp.max() - xs), abs(xs - gxp.min()))
    win, nx, nz, xsg, zsg, gxg, gzg = window_shot(models, xs, zs, gxp, gzp, pml, dx, dz, sroffmx)
    d = dict(kind=kind, nxx=nx + 2 * pml, nzz=nz + 2 * pml, pml=pml, dx=dx, dz=dz, dt=dt, fd=fd,
             nt=nt, rik=ricker(nt, dt, fd, 2), xsg=xsg, zsg=zsg, gxg=gxg, gzg=gzg, snaps=snaps,
             etas=1e-20, etar=1e-20, taoc=0.0, seed=seed)
    for k, v in win.items():
        d[k] = v.ravel()
    if visco:
        d["taoc"] = float(win["tao"].max())
    return d


def qrtm4_shots(nt: int = 5000, snaps: int = 30, n: int = 64, seed: int = 1004, kind: int = 3):
    """The batched Q-RTM workload: n shots with uneven windows, nx ~ U(600, 2000)
    columns at a random offset of a seeded 600 (z) x 6000 (x) parent model, CPML
    30, dt 0.5 ms, fd 20 Hz, the source at the window centre and a receiver in
    every window column at z = 2 cells.  The draws do not depend on nt or snaps,
    so a shortened run of shot i has shot i's window."""
    rng = np.random.default_rng(seed)
    parent = parent_model(6000, 600, seed, nlayers=12, nanom=3)
    shots = []
    for _ in range(n):
        nx = int(rng.integers(600, 2001))
        x0 = int(rng.integers(0, 6000 - nx + 1))
        shots.append(window_of_parent(kind, parent, x0, nx, 30, nt, 0.0005, 20.0, snaps))
    return shots


def artm3_shots(nt: int = 6000, snaps: int = 40, seed: int = 1003):
    """The large acoustic RTM shot: 800 (z) x 2400 (x) model, 12 seeded layers and 3
    anomalies, CPML 30, dt 0.5 ms.  Returns (migration shot on the 8-cell Gaussian
    blurred model, the same shot on the unblurred model that makes the observed
    data)."""
    mig = make_shot(2, 2400, 800, 30, nt, 0.0005, 20.0, seed=seed, nlayers=12, nanom=3,
                    smooth_cells=8.0, snaps=snaps)
    true = make_shot(0, 2400, 800, 30, nt, 0.0005, 20.0, seed=seed, nlayers=12, nanom=3)
    return mig, true


def synthetic_obs(d: dict, seed: int) -> np.ndarray:
    """Observed data with the shape of a Q-RTM gather (nt x nr): a few
    hyperbolic reflections of the source wavelet.  The cost of RTM does not
    depend on the values, so the batch does not need 64 modeling runs."""
    rng = np.random.default_rng(seed)
    nt, nr, dt = d["nt"], len(d["gxg"]), d["dt"]
    w = ricker(nt, dt, d["fd"])
    off = (np.asarray(d["gxg"]) - d["xsg"]) * d["dx"]
    obs = np.zeros((nt, nr))
    t = np.arange(nt) * dt
    for _ in range(4):
        t0, v = rng.uniform(0.2, 1.8), rng.uniform(1800.0, 4000.0)
        tr = np.sqrt(t0 ** 2 + (off / v) ** 2)
        idx = np.clip(np.rint(tr / dt).astype(int), 0, nt - 1)
        for j in range(nr):
            k = idx[j]
            obs[k:, j] += rng.uniform(-1, 1) * w[: nt - k]
    return obs.astype(np.float32)
