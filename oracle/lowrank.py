"""FP64 restatement of the reference's low-rank form (TEST INFRASTRUCTURE ONLY).

Only tests/ may import this module; it is the checker of the library's
low-rank decomposition and of its device operator, never a product path.

Follows sgpstd-qmodeling/sglowrank.c:
  * the symbol W(x, k) = sinc(vp dt k^(1+g)/2) k^g sqrt(1 + dt tau k^1.01/2),
    sinc(u) = sin(u)/u                                   (:251-257, 301, 339, 398)
  * acsglowrank2d: random samples, greedy column / row selection with
    projection removal, A = pinv(Us) Mes pinv(Vs)        (:148-480)
  * checka_error: exact row against the approximation   (:61-101)
  * consist_Vt: the half-grid factors mirrored to the full grid (:103-145)
and the apply kernels of sgpstd-qmodeling/acsglw.cu:1375-1497 (multv_kernel,
fuzhi_to_ifftrow, sumlw_kernel, sumlw2_kernel): out = sum_a U[x,a] sum_b
A[a,b] Re IFFT2(FFT2(p) Vt_b) (numpy's ifft2 carries the 1/N of multv_kernel).
The half-grid |k| is cal_k2dh (sgpstd-qmodeling/func.c:783-811), pinned to the
reference's own compiled function through tests/golden.

Parity of the decomposition itself is unpinned: sglowrank.c does not compile
(it includes 4GINV.C, which is not in the reference tree) and it draws its
samples from rand() seeded by the clock.  This restatement therefore uses the
same seeded splitmix64 draws as the library, so the two must choose the same
wavenumbers and points, and the tests add properties that hold for any
correct decomposition (exactness for piecewise-constant models of at most
rank materials, small approximation error on smooth models).
"""
from __future__ import annotations

import numpy as np

REF_PI = 3.1415926  # func.c:6
MASK = (1 << 64) - 1


class SplitMix64:
    def __init__(self, seed: int):
        self.s = seed & MASK

    def next(self) -> int:
        self.s = (self.s + 0x9E3779B97F4A7C15) & MASK
        z = self.s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK
        return z ^ (z >> 31)


def draw_distinct(g: SplitMix64, n: int, count: int) -> list:
    """random_select (sglowrank.c:5-22) on the seeded generator."""
    count = min(count, n)
    out, seen = [], set()
    while len(out) < count:
        v = g.next() % n
        if v not in seen:
            seen.add(v)
            out.append(v)
    return out


def khalf(nxx: int, nzz: int, dx: float, dz: float) -> np.ndarray:
    """cal_k2dh: |k| on the half grid (nxx//2+1) x (nzz//2+1), k[0] = 1e-6."""
    def kk(n, d):
        dk = 2.0 * REF_PI / (n * d)
        i = np.arange(n // 2 + 1)
        return i * dk
    kx, kz = kk(nxx, dx), kk(nzz, dz)
    k = np.sqrt(kx[:, None] ** 2 + kz[None, :] ** 2).ravel()
    k[0] = 1.0e-6
    return k


def symbol(vp, gam, tao, dt, k):
    vp, gam, tao, k = (np.asarray(a, dtype=np.float64) for a in (vp, gam, tao, k))
    u = 0.5 * vp * dt * k ** (1.0 + gam)
    sinc = np.where(u == 0.0, 1.0, np.sin(u) / np.where(u == 0.0, 1.0, u))
    return sinc * k ** gam * np.sqrt(1.0 + 0.5 * dt * tao * k ** 1.01)


def _greedy(S: np.ndarray, count: int) -> list:
    """S: candidates x samples (float64, deflated in place)."""
    ncand = S.shape[0]
    taken = np.zeros(ncand, dtype=bool)
    chosen, kept = [], []
    for n in range(count):
        nrm = np.einsum("ij,ij->i", S, S)
        pick, mx = -1, 0.0
        for c in np.argsort(-nrm, kind="stable"):
            if not taken[c]:
                if nrm[c] - mx > 0.0:
                    pick = int(c)
                break
        if pick < 0:
            pick = int(np.flatnonzero(~taken)[0])
        chosen.append(pick)
        taken[pick] = True
        if n == count - 1:
            break
        kept.append(S[pick].copy())
        rest = np.flatnonzero(~taken)
        for kb in kept:
            kk = kb @ kb
            if kk == 0.0:
                continue
            t = (S[rest] @ kb) / kk
            S[rest] -= t[:, None] * kb[None, :]
    return chosen


def decompose(nxx, nzz, dx, dz, dt, vp, tao, gam, row, col, seed=1):
    """acsglowrank2d in FP64; returns dict U (N1 x col), V (row x N2), A, jrr, irr."""
    vp, tao, gam = (np.asarray(a, dtype=np.float64).ravel() for a in (vp, tao, gam))
    N1 = nxx * nzz
    k = khalf(nxx, nzz, dx, dz)
    N2 = k.size
    g = SplitMix64(seed)
    W = lambda xs, ks: symbol(vp[xs][:, None], gam[xs][:, None], tao[xs][:, None], dt, k[ks][None, :])
    mm = min(N1, int(col * np.log(N1)))
    r1 = draw_distinct(g, N1, mm)
    Sr = W(np.array(r1), np.arange(N2)).T.copy()  # wavenumber-major
    jrr = _greedy(Sr, col)
    U = W(np.arange(N1), np.array(jrr))
    nn = min(N2, int(row * np.log(N2)))
    r2 = draw_distinct(g, N2, nn)
    Sc = W(np.arange(N1), np.array(r2)).copy()   # point-major
    irr = _greedy(Sc, row)
    V = W(np.array(irr), np.arange(N2))
    npn = min(mm, nn)
    r3 = np.array(draw_distinct(g, N1, npn))
    r4 = np.array(draw_distinct(g, N2, npn))
    Us = W(r3, np.array(jrr))
    Vs = W(np.array(irr), r4)
    Mes = W(r3, r4)
    A = np.linalg.pinv(Us, rcond=1e-8) @ Mes @ np.linalg.pinv(Vs, rcond=1e-8)
    return {"U": U, "V": V, "A": A, "jrr": np.array(jrr), "irr": np.array(irr)}


def mirror(V: np.ndarray, nxx: int, nzz: int) -> np.ndarray:
    """consist_Vt: row x (nxh*nzh) -> row x nxx x nzz."""
    nxh, nzh = nxx // 2 + 1, nzz // 2 + 1
    ix = np.arange(nxx)
    ix = np.where(ix < nxh, ix, nxx - ix)
    iz = np.arange(nzz)
    iz = np.where(iz < nzh, iz, nzz - iz)
    Vh = np.asarray(V, dtype=np.float64).reshape(-1, nxh, nzh)
    return Vh[:, ix][:, :, iz]


def apply(U, V, A, field, nxx, nzz):
    """out = sum_a U[x,a] sum_b A[a,b] Re IFFT2(FFT2(field) Vt_b), FP64."""
    P = np.fft.fft2(np.asarray(field, dtype=np.float64).reshape(nxx, nzz))
    Vt = mirror(V, nxx, nzz)
    q = np.stack([np.fft.ifft2(P * Vt[b]).real.ravel() for b in range(Vt.shape[0])])  # row x N1
    pst = np.asarray(A, dtype=np.float64) @ q                                        # col x N1
    return np.einsum("xa,ax->x", np.asarray(U, dtype=np.float64), pst).reshape(nxx, nzz)


def apply_exact(vp, tao, gam, dt, dx, dz, field, nxx, nzz):
    """The mixed-domain operator itself: sum_k W(x,k) P(k) e^{ikx} / N (small grids)."""
    k = khalf(nxx, nzz, dx, dz)
    vp, tao, gam = (np.asarray(a, dtype=np.float64).ravel() for a in (vp, tao, gam))
    P = np.fft.fft2(np.asarray(field, dtype=np.float64).reshape(nxx, nzz)).ravel()
    N = nxx * nzz
    Wh = symbol(vp[:, None], gam[:, None], tao[:, None], dt, k[None, :])           # N x N2
    Wf = mirror(Wh, nxx, nzz).reshape(N, N)                                          # N x N
    xi, zi = np.divmod(np.arange(N), nzz)
    ph = np.exp(2j * np.pi * (np.outer(xi, xi) / nxx + np.outer(zi, zi) / nzz))     # e^{i k x}
    return (np.einsum("xk,xk->x", Wf, ph * P[None, :]).real / N).reshape(nxx, nzz)


def check(U, V, A, vp, tao, gam, dt, dx, dz, nxx, nzz, point):
    """checka_error: exact row W(x_point, k) and its approximation."""
    k = khalf(nxx, nzz, dx, dz)
    vp, tao, gam = (np.asarray(a, dtype=np.float64).ravel() for a in (vp, tao, gam))
    We = symbol(vp[point], gam[point], tao[point], dt, k)
    tp = np.asarray(U, dtype=np.float64)[point] @ np.asarray(A, dtype=np.float64)
    return We, tp @ np.asarray(V, dtype=np.float64)
