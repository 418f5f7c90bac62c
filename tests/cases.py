"""Seeded shot cases shared by the parity tests (small enough for the oracle)."""
import numpy as np

import workloads as W


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def small_shot(kind, nx=60, nz=40, pml=10, nt=240, seed=11, **kw):
    return W.make_shot(kind, nx, nz, pml, nt, 0.001, 25.0, seed, **kw)


def grid439_shot(kind=0, nt=2000, seed=1001):
    """The 160 x 398 model geometry: CPML 20 -> padded 439 x 200, 398 receivers."""
    return W.make_shot(kind, 398, 160, 20, nt, 0.001, 20.0, seed, nlayers=5, nanom=1, fo=20.0)
