"""Fused passes on x lines longer than one butterfly per thread covers (GPU).

Windows of about 3000 to 4600 points need convolution / Bluestein lengths
(6144 .. 9216) whose smallest radix has more butterflies than a CTA has
threads; the compiled long plans (xplans_list.h, group 3) give each thread
several butterflies per pass.  The tests check such windows against the FP64
oracle (relative L2 <= 1e-4) for the acoustic and the constant-Q step, and that
a 4096-column request of the serving mix is planned in the fused form.
"""
import ctypes as C

import numpy as np
import pytest

import oracle as O
import qpstd
import workloads as W
from cases import rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-4


@pytest.fixture(scope="module", autouse=True)
def _lib():
    qpstd.lib()


def _wide(kind, nx, nz, nt):
    return W.make_shot(kind, nx, nz, 20, nt, 0.0005, 20.0, seed=nx + nz, nlayers=4, nanom=1)


@pytest.mark.parametrize("kind,nx,nz", [(qpstd.APS, 4096, 24), (qpstd.VAPS, 3300, 20), (qpstd.ARTM, 3900, 16)])
def test_long_x_lines_steps_from_random_state(kind, nx, nz):
    d = _wide(kind, nx, nz, 8)
    visco = kind in (qpstd.VAPS, qpstd.QRTM)
    rng = np.random.default_rng(nx)
    st0 = rng.standard_normal((8, d["nxx"], d["nzz"]))
    st0 *= np.array([1.0, 1e-3, 1e-3, 1e-4, 1e-4, 1e-4, 1e-4, 1e-2 if visco else 0.0])[:, None, None]
    ref_st, ref_g = O.OracleShot(d).steps(st0, 0, 4)
    sh = qpstd.Shot(d)
    info = sh.info()
    assert info["x_conv_m"] >= 2 * d["nxx"] - 1 and info["x_conv_m"] > 6000  # a long compiled plan
    sh.set_state(st0.astype(np.float32))
    g = sh.advance(0, 4)
    st = sh.get_state()
    sh.close()
    for f in range(8 if visco else 7):
        assert rel_l2(st[f], ref_st[f]) < TOL, (f, rel_l2(st[f], ref_st[f]))
    assert rel_l2(g, ref_g) < TOL


def test_widest_serving_request_is_fused():
    """The serving mix draws x up to 4096 cells (+ 2 x 20 CPML): fused plans exist
    (qpstd_shot_bytes >= 0), and the served gather equals the oracle's."""
    d = _wide(qpstd.APS, 4096, 20, 40)
    D = qpstd.Desc(d)
    assert qpstd.lib().qpstd_shot_bytes(C.byref(D.s)) > 0
    sv = qpstd.Server(mem_budget=0, max_active=4)
    rid = sv.submit(d, None)
    sv.wait()
    st, _, _ = sv.status(rid)
    assert st == 2
    g = sv.result(rid)
    sv.close()
    ref = O.OracleShot(d).model()
    assert rel_l2(g, ref) < TOL, rel_l2(g, ref)
