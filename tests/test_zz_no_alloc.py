"""The allocation-free acoustic entry point (qpstd_ac_advance_noalloc).

It serves callers that cannot call cudaMalloc (code running beside a CUDA
graph capture, plug-ins restricted to the buffers their host hands them,
hosts whose device memory belongs to a pool they do not own).  The test calls
it through the C ABI with device buffers the test owns (torch tensors) and
checks gathers and wavefield state against qpstd_shot_advance on the same
shot, for two calls in a row (steps 0..39, then 40..79), at the tolerance of
the other parity tests (relative L2 <= 1e-4).  This file sorts last so a run
that stops at the first failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

import qpstd
import workloads as W
from cases import rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-4


def _bind():
    f = qpstd.lib().qpstd_ac_advance_noalloc
    f.restype = C.c_int
    f.argtypes = [C.POINTER(qpstd.ShotDesc)] + [C.c_void_p] * 5 + [C.c_int, C.c_int, C.c_void_p, C.c_void_p]
    return f


def test_noalloc_matches_shot_advance_two_calls():
    import torch

    d = W.make_shot(qpstd.APS, 90, 52, 12, 80, 0.001, 25.0, seed=77)
    nxx, nzz, nr = d["nxx"], d["nzz"], len(d["gxg"])
    ref = qpstd.Shot(d)
    dev = torch.device("cuda:0")
    t = lambda a: torch.tensor(np.asarray(a, dtype=np.float32).ravel(), device=dev)
    vp, rho, bbx, bbz = t(d["vp"]), t(d["rho"]), t(d["bbx"]), t(d["bbz"])
    state = torch.zeros(8 * nxx * nzz, dtype=torch.float32, device=dev)
    gather = torch.zeros(40 * nr, dtype=torch.float32, device=dev)
    desc = qpstd.Desc(d)
    fn = _bind()
    stream = torch.cuda.current_stream(dev).cuda_stream
    for t0 in (0, 40):
        g_ref = ref.advance(t0, 40)
        st_ref = ref.get_state()
        rc = fn(C.byref(desc.s), vp.data_ptr(), rho.data_ptr(), bbx.data_ptr(), bbz.data_ptr(),
                state.data_ptr(), t0, 40, gather.data_ptr(), stream)
        assert rc == 0, qpstd.lib().qpstd_last_error().decode()
        torch.cuda.synchronize()
        g = gather.cpu().numpy().reshape(40, nr)
        st = state.cpu().numpy().reshape(8, nxx, nzz)
        assert rel_l2(g, g_ref) < TOL
        for f in range(7):
            assert rel_l2(st[f], st_ref[f]) < TOL, f
    ref.close()


def test_noalloc_rejects_oversized_grid():
    d = W.make_shot(qpstd.APS, 60, 40, 10, 10, 0.001, 25.0, seed=3)
    d = dict(d, nxx=2048, nzz=1024)  # 2 Mi points > QPSTD_NOALLOC_MAX_POINTS
    desc = qpstd.Desc(d)
    fn = _bind()
    one = C.c_void_p(1)
    rc = fn(C.byref(desc.s), one, one, one, one, one, 0, 1, None, None)
    assert rc == -1
    assert "static scratch" in qpstd.lib().qpstd_last_error().decode()
