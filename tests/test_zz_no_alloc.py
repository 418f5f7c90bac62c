"""The allocation-free acoustic entry point (qpstd_ac_advance_noalloc).

It serves callers that cannot call cudaMalloc: plug-ins restricted to the
buffers their host application hands them, hosts whose device memory belongs
to a pool they do not own, and latency-critical callers that may not allocate.
The tests call it through the C ABI with device buffers the test owns (torch
tensors) and check gathers and wavefield state against qpstd_shot_advance on
the same shot, at the tolerance of the other parity tests (relative L2 <=
1e-4):
  * two calls in a row on one shot (steps 0..39, then 40..79);
  * an artm source side with no gather, then a second shot of another grid
    shape (the static array keeps the previous call's contents, so stale
    state would show);
  * a grid at the size limit (1023 x 1024 points);
  * a grid above the limit is rejected with a status and a message.
This file sorts last so a run that stops at the first failure has already run
every other test.
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


class _Dev:
    """The device buffers a caller of the entry point owns for one shot."""

    def __init__(self, d):
        import torch

        dev = torch.device("cuda:0")
        t = lambda a: torch.tensor(np.asarray(a, dtype=np.float32).ravel(), device=dev)
        self.d = d
        self.vp, self.rho, self.bbx, self.bbz = t(d["vp"]), t(d["rho"]), t(d["bbx"]), t(d["bbz"])
        self.state = torch.zeros(8 * d["nxx"] * d["nzz"], dtype=torch.float32, device=dev)
        self.desc = qpstd.Desc(d)
        self.stream = torch.cuda.current_stream(dev).cuda_stream

    def run(self, t0, n, gather):
        rc = _bind()(C.byref(self.desc.s), self.vp.data_ptr(), self.rho.data_ptr(), self.bbx.data_ptr(),
                     self.bbz.data_ptr(), self.state.data_ptr(), t0, n,
                     gather.data_ptr() if gather is not None else None, self.stream)
        assert rc == 0, qpstd.lib().qpstd_last_error().decode()

    def state_np(self):
        import torch

        torch.cuda.synchronize()
        return self.state.cpu().numpy().reshape(8, self.d["nxx"], self.d["nzz"])


def _compare_state(st, st_ref):
    for f in range(7):
        assert rel_l2(st[f], st_ref[f]) < TOL, (f, rel_l2(st[f], st_ref[f]))


def test_noalloc_matches_shot_advance_two_calls():
    import torch

    d = W.make_shot(qpstd.APS, 90, 52, 12, 80, 0.001, 25.0, seed=77)
    nr = len(d["gxg"])
    ref = qpstd.Shot(d)
    dv = _Dev(d)
    gather = torch.zeros(40 * nr, dtype=torch.float32, device="cuda:0")
    for t0 in (0, 40):
        g_ref = ref.advance(t0, 40)
        st_ref = ref.get_state()
        dv.run(t0, 40, gather)
        st = dv.state_np()
        g = gather.cpu().numpy().reshape(40, nr)
        assert rel_l2(g, g_ref) < TOL
        _compare_state(st, st_ref)
    ref.close()


def test_noalloc_artm_without_gather_then_other_grid():
    """An artm source side with gather=NULL, then an aps shot of another shape
    on the same static array, each against its own qpstd_shot_advance run."""
    import torch

    d1 = W.make_shot(qpstd.ARTM, 120, 70, 15, 60, 0.001, 25.0, seed=78, snaps=4)
    ref1 = qpstd.Shot(d1)
    ref1.advance(0, 60, want_gather=False)
    st_ref1 = ref1.get_state()
    ref1.close()
    dv1 = _Dev(d1)
    dv1.run(0, 60, None)
    _compare_state(dv1.state_np(), st_ref1)

    d2 = W.make_shot(qpstd.APS, 71, 95, 10, 50, 0.001, 25.0, seed=79)
    nr2 = len(d2["gxg"])
    ref2 = qpstd.Shot(d2)
    g_ref2 = ref2.advance(0, 50)
    st_ref2 = ref2.get_state()
    ref2.close()
    dv2 = _Dev(d2)
    gather = torch.zeros(50 * nr2, dtype=torch.float32, device="cuda:0")
    dv2.run(0, 50, gather)
    _compare_state(dv2.state_np(), st_ref2)
    assert rel_l2(gather.cpu().numpy().reshape(50, nr2), g_ref2) < TOL


def test_noalloc_grid_at_the_size_limit():
    """A 999 x 1000 model with CPML 12: 1023 x 1024 padded points, within 0.1 % of
    QPSTD_NOALLOC_MAX_POINTS (the reference's window width is always odd)."""
    import torch

    d = W.make_shot(qpstd.APS, 999, 1000, 12, 12, 0.001, 20.0, seed=80)
    assert (d["nxx"], d["nzz"]) == (1023, 1024)
    nr = len(d["gxg"])
    ref = qpstd.Shot(d)
    g_ref = ref.advance(0, 12)
    st_ref = ref.get_state()
    ref.close()
    dv = _Dev(d)
    gather = torch.zeros(12 * nr, dtype=torch.float32, device="cuda:0")
    dv.run(0, 12, gather)
    _compare_state(dv.state_np(), st_ref)
    assert rel_l2(gather.cpu().numpy().reshape(12, nr), g_ref) < TOL


def test_noalloc_rejects_oversized_grid():
    d = W.make_shot(qpstd.APS, 60, 40, 10, 10, 0.001, 25.0, seed=3)
    d = dict(d, nxx=2048, nzz=1024)  # 2 Mi points > QPSTD_NOALLOC_MAX_POINTS
    desc = qpstd.Desc(d)
    fn = _bind()
    one = C.c_void_p(1)
    rc = fn(C.byref(desc.s), one, one, one, one, one, 0, 1, None, None)
    assert rc == -1
    assert "static scratch" in qpstd.lib().qpstd_last_error().decode()
