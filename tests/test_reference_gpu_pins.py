"""The oracle's step equations pinned to the reference's own cuFFT programs.

tests/golden/reference_gpu_gathers.npz holds the gathers that the reference's
aps (acoustic, 400 steps) and vaps (constant-Q power-expansion form, 300 steps)
wrote when built from their own sources for sm_103a and run on a GB300, on
the seeded one-shot case of tests/refgpu_case.py (CPML 10, as the programs
ship).  tests/golden/make_reference_gpu.py made it.  The reference computes in
FP32 with cuFFT; the oracle in FP64.  Tolerance: relative L2 <= 1e-4 (the
path's stated tolerance), measured about 1e-6.

The CPU tests compare the FP64 oracle with the reference's gathers; the GPU
test compares the library's fused path with them.
"""
import os

import numpy as np
import pytest

import oracle as O
import refgpu_case as R
from cases import rel_l2

FIX = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_gpu_gathers.npz")
TOL = 1e-4


@pytest.fixture(scope="module")
def fix():
    if not os.path.exists(FIX):
        pytest.skip("reference GPU gathers not recorded")
    return np.load(FIX)


def test_fixture_geometry_is_the_case(fix):
    gx, gz = R.geometry()
    assert np.array_equal(fix["gx"], gx) and np.array_equal(fix["gz"], gz)
    assert int(fix["pml"]) == 10


@pytest.mark.parametrize("prog,kind", [("aps", R.APS), ("vaps", R.VAPS)])
def test_oracle_matches_reference_cufft_program(fix, prog, kind):
    nt = int(fix[f"{prog}_nt"])
    ref = fix[f"{prog}_gather"].astype(np.float64)
    d = R.shot_desc(kind, nt, 10)
    g = O.OracleShot(d).model()
    err = rel_l2(g, ref)
    assert err < TOL, (prog, err)


@pytest.mark.gpu
@pytest.mark.parametrize("prog,kind", [("aps", R.APS), ("vaps", R.VAPS)])
def test_fused_path_matches_reference_cufft_program(fix, prog, kind):
    import qpstd

    nt = int(fix[f"{prog}_nt"])
    ref = fix[f"{prog}_gather"].astype(np.float64)
    d = R.shot_desc(kind, nt, 10)
    g = qpstd.model_shot(d)
    err = rel_l2(g, ref)
    assert err < TOL, (prog, err)
