"""CPU-side checks of the C ABI: the library loads and exports every symbol
that include/qpstd.h declares (no compute calls without a GPU)."""
import ctypes as C
import os
import re

import pytest

import qpstd

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    inc = os.path.join(ROOT, "include")
    for fn in os.listdir(inc):
        if fn.endswith(".h"):
            src = open(os.path.join(inc, fn)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names |= set(re.findall(r"\b(qpstd_\w+)\s*\(", src))
    return sorted(names)


def test_library_exports_every_declared_symbol():
    if not os.path.exists(qpstd.LIB_PATH):
        qpstd.build()
    lib = C.CDLL(qpstd.LIB_PATH)
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing
    assert len(declared_symbols()) >= 15


def test_python_bindings_cover_the_header():
    assert set(declared_symbols()) <= set(qpstd.EXPORTS)


def test_version_without_gpu():
    assert qpstd.lib().qpstd_version() >= 100


def test_shot_bytes_grows_by_the_snapshot_pool():
    """Host-only estimate (no GPU): each RTM snapshot holds 8 fields of N floats."""
    import workloads as W
    d = W.make_shot(qpstd.QRTM, 60, 40, 10, 50, 0.001, 25.0, seed=3, snaps=4)
    n = d["nxx"] * d["nzz"]
    b4 = qpstd.shot_bytes(d)
    b9 = qpstd.shot_bytes(dict(d, snaps=9))
    assert b9 - b4 == 5 * 32 * n
    assert qpstd.shot_bytes(dict(d, kind=qpstd.VAPS)) < b4


def test_shot_bytes_marks_windows_the_fused_passes_cannot_plan():
    import workloads as W
    # x lines up to about 4600 points plan (compiled long plans); 6000 do not
    d = W.make_shot(qpstd.APS, 4096, 24, 10, 40, 0.0005, 25.0, seed=9)
    assert qpstd.shot_bytes(d) > 0
    d = W.make_shot(qpstd.APS, 6000, 24, 10, 40, 0.0005, 25.0, seed=9)
    assert qpstd.shot_bytes(d) == -1
    assert qpstd.shot_bytes(dict(d, method=qpstd.PLAIN)) > 0


def test_pml_profiles_match_the_oracle():
    """qpstd_pml_profiles (the tables the library applies; the acforward shims
    warn when their caller's differ) against the FP64 oracle's restatement of
    get_pml_parameters."""
    import numpy as np

    import oracle as O
    nxx, nzz, pml = 139, 97, 20
    out = np.zeros(4 * (nxx + nzz), dtype=np.float32)
    assert qpstd.lib().qpstd_pml_profiles(pml, 20.0, nxx, nzz, 10.0, 12.0, 0.001, out.ctypes.data_as(qpstd._fp)) == 0
    ref = O.pml_coeffs(pml, 20.0, nxx, nzz, 10.0, 12.0, 0.001)
    order = ["i_ax", "i_bx", "h_ax", "h_bx", "i_az", "i_bz", "h_az", "h_bz"]
    q = 0
    for name in order:
        n = nxx if name.endswith("x") else nzz
        assert np.allclose(out[q:q + n], ref[name], rtol=1e-6, atol=1e-7), name
        q += n
