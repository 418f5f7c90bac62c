"""Known-answer checks of the oracle's operators (no GPU).

The reference ships no golden outputs for its stepping path, so besides the
coefficient pins the oracle is checked against answers known in closed form:
the half-cell shifted spectral derivatives that the shift tables define
(cal_shift_parameters, sgpstd-qmodeling/funca.c:342-432, applied as in
shift_vxz_kernel / shift_pxz_kernel, acps4.cu:1047-1108) differentiate every
resolved Fourier mode exactly, at x - dx/2 ("m" tables, velocity divergence)
and at x + dx/2 ("c" tables, pressure gradient).  For odd n the reference
mirrors the shift phases at index n/2*2-i (funca.c:397), so its symbol is not
the shifted derivative there; even lengths carry the exact answer.
"""
import numpy as np
import pytest

import oracle as O


def _apply(a, b, u):
    """Re IFFT(H FFT(u)) with the reference's symbol H = -b + i a below n/2+1, b - i a above."""
    n = u.size
    i = np.arange(n)
    H = np.where(i < n // 2 + 1, -b + 1j * a, b - 1j * a)
    return np.fft.ifft(H * np.fft.fft(u)).real


@pytest.mark.parametrize("n", [64, 200, 440, 860])
def test_shifted_spectral_derivatives_are_exact(n):
    dx = 10.0
    t = O.shift_tables(n, n, dx, dx)
    x = np.arange(n) * dx
    L = n * dx
    for m0 in (1, 5, n // 4, n // 2 - 1):
        k = 2 * np.pi * m0 / L
        u = np.sin(k * x)
        # the reference's pi is 3.1415926, so its wavenumbers are k * 3.1415926 / pi
        ks = k * 3.1415926 / np.pi
        dm = _apply(t["kxsmr"], t["kxsmi"], u)
        dc = _apply(t["kxscr"], t["kxsci"], u)
        assert np.abs(dm - ks * np.cos(k * (x - dx / 2))).max() < 1e-6 * ks, (n, m0)
        assert np.abs(dc - ks * np.cos(k * (x + dx / 2))).max() < 1e-6 * ks, (n, m0)
