"""Synthetic initial conditions of the benchmark problems (CPU)."""
import numpy as np
import pytest

from pluto_gb300 import problems


@pytest.mark.parametrize("n", [8, 12])
def test_turbulence_fft_equals_direct_mode_sum(n):
    """The inverse-FFT evaluation of the turbulence mode table gives the
    term-by-term sum to round-off, cell and face fields alike, and the face
    field stays divergence-free."""
    sd, vd, fd = problems.turbulence3d(n, fft=False)
    sf, vf, ff = problems.turbulence3d(n, fft=True)
    assert sd == sf
    assert np.abs(vf - vd).max() <= 1e-12 * np.abs(vd).max()
    for a, b in zip(ff, fd):
        assert a.shape == b.shape
        assert np.abs(a - b).max() <= 1e-12 * np.abs(b).max()
    bx, by, bz = ff
    div = (bx[:, :, 1:] - bx[:, :, :-1]) + (by[:, 1:, :] - by[:, :-1, :]) + (bz[1:] - bz[:-1])
    assert np.abs(div).max() <= 1e-12 * np.abs(bx).max()
