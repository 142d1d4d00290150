"""The wall-pressure spectrum (accuracy.wall_psd), the surface-pressure PSD
output of the mixed-precision error report (no counterpart in the reference,
which writes whole fields at intervals): known answers on synthetic series
sampled at a varying time step, as the CFL time step samples the recorder."""
import numpy as np
import pytest

from tandemproject_gb300.accuracy import wall_psd


def varying_times(n, t_end, seed=3):
    rng = np.random.default_rng(seed)
    dt = 1.0 + 0.3 * rng.random(n - 1)  # steps vary by 30 %, as CFL time steps do
    t = np.concatenate([[0.0], np.cumsum(dt)])
    return t * (t_end / t[-1])


def test_sinusoid_peak_and_power():
    """A sinusoid of amplitude A at f0: the spectrum peaks within one bin of
    f0, and its integral is the variance A^2 / 2 (to the Hann window's
    leakage and the resampling, 2 %)."""
    n, t_end, f0 = 4000, 50.0, 1.7
    t = varying_times(n, t_end)
    amps = np.array([0.3, 0.05])
    p = 1 / 1.4 + amps[None, :] * np.sin(2 * np.pi * f0 * t[:, None] + np.array([0.2, 1.1])[None, :])
    f, s = wall_psd(t, p)
    df = f[1] - f[0]
    assert abs(f[np.argmax(s)] - f0) <= df
    power = float(np.sum(s) * df)
    assert power == pytest.approx(np.mean(amps ** 2 / 2), rel=0.02)
    # nothing far from f0
    far = np.abs(f - f0) > 10 * df
    assert np.sum(s[far]) * df < 1e-3 * power


def test_two_tones_power_ratio():
    """Two tones of amplitudes 1 and 0.25: the power near each peak is in the
    ratio 16 : 1."""
    n, t_end = 8000, 80.0
    t = varying_times(n, t_end, seed=11)
    p = (np.sin(2 * np.pi * 0.9 * t) + 0.25 * np.sin(2 * np.pi * 3.1 * t))[:, None]
    f, s = wall_psd(t, p)
    df = f[1] - f[0]

    def band(fc):
        m = np.abs(f - fc) <= 5 * df
        return float(np.sum(s[m]) * df)

    assert band(0.9) / band(3.1) == pytest.approx(16.0, rel=0.03)
    assert band(0.9) == pytest.approx(0.5, rel=0.02)


def test_constant_and_frequency_axis():
    """A constant series has no power; the frequency axis is the uniform
    resampling's rfft axis (n points over the recorded time span)."""
    t = varying_times(1000, 10.0)
    f, s = wall_psd(t, np.full((1000, 3), 0.71))
    assert np.max(s) < 1e-28  # (the mean's rounding leaves ~1e-17)
    assert f.size == 501 and f[1] == pytest.approx(1.0 / (10.0 * 1000 / 999), rel=1e-12)
