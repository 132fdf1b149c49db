"""The FEL figures of merit (puffin_gb300.fel) on synthetic pulse-energy
curves with known answers: exponential growth with a chosen gain length,
saturation and synchrotron oscillation."""
import numpy as np
import pytest

from puffin_gb300 import fel


def _curve(lg=0.7, zsat=8.0, esat=1.0, n=600, zmax=12.0):
    z = np.linspace(0.05, zmax, n)
    grow = esat * np.exp((z - zsat) / lg)
    osc = esat * (0.75 + 0.25 * np.cos(2 * np.pi * (z - zsat) / 2.5))
    return z, np.where(z < zsat, grow, osc)


def test_gain_length_and_saturation():
    z, e = _curve()
    zs, es = fel.saturation(z, e)
    assert zs == pytest.approx(8.0, abs=0.05)
    assert es == pytest.approx(1.0, rel=1e-3)
    lg, za, zb = fel.gain_length(z, e)
    assert lg == pytest.approx(0.7, rel=1e-6)
    assert za < zb < zs


def test_compare_reports_relative_differences():
    z, e0 = _curve(lg=0.7)
    _, e1 = _curve(lg=0.7035, esat=1.005)
    c = fel.compare(z, e0, e1)
    assert c["gain_length"]["rel_diff"] == pytest.approx(0.005, rel=1e-3)
    assert c["saturated_energy"]["rel_diff"] == pytest.approx(0.005, rel=0.05)


def test_noisy_start_is_not_saturation():
    z, e = _curve()
    e = e * (1.0 + 0.2 * np.sin(40 * z) * (z < 1.0))  # wiggles in the lethargy
    zs, _ = fel.saturation(z, e)
    assert zs == pytest.approx(8.0, abs=0.05)
