"""Pin the oracle's diagnostics against the reference's golden integrated
dump (f1main_expected_integrated.h5): the bunching factor per slice and the
1D power (which the writer scales by the transverse area 2 pi sigma_x sigma_y,
av_write.f90:396, with the single-precision pi)."""
import os

import numpy as np

from oracle import oracle as O
from tests import golden_beam as GB

GOLD = os.path.join(os.path.dirname(__file__), "golden", "f1main_expected.npz")


def test_bunching_matches_golden():
    g = np.load(GOLD)
    cfg, _ = GB.config()
    e = g["electrons"]
    b1 = O.bunching(cfg, e[:, 2], e[:, 6], harmonic=1)
    assert O.num_slices(cfg) == len(g["int_bunchingFundamental"]) == 32
    np.testing.assert_allclose(b1, g["int_bunchingFundamental"], rtol=1e-10, atol=1e-16)


def test_power_1d_matches_golden():
    g = np.load(GOLD)
    cfg, _ = GB.config()
    p = O.power(cfg, g["aperp"][0].copy(), g["aperp"][1].copy())
    ata = float(g["attr_transArea"])
    assert ata == 2.0 * O.PUFFIN_PI * 0.1 * 0.1
    np.testing.assert_allclose(p * ata, g["int_power"], rtol=1e-14, atol=0)


def test_power_3d_uses_single_precision_trapezoid():
    cfg = O.Config(rho=0.005, aw=1.0, gamma_r=500.0, eta=1e-5, kappa=0.2, nx=5, ny=4, nz2=3,
                   dx=0.3, dy=0.2, dz2=0.01)
    rng = np.random.default_rng(0)
    re = rng.standard_normal(60)
    im = rng.standard_normal(60)
    p = O.power(cfg, re, im)
    # against a double-precision trapezoid: equal to single-precision rounding
    inten = (re ** 2 + im ** 2).reshape(3, 4, 5)
    xa = np.linspace(-0.6, 0.6, 5)
    ya = np.linspace(-0.3, 0.3, 4)
    ref = np.trapezoid(np.trapezoid(inten, xa, axis=2), ya, axis=1)
    np.testing.assert_allclose(p, ref, rtol=1e-6)
    assert all(float(np.float32(v)) == v for v in p)
