"""GPU diagnostics (pf_power, pf_bunching, pf_spectrum) against the oracle's
restatement of the reference writer, and against the reference's own golden
integrated dump for the 1D run.

Tolerances:
* power: the reference accumulates the 2D trapezoid in single precision, so
  GPU and oracle agree to a few single-precision ulps (rtol 1e-6); the 1D
  power |A|^2 is exact to 1e-14;
* bunching: FP64 atomics reorder the slice sums, rtol 1e-9 of the largest
  slice value;
* spectrum: a direct DFT on the GPU against numpy's FFT, 1e-10 of the
  largest bin.
"""
import os

import numpy as np
import pytest

import puffin_gb300 as P
from puffin_gb300 import configs
from oracle import oracle as O
from tests import golden_beam as GB
from tests.oracle_bridge import oracle_config

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden", "f1main_expected.npz")


def _state(params, beam, field, steps=0, h=0.0):
    with P.Puffin(params) as sim:
        sim.set_particles(*(beam[k] for k in P.PARTICLE_KEYS))
        sim.set_field(*field)
        szl = 0.0
        for _ in range(steps):
            assert sim.rk4par(szl, h)
            szl += h
        beam_out = sim.get_particles()
        field_out = sim.get_field()
        return (beam_out, field_out, sim.power(), sim.bunching(1), sim.bunching(3),
                sim.spectrum())


def _close(got, want, rel):
    scale = max(float(np.max(np.abs(want))), 1e-300)
    np.testing.assert_allclose(got, want, rtol=0, atol=rel * scale)


def test_golden_1d_power_and_bunching():
    """The reference's end-of-run dump: power x transverse area and the
    fundamental bunching, computed on the GPU from the dumped state."""
    g = np.load(GOLD)
    cfg, _ = GB.config()
    e = g["electrons"]
    beam = {k: np.ascontiguousarray(e[:, j]) for j, k in enumerate(P.PARTICLE_KEYS)}
    p = P.default_params(rho=cfg.rho, aw=cfg.aw, gamma_r=cfg.gamma_r, eta=cfg.eta,
                         kappa=cfg.kappa, fx=cfg.fx, fy=cfg.fy, und_type=P.UND_PUFFIN,
                         nx=1, ny=1, nz2=cfg.nz2, dx=1.0, dy=1.0, dz2=cfg.dz2, one_d=1)
    _, _, pw, b1, _, _ = _state(p, beam, (g["aperp"][0].copy(), g["aperp"][1].copy()))
    np.testing.assert_allclose(pw * float(g["attr_transArea"]), g["int_power"], rtol=1e-14)
    assert len(b1) == 32
    np.testing.assert_allclose(b1, g["int_bunchingFundamental"], rtol=1e-9, atol=1e-15)


@pytest.mark.parametrize("precision", [P.FP64, P.MIXED])
def test_periodic_3d_after_steps(precision):
    w = configs.config1(np_=4000, seed=3)
    w.params.precision = precision
    rng = np.random.default_rng(3)
    n = w.params.nx * w.params.ny * w.params.nz2
    field = (1e-3 * rng.standard_normal(n), 1e-3 * rng.standard_normal(n))
    beam, (fr, fi), pw, b1, b3, (sx, sy) = _state(w.params, w.beam, field, steps=3, h=w.h)
    cfg = oracle_config(w.params)
    np.testing.assert_allclose(pw, O.power(cfg, fr, fi), rtol=1e-6)
    _close(b1, O.bunching(cfg, beam["z2"], beam["chi"], 1), 1e-9)
    _close(b3, O.bunching(cfg, beam["z2"], beam["chi"], 3), 1e-9)
    ox, oy = O.spectrum(cfg, fr, fi)
    _close(sx, ox, 1e-10)
    _close(sy, oy, 1e-10)


def test_temporal_planepole_even_and_odd_nz2():
    for nz2 in (96, 97):
        w = configs.config2(np_=6000, seed=5, nperiods=2, nz2=nz2)
        rng = np.random.default_rng(nz2)
        n = w.params.nx * w.params.ny * w.params.nz2
        field = (1e-3 * rng.standard_normal(n), 1e-3 * rng.standard_normal(n))
        beam, (fr, fi), pw, b1, b3, (sx, sy) = _state(w.params, w.beam, field)
        cfg = oracle_config(w.params)
        np.testing.assert_allclose(pw, O.power(cfg, fr, fi), rtol=1e-6)
        _close(b1, O.bunching(cfg, beam["z2"], beam["chi"], 1), 1e-9)
        _close(b3, O.bunching(cfg, beam["z2"], beam["chi"], 3), 1e-9)
        ox, oy = O.spectrum(cfg, fr, fi)
        assert len(sx) == len(ox) == (nz2 + 2) // 2
        _close(sx, ox, 1e-10)
        _close(sy, oy, 1e-10)


def test_bad_arguments():
    w = configs.config1(np_=500, seed=1)
    with P.Puffin(w.params) as sim:
        sim.set_particles(*(w.beam[k] for k in P.PARTICLE_KEYS))
        with pytest.raises(P.PuffinError):
            sim.bunching(0)
