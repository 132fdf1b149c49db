"""Pin the CPU oracle against the reference's own golden dump.

Mirrors test/testMPIIntegration.pf:84-128: 319 macroparticles, 511 z2 nodes,
every coordinate and both field components within 1e-10 of the expected
values.  The oracle actually matches far tighter, so the ordered comparison
below also asserts 1e-14.
"""
import os

import numpy as np
import pytest

from oracle import oracle as O
from tests import golden_beam as GB

GOLD = os.path.join(os.path.dirname(__file__), "golden", "f1main_expected.npz")


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLD)


@pytest.fixture(scope="module")
def oracle_run(golden):
    O.set_threads(1)
    cfg, h = GB.config()
    beam = GB.initial_beam(cfg, golden["electrons"][:, 6])
    wr = np.zeros(cfg.nplanes)
    wi = np.zeros(cfg.nplanes)
    taper = O.Taper(1.0, 1.0, 0.0)
    szl = 0.0
    for _ in range(GB.NSTEPS):
        assert O.rk4_step(cfg, taper, szl, h, beam, wr, wi, 1, 1) == 0
        szl = szl + h
    O.match_out(cfg, beam, szl, taper.n2col)
    O.correct_trans(beam)
    return cfg, h, szl, beam, wr, wi


def test_scaling_constants(golden):
    cfg, h = GB.config()
    assert cfg.eta == float(golden["attr_eta"])
    assert cfg.kappa == float(golden["attr_kappa"])
    assert h == float(golden["attr_sStepSize"])
    assert cfg.dz2 == float(golden["attr_sLengthOfElmZ2"])
    assert cfg.nz2 == int(golden["attr_nZ2"]) == 511


def test_counts_and_zbar(golden, oracle_run):
    _, _, szl, beam, _, _ = oracle_run
    assert beam.n == golden["electrons"].shape[0] == 319
    assert szl == float(golden["attr_zbarTotal"])


def test_electrons_match_reference_tolerance(golden, oracle_run):
    """The reference test's own, order-insensitive 1e-10 check."""
    e = golden["electrons"]
    beam = oracle_run[3]
    for j, k in enumerate(("x", "y", "z2", "px", "py", "gam")):
        got = getattr(beam, k)
        for v in got:
            assert np.any(np.abs(e[:, j] - v) <= 1e-10), k


def test_electrons_ordered_tight(golden, oracle_run):
    e = golden["electrons"]
    beam = oracle_run[3]
    for j, k in enumerate(("x", "y", "z2", "px", "py", "gam")):
        np.testing.assert_allclose(getattr(beam, k), e[:, j], rtol=0, atol=1e-14, err_msg=k)
    # z2 and Gamma reproduce the reference bit for bit
    np.testing.assert_array_equal(beam.z2, e[:, 2])
    np.testing.assert_array_equal(beam.gam, e[:, 5])


def test_field_matches(golden, oracle_run):
    _, _, _, _, wr, wi = oracle_run
    np.testing.assert_allclose(wr, golden["aperp"][0], rtol=0, atol=1e-10)
    np.testing.assert_allclose(wi, golden["aperp"][1], rtol=0, atol=1e-10)
    np.testing.assert_allclose(wr, golden["aperp"][0], rtol=0, atol=1e-15)
    np.testing.assert_allclose(wi, golden["aperp"][1], rtol=0, atol=1e-15)
