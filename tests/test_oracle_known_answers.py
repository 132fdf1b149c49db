"""The reference's known answers for its helper formulas, restated in the
oracle: the values test/testFFunctions.pf asserts (testDiffractionLength,
testGainLength, testRaleighLength).  The GPU tests of the diffraction step and
of the cold-beam gain use these formulas as their expected values."""
import math

from oracle import oracle as O


def test_diffraction_length_known_answer():
    # testFFunctions.pf: z = 1, sRaleighLength = 1, sigma = 3 -> 36
    assert abs(O.diffraction_length(1.0, 1.0, 3.0) - 36.0) < 1e-7


def test_gain_length_known_answer():
    # testFFunctions.pf: sWigglerWaveLength = 100e-9, rho = 0.05 ->
    # 1.5915494309189532e-07 (the reference's tolerance is 1e-7 absolute;
    # here 1e-7 relative, which the single-precision pi of the module meets)
    got = O.gain_length(100e-9, 0.05)
    assert abs(got / 1.5915494309189532e-07 - 1.0) < 1e-7


def test_raleigh_length_known_answer():
    # testFFunctions.pf: srho = 0.05, sigma = 1 -> 10
    assert abs(O.raleigh_length(0.05, 1.0) - 10.0) < 1e-7


def test_gaussian_width_growth_from_diffraction_length():
    zr = O.raleigh_length(0.005, 0.75)
    for z in (0.0, 0.5 * zr, zr, 3.0 * zr):
        ratio = O.diffraction_length(z, zr, 0.75) / O.diffraction_length(0.0, zr, 0.75)
        assert abs(ratio - math.sqrt(1.0 + (z / zr) ** 2)) < 1e-15


def test_cold_beam_growth_limits():
    assert abs(O.cold_beam_power_growth(10 ** 6) - math.sqrt(3.0)) < 1e-9
    assert 0.991 < O.cold_beam_power_growth(16) / math.sqrt(3.0) < 0.992
