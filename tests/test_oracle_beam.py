"""The oracle's quiet-start generator on its own: Halton values against the
sequence's definition (radical inverse), the Gaussian projection against the
inverse CDF, and the statistics of the shot noise."""
import math
from statistics import NormalDist

import numpy as np

from oracle import oracle as O


def test_halton_is_the_radical_inverse():
    assert O.halton(1, 2) == 0.5
    assert O.halton(2, 2) == 0.25
    assert O.halton(3, 2) == 0.75
    assert O.halton(1, 3) == 1.0 / 3.0
    assert abs(O.halton(7, 3) - (1.0 / 3.0 + 2.0 / 9.0)) < 1e-16   # 7 = 21 (base 3)
    assert abs(O.halton(12, 13) - 12.0 / 13.0) < 1e-16


def test_projection_inverts_the_gaussian_cdf():
    u = np.linspace(0.01, 0.99, 99)
    got = O.project_gauss(u)
    want = np.array([NormalDist().inv_cdf(v) for v in u])
    np.testing.assert_allclose(got, want, atol=5e-5)   # linear on a 0.004-wide mesh
    assert O.project_gauss([0.0])[0] == -4.0 and abs(O.project_gauss([1.0])[0] - 4.0) < 1e-14


def test_generator_layout_and_noise_statistics():
    ns, nseq = 40, 50
    z2m = (np.arange(ns) + 0.5) * 0.1
    ne = np.full(ns, 5.0e3)     # 100 electrons per beamlet: the normal branch
    mean = [0.0, 0.1, 0.0, 0.0, 1.0]
    sig = [1.0, 0.5, 0.01, 0.01, 1e-3]
    quiet = O.generate_beam(z2m, ne, 0.1, nseq, mean, sig, False, 7, 2.0)
    assert quiet.n == ns * nseq
    np.testing.assert_allclose(quiet.chi, 2.0 * 100.0)
    # the same sequence in every slice, shifted to the slice centre
    np.testing.assert_allclose(quiet.x[:nseq], quiet.x[nseq:2 * nseq])
    np.testing.assert_allclose(quiet.z2[nseq:2 * nseq] - quiet.z2[:nseq], 0.1, atol=1e-15)
    noisy = O.generate_beam(z2m, ne, 0.1, nseq, mean, sig, True, 7, 2.0)
    again = O.generate_beam(z2m, ne, 0.1, nseq, mean, sig, True, 7, 2.0)
    np.testing.assert_array_equal(noisy.z2, again.z2)       # seeded: reproducible
    dev = (noisy.z2 - quiet.z2) * np.sqrt(noisy.chi / 2.0) / 0.1   # (u - 1/2)
    assert np.all(np.abs(dev) <= 0.5)
    assert abs(np.mean(dev)) < 0.02 and abs(np.var(dev) - 1.0 / 12.0) < 0.01
    counts = noisy.chi / 2.0
    assert abs(np.mean(counts) - 100.0) < 1.0 and abs(np.var(counts) / 100.0 - 1.0) < 0.1
    # small counts: Knuth's branch; a zero draw keeps the beamlet's count
    # (noise.f90:55-58), so the mean is 3 + 3 exp(-3)
    low = O.generate_beam(z2m, np.full(ns, 150.0), 0.1, nseq, mean, sig, True, 11, 1.0)
    c = low.chi
    assert abs(np.mean(c) - (3.0 + 3.0 * math.exp(-3.0))) < 0.1
    assert np.all(c >= 1.0)
