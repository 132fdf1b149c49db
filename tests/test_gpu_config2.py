"""The FP64 drop-in configuration at its own size against the oracle.

Temporal 129 x 129 x 4096 mesh, planepole undulator (aw_rms 0.8), rho =
0.002, gamma_r = 2000, -1 % linear taper, 2^23 macroparticles on a flat top
over 80 % of z2: eight RK4 steps with diffraction every eight (the first half
step, then the merged half steps of UndSection, puffin/lib/undulator.f90:
106-331) through pf_run, against the oracle's UndSection on the same seeded
beam at the reference's own tolerance of 1e-10 relative
(test/testMPIIntegration.pf:94-128), and a second GPU run that must give the
same bits (the FP64 path is bit-reproducible run to run: integer deposit).

This runs the dense path of the headline benchmark as one piece: the 37 x 37
x 4096 window, the prime-factor 129-point transverse FFT and the four-step
4096-point z2 transform, the temporal mask, the taper and the planepole
b-fields.  The oracle takes about 10-20 s on 16 host cores.
"""
import numpy as np
import pytest

import puffin_gb300 as P
from puffin_gb300 import configs
from oracle import oracle as O
from tests.oracle_bridge import oracle_beam, oracle_config

pytestmark = pytest.mark.gpu

NSTEPS, EVERY = 8, 8


def _gpu_run(w):
    with P.Puffin(w.params) as sim:
        sim.set_particles(*(w.beam[k] for k in P.PARTICLE_KEYS))
        sim.set_field(*w.field)
        z = sim.und_section(NSTEPS, EVERY, True, w.h, 0.0)
        parts = sim.get_particles()
        fr, fi = sim.get_field()
        win = sim.window
    return parts, (fr, fi), win, z


@pytest.fixture(scope="module")
def config2_runs():
    w = configs.config2()
    assert w.np == 2 ** 23 and (w.params.nx, w.params.ny, w.params.nz2) == (129, 129, 4096)
    first = _gpu_run(w)
    second = _gpu_run(w)
    return w, first, second


def test_config2_is_bit_reproducible_run_to_run(config2_runs):
    _, (p1, f1, w1, z1), (p2, f2, w2, z2) = config2_runs
    assert w1 == w2 and z1 == z2
    for k in P.PARTICLE_KEYS:
        assert np.array_equal(p1[k].view(np.int64), p2[k].view(np.int64)), k
    assert np.array_equal(f1[0].view(np.int64), f2[0].view(np.int64))
    assert np.array_equal(f1[1].view(np.int64), f2[1].view(np.int64))


def test_config2_matches_the_oracle_at_1e10(config2_runs):
    w, (parts, (fr, fi), win, z), _ = config2_runs
    O.set_threads(max(1, __import__("os").cpu_count() or 1))
    cfg = oracle_config(w.params)
    beam = oracle_beam(w.beam)
    re, im = (np.array(a) for a in w.field)
    r = O.undulator_run(cfg, beam, re, im, w.h, NSTEPS, EVERY, True)
    assert r.status == 0 and r.steps == NSTEPS
    assert tuple(r.window) == tuple(win)
    for k in ("x", "y", "z2", "px", "py", "gam"):
        want = getattr(beam, k)
        np.testing.assert_allclose(parts[k], want, rtol=1e-10,
                                   atol=1e-10 * max(np.max(np.abs(want)), 1e-300), err_msg=k)
    scale = max(np.max(np.abs(re)), np.max(np.abs(im)))
    assert scale > 0.0                   # the beam has radiated into the zero seed
    np.testing.assert_allclose(fr, re, rtol=0, atol=1e-10 * scale)
    np.testing.assert_allclose(fi, im, rtol=0, atol=1e-10 * scale)
