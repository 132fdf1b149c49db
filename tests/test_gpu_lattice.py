"""Beam-line elements on the GPU against the oracle's restatement of
acc_lattice.f90 (drift, chicane, quad, modulation, matchIn/matchOut,
correctTrans) and the element loop of puffin_module.f90 over a short line.

Tolerances: drift, chicane and quad use only +, -, *, / and sqrt, which the
GPU rounds exactly as the oracle (no FMA contraction), so they must agree
bit for bit; modulation and the matching use the CUDA library's cos/sin
(rtol 1e-15); correctTrans reduces in a different order (1e-15 of the
coordinate scale); the line with two undulator modules is held to the same
1e-9 as the single-module run (the FEL instability amplifies rounding).
"""
import numpy as np
import pytest

import puffin_gb300 as P
from puffin_gb300 import configs, lattice
from oracle import oracle as O
from tests.oracle_bridge import assert_beam_close, oracle_beam, oracle_config

pytestmark = pytest.mark.gpu
KEYS = ("x", "y", "z2", "px", "py", "gam")


@pytest.fixture(scope="module", autouse=True)
def _threads():
    O.set_threads(1)


def _field(params, seed, amp=1e-3):
    rng = np.random.default_rng(seed)
    n = params.nx * params.ny * params.nz2
    re, im = amp * rng.standard_normal(n), amp * rng.standard_normal(n)
    if params.mesh_type == P.MESH_PERIODIC:
        p = params.nx * params.ny
        re[-p:] = re[:p]
        im[-p:] = im[:p]
    return re, im


def _apply(params, beam, fn, field=None):
    with P.Puffin(params) as sim:
        sim.set_particles(*(beam[k] for k in P.PARTICLE_KEYS))
        if field is not None:
            sim.set_field(*field)
        fn(sim)
        return sim.get_particles(), (sim.get_field() if field is not None else None)


def _exact(got, b, keys=KEYS):
    for k in keys:
        np.testing.assert_array_equal(got[k], getattr(b, k), err_msg=k)


def _one_d(w):
    """The same beam on a 1D mesh (nx = ny = 1)."""
    p = w.params
    p.one_d, p.nx, p.ny, p.nix, p.niy = 1, 1, 1, 1, 1
    return w


@pytest.mark.parametrize("one_d", [0, 1])
def test_drift_particles_bit_exact(one_d):
    w = configs.config1(np_=5000, seed=11)
    if one_d:
        w = _one_d(w)
    got, _ = _apply(w.params, w.beam, lambda s: s.drift(0.37, qdiffraction=False))
    cfg = oracle_config(w.params)
    b = oracle_beam(w.beam)
    O.drift(cfg, b, 0.37)
    _exact(got, b)


def test_drift_with_diffraction():
    w = configs.config1(np_=3000, seed=12)
    field = _field(w.params, 12)
    got, gf = _apply(w.params, w.beam, lambda s: s.drift(0.25), field)
    cfg = oracle_config(w.params)
    b = oracle_beam(w.beam)
    O.drift(cfg, b, 0.25)
    re, im = (a.copy() for a in field)
    O.diffract(cfg, re, im, 0.25)
    _exact(got, b)
    scale = max(np.abs(re).max(), np.abs(im).max())
    np.testing.assert_allclose(gf[0], re, rtol=0, atol=1e-12 * scale)
    np.testing.assert_allclose(gf[1], im, rtol=0, atol=1e-12 * scale)


@pytest.mark.parametrize("periodic", [False, True])
def test_chicane(periodic):
    if periodic:
        w = configs.config1(np_=4000, seed=13)
    else:
        w = configs.config2(np_=4000, seed=13, nperiods=2, nz2=128)
    disp, slip = 0.8, 0.05
    got, _ = _apply(w.params, w.beam, lambda s: s.disperse(disp, slip, 0.0, False))
    cfg = oracle_config(w.params)
    b = oracle_beam(w.beam)
    O.chicane(cfg, b, disp, slip)
    if periodic:
        O.wrap_z2(cfg, b.z2)
    _exact(got, b)


def test_quad_bit_exact():
    w = configs.config1(np_=4000, seed=14)
    got, _ = _apply(w.params, w.beam, lambda s: s.quad(3.5, -2.25))
    cfg = oracle_config(w.params)
    b = oracle_beam(w.beam)
    O.quad(cfg, b, 3.5, -2.25)
    _exact(got, b)


def test_modulation():
    w = configs.config1(np_=4000, seed=15)
    got, _ = _apply(w.params, w.beam, lambda s: s.modulation(2e-3, 25.0))
    b = oracle_beam(w.beam)
    O.modulation(b, 2e-3, 25.0)
    assert_beam_close(got, b, rtol=1e-15, atol=0)


@pytest.mark.parametrize("und", [P.UND_PUFFIN, P.UND_HELICAL, P.UND_PLANEPOLE, P.UND_CURVED])
@pytest.mark.parametrize("direction", ["in", "out"])
def test_match(und, direction):
    w = configs.config1(np_=3000, seed=16)
    w.params.und_type = und
    w.params.fx, w.params.fy = (1.0, 1.0) if und == P.UND_HELICAL else (0.0, 1.0)
    w.params.kx_und, w.params.ky_und = 0.3, 0.4
    sz = 0.61

    def fn(s):
        s.set_taper(0.97, 0.97, 0.0)
        (s.matchIn if direction == "in" else s.matchOut)(sz)

    got, _ = _apply(w.params, w.beam, fn)
    cfg = oracle_config(w.params)
    b = oracle_beam(w.beam)
    (O.match_in if direction == "in" else O.match_out)(cfg, b, sz, 0.97)
    assert_beam_close(got, b, rtol=1e-15, atol=1e-17)


def test_correct_trans():
    w = configs.config1(np_=50000, seed=17)
    beam = {k: v.copy() for k, v in w.beam.items()}
    beam["px"] += 0.3
    beam["x"] -= 0.1
    got, _ = _apply(w.params, beam, lambda s: s.correctTrans())
    b = oracle_beam(beam)
    O.correct_trans(b)
    for k in ("x", "y", "px", "py"):
        scale = np.abs(beam[k]).max()
        np.testing.assert_allclose(got[k], getattr(b, k), rtol=0, atol=1e-15 * scale, err_msg=k)
    for k in ("z2", "gam"):
        np.testing.assert_array_equal(got[k], beam[k])
    wsum = np.sum(beam["chi"])
    assert abs(np.sum(got["px"] * beam["chi"]) / wsum) < 1e-15


def test_beam_line_two_modules():
    """Undulator, chicane, quad, drift, modulation, undulator: the element
    loop on the GPU against the oracle's, particles and field."""
    w = configs.config1(np_=4096, seed=18, nsteps=16)
    field = _field(w.params, 18, amp=1e-2)
    und = lattice.Undulator(P.UND_HELICAL, 1.0, 1.0, 0.0, 0.0, 1.0, -1e-3, 16, w.h, 8)
    line = [und,
            lattice.Chicane(zbar=0.2, disp=0.05, slip=0.01),
            lattice.Quad(5.0, -5.0),
            lattice.Drift(0.3),
            lattice.Modulation(1e-4, 1.0 / (2.0 * w.params.rho)),
            lattice.Undulator(P.UND_HELICAL, 1.0, 1.0, 0.0, 0.0, 0.99, 0.0, 16, w.h, 8)]
    with P.Puffin(w.params) as sim:
        sim.set_particles(*(w.beam[k] for k in P.PARTICLE_KEYS))
        sim.set_field(*field)
        sz = lattice.run(sim, line)
        got = sim.get_particles()
        gf = sim.get_field()
        csteps = sim.step_count
    cfg = oracle_config(w.params)
    b = oracle_beam(w.beam)
    re, im = (a.copy() for a in field)
    osz, ocs = O.run_lattice(cfg, b, re, im, [lattice.as_tuple(e) for e in line])
    assert csteps == ocs == 32
    assert sz == osz
    assert_beam_close(got, b, rtol=1e-9, atol=1e-12)
    scale = max(np.abs(re).max(), np.abs(im).max())
    np.testing.assert_allclose(gf[0], re, rtol=0, atol=1e-9 * scale)
    np.testing.assert_allclose(gf[1], im, rtol=0, atol=1e-9 * scale)


def test_lattice_bad_args():
    w = configs.config1(np_=100, seed=1)
    with P.Puffin(w.params) as sim:
        with pytest.raises(P.PuffinError):
            sim.drift(0.1)            # no particles yet
        sim.set_particles(*(w.beam[k] for k in P.PARTICLE_KEYS))
        with pytest.raises(P.PuffinError):
            sim.quad(0.0, 1.0)
        with pytest.raises(P.PuffinError):
            sim.init_undulator(9, 1, 1, 0, 0, 1, 0, 10, 0.1, False)
