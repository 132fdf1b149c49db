"""The inner-window field through the C ABI (pf_set/get_window_field): the
arrays rk4par advances, in outer2Inner's layout.

* get_window_field after set_field is the oracle's outer_to_inner of the
  outer field (exact in FP64; in mixed precision the FP32 rounding of it);
* set_window_field, then get_field, is the oracle's inner_to_outer;
* a host driver that keeps the particles and the window field on the host,
  hands them in and reads them back around every rk4par call, and exchanges
  the outer field only around diffraction calls (UndSection's data flow,
  the end-to-end bench pattern) gives the same bits as the resident run.
"""
import numpy as np
import pytest

import puffin_gb300 as P
from puffin_gb300 import configs
from oracle import oracle as O
from tests.oracle_bridge import oracle_config

pytestmark = pytest.mark.gpu


def _setup(precision, seed=5, np_=4096):
    w = configs.config1(np_=np_, seed=seed, nsteps=32)
    w.params.precision = precision
    rng = np.random.default_rng(seed)
    n = w.params.nx * w.params.ny * w.params.nz2
    field = (1e-2 * rng.standard_normal(n), 1e-2 * rng.standard_normal(n))
    return w, field


def _mirrored(cfg, field):
    re, im = (np.array(a) for a in field)
    if cfg.mesh_type == O.MESH_PERIODIC:
        n = cfg.nx * cfg.ny
        re[-n:] = re[:n]
        im[-n:] = im[:n]
    return re, im


@pytest.mark.parametrize("precision", [P.FP64, P.MIXED])
def test_window_field_is_outer_to_inner(precision):
    w, field = _setup(precision)
    cfg = oracle_config(w.params)
    with P.Puffin(w.params) as sim:
        sim.set_particles(*(w.beam[k] for k in P.PARTICLE_KEYS))
        if precision == P.MIXED:  # the mixed path holds the field in FP32
            field = tuple(a.astype(np.float32).astype(np.float64) for a in field)
        sim.set_field(*field)
        nix, niy = sim.window
        assert sim.n_window == nix * niy * cfg.nplanes
        wr, wi = sim.get_window_field()
    re, im = _mirrored(cfg, field)
    er, ei = O.outer_to_inner(cfg, re, im, nix, niy)
    np.testing.assert_array_equal(wr, er)
    np.testing.assert_array_equal(wi, ei)


@pytest.mark.parametrize("precision", [P.FP64, P.MIXED])
def test_set_window_field_then_outer(precision):
    w, field = _setup(precision, seed=9)
    cfg = oracle_config(w.params)
    if precision == P.MIXED:
        field = tuple(a.astype(np.float32).astype(np.float64) for a in field)
    with P.Puffin(w.params) as sim:
        sim.set_particles(*(w.beam[k] for k in P.PARTICLE_KEYS))
        sim.set_field(*field)
        nix, niy = sim.window
        rng = np.random.default_rng(3)
        nw = sim.n_window
        wr = rng.standard_normal(nw).astype(np.float32).astype(np.float64)
        wi = rng.standard_normal(nw).astype(np.float32).astype(np.float64)
        sim.set_window_field(wr, wi)
        gr, gi = sim.get_window_field()
        fr, fi = sim.get_field()
        with pytest.raises(ValueError):
            sim.set_window_field(wr[:-1], wi[:-1])
    np.testing.assert_array_equal(gr, wr)
    np.testing.assert_array_equal(gi, wi)
    re, im = _mirrored(cfg, field)
    O.inner_to_outer(cfg, re, im, wr, wi, nix, niy)
    np.testing.assert_array_equal(fr, re)
    np.testing.assert_array_equal(fi, im)


def test_window_field_needs_particles():
    w, _ = _setup(P.FP64)
    with P.Puffin(w.params) as sim:
        with pytest.raises(P.PuffinError):
            sim.get_window_field()


def test_host_driver_matches_resident_run_bitwise():
    """12 FP64 steps, diffraction every 4: resident state against a host
    driver holding particles and window field on the host (the outer field
    exchanged only around the diffraction calls)."""
    w, field = _setup(P.FP64, seed=13)
    h, every, nsteps = w.h, 4, 12
    with P.Puffin(w.params) as sim:
        sim.set_particles(*(w.beam[k] for k in P.PARTICLE_KEYS))
        sim.set_field(*field)
        szl = 0.0
        for i in range(1, nsteps + 1):
            assert sim.rk4par(szl, h)
            szl += h
            if i % every == 0:
                sim.diffractIM(every * h)
        want_p, want_f = sim.get_particles(), sim.get_field()
    beam = {k: np.array(w.beam[k]) for k in P.PARTICLE_KEYS}
    outer = tuple(np.array(a) for a in field)
    with P.Puffin(w.params) as sim:
        sim.set_particles(*(beam[k] for k in P.PARTICLE_KEYS))
        sim.set_field(*outer)
        outer = sim.get_field()
        win = sim.get_window_field()
        szl = 0.0
        for i in range(1, nsteps + 1):
            diff = i % every == 0
            # outer field, then window, then particles: a window that the
            # particles need larger is re-made from the handle's current
            # field (the driver then reads it back at the new size)
            if diff:
                sim.set_field(*outer)
            sim.set_window_field(*win)
            sim.set_particles(*(beam[k] for k in P.PARTICLE_KEYS))
            assert sim.rk4par(szl, h)
            szl += h
            if diff:
                sim.diffractIM(every * h)
            got = sim.get_particles()
            for k in P.PARTICLE_KEYS:
                beam[k] = got[k]
            win = sim.get_window_field()
            if diff:
                outer = sim.get_field()
        got_f = sim.get_field()
    for k in ("x", "y", "z2", "px", "py", "gam"):
        np.testing.assert_array_equal(beam[k], want_p[k], err_msg=k)
    np.testing.assert_array_equal(got_f[0], want_f[0])
    np.testing.assert_array_equal(got_f[1], want_f[1])
    np.testing.assert_array_equal(outer[0], want_f[0])


def test_host_driver_golden_1d_run():
    """The reference's own 1D end-to-end case (test/testMPIIntegration.pf)
    driven through the host pattern: particles and the window field (here
    the whole 1D field, one node per z2 plane) handed in and read back around
    every rk4par call; the result matches the reference's golden dump to its
    own 1e-10."""
    import os
    from tests import golden_beam as GB
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "f1main_expected.npz"))
    cfg, h = GB.config()
    ob = GB.initial_beam(cfg, g["electrons"][:, 6])
    beam = {k: getattr(ob, k).copy() for k in P.PARTICLE_KEYS}
    p = P.default_params(rho=cfg.rho, aw=cfg.aw, gamma_r=cfg.gamma_r, eta=cfg.eta,
                         kappa=cfg.kappa, fx=cfg.fx, fy=cfg.fy, und_type=P.UND_PUFFIN,
                         nx=1, ny=1, nz2=cfg.nz2, dx=1.0, dy=1.0, dz2=cfg.dz2, one_d=1,
                         szfs=0.0, szfe=cfg.szfe)
    with P.Puffin(p) as sim:
        sim.set_particles(*(beam[k] for k in P.PARTICLE_KEYS))
        sim.set_field(np.zeros(cfg.nz2), np.zeros(cfg.nz2))
        assert sim.window == (1, 1) and sim.n_window == cfg.nz2
        win = sim.get_window_field()
        szl = 0.0
        for _ in range(GB.NSTEPS):
            sim.set_window_field(*win)
            # chi, which rk4par never changes, stays on the device
            sim.set_particles(*(beam[k] for k in P.PARTICLE_KEYS[:6]))
            assert sim.rk4par(szl, h)
            szl += h
            got = sim.get_particles()
            for k in P.PARTICLE_KEYS:
                beam[k] = got[k]
            win = sim.get_window_field()
        taper = sim.get_taper()
    b = O.Beam(*(beam[k] for k in P.PARTICLE_KEYS))
    O.match_out(cfg, b, szl, taper[0])
    O.correct_trans(b)
    e = g["electrons"]
    for j, k in enumerate(("x", "y", "z2", "px", "py", "gam")):
        np.testing.assert_allclose(getattr(b, k), e[:, j], rtol=0, atol=1e-10, err_msg=k)
    np.testing.assert_allclose(win[0], g["aperp"][0], rtol=0, atol=1e-10)
    np.testing.assert_allclose(win[1], g["aperp"][1], rtol=0, atol=1e-10)


def test_host_driver_mixed_matches_resident_run():
    """The same host pattern on the mixed path (FP32 window field: the FP64
    host copy holds FP32 values, so the hand-over is exact): 12 steps with
    diffraction every 4 against the resident mixed run, to the mixed path's
    own run-to-run spread (FP32 atomics land in any order)."""
    w, field = _setup(P.MIXED, seed=21)
    h, every, nsteps = w.h, 4, 12
    with P.Puffin(w.params) as sim:
        sim.set_particles(*(w.beam[k] for k in P.PARTICLE_KEYS))
        sim.set_field(*field)
        szl = 0.0
        for i in range(1, nsteps + 1):
            assert sim.rk4par(szl, h)
            szl += h
            if i % every == 0:
                sim.diffractIM(every * h)
        want_p, want_f = sim.get_particles(), sim.get_field()
    beam = {k: np.array(w.beam[k]) for k in P.PARTICLE_KEYS}
    with P.Puffin(w.params) as sim:
        sim.set_particles(*(beam[k] for k in P.PARTICLE_KEYS))
        sim.set_field(*field)
        outer = sim.get_field()
        win = sim.get_window_field()
        szl = 0.0
        for i in range(1, nsteps + 1):
            diff = i % every == 0
            if diff:
                sim.set_field(*outer)
            sim.set_window_field(*win)
            sim.set_particles(*(beam[k] for k in P.PARTICLE_KEYS))
            assert sim.rk4par(szl, h)
            szl += h
            if diff:
                sim.diffractIM(every * h)
            got = sim.get_particles()
            for k in P.PARTICLE_KEYS:
                beam[k] = got[k]
            win = sim.get_window_field()
            if diff:
                outer = sim.get_field()
    for k in ("x", "y", "z2", "px", "py", "gam"):
        # the tolerances of the mixed graph-block test: FP32 rounding of
        # differently ordered atomics, to 1e-5 of each coordinate's scale
        np.testing.assert_allclose(beam[k], want_p[k], rtol=1e-5, atol=1e-7, err_msg=k)
    scale = max(np.max(np.abs(want_f[0])), np.max(np.abs(want_f[1])))
    np.testing.assert_allclose(outer[0], want_f[0], rtol=0, atol=1e-4 * scale)
    np.testing.assert_allclose(outer[1], want_f[1], rtol=0, atol=1e-4 * scale)


def test_set_particles_keeps_a_covering_window():
    """pf_set_particles computes the window (getInNode) for the first beam,
    grows it for a wider one and keeps it for a narrower one; pf_redistribute
    recomputes it from the particles, as the reference does."""
    w, field = _setup(P.FP64, seed=31, np_=2048)
    beam = {k: np.array(v) for k, v in w.beam.items()}
    narrow = dict(beam, x=0.5 * beam["x"], y=0.5 * beam["y"])
    with P.Puffin(w.params) as sim:
        sim.set_particles(*(narrow[k] for k in P.PARTICLE_KEYS))
        sim.set_field(*field)
        w0 = sim.window
        sim.set_particles(*(beam[k] for k in P.PARTICLE_KEYS))
        w1 = sim.window
        assert w1[0] > w0[0] and w1[1] > w0[1]
        sim.set_particles(*(narrow[k] for k in P.PARTICLE_KEYS))
        assert sim.window == w1
        sim.redistribute()
        assert sim.window == w0
        # the field survives the window changes (inner2Outer before each)
        fr, fi = sim.get_field()
    cfg = oracle_config(w.params)
    re, im = _mirrored(cfg, field)
    np.testing.assert_array_equal(fr, re)
    np.testing.assert_array_equal(fi, im)


def test_keeping_chi_needs_the_same_macroparticles():
    w, field = _setup(P.FP64, seed=33, np_=1024)
    b = w.beam
    with P.Puffin(w.params) as sim:
        with pytest.raises(P.PuffinError):      # no chi on the handle yet
            sim.set_particles(*(b[k] for k in P.PARTICLE_KEYS[:6]))
        sim.set_particles(*(b[k] for k in P.PARTICLE_KEYS))
        sim.set_particles(*(b[k] for k in P.PARTICLE_KEYS[:6]))
        with pytest.raises(P.PuffinError):      # a different count needs its chi
            sim.set_particles(*(b[k][:-1] for k in P.PARTICLE_KEYS[:6]))
        got = sim.get_particles()
    np.testing.assert_array_equal(got["chi"], b["chi"])
