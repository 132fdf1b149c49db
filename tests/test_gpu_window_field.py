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
