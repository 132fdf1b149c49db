"""Host-side beam-line logic (no GPU): the element records, their plain form
for the oracle, and the oracle's element loop without undulator modules."""
import math

import numpy as np

from puffin_gb300 import lattice
from oracle import oracle as O


def _beam(n=64, seed=0):
    rng = np.random.default_rng(seed)
    return O.Beam(rng.standard_normal(n) * 0.3, rng.standard_normal(n) * 0.3,
                  rng.uniform(0.0, 0.4, n), rng.standard_normal(n) * 0.1,
                  rng.standard_normal(n) * 0.1, 1.0 + 1e-3 * rng.standard_normal(n),
                  np.full(n, 2.0))


def _cfg(**kw):
    return O.Config(rho=0.005, aw=1.0, gamma_r=500.0, eta=1e-5, kappa=0.2, nx=25, ny=25, nz2=9,
                    dx=0.2, dy=0.2, dz2=0.05, mesh_type=O.MESH_PERIODIC, **kw)


def test_as_tuple():
    assert lattice.as_tuple(lattice.Drift(0.5)) == ("drift", 0.5)
    assert lattice.as_tuple(lattice.Chicane(0.1, 0.2, 0.3)) == ("chicane", 0.1, 0.2, 0.3)
    u = lattice.Undulator(1, 1.0, 1.0, 0.0, 0.0, 1.0, 0.0, 10, 0.01, 5)
    assert lattice.as_tuple(u)[0] == "undulator" and len(lattice.as_tuple(u)) == 11


def test_oracle_line_without_undulators():
    cfg = _cfg()
    b = _beam()
    ref = _beam()
    line = [("quad", 2.0, -3.0), ("chicane", 0.0, 0.5, 0.02), ("drift", 0.1),
            ("modulation", 1e-3, 7.0)]
    n = cfg.nx * cfg.ny * cfg.nz2
    re, im = np.zeros(n), np.zeros(n)
    sz, csteps = O.run_lattice(cfg, b, re, im, line, qdiffraction=False)
    assert csteps == 0 and sz == 0.1
    O.quad(cfg, ref, 2.0, -3.0)
    O.chicane(cfg, ref, 0.5, 0.02)
    O.wrap_z2(cfg, ref.z2)
    O.drift(cfg, ref, 0.1)
    O.modulation(ref, 1e-3, 7.0)
    for k in ("x", "y", "z2", "px", "py", "gam"):
        np.testing.assert_array_equal(getattr(b, k), getattr(ref, k))
    lenz2 = cfg.dz2 * (cfg.nz2 - 1)
    assert np.all(ref.z2 >= -1e-12)
    assert math.isfinite(lenz2)


def test_init_undulator_ends():
    cfg = _cfg()
    t = O.Taper(1.0, 1.0, 0.0)
    O.init_undulator(cfg, t, O.UND_PLANEPOLE, 0.0, 1.0, 0.0, 0.0, 0.98, -1e-3, 100, 0.01, True)
    assert t.n2col == t.n2col0 == 0.98 and t.undgrad == -1e-3
    assert cfg.szfs == 4.0 * O.PUFFIN_PI * cfg.rho * 2.0
    assert cfg.szfe == 100 * 0.01 - 4.0 * O.PUFFIN_PI * cfg.rho * 2.0
    O.init_undulator(cfg, t, O.UND_HELICAL, 1.0, 1.0, 0.0, 0.0, 1.0, 0.0, 100, 0.01, False)
    assert cfg.szfs == 0.0 and cfg.szfe == 1.0
