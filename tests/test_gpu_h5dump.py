"""Starting GPU runs from Puffin dump files and writing them back
(Puffin.load_dump / save_dump over the C ABI; the reference's layout of
hdf5_puff_coll.f90:43,672 and h5_in.f90:133-370).

* The reference's golden 1D dump (the 2-rank end-to-end test, kept as the
  committed fixture tests/golden/f1main_expected.npz) written in the dump
  layout and loaded into a GPU handle comes back bit for bit, with the
  cumulative step count (iCsteps) it carries.
* A 3D run saved mid-way and resumed in a new handle continues bit for bit
  like the run that never stopped (FP64: deterministic deposit).
"""
import numpy as np
import pytest

import puffin_gb300 as P
from puffin_gb300 import configs
from puffin_gb300 import h5dump as H
from tests import golden_beam as GB

pytestmark = pytest.mark.gpu
GOLD = GB.__file__.replace("golden_beam.py", "golden/f1main_expected.npz")


def test_golden_dump_loads_into_a_gpu_handle(tmp_path):
    g = np.load(GOLD)
    e = g["electrons"]
    beam = {k: e[:, j].copy() for j, k in enumerate(H.PARTICLE_COLUMNS)}
    H.write_particles(tmp_path / "e.h5", beam, {"iCsteps": 30, "zbarLocal": 0.0})
    H.write_field(tmp_path / "f.h5", g["aperp"][0], g["aperp"][1], (1, 1, 511))
    cfg, _ = GB.config()
    p = P.default_params(rho=cfg.rho, aw=cfg.aw, gamma_r=cfg.gamma_r, eta=cfg.eta,
                         kappa=cfg.kappa, fx=cfg.fx, fy=cfg.fy, und_type=P.UND_PUFFIN,
                         nx=1, ny=1, nz2=cfg.nz2, dx=1.0, dy=1.0, dz2=cfg.dz2, one_d=1)
    with P.Puffin(p) as sim:
        attrs = sim.load_dump(tmp_path / "e.h5", tmp_path / "f.h5")
        assert int(attrs["iCsteps"]) == 30 and sim.step_count == 30
        got = sim.get_particles()
        for j, k in enumerate(H.PARTICLE_COLUMNS):
            assert np.array_equal(got[k], e[:, j]), k
        fr, fi = sim.get_field()
        assert np.array_equal(fr, g["aperp"][0]) and np.array_equal(fi, g["aperp"][1])


def test_save_and_resume_continues_bit_for_bit(tmp_path):
    w = configs.config1(np_=20000, seed=12)
    rng = np.random.default_rng(3)
    n = w.params.nx * w.params.ny * w.params.nz2
    field = (1e-3 * rng.standard_normal(n), 1e-3 * rng.standard_normal(n))
    field[0][-w.params.nx * w.params.ny:] = field[0][:w.params.nx * w.params.ny]   # periodic
    field[1][-w.params.nx * w.params.ny:] = field[1][:w.params.nx * w.params.ny]
    with P.Puffin(w.params) as a:
        a.set_particles(*(w.beam[k] for k in P.PARTICLE_KEYS))
        a.set_field(*field)
        z = a.und_section(32, 16, True, w.h, 0.0)
        a.save_dump(tmp_path / "e.h5", tmp_path / "f.h5", {"zbarLocal": z})
        z_a = a.und_section(32, 16, True, w.h, z)
        pa = a.get_particles()
        fa = a.get_field()
    with P.Puffin(w.params) as b:
        attrs = b.load_dump(tmp_path / "e.h5", tmp_path / "f.h5")
        assert b.step_count == 32
        z_b = b.und_section(32, 16, True, w.h, float(attrs["zbarLocal"]))
        pb = b.get_particles()
        fb = b.get_field()
    assert z_a == z_b
    for k in P.PARTICLE_KEYS:
        assert np.array_equal(pa[k], pb[k]), k
    assert np.array_equal(fa[0], fb[0]) and np.array_equal(fa[1], fb[1])
