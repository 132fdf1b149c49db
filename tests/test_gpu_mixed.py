"""Mixed-precision path (FP32 field, weights, deposit and FFT; FP64 state,
p2 and RK4 combination) against the FP64 CPU oracle.

Tolerances are FP32-level and stated per quantity: one RK4 step moves the
particles by h * slope, and the slopes carry FP32 relative error (~1e-7), so
particle coordinates agree to rtol 1e-6 / atol 1e-8; the field (stored in
FP32) to 2e-5 of its scale; a diffraction call (FP32 FFT of ~10^5 points) to
2e-5 of the field scale; after 32 steps with diffraction the radiated power
(sum |A|^2 over the mesh) to 1e-4 relative.
"""
import numpy as np
import pytest

import puffin_gb300 as P
from puffin_gb300 import configs
from oracle import oracle as O
from tests.oracle_bridge import assert_beam_close, oracle_beam, oracle_config
from tests.test_gpu_parity import (field_close, random_field, run_gpu_steps,
                                   run_oracle_steps)

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _threads():
    O.set_threads(1)


def mixed(params):
    q = P.Params.from_buffer_copy(params)
    q.precision = P.MIXED
    return q


@pytest.mark.parametrize("seed", [1, 2])
def test_mixed_one_step_periodic_helical(seed):
    w = configs.config1(np_=3000, seed=seed)
    field = random_field(w.params, seed)
    got, gf, (nix, niy), _ = run_gpu_steps(mixed(w.params), w.beam, field, w.h, 1)
    b, of, _ = run_oracle_steps(w.params, w.beam, field, w.h, 1, nix, niy)
    assert_beam_close(got, b, rtol=1e-6, atol=1e-8)
    field_close(gf, of, 2e-5)


def test_mixed_one_step_planepole_temporal():
    from tests.test_gpu_parity import _beam3d, _planepole_params
    lamr = 4.0 * configs.PUFFIN_PI * 0.004
    p = _planepole_params(undgrad=-0.05, szfe=0.8)
    lz2 = (p.nz2 - 1) * p.dz2
    beam = _beam3d(p, 2500, 7, 0.2 * lz2, 0.8 * lz2)
    field = random_field(p, 3)
    h = lamr / 24.0
    got, gf, (nix, niy), _ = run_gpu_steps(mixed(p), beam, field, h, 2)
    b, of, _ = run_oracle_steps(p, beam, field, h, 2, nix, niy)
    assert_beam_close(got, b, rtol=1e-6, atol=1e-8)
    field_close(gf, of, 2e-5)


@pytest.mark.parametrize("mesh", [P.MESH_PERIODIC, P.MESH_TEMPORAL])
def test_mixed_diffraction(mesh):
    rho = 0.005
    lamr = 4.0 * configs.PUFFIN_PI * rho
    if mesh == P.MESH_PERIODIC:
        p = P.default_params(rho=rho, eta=1e-5, kappa=0.2, nx=21, ny=21, nz2=65, dx=0.2, dy=0.2,
                             dz2=lamr / 16, mesh_type=mesh, sperwaves=4.0, precision=P.MIXED)
    else:
        p = P.default_params(rho=rho, eta=1e-5, kappa=0.2, nx=33, ny=35, nz2=128, dx=0.3,
                             dy=0.25, dz2=lamr / 16, mesh_type=mesh, precision=P.MIXED)
    field = random_field(p, 9, amp=1.0)
    with P.Puffin(p) as sim:
        sim.set_field(*field)
        sim.diffractIM(0.37)
        gf = sim.get_field()
    cfg = oracle_config(p)
    re, im = (a.copy() for a in field)
    if mesh == P.MESH_PERIODIC:
        n = p.nx * p.ny
        re[-n:] = re[:n]
        im[-n:] = im[:n]
    O.diffract(cfg, re, im, 0.37)
    field_close(gf, (re, im), 2e-5)


def test_mixed_run_power_matches_fp64():
    w = configs.config1(np_=8192, seed=21, nsteps=32)
    field = random_field(w.params, 4, amp=1e-2)
    outs = {}
    for name, prm in (("fp64", w.params), ("mixed", mixed(w.params))):
        with P.Puffin(prm) as sim:
            sim.set_particles(*(w.beam[k] for k in P.PARTICLE_KEYS))
            sim.set_field(*field)
            sim.und_section(w.nsteps, w.isteps4diff, True, w.h)
            outs[name] = (sim.get_particles(), sim.get_field())
    pw = {k: float(np.sum(v[1][0] ** 2 + v[1][1] ** 2)) for k, v in outs.items()}
    assert abs(pw["mixed"] - pw["fp64"]) <= 1e-4 * pw["fp64"]
    np.testing.assert_allclose(outs["mixed"][0]["z2"], outs["fp64"][0]["z2"], rtol=1e-7, atol=1e-9)
    np.testing.assert_allclose(outs["mixed"][0]["gam"], outs["fp64"][0]["gam"], rtol=1e-7, atol=1e-9)


def test_mixed_gain_length_and_saturation_match_fp64():
    """The mixed form's physics targets on the config-1 mesh run to
    saturation from a shot-noise start (2^16 macroparticles, 5120 steps,
    zbar 0 to 10): power gain length of the exponential regime within 0.5 %
    and saturated energy within 1 % of the FP64 run."""
    from puffin_gb300 import fel
    w = configs.config1(np_=2 ** 16, nsteps=5120)
    curves = {}
    for name, prm in (("fp64", w.params), ("mixed", mixed(w.params))):
        curves[name] = fel.power_curve(prm, w.beam, w.field, w.h, w.nsteps)
    z = curves["fp64"][0]
    c = fel.compare(z, curves["fp64"][1], curves["mixed"][1])
    zs = c["saturated_energy"]["zbar_ref"]
    assert zs < z[-1] - 0.5, "the run must pass the first saturation"
    assert abs(c["gain_length"]["rel_diff"]) <= 5e-3, c
    assert abs(c["saturated_energy"]["rel_diff"]) <= 1e-2, c
