"""GPU parity: the puffgpu C ABI against the CPU oracle on the same seeded
inputs, and against the reference's own golden dump for the 1D path.

Tolerances (floating point; the GPU uses FMA contraction and an exact
fixed-point deposit sum, the oracle sequential FP64 sums):
* one RK4 step: rtol 1e-12 on particles, 1e-12 of the field scale;
* 32 steps with diffraction: rtol 1e-9 (the FEL instability amplifies
  rounding differences step by step);
* the reference's own 1D end-to-end test: 1e-10 absolute, as in
  test/testMPIIntegration.pf:94-128.
"""
import math
import os

import numpy as np
import pytest

import puffin_gb300 as P
from puffin_gb300 import configs
from oracle import oracle as O
from tests import golden_beam as GB
from tests.oracle_bridge import assert_beam_close, oracle_beam, oracle_config

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden", "f1main_expected.npz")


@pytest.fixture(scope="module", autouse=True)
def _threads():
    O.set_threads(1)


def run_gpu_steps(params, beam, field, h, nsteps, szl=0.0, taper=None):
    with P.Puffin(params) as sim:
        sim.set_particles(*(beam[k] for k in P.PARTICLE_KEYS))
        sim.set_field(*field)
        if taper is not None:
            sim.set_taper(*taper)
        for _ in range(nsteps):
            assert sim.rk4par(szl, h)
            szl += h
        return sim.get_particles(), sim.get_field(), sim.window, sim.get_taper()


def run_oracle_steps(params, beam, field, h, nsteps, nix, niy, szl=0.0, taper=None):
    cfg = oracle_config(params)
    b = oracle_beam(beam)
    re, im = (np.array(a, dtype=np.float64) for a in field)
    if cfg.mesh_type == O.MESH_PERIODIC:
        n = cfg.nx * cfg.ny
        re[-n:] = re[:n]
        im[-n:] = im[:n]
    wr, wi = O.outer_to_inner(cfg, re, im, nix, niy)
    t = O.Taper(*(taper or (params.n2col0, params.n2col0, params.undgrad)))
    for _ in range(nsteps):
        assert O.rk4_step(cfg, t, szl, h, b, wr, wi, nix, niy) == 0
        szl += h
    O.inner_to_outer(cfg, re, im, wr, wi, nix, niy)
    return b, (re, im), t


def random_field(params, seed, amp=1e-3):
    rng = np.random.default_rng(seed)
    n = params.nx * params.ny * params.nz2
    return amp * rng.standard_normal(n), amp * rng.standard_normal(n)


def field_close(got, want, rel):
    scale = max(np.max(np.abs(want[0])), np.max(np.abs(want[1])), 1e-300)
    np.testing.assert_allclose(got[0], want[0], rtol=0, atol=rel * scale)
    np.testing.assert_allclose(got[1], want[1], rtol=0, atol=rel * scale)


# ---------------------------------------------------------------------------
def test_golden_1d_reference_run():
    """The reference's 2-rank end-to-end test, run through the GPU library."""
    g = np.load(GOLD)
    cfg, h = GB.config()
    ob = GB.initial_beam(cfg, g["electrons"][:, 6])
    beam = {k: getattr(ob, k).copy() for k in P.PARTICLE_KEYS}
    p = P.default_params(rho=cfg.rho, aw=cfg.aw, gamma_r=cfg.gamma_r, eta=cfg.eta,
                         kappa=cfg.kappa, fx=cfg.fx, fy=cfg.fy, und_type=P.UND_PUFFIN,
                         nx=1, ny=1, nz2=cfg.nz2, dx=1.0, dy=1.0, dz2=cfg.dz2, one_d=1,
                         szfs=0.0, szfe=cfg.szfe)
    got, (fr, fi), win, taper = run_gpu_steps(p, beam, (np.zeros(cfg.nz2), np.zeros(cfg.nz2)),
                                              h, GB.NSTEPS)
    assert win == (1, 1)
    szl = 0.0
    for _ in range(GB.NSTEPS):
        szl = szl + h
    b = O.Beam(*(got[k] for k in P.PARTICLE_KEYS))
    O.match_out(cfg, b, szl, taper[0])
    O.correct_trans(b)
    e = g["electrons"]
    assert b.n == 319
    for j, k in enumerate(("x", "y", "z2", "px", "py", "gam")):
        np.testing.assert_allclose(getattr(b, k), e[:, j], rtol=0, atol=1e-10, err_msg=k)
    np.testing.assert_allclose(fr, g["aperp"][0], rtol=0, atol=1e-10)
    np.testing.assert_allclose(fi, g["aperp"][1], rtol=0, atol=1e-10)


@pytest.mark.parametrize("seed", [1, 2])
def test_one_step_periodic_helical(seed):
    w = configs.config1(np_=3000, seed=seed)
    field = random_field(w.params, seed)
    got, gf, (nix, niy), _ = run_gpu_steps(w.params, w.beam, field, w.h, 1)
    b, of, _ = run_oracle_steps(w.params, w.beam, field, w.h, 1, nix, niy)
    assert_beam_close(got, b, rtol=1e-12, atol=1e-15)
    field_close(gf, of, 1e-12)


def _planepole_params(**kw):
    rho, aw, gr = 0.004, 1.2, 800.0
    eta, kappa, fx, fy = configs.calc_scaling(rho, aw, gr, P.UND_PLANEPOLE)
    lamr = 4.0 * configs.PUFFIN_PI * rho
    p = P.default_params(rho=rho, aw=aw, gamma_r=gr, eta=eta, kappa=kappa, fx=fx, fy=fy,
                         und_type=P.UND_PLANEPOLE, nx=33, ny=33, nz2=96, dx=0.3, dy=0.3,
                         dz2=lamr / 16.0, mesh_type=P.MESH_TEMPORAL)
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def _beam3d(p, n, seed, zlo, zhi, sig=1.0):
    rng = np.random.default_rng(seed)
    beam = {"x": sig * np.clip(rng.standard_normal(n), -3, 3),
            "y": sig * np.clip(rng.standard_normal(n), -3, 3),
            "z2": rng.uniform(zlo, zhi, n),
            "px": 0.02 * rng.standard_normal(n), "py": 0.02 * rng.standard_normal(n),
            "gam": 1.0 + 1e-3 * rng.standard_normal(n),
            "chi": rng.uniform(0.5, 1.5, n) * 1e-3}
    configs.match_in(p, beam)
    return beam


def test_cell_edges_and_periodic_images():
    """The cell index and fraction come from the bits of the scaled
    coordinate: macroparticles exactly on cell boundaries (transverse and
    z2), at negative z2 and beyond the first period of the periodic mesh
    (their images), against the oracle's floor arithmetic at 1e-12.

    Which behaviour this pins: on cell boundaries at non-negative
    coordinates it is the reference's own -- there its node index from
    truncating int() (rhs.f90:174-178) and its weights from floor
    (system_interpolation.f90:45-58) agree.  Negative z2 and z2 beyond the
    first period are inputs the reference does not define (int() and floor
    part ways and its node index leaves the mesh); here the periodic mesh
    reads them as their images, plane modulo nz2 - 1, which is where the
    reference's own wrap (para_field.f90:212-215) puts them.  On the
    temporal mesh z2 < 0 returns PF_OUT_OF_Z2 (a deliberate deviation: the
    reference neither checks nor defines it)."""
    w = configs.config1(np_=4096, seed=5, nsteps=2)
    p = w.params
    beam = {k: v.copy() for k, v in w.beam.items()}
    n = len(beam["x"])
    lz2 = (p.nz2 - 1) * p.dz2
    rng = np.random.default_rng(9)
    k = np.arange(n)
    # a quarter on z2 cell boundaries, a quarter shifted by -1 or +2 periods
    on = k % 4 == 0
    beam["z2"][on] = np.round(beam["z2"][on] / p.dz2) * p.dz2
    img = k % 4 == 1
    beam["z2"][img] += np.where(rng.random(img.sum()) < 0.5, -lz2, 2.0 * lz2)
    # transverse boundaries: x on a node of the window (cells of dx = 0.2)
    xb = k % 4 == 2
    beam["x"][xb] = np.round(beam["x"][xb] / p.dx) * p.dx
    beam["y"][xb] = np.round(beam["y"][xb] / p.dy) * p.dy
    field = random_field(p, 4, amp=1e-2)
    got, gf, (nix, niy), _ = run_gpu_steps(p, beam, field, w.h, 2)
    b, of, _ = run_oracle_steps(p, beam, field, w.h, 2, nix, niy)
    assert_beam_close(got, b, rtol=1e-12, atol=1e-15)
    field_close(gf, of, 1e-12)


@pytest.mark.parametrize("place_sz", [0.0, 0.05, 0.9])
def test_one_step_planepole_taper_ends_focusing(place_sz):
    """Temporal mesh, planepole with undulator ends (start/main/end sections),
    a linear taper and strong focusing."""
    lamr = 4.0 * configs.PUFFIN_PI * 0.004
    p = _planepole_params(und_ends=1, szfs=2 * lamr, szfe=0.8, undgrad=-0.05, focusing=1,
                          kbxsf=0.3, kbysf=0.4)
    lz2 = (p.nz2 - 1) * p.dz2
    beam = _beam3d(p, 2500, 7, 0.2 * lz2, 0.8 * lz2)
    field = random_field(p, 3)
    h = lamr / 24.0
    taper = (1.0, 1.0, p.undgrad)
    got, gf, (nix, niy), gt = run_gpu_steps(p, beam, field, h, 2, szl=place_sz, taper=taper)
    b, of, ot = run_oracle_steps(p, beam, field, h, 2, nix, niy, szl=place_sz, taper=taper)
    assert_beam_close(got, b, rtol=1e-12, atol=1e-15)
    field_close(gf, of, 1e-12)
    assert gt[0] == ot.n2col and gt[1] == ot.n2col0


def test_taper_profile_steps():
    """A 16-point piecewise-linear taper profile alpha(z) across the steps."""
    lamr = 4.0 * configs.PUFFIN_PI * 0.004
    p = _planepole_params()
    lz2 = (p.nz2 - 1) * p.dz2
    beam = _beam3d(p, 2500, 17, 0.2 * lz2, 0.8 * lz2)
    field = random_field(p, 8)
    h = lamr / 24.0
    rng = np.random.default_rng(4)
    pz = np.linspace(0.0, 6 * h, 16)
    pa = 1.0 + 0.05 * rng.standard_normal(16)
    with P.Puffin(p) as sim:
        sim.set_particles(*(beam[k] for k in P.PARTICLE_KEYS))
        sim.set_field(*field)
        sim.set_taper_profile(pz, pa)
        szl = 0.0
        for _ in range(5):
            assert sim.rk4par(szl, h)
            szl += h
        got, gf, (nix, niy) = sim.get_particles(), sim.get_field(), sim.window
    cfg = oracle_config(p)
    b = oracle_beam(beam)
    re, im = (a.copy() for a in field)
    wr, wi = O.outer_to_inner(cfg, re, im, nix, niy)
    t = O.Taper(pa[0], pa[0], 0.0, pz, pa)
    szl = 0.0
    for _ in range(5):
        assert O.rk4_step(cfg, t, szl, h, b, wr, wi, nix, niy) == 0
        szl += h
    O.inner_to_outer(cfg, re, im, wr, wi, nix, niy)
    assert_beam_close(got, b, rtol=1e-12, atol=1e-15)
    field_close(gf, (re, im), 1e-12)


@pytest.mark.parametrize("und", [P.UND_HELICAL, P.UND_PUFFIN, P.UND_CURVED])
@pytest.mark.parametrize("place_sz", [0.0, 0.03, 0.5])
def test_one_step_undulator_types(und, place_sz):
    rho, aw, gr = 0.005, 1.0, 400.0
    eta, kappa, fx, fy = configs.calc_scaling(rho, aw, gr, und, 0.8, 0.6)
    lamr = 4.0 * configs.PUFFIN_PI * rho
    kw = {}
    if und == P.UND_CURVED:
        kx = math.sqrt(eta / (8.0 * rho ** 2))
        kw = dict(kx_und=kx, ky_und=kx)
    p = P.default_params(rho=rho, aw=aw, gamma_r=gr, eta=eta, kappa=kappa, fx=fx, fy=fy,
                         und_type=und, nx=25, ny=25, nz2=65, dx=0.25, dy=0.25, dz2=lamr / 16,
                         mesh_type=P.MESH_PERIODIC, sperwaves=4.0, und_ends=1,
                         szfs=2 * lamr, szfe=0.4, **kw)
    beam = _beam3d(p, 2000, 11, 0.0, 4 * lamr, sig=0.7)
    field = random_field(p, 5)
    h = lamr / 30.0
    got, gf, (nix, niy), _ = run_gpu_steps(p, beam, field, h, 2, szl=place_sz)
    b, of, _ = run_oracle_steps(p, beam, field, h, 2, nix, niy, szl=place_sz)
    assert_beam_close(got, b, rtol=1e-12, atol=1e-15)
    field_close(gf, of, 1e-12)


@pytest.mark.parametrize("mesh", [P.MESH_PERIODIC, P.MESH_TEMPORAL])
def test_diffraction_matches_oracle(mesh):
    rho = 0.005
    lamr = 4.0 * configs.PUFFIN_PI * rho
    if mesh == P.MESH_PERIODIC:
        p = P.default_params(rho=rho, eta=1e-5, kappa=0.2, nx=21, ny=21, nz2=65, dx=0.2, dy=0.2,
                             dz2=lamr / 16, mesh_type=mesh, sperwaves=4.0)
    else:
        p = P.default_params(rho=rho, eta=1e-5, kappa=0.2, nx=33, ny=35, nz2=128, dx=0.3,
                             dy=0.25, dz2=lamr / 16, mesh_type=mesh)
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
    field_close(gf, (re, im), 1e-12)


@pytest.mark.parametrize("precision", [P.FP64, P.MIXED])
@pytest.mark.parametrize("shape", [(17, 21, 4096), (129, 129, 8), (129, 17, 1536), (17, 33, 600),
                                   (33, 33, 64), (65, 65, 32), (17, 17, 2048)])
def test_diffraction_kernel_shapes(shape, precision):
    """Meshes that select each diffraction kernel form: the transverse-plane
    pass (plane in shared memory), the nine line passes with the radix-43
    butterfly, and the long z2 lines with several adjacent lines per block.
    FP64 to 1e-12 of the field scale, the mixed (FP32) transform to 2e-5."""
    nx, ny, nz2 = shape
    rho = 0.005
    lamr = 4.0 * configs.PUFFIN_PI * rho
    p = P.default_params(rho=rho, eta=1e-5, kappa=0.2, nx=nx, ny=ny, nz2=nz2, dx=0.3, dy=0.25,
                         dz2=lamr / 16, mesh_type=P.MESH_TEMPORAL, precision=precision)
    field = random_field(p, 11, amp=1.0)
    with P.Puffin(p) as sim:
        sim.set_field(*field)
        sim.diffractIM(0.29)
        gf = sim.get_field()
    re, im = (a.copy() for a in field)
    O.diffract(oracle_config(p), re, im, 0.29)
    field_close(gf, (re, im), 1e-12 if precision == P.FP64 else 2e-5)


def test_run_with_diffraction_matches_oracle():
    """pf_run (UndSection's loop) against oracle.undulator_run: 32 steps with
    diffraction every 16 steps and merged half steps."""
    w = configs.config1(np_=4096, seed=21, nsteps=32)
    field = random_field(w.params, 4, amp=1e-2)
    with P.Puffin(w.params) as sim:
        sim.set_particles(*(w.beam[k] for k in P.PARTICLE_KEYS))
        sim.set_field(*field)
        szl = sim.und_section(w.nsteps, w.isteps4diff, True, w.h)
        got = sim.get_particles()
        gf = sim.get_field()
    cfg = oracle_config(w.params)
    b = oracle_beam(w.beam)
    re, im = (a.copy() for a in field)
    n = cfg.nx * cfg.ny
    re[-n:] = re[:n]
    im[-n:] = im[:n]
    r = O.undulator_run(cfg, b, re, im, w.h, w.nsteps, w.isteps4diff, True)
    assert r.status == 0
    assert abs(szl - w.nsteps * w.h) < 1e-12
    assert_beam_close(got, b, rtol=1e-9, atol=1e-12)
    field_close(gf, (re, im), 1e-9)


@pytest.mark.parametrize("precision", [P.FP64, P.MIXED])
def test_run_graph_blocks_match_step_by_step(precision):
    """pf_run replays its 8-step blocks as captured CUDA graphs with the stage
    coefficients from a device table; the result matches the same schedule
    driven one call at a time (rk4par, diffractIM, wrap): bit for bit in
    FP64."""
    w = configs.config1(np_=8192, seed=41, nsteps=64)
    w.params.precision = precision
    field = random_field(w.params, 3, amp=1e-2)
    h = w.h
    with P.Puffin(w.params) as sim:
        sim.set_particles(*(w.beam[k] for k in P.PARTICLE_KEYS))
        sim.set_field(*field)
        sim.und_section(64, 8, True, h)
        got, gf = sim.get_particles(), sim.get_field()
    with P.Puffin(w.params) as sim:
        sim.set_particles(*(w.beam[k] for k in P.PARTICLE_KEYS))
        sim.set_field(*field)
        sim.diffractIM(8 * h / 2)
        szl = 0.0
        for i in range(1, 65):
            assert sim.rk4par(szl, h)
            szl = szl + h
            if i % 8 == 0:
                sim.diffractIM(8 * h / 2 + (8 * h / 2 if i < 64 else 0.0))
            if i % 60 == 0:
                sim.wrap_z2()
        want, wf = sim.get_particles(), sim.get_field()
    if precision == P.FP64:  # the fixed-point deposit makes FP64 runs reproducible bit for bit
        for k in ("x", "y", "z2", "px", "py", "gam"):
            np.testing.assert_array_equal(got[k], want[k], err_msg=k)
        np.testing.assert_array_equal(gf[0], wf[0])
        np.testing.assert_array_equal(gf[1], wf[1])
    else:  # FP32 atomics land in any order: FP32 rounding, grown over 64 steps,
        # to 1e-5 of each coordinate's scale (momenta ~1e-2: atol 1e-7)
        assert_beam_close(got, oracle_beam(want), rtol=1e-5, atol=1e-7)
        field_close(gf, wf, 1e-4)


def test_deposit_is_bit_reproducible():
    w = configs.config1(np_=20000, seed=3, nsteps=4)
    field = random_field(w.params, 2)
    outs = []
    for _ in range(2):
        got, gf, _, _ = run_gpu_steps(w.params, w.beam, field, w.h, 4)
        outs.append((got, gf))
    for k in ("x", "y", "z2", "px", "py", "gam"):
        np.testing.assert_array_equal(outs[0][0][k], outs[1][0][k])
    np.testing.assert_array_equal(outs[0][1][0], outs[1][1][0])
    np.testing.assert_array_equal(outs[0][1][1], outs[1][1][1])


@pytest.mark.parametrize("npart", [2 ** 18, 3_500_000])
def test_dense_beam_tiled_deposit(npart):
    """Dense beams on the config-1 mesh select the shared-memory deposit
    tile: 2^18 macroparticles (about ten per window cell) in blocks sized to
    fill a wave of resident blocks (342 blocks of 768 macroparticles, the
    last one holding 256), 3.5 M in the full blocks of 8192 (428 blocks,
    94 % of a wave; the last one holding 2016).  One RK4 step against the
    oracle (rtol 1e-12) and bit-identical repeats."""
    w = configs.config1(np_=npart, seed=9, nsteps=2)
    field = random_field(w.params, 5)
    outs = []
    for _ in range(2):
        got, gf, (nix, niy), _ = run_gpu_steps(w.params, w.beam, field, w.h, 1)
        outs.append((got, gf))
    assert w.np >= 8 * (w.params.nz2 - 1) * nix * niy      # the dense mode is selected
    for k in ("x", "y", "z2", "px", "py", "gam"):
        np.testing.assert_array_equal(outs[0][0][k], outs[1][0][k])
    np.testing.assert_array_equal(outs[0][1][0], outs[1][1][0])
    b, of, _ = run_oracle_steps(w.params, w.beam, field, w.h, 1, nix, niy)
    if npart < 10 ** 6:
        assert_beam_close(outs[0][0], b, rtol=1e-12, atol=1e-15)
    else:
        # p2 = (1/sqrt(1 - u) - 1)/eta cancels seven digits (u ~ 4e-6 here),
        # so an ulp of difference upstream flips its rounding for a few
        # macroparticles in millions: 2^-52/u ~ 6e-11 of p2, h = 0.002 times
        # that in z2, 1.1e-13 absolute (z2 near zero makes it large relative)
        assert_beam_close(outs[0][0], b, rtol=1e-12, atol=1e-15,
                          keys=("x", "y", "px", "py", "gam"))
        np.testing.assert_allclose(outs[0][0]["z2"], b.z2, rtol=1e-12, atol=2e-13)
    field_close(outs[0][1], of, 1e-12)


def test_out_of_window_leaves_state_and_recovers():
    w = configs.config1(np_=1000, seed=5)
    beam = {k: v.copy() for k, v in w.beam.items()}
    field = random_field(w.params, 6)
    with P.Puffin(w.params, nix=11, niy=11) as sim:
        sim.set_particles(*(beam[k] for k in P.PARTICLE_KEYS))
        sim.set_field(*field)
        assert sim.window == (11, 11)
        before = sim.get_particles()
        f0 = sim.get_field()
        assert sim.rk4par(0.0, w.h) is False          # qPArrOK_G = .false.
        after = sim.get_particles()
        for k in P.PARTICLE_KEYS:
            np.testing.assert_array_equal(before[k], after[k])
        f1 = sim.get_field()
        np.testing.assert_array_equal(f0[0], f1[0])
        sim.redistribute()                             # getInNode + wrap
        assert sim.window == (21, 21)
        assert sim.rk4par(0.0, w.h) is True


def test_run_recovers_when_particles_leave_the_window_mid_block():
    """A beam whose outer particles drift across the inner window edge during
    pf_run: the asynchronous step block that fails is restored and replayed
    step by step with the reference's window recomputation (two retries in
    32 steps), and the result matches the oracle's UndSection restatement."""
    w = configs.config1(np_=2000, seed=7, nsteps=32)
    w.params.nx = w.params.ny = 39
    beam = {k: a.copy() for k, a in w.beam.items()}
    beam["px"] = beam["px"] + 20.0 * (beam["x"] > 0.8)
    field = random_field(w.params, 1)
    n = w.params.nx * w.params.ny
    for f in field:
        f[-n:] = f[:n]
    with P.Puffin(w.params) as sim:
        sim.set_particles(*(beam[k] for k in P.PARTICLE_KEYS))
        sim.set_field(*field)
        assert sim.window == (21, 21)
        sim.und_section(32, 16, True, w.h)
        got, gf, win = sim.get_particles(), sim.get_field(), sim.window
    cfg = oracle_config(w.params)
    b = oracle_beam(beam)
    re, im = (a.copy() for a in field)
    r = O.undulator_run(cfg, b, re, im, w.h, 32, 16, True)
    assert r.status == 0 and r.retries == 2
    assert win == r.window
    assert_beam_close(got, b, rtol=1e-9, atol=1e-12)
    field_close(gf, (re, im), 1e-9)


def test_out_of_temporal_mesh_raises():
    p = _planepole_params()
    lz2 = (p.nz2 - 1) * p.dz2
    beam = _beam3d(p, 100, 1, 0.1 * lz2, 0.5 * lz2)
    beam["z2"][7] = (p.nz2 - 1) * p.dz2 + 0.5 * p.dz2   # beyond the last node
    with P.Puffin(p) as sim:
        sim.set_particles(*(beam[k] for k in P.PARTICLE_KEYS))
        with pytest.raises(P.PuffinError) as e:
            sim.rk4par(0.0, 1e-3)
        assert e.value.code == P.lib.PF_OUT_OF_Z2


def test_empty_beam_is_a_no_op_on_the_field():
    p = _planepole_params(nix=9, niy=9)
    field = random_field(p, 8)
    with P.Puffin(p) as sim:
        e = np.zeros(0)
        sim.set_particles(e, e, e, e, e, e, e)
        sim.set_field(*field)
        assert sim.rk4par(0.0, 1e-3)
        gf = sim.get_field()
    np.testing.assert_array_equal(gf[0], field[0])
    np.testing.assert_array_equal(gf[1], field[1])


def test_device_arrays_round_trip():
    torch = pytest.importorskip("torch")
    w = configs.config1(np_=777, seed=9)
    t = {k: torch.tensor(w.beam[k], dtype=torch.float64, device="cuda") for k in P.PARTICLE_KEYS}
    with P.Puffin(w.params) as sim:
        sim.set_particles(*(t[k] for k in P.PARTICLE_KEYS))
        out = {k: torch.empty_like(t[k]) for k in P.PARTICLE_KEYS}
        sim.get_particles(out)
    torch.cuda.synchronize()
    for k in P.PARTICLE_KEYS:
        assert torch.equal(out[k], t[k])


@pytest.mark.parametrize("noise", [False, True])
def test_generate_beam_matches_oracle(noise):
    """The device beam generator against the oracle's restatement: the quiet
    beam bit for bit, the shot noise to the transcendental functions' last
    bits (normal branch) and exactly where the counts agree."""
    ns, nseq = 64, 200
    z2m = (np.arange(ns) + 0.5) * 0.05
    ne = np.where(np.arange(ns) % 2 == 0, 8.0e4, 900.0)   # 400 and 4.5 per beamlet
    mean = np.stack([np.zeros(ns), np.full(ns, 0.2), np.zeros(ns), np.zeros(ns),
                     1.0 + 1e-3 * np.arange(ns)], axis=1)
    sig = np.array([0.8, 0.6, 0.01, 0.02, 5e-4])
    p = P.default_params(rho=0.005, eta=1e-5, kappa=0.2, nx=31, ny=31, nz2=80, dx=0.3, dy=0.3,
                         dz2=0.05)
    with P.Puffin(p) as sim:
        sim.generate_beam(z2m, ne, 0.05, nseq, mean, sig, noise=noise, seed=99, chi_per_electron=3.0)
        got = sim.get_particles()
    want = O.generate_beam(z2m, ne, 0.05, nseq, mean, sig, noise, 99, 3.0)
    for k in ("x", "y", "px", "py", "gam"):
        np.testing.assert_array_equal(got[k], getattr(want, k), err_msg=k)
    if not noise:
        np.testing.assert_array_equal(got["z2"], want.z2)
        np.testing.assert_array_equal(got["chi"], want.chi)
    else:
        same = got["chi"] == want.chi
        assert np.mean(same) > 0.999
        np.testing.assert_allclose(got["z2"][same], want.z2[same], rtol=0, atol=1e-15)


@pytest.mark.parametrize("precision", [P.FP64, P.MIXED])
def test_run_with_z2_ordering_matches_step_by_step(precision):
    """pf_run re-orders beams of 2^15 macroparticles or more by z2 plane at
    the wrap cadence (the caller's order is restored by pf_get_particles);
    130 steps (two orderings) against the same schedule driven one call at a
    time, which never re-orders: bit for bit in FP64."""
    w = configs.config1(np_=2 ** 15, seed=43, nsteps=130)
    w.params.precision = precision
    field = random_field(w.params, 5, amp=1e-2)
    h = w.h
    with P.Puffin(w.params) as sim:
        sim.set_particles(*(w.beam[k] for k in P.PARTICLE_KEYS))
        sim.set_field(*field)
        sim.und_section(130, 10, True, h)
        got, gf = sim.get_particles(), sim.get_field()
        # a second read and a chi-keeping hand-over see the caller's order too
        again = sim.get_particles()
        sim.set_particles(*(got[k] for k in P.PARTICLE_KEYS[:6]))
        kept = sim.get_particles()
    for k in P.PARTICLE_KEYS:
        np.testing.assert_array_equal(again[k], got[k], err_msg=k)
        np.testing.assert_array_equal(kept[k], got[k], err_msg=k)
    np.testing.assert_array_equal(got["chi"], w.beam["chi"])
    with P.Puffin(w.params) as sim:
        sim.set_particles(*(w.beam[k] for k in P.PARTICLE_KEYS))
        sim.set_field(*field)
        sim.diffractIM(10 * h / 2)
        szl = 0.0
        for i in range(1, 131):
            assert sim.rk4par(szl, h)
            szl = szl + h
            if i % 10 == 0:
                sim.diffractIM(10 * h / 2 + (10 * h / 2 if i < 130 else 0.0))
            if i % 60 == 0:
                sim.wrap_z2()
        want, wf = sim.get_particles(), sim.get_field()
    if precision == P.FP64:
        for k in ("x", "y", "z2", "px", "py", "gam"):
            np.testing.assert_array_equal(got[k], want[k], err_msg=k)
        np.testing.assert_array_equal(gf[0], wf[0])
        np.testing.assert_array_equal(gf[1], wf[1])
    else:
        assert_beam_close(got, oracle_beam(want), rtol=1e-5, atol=1e-7)
        field_close(gf, wf, 1e-4)


def test_z2_ordering_is_the_same_every_run():
    """The z2 ordering inside pf_run is a stable counting sort (the slots of
    a plane keep their order), so the device order after a run depends on
    the input only: reductions over the macroparticles in device order, such
    as correctTrans's chi-weighted means (acc_lattice.f90:601-623), give the
    same bits in two identical runs."""
    w = configs.config1(np_=3 * 2 ** 15, seed=44, nsteps=130)
    field = random_field(w.params, 6, amp=1e-2)
    outs = []
    for _ in range(2):
        with P.Puffin(w.params) as sim:
            sim.set_particles(*(w.beam[k] for k in P.PARTICLE_KEYS))
            sim.set_field(*field)
            sim.und_section(130, 10, True, w.h)
            sim.correctTrans()
            outs.append(sim.get_particles())
    for k in P.PARTICLE_KEYS:
        np.testing.assert_array_equal(outs[0][k], outs[1][k], err_msg=k)


@pytest.mark.parametrize("mesh", ["periodic", (17, 21, 4096), (129, 129, 8), (129, 17, 1536),
                                  (17, 33, 600), (33, 33, 64), (65, 65, 32), (17, 17, 2048)])
def test_paired_fp32_diffraction_matches_oracle(mesh):
    """The FP64 path's diffraction with its FFTs in paired-FP32 arithmetic
    (pf_set_fft_arithmetic): every kernel form against the oracle's FP64
    diffraction step to 2e-12 of the field scale, and two calls in a row
    give the same bits."""
    rho = 0.005
    lamr = 4.0 * configs.PUFFIN_PI * rho
    if mesh == "periodic":
        p = P.default_params(rho=rho, eta=1e-5, kappa=0.2, nx=21, ny=21, nz2=65, dx=0.2, dy=0.2,
                             dz2=lamr / 16, mesh_type=P.MESH_PERIODIC, sperwaves=4.0)
    else:
        nx, ny, nz2 = mesh
        p = P.default_params(rho=rho, eta=1e-5, kappa=0.2, nx=nx, ny=ny, nz2=nz2, dx=0.3,
                             dy=0.25, dz2=lamr / 16, mesh_type=P.MESH_TEMPORAL)
    field = random_field(p, 13, amp=1.0)
    if mesh == "periodic":
        n = p.nx * p.ny
        field[0][-n:] = field[0][:n]
        field[1][-n:] = field[1][:n]
    outs = []
    for _ in range(2):
        with P.Puffin(p) as sim:
            sim.set_fft_arithmetic(P.lib.FFT_PAIRED_FP32)
            sim.set_field(*field)
            sim.diffractIM(0.31)
            outs.append(sim.get_field())
    re, im = (a.copy() for a in field)
    O.diffract(oracle_config(p), re, im, 0.31)
    field_close(outs[0], (re, im), 2e-12)
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])
