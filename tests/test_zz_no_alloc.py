"""The allocation-free RK4 step (pf_rk4_step_noalloc) against pf_rk4_step.

pf_rk4_step_noalloc exists for callers that cannot allocate device memory:
their device memory is owned by their own allocator, or they cannot take the
implicit synchronisation of cudaMalloc.  It runs the same kernels with its
temporaries in the library's fixed-size static device array, so on the same
inputs it must give the results of the handle-based pf_rk4_step.  Two calls
in a row check that contents left in the shared array by one call do not leak
into the next.  This file is collected last so that a stop at the first
failure has already run every other test.
"""
import numpy as np
import pytest

import puffin_gb300 as P
from puffin_gb300 import configs

pytestmark = pytest.mark.gpu


def test_noalloc_matches_handle_path_two_calls():
    torch = pytest.importorskip("torch")
    w = configs.config1(np_=5000, seed=17)
    rng = np.random.default_rng(4)
    n_out = w.params.nx * w.params.ny * w.params.nz2
    field = (1e-3 * rng.standard_normal(n_out), 1e-3 * rng.standard_normal(n_out))

    # reference: the handle-based entry point, two steps
    with P.Puffin(w.params) as sim:
        sim.set_particles(*(w.beam[k] for k in P.PARTICLE_KEYS))
        sim.set_field(*field)
        nix, niy = sim.window
        ref = []
        szl = 0.0
        for _ in range(2):
            assert sim.rk4par(szl, w.h)
            szl += w.h
            parts = sim.get_particles()
            fr, fi = sim.get_field()
            ref.append((parts, fr, fi))

    # allocation-free entry point on caller-owned device buffers
    p = w.params
    npl = p.nz2 - 1 if p.mesh_type == P.MESH_PERIODIC else p.nz2
    assert w.np <= P.lib.NOALLOC_MAX_PARTICLES and nix * niy * npl <= P.lib.NOALLOC_MAX_NODES
    ox, oy = (p.nx - nix) // 2, (p.ny - niy) // 2

    def window(a):
        return a.reshape(p.nz2, p.ny, p.nx)[:npl, oy:oy + niy, ox:ox + nix].reshape(-1)

    dev = {k: torch.tensor(w.beam[k], dtype=torch.float64, device="cuda") for k in P.PARTICLE_KEYS}
    wr = torch.tensor(np.ascontiguousarray(window(field[0])), dtype=torch.float64, device="cuda")
    wi = torch.tensor(np.ascontiguousarray(window(field[1])), dtype=torch.float64, device="cuda")
    taper = [p.n2col0, p.n2col0]
    szl = 0.0
    for step in range(2):
        torch.cuda.synchronize()
        assert P.rk4_step_noalloc(p, taper, szl, w.h, dev, wr, wi, nix, niy)
        szl += w.h
        torch.cuda.synchronize()
        parts, fr, fi = ref[step]
        for k in ("x", "y", "z2", "px", "py", "gam"):
            np.testing.assert_allclose(dev[k].cpu().numpy(), parts[k], rtol=1e-12, atol=1e-15,
                                       err_msg=f"step {step}: {k}")
        scale = max(np.abs(fr).max(), np.abs(fi).max())
        np.testing.assert_allclose(wr.cpu().numpy(), window(fr), rtol=0, atol=1e-12 * scale)
        np.testing.assert_allclose(wi.cpu().numpy(), window(fi), rtol=0, atol=1e-12 * scale)


def test_noalloc_rejects_sizes_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    w = configs.config1(np_=P.lib.NOALLOC_MAX_PARTICLES + 1, seed=2)
    p = w.params
    dev = {k: torch.tensor(w.beam[k], dtype=torch.float64, device="cuda") for k in P.PARTICLE_KEYS}
    npl = p.nz2 - 1
    wr = torch.zeros(21 * 21 * npl, dtype=torch.float64, device="cuda")
    wi = torch.zeros_like(wr)
    with pytest.raises(P.PuffinError) as e:
        P.rk4_step_noalloc(p, [1.0, 1.0], 0.0, w.h, dev, wr, wi, 21, 21)
    assert e.value.code == P.lib.PF_BAD_ARG


def _window_of(p, a, nix, niy):
    npl = p.nz2 - 1 if p.mesh_type == P.MESH_PERIODIC else p.nz2
    ox, oy = (p.nx - nix) // 2, (p.ny - niy) // 2
    return np.ascontiguousarray(a.reshape(p.nz2, p.ny, p.nx)[:npl, oy:oy + niy, ox:ox + nix]
                                .reshape(-1))


def test_noalloc_out_of_window_leaves_caller_arrays_unchanged():
    """A macroparticle beyond the last full cell of the window makes the step
    fail (the reference's qInnerXYOK_G = .false.): the call reports it and
    the caller's particle and window arrays keep their bits."""
    torch = pytest.importorskip("torch")
    w = configs.config1(np_=4000, seed=23)
    p = w.params
    nix = niy = 15
    beam = {k: np.array(v) for k, v in w.beam.items()}
    halfx = (nix - 1) / 2.0 * p.dx
    beam["x"][1234] = halfx + 0.25 * p.dx   # past the last full cell: x node + 1 == nix
    rng = np.random.default_rng(5)
    n_out = p.nx * p.ny * p.nz2
    field = (1e-3 * rng.standard_normal(n_out), 1e-3 * rng.standard_normal(n_out))
    dev = {k: torch.tensor(beam[k], dtype=torch.float64, device="cuda") for k in P.PARTICLE_KEYS}
    wr = torch.tensor(_window_of(p, field[0], nix, niy), dtype=torch.float64, device="cuda")
    wi = torch.tensor(_window_of(p, field[1], nix, niy), dtype=torch.float64, device="cuda")
    before = {k: v.clone() for k, v in dev.items()}
    wr0, wi0 = wr.clone(), wi.clone()
    taper = [p.n2col0, p.n2col0]
    for _ in range(2):   # twice: the failed call leaves nothing behind for the next
        torch.cuda.synchronize()
        assert not P.rk4_step_noalloc(p, taper, 0.0, w.h, dev, wr, wi, nix, niy)
        torch.cuda.synchronize()
        for k in P.PARTICLE_KEYS:
            assert torch.equal(dev[k], before[k]), k
        assert torch.equal(wr, wr0) and torch.equal(wi, wi0)


def test_noalloc_one_d_matches_handle_path():
    """The 1D mesh (nx = ny = 1, two-point interpolation along z2): two
    calls in a row against the handle's pf_rk4_step."""
    torch = pytest.importorskip("torch")
    from tests import golden_beam as GB
    g = np.load(GB.__file__.replace("golden_beam.py", "golden/f1main_expected.npz"))
    cfg, h = GB.config()
    ob = GB.initial_beam(cfg, g["electrons"][:, 6])
    beam = {k: getattr(ob, k).copy() for k in P.PARTICLE_KEYS}
    p = P.default_params(rho=cfg.rho, aw=cfg.aw, gamma_r=cfg.gamma_r, eta=cfg.eta,
                         kappa=cfg.kappa, fx=cfg.fx, fy=cfg.fy, und_type=P.UND_PUFFIN,
                         nx=1, ny=1, nz2=cfg.nz2, dx=1.0, dy=1.0, dz2=cfg.dz2, one_d=1,
                         szfs=0.0, szfe=cfg.szfe)
    rng = np.random.default_rng(8)
    field = (1e-2 * rng.standard_normal(cfg.nz2), 1e-2 * rng.standard_normal(cfg.nz2))
    ref = []
    with P.Puffin(p) as sim:
        sim.set_particles(*(beam[k] for k in P.PARTICLE_KEYS))
        sim.set_field(*field)
        assert sim.window == (1, 1)
        szl = 0.0
        for _ in range(2):
            assert sim.rk4par(szl, h)
            szl += h
            ref.append((sim.get_particles(), sim.get_field()))
    dev = {k: torch.tensor(beam[k], dtype=torch.float64, device="cuda") for k in P.PARTICLE_KEYS}
    wr = torch.tensor(field[0], dtype=torch.float64, device="cuda")
    wi = torch.tensor(field[1], dtype=torch.float64, device="cuda")
    taper = [p.n2col0, p.n2col0]
    szl = 0.0
    for step in range(2):
        torch.cuda.synchronize()
        assert P.rk4_step_noalloc(p, taper, szl, h, dev, wr, wi, 1, 1)
        szl += h
        torch.cuda.synchronize()
        parts, (fr, fi) = ref[step]
        for k in ("x", "y", "z2", "px", "py", "gam"):
            np.testing.assert_allclose(dev[k].cpu().numpy(), parts[k], rtol=1e-12, atol=1e-15,
                                       err_msg=f"step {step}: {k}")
        scale = max(np.abs(fr).max(), np.abs(fi).max())
        np.testing.assert_allclose(wr.cpu().numpy(), fr, rtol=0, atol=1e-12 * scale)
        np.testing.assert_allclose(wi.cpu().numpy(), fi, rtol=0, atol=1e-12 * scale)
