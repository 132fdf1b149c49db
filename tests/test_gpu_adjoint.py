"""Adjoint of the RK4/diffraction run against central finite differences of
the FP64 forward run, and the forward of the adjoint driver against pf_run
on the same inputs, for FP64 and mixed-precision handles.

Workload: the config-1 mesh (periodic, helical, 21 x 21 x 64 unique planes),
4096 macroparticles, 32 steps with diffraction every 8 and checkpoints every
8, a 16-point taper profile, a Gaussian seed (waist 1.0) at amplitude 1e-2
and an energy chirp.  Tolerance (the adjoint form's target): the adjoint
gradient within 1e-4 relative of central differences with steps of 1e-6, for
every component larger than 1e-3 of the largest.  The mixed-precision
adjoint is checked against the FP64 forward's differences: a step of 1e-6
of a taper value is below the FP32 resolution of the mixed forward's
coefficients (2^-24 relative), so its own energy cannot be differenced at
that step.
"""
import numpy as np
import pytest
import torch

import puffin_gb300 as P
from puffin_gb300 import configs
from puffin_gb300.adjoint import pulse_energy

pytestmark = pytest.mark.gpu
NSTEPS, EVERY, K = 32, 8, 8


def _setup():
    w = configs.config1(np_=4096, seed=31, nsteps=NSTEPS)
    p = w.params
    nx, ny, nz2 = p.nx, p.ny, p.nz2
    xs = (np.arange(nx) - (nx - 1) / 2) * p.dx
    ys = (np.arange(ny) - (ny - 1) / 2) * p.dy
    g = np.exp(-(xs[None, :] ** 2 + ys[:, None] ** 2) / 2.0).ravel()
    # carrier at the resonant wavelength (4 pi rho in z2), which the high-pass
    # filter of the diffraction step passes
    ph = np.arange(nz2) * p.dz2 / (2.0 * p.rho)
    seed_re = (np.cos(ph)[:, None] * g[None, :]).ravel()
    seed_im = (np.sin(ph)[:, None] * g[None, :]).ravel()
    taper_z = np.linspace(0.0, NSTEPS * w.h, 16)
    alpha = 1.0 + 0.02 * np.sin(np.arange(16) * 0.7)
    return w, (seed_re, seed_im), taper_z, alpha


def _mixed(params):
    q = P.Params.from_buffer_copy(params)
    q.precision = P.MIXED
    return q


def _run_energy(params, w, seed, taper_z, alpha, amp, chirp):
    """Pulse energy of the same run through pf_run (und_section)."""
    beam = {k: v.copy() for k, v in w.beam.items()}
    beam["gam"] = beam["gam"] + chirp * (beam["z2"] - np.sum(beam["z2"]) / len(beam["z2"]))
    with P.Puffin(params) as sim:
        sim.set_particles(*(beam[k] for k in P.PARTICLE_KEYS))
        sim.set_field(amp * seed[0], amp * seed[1])
        sim.set_taper_profile(taper_z, alpha)
        sim.und_section(NSTEPS, EVERY, True, w.h)
        fr, fi = sim.get_field()
    p = w.params
    n = p.nx * p.ny * (p.nz2 - 1)  # unique planes of the periodic mesh
    return p.dx * p.dy * p.dz2 * float(np.sum(fr[:n] ** 2 + fi[:n] ** 2))


def _fd_checks(sim, w, seed, taper_z, alpha, amp, chirp):
    """(name, central difference) of the energy on the handle sim."""
    def fd(f, x, d):
        return (f(x + d) - f(x - d)) / (2.0 * d)

    out = [
        ("seed_amp", fd(lambda a: _energy(sim, w, seed, taper_z, alpha, a, chirp),
                        amp, 1e-6 * amp)),
        ("chirp", fd(lambda c: _energy(sim, w, seed, taper_z, alpha, amp, c), chirp, 1e-6)),
    ]
    for k in (1, 6, 11, 15):
        def e_k(v, k=k):
            a = alpha.copy()
            a[k] = v
            return _energy(sim, w, seed, taper_z, a, amp, chirp)
        out.append((f"taper[{k}]", fd(e_k, alpha[k], 1e-6)))
    return out


def _energy(sim, w, seed, taper_z, alpha, amp, chirp):
    sim.set_taper_profile(taper_z, alpha)
    return sim.adjoint_forward(NSTEPS, EVERY, True, w.h, K, seed[0], seed[1], amp, chirp)


def test_adjoint_forward_matches_pf_run():
    w, seed, taper_z, alpha = _setup()
    amp, chirp = 1e-2, 0.05
    with P.Puffin(w.params) as sim:
        sim.set_particles(*(w.beam[k] for k in P.PARTICLE_KEYS))
        e_adj = _energy(sim, w, seed, taper_z, alpha, amp, chirp)
    e_run = _run_energy(w.params, w, seed, taper_z, alpha, amp, chirp)
    assert e_adj == pytest.approx(e_run, rel=1e-9)


def test_adjoint_gradient_matches_central_differences():
    w, seed, taper_z, alpha = _setup()
    amp, chirp = 1e-2, 0.05
    with P.Puffin(w.params) as sim:
        sim.set_particles(*(w.beam[k] for k in P.PARTICLE_KEYS))
        e0 = _energy(sim, w, seed, taper_z, alpha, amp, chirp)
        g_taper, g_amp, g_chirp = sim.adjoint_backward(len(alpha))
        assert e0 > 0.0
        num = _fd_checks(sim, w, seed, taper_z, alpha, amp, chirp)
    adj = {"seed_amp": g_amp, "chirp": g_chirp}
    adj.update({f"taper[{k}]": g_taper[k] for k in range(len(alpha))})
    scale = max(abs(v) for _, v in num)
    for name, v in num:
        if abs(v) < 1e-3 * scale:
            continue
        assert abs(adj[name] - v) <= 1e-4 * abs(v), f"{name}: adjoint {adj[name]!r} vs differences {v!r}"


def test_mixed_adjoint_forward_matches_pf_run():
    """The mixed adjoint's recorded forward runs the mixed stage kernels and
    the FP32 diffraction: its energy is pf_run's on a mixed handle, to the
    rounding of the FP32 float atomics (deposits outside the shared tiles)."""
    w, seed, taper_z, alpha = _setup()
    amp, chirp = 1e-2, 0.05
    with P.Puffin(_mixed(w.params)) as sim:
        sim.set_particles(*(w.beam[k] for k in P.PARTICLE_KEYS))
        e_adj = _energy(sim, w, seed, taper_z, alpha, amp, chirp)
    e_run = _run_energy(_mixed(w.params), w, seed, taper_z, alpha, amp, chirp)
    e_64 = _run_energy(w.params, w, seed, taper_z, alpha, amp, chirp)
    assert e_adj == pytest.approx(e_run, rel=1e-5)
    assert e_adj == pytest.approx(e_64, rel=1e-4)


def test_mixed_adjoint_gradient_matches_fp64_differences():
    w, seed, taper_z, alpha = _setup()
    amp, chirp = 1e-2, 0.05
    with P.Puffin(_mixed(w.params)) as sim:
        sim.set_particles(*(w.beam[k] for k in P.PARTICLE_KEYS))
        assert _energy(sim, w, seed, taper_z, alpha, amp, chirp) > 0.0
        g_taper, g_amp, g_chirp = sim.adjoint_backward(len(alpha))
        # the backward pass leaves the handle usable for another run
        e_again = _energy(sim, w, seed, taper_z, alpha, amp, chirp)
        g2 = sim.adjoint_backward(len(alpha))
    np.testing.assert_allclose(g2[0], g_taper, rtol=1e-5, atol=1e-5 * np.max(np.abs(g_taper)))
    assert e_again > 0.0
    with P.Puffin(w.params) as sim:
        sim.set_particles(*(w.beam[k] for k in P.PARTICLE_KEYS))
        num = _fd_checks(sim, w, seed, taper_z, alpha, amp, chirp)
    adj = {"seed_amp": g_amp, "chirp": g_chirp}
    adj.update({f"taper[{k}]": g_taper[k] for k in range(len(alpha))})
    scale = max(abs(v) for _, v in num)
    for name, v in num:
        if abs(v) < 1e-3 * scale:
            continue
        assert abs(adj[name] - v) <= 1e-4 * abs(v), f"{name}: mixed adjoint {adj[name]!r} vs FP64 differences {v!r}"


def test_autograd_function():
    w, seed, taper_z, alpha = _setup()
    with P.Puffin(w.params) as sim:
        sim.set_particles(*(w.beam[k] for k in P.PARTICLE_KEYS))
        a = torch.tensor(alpha, dtype=torch.float64, requires_grad=True)
        s = torch.tensor(1e-2, dtype=torch.float64, requires_grad=True)
        c = torch.tensor(0.05, dtype=torch.float64, requires_grad=True)
        e = pulse_energy(sim, a, s, c, taper_z, seed, NSTEPS, EVERY, w.h, checkpoint_every=K)
        (3.0 * e).backward()
        e2 = _energy(sim, w, seed, taper_z, alpha, 1e-2, 0.05)
        g_taper, g_amp, g_chirp = sim.adjoint_backward(len(alpha), 3.0)
    assert float(e.detach()) == pytest.approx(e2, rel=1e-13)
    np.testing.assert_allclose(a.grad.numpy(), g_taper, rtol=1e-12, atol=0)
    assert float(s.grad) == pytest.approx(g_amp, rel=1e-12)
    assert float(c.grad) == pytest.approx(g_chirp, rel=1e-12)
