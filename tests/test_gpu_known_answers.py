"""The diffraction step and the 3D coupling against the reference's own known
answers (the formulas of puffin/lib/utilities/base_functions.f90 that its
unit tests pin, test/testFFunctions.pf; restated in oracle/oracle.py and
checked there against those values).

* Free-space diffraction: a Gaussian seed of field amplitude
  exp(-r^2 / (2 sigma^2)) on the resonant carrier, the electrons absent,
  propagated through pf_diffract over one Rayleigh range
  zR = RaleighLength(rho, sigma): its rms width grows by
  DiffractionLength(z, zR, sigma) / DiffractionLength(0, zR, sigma) =
  sqrt(1 + (z / zR)^2).  Periodic and temporal meshes (the latter through
  the 129-point prime-factor transform and the z2 absorbing mask), FP64 and
  FP32.  This pins the propagator, the k-values, the filter and the
  absorbing step (diffraction.f90:111-523) to the paraxial optics the
  scaled units are built on.
* Exponential gain: a cold resonant beam seeded at the resonant wavenumber
  grows in power as exp(g zbar) with g = sqrt(3) (1D high-gain theory: the
  power gain length is GainLength(lambda_w, rho) / sqrt(3)) times the
  attenuation of linear interpolation at 16 nodes per wavelength
  (oracle.cold_beam_power_growth).  On the 1D mesh this pins the 1D
  coupling; on a 3D mesh with the beam on the axis node and no diffraction
  the axis column is that same 1D FEL, which pins the trilinear gather and
  deposit, dV3 and the 3D source term (system_interpolation.f90:25-248,
  rhs.f90:60-330) in both precisions.
"""
import math

import numpy as np
import pytest

import puffin_gb300 as P
from puffin_gb300 import configs
from oracle import oracle as O

pytestmark = pytest.mark.gpu


# ---------------------------------------------------------------------------
def _carrier_seed(p, sigma, rho):
    xs = (np.arange(p.nx) - (p.nx - 1) / 2) * p.dx
    ys = (np.arange(p.ny) - (p.ny - 1) / 2) * p.dy
    g = np.exp(-(xs[None, :] ** 2 + ys[:, None] ** 2) / (2.0 * sigma ** 2))
    z = np.arange(p.nz2) * p.dz2
    re = (np.cos(z / (2.0 * rho))[:, None, None] * g).ravel()
    im = (-np.sin(z / (2.0 * rho))[:, None, None] * g).ravel()
    return re, im, xs, ys


def _widths(p, re, im, xs, ys, planes):
    inten = (re ** 2 + im ** 2).reshape(p.nz2, p.ny, p.nx)[planes]
    ix = inten.sum(axis=(0, 1))
    iy = inten.sum(axis=(0, 2))
    return (math.sqrt(float((xs ** 2 * ix).sum() / ix.sum())),
            math.sqrt(float((ys ** 2 * iy).sum() / iy.sum())))


CASES = {
    # name: (mesh, nx, dx, rho, sigma, resonant wavelengths in z2)
    "periodic65": (P.MESH_PERIODIC, 65, 0.25, 0.005, 0.75, 2),
    "temporal129": (P.MESH_TEMPORAL, 129, 0.5, 0.002, 1.5, 16),
}
TOL = {("periodic65", P.FP64): 1e-7, ("periodic65", P.MIXED): 2e-5,
       ("temporal129", P.FP64): 1e-5, ("temporal129", P.MIXED): 3e-5}


@pytest.mark.parametrize("prec", [P.FP64, P.MIXED])
@pytest.mark.parametrize("case,ncalls", [("periodic65", 1), ("periodic65", 4),
                                         ("temporal129", 1)])
def test_gaussian_seed_follows_the_diffraction_length(case, prec, ncalls):
    """One call over zR, or four over zR / 4.  The temporal mesh runs one
    call only: each call splits the field of the 37 absorbing z2 end planes
    off and damps it in the full 3D spectrum, which leaks into the interior
    planes at about 6e-5 per call here (the reference's AbsorptionStep,
    diffraction.f90:367-523, does the same; the oracle agrees)."""
    mesh, nx, dx, rho, sigma, nwaves = CASES[case]
    lamr = 4.0 * configs.PUFFIN_PI * rho
    eta, kappa, fx, fy = configs.calc_scaling(rho, 1.0, 500.0, P.UND_HELICAL)
    nz2 = 16 * nwaves + (1 if mesh == P.MESH_PERIODIC else 0)
    p = P.default_params(rho=rho, aw=1.0, gamma_r=500.0, eta=eta, kappa=kappa, fx=fx, fy=fy,
                         und_type=P.UND_HELICAL, nx=nx, ny=nx, nz2=nz2, dx=dx, dy=dx,
                         dz2=lamr / 16.0, mesh_type=mesh, sperwaves=float(nwaves),
                         precision=prec)
    re, im, xs, ys = _carrier_seed(p, sigma, rho)
    # planes away from the temporal mesh's z2 absorbing ends (37 nodes)
    planes = slice(0, nz2 - 1) if mesh == P.MESH_PERIODIC else slice(40, nz2 - 40)
    w0 = _widths(p, re, im, xs, ys, planes)
    zr = O.raleigh_length(rho, sigma)
    with P.Puffin(p) as sim:
        sim.set_field(re, im)
        for _ in range(ncalls):
            sim.diffractIM(zr / ncalls)
        gr, gi = sim.get_field()
    w1 = _widths(p, gr, gi, xs, ys, planes)
    want = O.diffraction_length(zr, zr, sigma) / O.diffraction_length(0.0, zr, sigma)
    assert abs(want - math.sqrt(2.0)) < 1e-15
    for a, b in zip(w1, w0):
        assert abs(a / b / want - 1.0) < TOL[(case, prec)], (a / b, want)


# ---------------------------------------------------------------------------
RHO, NPER = 0.005, 4


def _cold_params(nx, dx, prec):
    eta, kappa, fx, fy = configs.calc_scaling(RHO, 1.0, 500.0, P.UND_HELICAL)
    lamr = 4.0 * configs.PUFFIN_PI * RHO
    return P.default_params(rho=RHO, aw=1.0, gamma_r=500.0, eta=eta, kappa=kappa, fx=fx, fy=fy,
                            und_type=P.UND_HELICAL, nx=nx, ny=nx, nz2=16 * NPER + 1, dx=dx,
                            dy=dx, dz2=lamr / 16.0, mesh_type=P.MESH_PERIODIC,
                            sperwaves=float(NPER), one_d=int(nx == 1), szfs=0.0,
                            szfe=1.0e30, precision=prec), lamr


def _growth(p, beam, line_of, nsteps, h, a0=1e-4):
    """Power of the resonant harmonic along z2 (the line of nodes
    line_of(field) picks) every 16 steps; fit of ln P between 1e-6 and 1e-2
    (the exponential regime, well before saturation near 1)."""
    z = np.arange(p.nz2) * p.dz2
    shape = (p.nz2, p.ny, p.nx)
    re = np.broadcast_to((a0 * np.cos(z / (2 * RHO)))[:, None, None], shape).ravel().copy()
    im = np.broadcast_to((-a0 * np.sin(z / (2 * RHO)))[:, None, None], shape).ravel().copy()
    zs, ps = [], []
    with P.Puffin(p) as sim:
        sim.set_particles(*(beam[k] for k in P.PARTICLE_KEYS))
        sim.set_field(re, im)
        szl = 0.0
        for _ in range(nsteps // 16):
            szl = sim.und_section(16, 16, False, h, szl)
            fr, fi = sim.get_field()
            line = line_of(fr.reshape(shape), fi.reshape(shape))[:p.nz2 - 1]
            f = np.fft.fft(line) / len(line)
            zs.append(szl)
            ps.append(abs(f[NPER]) ** 2 + abs(f[-NPER]) ** 2)
    zs, ps = np.array(zs), np.array(ps)
    sel = (ps > 1e-6) & (ps < 1e-2)
    assert np.count_nonzero(sel) > 50
    return float(np.polyfit(zs[sel], np.log(ps[sel]), 1)[0])


@pytest.mark.parametrize("prec", [P.FP64, P.MIXED])
def test_cold_beam_gain_1d(prec):
    p, lamr = _cold_params(1, 1.0, prec)
    n = 4096
    lz2 = (p.nz2 - 1) * p.dz2
    beam = {"x": np.zeros(n), "y": np.zeros(n), "z2": (np.arange(n) + 0.5) * lz2 / n,
            "px": np.zeros(n), "py": np.zeros(n), "gam": np.ones(n), "chi": np.full(n, lz2 / n)}
    configs.match_in(p, beam)
    g = _growth(p, beam, lambda r, i: r[:, 0, 0] + 1j * i[:, 0, 0], 6000, lamr / 32.0)
    want = O.cold_beam_power_growth(16)
    assert abs(g / want - 1.0) < 0.01, (g, want)
    # in physical units: the power gain length is GainLength(lambda_w, rho) / g
    lam_w = 0.03
    assert abs((O.gain_length(lam_w, RHO) / g) / (O.gain_length(lam_w, RHO) / want) - 1) < 0.01


@pytest.mark.parametrize("prec", [P.FP64, P.MIXED])
def test_cold_beam_gain_3d_on_the_axis_node(prec):
    """The 3D kernels (trilinear weights, 3D deposit with dV3 = dx dy dz2,
    the 3D equations with the off-axis undulator field) on a beam whose
    macroparticles sit on the axis node of a 15 x 15 transverse mesh with
    chi = dx dy L / N (unit density in that node's cells): without
    diffraction the axis column is the 1D FEL.  Cells of dx = 4 keep the
    helical orbit (amplitude 2 rho = 0.01) at 0.25 % of a cell, so the
    trilinear weights keep nearly all the coupling on the axis node (at
    dx = 1 the orbit takes 0.8 % of the growth rate off it).  A transversely
    uniform beam is not a 1D FEL here: the off-axis undulator field
    (bfields.f90:741-742) detunes macroparticles away from the axis."""
    p, lamr = _cold_params(15, 4.0, prec)
    lz2 = (p.nz2 - 1) * p.dz2
    n = 4096
    beam = {"x": np.zeros(n), "y": np.zeros(n), "z2": (np.arange(n) + 0.5) * lz2 / n,
            "px": np.zeros(n), "py": np.zeros(n), "gam": np.ones(n),
            "chi": np.full(n, p.dx * p.dy * lz2 / n)}
    configs.match_in(p, beam)
    c = p.nx // 2
    grow = _growth(p, beam, lambda r, i: r[:, c, c] + 1j * i[:, c, c], 6000, lamr / 32.0)
    want = O.cold_beam_power_growth(16)
    assert abs(grow / want - 1.0) < 0.01, (grow, want)
