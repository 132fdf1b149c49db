"""Synthetic workloads in Puffin scaled units, and the host-side undulator
entry/exit matching that brackets the hot path.

The workloads stand in for the configurations the reference is quoted on; no
dataset or reference input deck is read.  Beams are drawn from a seeded
generator (numpy PCG64, seed 0x5EED unless given).

Choices the configurations leave open are fixed here and stated:
* momenta spread sigma_p = 0.01 (scaled p_perp) about the matched orbit;
* config 2's transverse cell size dx = dy = 0.5 (mesh 64 wide = +-21 sigma);
* config 1 truncates x, y to |x|,|y| <= 1.35 so the inner-window rule
  2 (ceil(max|x|/dx) + 3) fits the 21-node mesh;
* charge weights chi = 2 pi sigma_x sigma_y L_beam / Np (unit peak density).
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from . import lib as L

PUFFIN_PI = float(np.float32(3.14159265358979323846))
SEED = 0x5EED


def calc_scaling(rho, aw, gamma_r, und_type, fx=1.0, fy=1.0):
    """eta, kappa and the fx/fy overrides of calcScaling
    (puffin/lib/setup/setup_calcs.f90:722-803)."""
    if und_type in (L.UND_CURVED, L.UND_PLANEPOLE):
        aw_rms, fx, fy = aw / math.sqrt(2.0), 0.0, 1.0
    elif und_type == L.UND_HELICAL:
        aw_rms, fx, fy = aw, 1.0, 1.0
    else:
        aw_rms = aw * math.sqrt(fx ** 2 + fy ** 2) / math.sqrt(2.0)
    betaz = math.sqrt(gamma_r ** 2.0 - 1.0 - aw_rms ** 2.0) / gamma_r
    eta = (1.0 - betaz) / betaz
    kappa = aw / 2.0 / rho / gamma_r
    return eta, kappa, fx, fy


@dataclass
class Workload:
    name: str
    params: L.Params
    h: float             # RK4 step in zbar
    nsteps: int
    isteps4diff: int
    qdiffraction: bool
    beam: dict           # x, y, z2, px, py, gam, chi (numpy float64)
    field: tuple         # (re, im) outer mesh

    @property
    def np(self):
        return len(self.beam["x"])


def _base_params(rho, aw, gamma_r, und_type, nx, ny, nz2, dx, dy, dz2, mesh_type, **kw):
    eta, kappa, fx, fy = calc_scaling(rho, aw, gamma_r, und_type)
    p = L.default_params(rho=rho, aw=aw, gamma_r=gamma_r, eta=eta, kappa=kappa, fx=fx, fy=fy,
                         und_type=und_type, nx=nx, ny=ny, nz2=nz2, dx=dx, dy=dy, dz2=dz2,
                         mesh_type=mesh_type)
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def match_in(params, beam, sz=0.0, n2col=None):
    """matchIn (puffin/lib/acc_lattice.f90:743-846) with the offsets of
    init_conds.f90:70-203, on host arrays in place."""
    _match(params, beam, sz, params.n2col0 if n2col is None else n2col, +1.0)


def match_out(params, beam, sz, n2col):
    """matchOut (puffin/lib/acc_lattice.f90:638-741)."""
    _match(params, beam, sz, n2col, -1.0)


def _match(p, b, sz, n2col, sign):
    rho = p.rho
    pxo = -(p.fy * n2col * math.cos(sz / (2.0 * rho)))
    pyo = -(p.fx * n2col * math.sin(sz / (2.0 * rho)))
    n = len(b["x"])
    if p.und_type == L.UND_CURVED:
        kx, ky = p.kx_und, p.ky_und
        spx = pxo - 0.5 * kx ** 2 * b["x"] ** 2 - 0.5 * ky ** 2 * b["y"] ** 2
        spy = -1.0 * (pyo - kx ** 2 * b["x"] * b["y"])
    elif p.und_type == L.UND_PLANEPOLE:
        spx = pxo - 0.5 * (p.eta / (4 * rho ** 2)) * b["x"] ** 2
        spy = np.full(n, -1.0 * pyo)
    else:
        spx = np.full(n, pxo)
        spy = np.full(n, -1.0 * pyo)
    gj = p.gamma_r * b["gam"]
    pyarg = -spy if sign > 0 else spy
    common = 4.0 * p.kappa * rho ** 2 / math.sqrt(p.eta)
    nc_x = p.aw ** 2
    nc_y = 2.0 * p.aw ** 2 / (p.fx ** 2 + p.fy ** 2)
    xo = -(p.fy * common * (p.gamma_r / np.sqrt(gj * gj - (1.0 + nc_x * (spx * spx + pyarg * pyarg))))
           * n2col * math.sin(sz / (2.0 * rho)))
    yo = (p.fx * common * (p.gamma_r / np.sqrt(gj * gj - (1.0 + nc_y * (spx * spx + pyarg * pyarg))))
          * n2col * math.cos(sz / (2.0 * rho)))
    b["x"][:] = b["x"] + sign * xo
    b["y"][:] = b["y"] + sign * yo
    b["px"][:] = b["px"] + sign * spx
    b["py"][:] = b["py"] + sign * spy


def _quiet_z2(rng, n, start, length):
    """Quiet start: equally spaced macroparticles with a seeded shot-noise
    jitter of (u - 1/2) * dz / 10, in the spirit of noise.f90:65-80."""
    dz = length / n
    z = start + (np.arange(n) + 0.5) * dz
    z += (rng.random(n) - 0.5) * dz * 0.1
    return z


def config1(np_=2 ** 16, seed=SEED, nsteps=2000):
    """3D periodic single slice, helical, rho=0.005, aw=1, gamma_r=500,
    21x21 (dx=dy=0.2) x 65 z2 nodes (64 unique) over 4 resonant wavelengths,
    32 steps per period, diffraction every 16 steps."""
    rho, aw, gr = 0.005, 1.0, 500.0
    lamr = 4.0 * PUFFIN_PI * rho
    dz2 = lamr / 16.0                      # nodesPerLambdar = 17 (setup_calcs.f90:865)
    nz2 = int(round(4.0 * lamr / dz2)) + 1  # sPerWaves = 4
    p = _base_params(rho, aw, gr, L.UND_HELICAL, 21, 21, nz2, 0.2, 0.2, dz2, L.MESH_PERIODIC,
                     sperwaves=4.0, szfs=0.0, szfe=nsteps * lamr / 32.0)
    rng = np.random.default_rng(seed)
    lz2 = (nz2 - 1) * dz2
    sig = 1.0
    x = rng.standard_normal(np_ * 2)
    x = x[np.abs(x) <= 1.35][:np_]
    y = rng.standard_normal(np_ * 2)
    y = y[np.abs(y) <= 1.35][:np_]
    beam = {
        "x": x.copy(), "y": y.copy(),
        "z2": _quiet_z2(rng, np_, 0.0, lz2),
        "px": 0.01 * rng.standard_normal(np_), "py": 0.01 * rng.standard_normal(np_),
        "gam": 1.0 + 5e-4 * rng.standard_normal(np_),
        "chi": np.full(np_, 2.0 * math.pi * sig * sig * lz2 / np_),
    }
    match_in(p, beam)
    n = p.nx * p.ny * p.nz2
    return Workload("config1: periodic helical 21x21x64, rho=0.005, gamma_r=500", p,
                    lamr / 32.0, nsteps, 16, True, beam, (np.zeros(n), np.zeros(n)))


def config2(np_=2 ** 23, seed=SEED, nperiods=20, nz2=4096):
    """3D temporal planepole, aw_rms = 0.8 (peak 0.8*sqrt 2), rho=0.002,
    gamma_r=2000, linear taper -1% over the module, 129x129 (dx=dy=0.5) x 4096
    z2 nodes, flat-top beam over 80% of z2 with sigma_perp = 1.5 and 0.01%
    energy spread, 24 steps per period, diffraction every 8 steps."""
    rho, aw, gr = 0.002, 0.8 * math.sqrt(2.0), 2000.0
    lamr = 4.0 * PUFFIN_PI * rho
    dz2 = lamr / 16.0
    nsteps = nperiods * 24
    h = lamr / 24.0
    zlen = nsteps * h
    undgrad = -0.01 / zlen
    p = _base_params(rho, aw, gr, L.UND_PLANEPOLE, 129, 129, nz2, 0.5, 0.5, dz2,
                     L.MESH_TEMPORAL, szfs=0.0, szfe=zlen, undgrad=undgrad)
    rng = np.random.default_rng(seed)
    lz2 = (nz2 - 1) * dz2
    sig = 1.5
    beam = {
        "x": sig * np.clip(rng.standard_normal(np_), -5.0, 5.0),
        "y": sig * np.clip(rng.standard_normal(np_), -5.0, 5.0),
        "z2": _quiet_z2(rng, np_, 0.1 * lz2, 0.8 * lz2),
        "px": 0.01 * rng.standard_normal(np_), "py": 0.01 * rng.standard_normal(np_),
        "gam": 1.0 + 1e-4 * rng.standard_normal(np_),
        "chi": np.full(np_, 2.0 * math.pi * sig * sig * 0.8 * lz2 / np_),
    }
    match_in(p, beam)
    n = p.nx * p.ny * p.nz2
    return Workload(f"config2: temporal planepole 129x129x{nz2}, rho=0.002, gamma_r=2000, taper -1%",
                    p, h, nsteps, 8, True, beam, (np.zeros(n), np.zeros(n)))


def config3(np_=2 ** 24, seed=SEED, nsteps=2000):
    """Config-1 shapes at 2^24 macroparticles (same density)."""
    w = config1(np_=np_, seed=seed, nsteps=nsteps)
    w.name = "config3: config1 mesh, 2^24 macroparticles"
    return w


def config4(np_=2 ** 18, seed=SEED, nsteps=3000):
    """The adjoint form's mesh: periodic helical 33 x 33 x 129 nodes (128
    unique planes over 8 resonant wavelengths), dx = dy = 0.2, rho = 0.005,
    aw = 1, gamma_r = 500, 32 steps per period, diffraction every 16 steps,
    the config-1 beam at 2^18 macroparticles (sigma 1.0, |x|,|y| <= 1.35)."""
    w = config1(np_=np_, seed=seed, nsteps=nsteps)
    p = w.params
    lamr = 4.0 * PUFFIN_PI * p.rho
    p.nx = p.ny = 33
    p.nz2 = 129
    p.dz2 = 8.0 * lamr / 128.0
    p.sperwaves = 8.0
    rng = np.random.default_rng(seed)
    lz2 = (p.nz2 - 1) * p.dz2
    w.beam["z2"] = _quiet_z2(rng, np_, 0.0, lz2)
    w.beam["chi"] = np.full(np_, 2.0 * math.pi * lz2 / np_)
    n = p.nx * p.ny * p.nz2
    w.field = (np.zeros(n), np.zeros(n))
    w.name = "config4: periodic helical 33x33x128 (adjoint form)"
    return w


def config5(n_inst=128, seed=SEED, nsteps=1000, np_range=(2 ** 14, 2 ** 20)):
    """The batched form: n_inst independent periodic single-slice instances.
    Per instance, from the seed: macroparticles log-uniform in np_range;
    transverse mesh nx = ny in {17, 33, 65} with dx chosen so the inner-window
    rule fits the beam (|x|, |y| <= 1.35 sigma, sigma 1.0) on the mesh; z2
    mesh of {32, 64, 128} unique planes at 16 per resonant wavelength;
    rho uniform in [0.002, 0.01]; energy detuning uniform in +-2 rho; aw
    uniform in [0.7, 1.5]; helical or planepole with equal odds.  32 steps per
    period (h = 4 pi rho / 32), diffraction every 16 steps.  Returns the list
    of workloads (each with its own params, h and beam)."""
    rng = np.random.default_rng(seed)
    out = []
    lo, hi = math.log(np_range[0]), math.log(np_range[1])
    for k in range(n_inst):
        np_ = int(round(math.exp(rng.uniform(lo, hi))))
        nx = int(rng.choice([17, 33, 65]))
        nunique = int(rng.choice([32, 64, 128]))
        rho = float(rng.uniform(0.002, 0.01))
        detune = float(rng.uniform(-2.0 * rho, 2.0 * rho))
        aw = float(rng.uniform(0.7, 1.5))
        und = L.UND_HELICAL if rng.random() < 0.5 else L.UND_PLANEPOLE
        gr = 500.0
        lamr = 4.0 * PUFFIN_PI * rho
        dz2 = lamr / 16.0
        nz2 = nunique + 1
        # window rule 2 (ceil(1.35 / dx) + 3) <= nx - 1
        dx = 1.35 / ((nx - 1) / 2 - 3.5)
        p = _base_params(rho, aw, gr, und, nx, nx, nz2, dx, dx, dz2, L.MESH_PERIODIC,
                         sperwaves=nunique / 16.0, szfs=0.0, szfe=nsteps * lamr / 32.0)
        lz2 = nunique * dz2
        x = rng.standard_normal(np_ * 2)
        x = x[np.abs(x) <= 1.35][:np_]
        y = rng.standard_normal(np_ * 2)
        y = y[np.abs(y) <= 1.35][:np_]
        beam = {
            "x": x.copy(), "y": y.copy(),
            "z2": _quiet_z2(rng, np_, 0.0, lz2),
            "px": 0.01 * rng.standard_normal(np_), "py": 0.01 * rng.standard_normal(np_),
            "gam": 1.0 + detune + 5e-4 * rng.standard_normal(np_),
            "chi": np.full(np_, 2.0 * math.pi * lz2 / np_),
        }
        match_in(p, beam)
        n = p.nx * p.ny * p.nz2
        und_name = "helical" if und == L.UND_HELICAL else "planepole"
        out.append(Workload(f"batch instance {k}: periodic {und_name} {nx}x{nx}x{nunique}, "
                            f"rho={rho:.4f}, aw={aw:.3f}, detuning={detune:+.4f}, np={np_}",
                            p, lamr / 32.0, nsteps, 16, True, beam, (np.zeros(n), np.zeros(n))))
    return out
