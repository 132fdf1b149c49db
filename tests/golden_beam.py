"""Initial state of the reference's 1D end-to-end golden test.

test/inputs/f1main.in + beam_file.in + seed_file.in describe a deterministic
run (q_noise = .false., zero seed): a cold flat-top beam of 319 macroparticles
over z2 in [0, 2], generated on 2 MPI ranks, matched into a 'puffin'
(elliptical, ux = uy = 1) undulator with rho = 0.01, aw = 1, gamma_r = 100,
and pushed 30 RK4 steps (1 period at 30 steps per period) on a temporal
511-node z2 mesh.  The dump is taken after matchOut + correctTrans.

The z2 positions restate splitBeam (parBeam.f90:17-75) and PulseGrid +
genMacros midpoints (particleFunctions.f90:28-80, gen_macros.f90:206-212);
the charge weights are read from the golden dump itself (they do not change
during the run).
"""
import math

import numpy as np

from oracle import oracle as O

NMP, LEN_Z2, NRANKS = 319, 2.0, 2
NSTEPS = 30


def config():
    rho, aw, gr = 0.01, 1.0, 100.0
    eta, kappa, fx, fy = O.calc_scaling(rho, aw, gr, O.UND_PUFFIN, 1.0, 1.0)
    h = 4.0 * O.PUFFIN_PI * rho / 30.0
    cfg = O.Config(rho=rho, aw=aw, gamma_r=gr, eta=eta, kappa=kappa, nx=1, ny=1,
                   nz2=511, dx=1.0, dy=1.0, dz2=4.0 / 510, mesh_type=O.MESH_TEMPORAL,
                   und_type=O.UND_PUFFIN, fx=fx, fy=fy, one_d=True, szfs=0.0,
                   szfe=NSTEPS * h, nix=1, niy=1)
    return cfg, h


def initial_z2():
    frac = float(np.float32(NMP) / np.float32(NRANKS))
    lown, highn = math.floor(frac), math.ceil(frac)
    rem = NMP % NRANKS
    one = LEN_Z2 / NMP
    lower, upper = lown * one, highn * one
    out = []
    for rank in range(NRANKS):
        locn = highn if rank < rem else lown
        if rank >= rem:
            s = upper * rem + (rank - rem) * lower
            f = upper * rem + ((rank + 1) - rem) * lower
        else:
            s, f = rank * upper, (rank + 1) * upper
        d = (f - s) / float(locn)
        g = s + np.arange(locn + 1) * d
        out.append(g[:-1] + (g[1:] - g[:-1]) / 2.0)
    return np.concatenate(out)


def initial_beam(cfg, chi):
    z2 = initial_z2()
    n = len(z2)
    beam = O.Beam(np.zeros(n), np.zeros(n), z2, np.zeros(n), np.zeros(n),
                  np.ones(n), np.array(chi, dtype=np.float64))
    O.match_in(cfg, beam, 0.0, 1.0)
    return beam
