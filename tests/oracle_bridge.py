"""Helpers that run the CPU oracle on the same inputs as a puffgpu handle."""
import numpy as np

from oracle import oracle as O
import puffin_gb300 as P

CFG_KEYS = ("rho", "aw", "gamma_r", "eta", "kappa", "nx", "ny", "nz2", "dx", "dy", "dz2",
            "mesh_type", "und_type", "fx", "fy", "kx_und", "ky_und", "kbxsf", "kbysf",
            "szfs", "szfe", "n2col0", "undgrad", "sbeta", "sfilt_frac", "sperwaves",
            "nbx", "nby", "nbz2")
BOOL_KEYS = ("focusing", "und_ends", "one_d", "field_evolve", "electrons_evolve", "coupling",
             "qfilter")


def oracle_config(params):
    kw = {k: getattr(params, k) for k in CFG_KEYS}
    kw.update({k: bool(getattr(params, k)) for k in BOOL_KEYS})
    return O.Config(**kw)


def oracle_beam(beam):
    return O.Beam(*(np.array(beam[k], dtype=np.float64) for k in P.PARTICLE_KEYS))


def assert_beam_close(got, beam, rtol, atol, keys=("x", "y", "z2", "px", "py", "gam")):
    for k in keys:
        np.testing.assert_allclose(got[k], getattr(beam, k), rtol=rtol, atol=atol, err_msg=k)
