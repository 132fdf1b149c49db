"""FEL figures of merit from a run: the pulse energy along the undulator, the
power gain length of the exponential (linear) regime and the saturated
power.

The reference writes the same quantities through its integrated-data files
(power per z2 slice every write step, puffin/lib/io/hdf5PuffColl.f90); here
the pulse energy sum |A|^2 dx dy dz2 over the unique planes is sampled after
every block of steps between diffraction calls.
"""
from __future__ import annotations

import numpy as np

from . import lib as L
from .puffin import PARTICLE_KEYS, Puffin


def power_curve(params, beam, field, h: float, nsteps: int, every: int = 16,
                timings: bool = False):
    """Runs the module from (beam, field) in calls of `every` steps with
    diffraction every `every` steps; returns (zbar, energy) after each call,
    and with `timings` also the wall-clock seconds of each call (the steps'
    host and device time: each call ends with the device idle)."""
    import time

    p = params
    nuniq = p.nz2 - 1 if p.mesh_type == L.MESH_PERIODIC else p.nz2
    n = p.nx * p.ny * nuniq
    zs, es, ts = [], [], []
    with Puffin(p) as sim:
        sim.set_particles(*(beam[k] for k in PARTICLE_KEYS))
        sim.set_field(*field)
        szl = 0.0
        for _ in range(nsteps // every):
            t0 = time.perf_counter()
            szl = sim.und_section(every, every, True, h, szl)
            sim.sync()
            ts.append(time.perf_counter() - t0)
            fr, fi = sim.get_field()
            es.append(float(np.sum(fr[:n] ** 2 + fi[:n] ** 2)) * p.dx * p.dy * p.dz2)
            zs.append(szl)
    if timings:
        return np.array(zs), np.array(es), np.array(ts)
    return np.array(zs), np.array(es)


def saturation(z, e, dip=0.9, floor=0.1):
    """The first saturation: the first local maximum of the energy, at least
    floor times the largest energy of the run (wiggles of the start-up
    regime are far below), after which the energy falls below dip times that
    maximum before exceeding it again (the top of the first synchrotron
    oscillation).  Returns (zbar, energy)."""
    e = np.asarray(e)
    top = float(np.max(e))
    for k in range(1, len(e) - 1):
        if not (e[k] >= e[k - 1] and e[k] > e[k + 1]) or e[k] < floor * top:
            continue
        after = e[k + 1:]
        above = np.nonzero(after > e[k])[0]
        seg = after[:above[0]] if len(above) else after
        if len(seg) and np.min(seg) < dip * e[k]:
            return float(z[k]), float(e[k])
    k = int(np.argmax(e))
    return float(z[k]), float(e[k])


def gain_length(z, e, lo=1e-3, hi=1e-1):
    """Power gain length (zbar per e-folding) from a least-squares fit of
    ln(energy) over the samples before saturation whose energy lies between
    lo and hi times the saturated energy.  Returns (length, zbar_lo, zbar_hi)."""
    zs, es = saturation(z, e)
    sel = (z < zs) & (e >= lo * es) & (e <= hi * es)
    if np.count_nonzero(sel) < 3:
        raise ValueError("too few samples in the exponential regime")
    slope = np.polyfit(z[sel], np.log(e[sel]), 1)[0]
    return float(1.0 / slope), float(z[sel][0]), float(z[sel][-1])


def compare(z, e_ref, e_test):
    """Gain length and saturated energy of two runs and their relative
    differences (test against reference)."""
    g0, za, zb = gain_length(z, e_ref)
    g1, _, _ = gain_length(z, e_test)
    s0 = saturation(z, e_ref)
    s1 = saturation(z, e_test)
    return {
        "gain_length": {"ref": g0, "test": g1, "rel_diff": g1 / g0 - 1.0, "fit_zbar": [za, zb]},
        "saturated_energy": {"ref": s0[1], "test": s1[1], "rel_diff": s1[1] / s0[1] - 1.0,
                             "zbar_ref": s0[0], "zbar_test": s1[0]},
        "max_energy": {"ref": float(np.max(e_ref)), "test": float(np.max(e_test)),
                       "rel_diff": float(np.max(e_test) / np.max(e_ref) - 1.0)},
    }
