"""The reference's element loop over a beam line (puffin/lib/puffin_module.f90:57-89)
on one ``Puffin`` handle: undulator modules (initUndulator, matchIn, the
RK4/diffraction loop, matchOut, correctTrans; puffin/lib/undulator.f90:33-358),
quads, chicanes, drifts and energy modulations (puffin/lib/acc_lattice.f90).

Element parameters are the scaled quantities the reference's lattice reader
produces (acc_lattice.f90:131-410): zbar lengths, dispersion and slippage in
z2, quad focal factors, modulation amplitude and wavenumber.
"""
from __future__ import annotations

from dataclasses import astuple, dataclass


@dataclass
class Undulator:
    und_type: int
    fx: float
    fy: float
    kbxsf: float
    kbysf: float
    mf: float          # taper factor alpha at the module start
    taper: float       # d(alpha)/dzbar
    nsteps: int
    h: float           # RK4 step size (sStepSize, delmz)
    isteps4diff: int


@dataclass
class Quad:
    qfx: float
    qfy: float


@dataclass
class Chicane:
    zbar: float        # slippage length for the field's diffraction
    disp: float        # chic_disp
    slip: float        # chic_slip


@dataclass
class Drift:
    zbar: float


@dataclass
class Modulation:
    mag: float
    wavenum: float


_KIND = {Undulator: "undulator", Quad: "quad", Chicane: "chicane", Drift: "drift",
         Modulation: "modulation"}


def as_tuple(el):
    """(kind, *fields): the plain form the CPU restatement takes."""
    return (_KIND[type(el)],) + astuple(el)


def run(sim, elements, qdiffraction: bool = True, sz: float = 0.0) -> float:
    """Run the beam line on ``sim`` (a ``Puffin``); returns the final zbar."""
    und_ends = bool(sim.params.und_ends)
    for el in elements:
        if isinstance(el, Undulator):
            sim.init_undulator(el.und_type, el.fx, el.fy, el.kbxsf, el.kbysf, el.mf, el.taper,
                               el.nsteps, el.h, und_ends)
            sz0 = sz
            if not und_ends:
                sim.matchIn(0.0)
            sim.wrap_z2()  # getLocalFieldIndices at the module start (undulator.f90:102)
            szl = sim.und_section(el.nsteps, el.isteps4diff, qdiffraction, el.h, 0.0)
            sz = sz0 + szl
            if not und_ends:
                sim.matchOut(sz)
            sim.correctTrans()
        elif isinstance(el, Quad):
            sim.quad(el.qfx, el.qfy)
        elif isinstance(el, Chicane):
            sim.disperse(el.disp, el.slip, el.zbar, qdiffraction)
            sz = sz + el.zbar
        elif isinstance(el, Drift):
            sim.drift(el.zbar, qdiffraction)
            sz = sz + el.zbar
        elif isinstance(el, Modulation):
            sim.modulation(el.mag, el.wavenum)
        else:
            raise TypeError(f"unknown beam-line element {el!r}")
    return sz
