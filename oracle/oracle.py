"""CPU oracle for the Puffin hot path (TEST INFRASTRUCTURE ONLY).

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg may import this module, and only to compare against: the GPU library
never calls it.  It restates the reference's algorithm on the CPU:

* the RK4 particle/field push (``puffin_oracle.c``, reached through ctypes);
* the diffraction step in numpy (``diffract``), following
  puffin/lib/diffraction/diffraction.f90:111-523, masks.f90:50-430 and
  transforms.f90:472-590, with numpy's FFT standing in for FFTW (unnormalised
  forward -1 / backward +1 transforms, as FFTW's are);
* host helpers that the reference performs between kernels: the inner
  transverse window (``get_in_node``, para_field.f90:1432-1508), the
  inner/outer copies (para_field.f90:1352-1429) and the split-step schedule of
  ``UndSection`` (undulator.f90:106-331).

Parity status: the 1D RK4 path is pinned against the reference's golden dump
(tests/golden/).  The 3D gather/deposit, b-field and diffraction paths have no
golden vectors in the reference and are a restatement only (parity unpinned for
those rows).
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libpuffin_oracle.so")

# puffin/lib/common/puffin_constants.f90:22 declares pi with a default-kind
# (single precision) literal; every use of the global pi sees this value.
PUFFIN_PI = float(np.float32(3.14159265358979323846))

UND_PUFFIN, UND_HELICAL, UND_PLANEPOLE, UND_CURVED = 0, 1, 2, 3
MESH_TEMPORAL, MESH_PERIODIC = 0, 1
UND_NAMES = {"": UND_PUFFIN, "puffin": UND_PUFFIN, "helical": UND_HELICAL,
             "planepole": UND_PLANEPOLE, "curved": UND_CURVED}


class _Params(ctypes.Structure):
    _fields_ = [
        ("rho", ctypes.c_double), ("eta", ctypes.c_double),
        ("kappa", ctypes.c_double), ("aw", ctypes.c_double),
        ("gamma_r", ctypes.c_double),
        ("fx", ctypes.c_double), ("fy", ctypes.c_double),
        ("kx_und", ctypes.c_double), ("ky_und", ctypes.c_double),
        ("kbxsf", ctypes.c_double), ("kbysf", ctypes.c_double),
        ("und_type", ctypes.c_int), ("one_d", ctypes.c_int),
        ("focusing", ctypes.c_int), ("und_ends", ctypes.c_int),
        ("field_evolve", ctypes.c_int), ("electrons_evolve", ctypes.c_int),
        ("coupling", ctypes.c_int),
        ("szfs", ctypes.c_double), ("szfe", ctypes.c_double),
        ("mesh_type", ctypes.c_int),
        ("nz2", ctypes.c_int64), ("nix", ctypes.c_int64), ("niy", ctypes.c_int64),
        ("dx", ctypes.c_double), ("dy", ctypes.c_double), ("dz2", ctypes.c_double),
    ]


class _Taper(ctypes.Structure):
    _fields_ = [("n2col", ctypes.c_double), ("n2col0", ctypes.c_double),
                ("undgrad", ctypes.c_double), ("nprof", ctypes.c_int),
                ("pz", ctypes.c_void_p), ("pa", ctypes.c_void_p)]


class _Stage(ctypes.Structure):
    _fields_ = [("sz", ctypes.c_double), ("n2col", ctypes.c_double),
                ("place", ctypes.c_int)]


_lib = None


def build():
    """Compile the C restatement with its committed Makefile."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        dp = ctypes.POINTER(ctypes.c_double)
        L.or_rk4_step.argtypes = [ctypes.POINTER(_Params), ctypes.POINTER(_Taper),
                                  ctypes.c_double, ctypes.c_double, ctypes.c_int64,
                                  dp, dp, dp, dp, dp, dp, dp, dp, dp]
        L.or_rk4_step.restype = ctypes.c_int
        L.or_rhs.argtypes = [ctypes.POINTER(_Params), ctypes.POINTER(_Stage),
                             ctypes.c_int64, dp, dp, dp, dp, dp, dp, dp, dp, dp,
                             dp, dp, dp, dp, dp, dp, dp, dp]
        L.or_rhs.restype = ctypes.c_int
        L.or_stage_setup.argtypes = [ctypes.POINTER(_Params), ctypes.POINTER(_Taper),
                                     ctypes.c_double, ctypes.POINTER(_Stage)]
        L.or_p2.argtypes = [ctypes.c_double] * 6
        L.or_p2.restype = ctypes.c_double
        L.or_wrap_z2.argtypes = [ctypes.POINTER(_Params), ctypes.c_int64, dp]
        L.or_set_threads.argtypes = [ctypes.c_int]
        L.or_bfield.argtypes = [ctypes.POINTER(_Params), ctypes.POINTER(_Stage),
                                ctypes.c_double, ctypes.c_double, dp, dp, dp]
        _lib = L
    return _lib


def _ptr(a):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def set_threads(n: int):
    lib().or_set_threads(int(n))


# ---------------------------------------------------------------------------
# Configuration (scaled units), mirroring the reference's global state.
# ---------------------------------------------------------------------------
@dataclass
class Config:
    rho: float
    aw: float                 # peak undulator parameter (saw_G)
    gamma_r: float
    eta: float
    kappa: float
    nx: int
    ny: int
    nz2: int
    dx: float
    dy: float
    dz2: float
    mesh_type: int = MESH_TEMPORAL
    und_type: int = UND_HELICAL
    fx: float = 1.0
    fy: float = 1.0
    kx_und: float = 0.0
    ky_und: float = 0.0
    kbxsf: float = 0.0
    kbysf: float = 0.0
    focusing: bool = False
    und_ends: bool = False
    one_d: bool = False
    field_evolve: bool = True
    electrons_evolve: bool = True
    coupling: bool = True
    szfs: float = 0.0
    szfe: float = 1.0e30
    n2col0: float = 1.0
    undgrad: float = 0.0
    # diffraction
    sbeta: float = 1.0
    sfilt_frac: float = 0.3
    qfilter: bool = True
    sperwaves: float = -1.0
    nbx: int = 16
    nby: int = 16
    nbz2: int = 37
    nix: int = 0
    niy: int = 0

    @property
    def nplanes(self):
        return self.nz2 - 1 if self.mesh_type == MESH_PERIODIC else self.nz2

    def cparams(self, nix=None, niy=None):
        p = _Params()
        for k in ("rho", "eta", "kappa", "aw", "gamma_r", "fx", "fy", "kx_und",
                  "ky_und", "kbxsf", "kbysf", "szfs", "szfe", "dx", "dy", "dz2"):
            setattr(p, k, float(getattr(self, k)))
        p.und_type = int(self.und_type)
        p.one_d = int(self.one_d)
        p.focusing = int(self.focusing)
        p.und_ends = int(self.und_ends)
        p.field_evolve = int(self.field_evolve)
        p.electrons_evolve = int(self.electrons_evolve)
        p.coupling = int(self.coupling)
        p.mesh_type = int(self.mesh_type)
        p.nz2 = int(self.nz2)
        p.nix = int(self.nix if nix is None else nix)
        p.niy = int(self.niy if niy is None else niy)
        return p


def calc_scaling(rho, aw, gamma_r, und_type, fx=1.0, fy=1.0):
    """eta and kappa (setup_calcs.f90 calcScaling, :722-803), with the same
    per-type fx/fy overrides."""
    if und_type == UND_CURVED:
        aw_rms, fx, fy = aw / math.sqrt(2.0), 0.0, 1.0
    elif und_type == UND_PLANEPOLE:
        aw_rms, fx, fy = aw / math.sqrt(2.0), 0.0, 1.0
    elif und_type == UND_HELICAL:
        aw_rms, fx, fy = aw, 1.0, 1.0
    else:
        aw_rms = aw * math.sqrt(fx ** 2 + fy ** 2) / math.sqrt(2.0)
    betaz = math.sqrt(gamma_r ** 2.0 - 1.0 - aw_rms ** 2.0) / gamma_r
    eta = (1.0 - betaz) / betaz
    kappa = aw / 2.0 / rho / gamma_r
    return eta, kappa, fx, fy


def get_in_node(cfg: Config, x, y):
    """Inner transverse window (nspinDX, nspinDY): para_field.f90:1432-1508."""
    if cfg.nx * cfg.ny == 1:
        return 1, 1
    inbuf = 3
    if len(x) > 0:
        smaxx, sminx = abs(np.max(x)), abs(np.min(x))
        smaxy, sminy = abs(np.max(y)), abs(np.min(y))
        imaxx, iminx = math.ceil(smaxx / cfg.dx), math.floor(sminx / cfg.dx)
        imaxy, iminy = math.ceil(smaxy / cfg.dy), math.floor(sminy / cfg.dy)
        nix = (max(imaxx, iminx) + inbuf) * 2
        niy = (max(imaxy, iminy) + inbuf) * 2
    else:
        nix = niy = 2
    if cfg.nx % 2 != nix % 2:
        nix += 1
    if cfg.ny % 2 != niy % 2:
        niy += 1
    if nix > cfg.nx or niy > cfg.ny:
        raise ValueError(f"transverse grid not large enough: nspinDX={nix}, nspinDY={niy}")
    return nix, niy


def outer_to_inner(cfg: Config, re, im, nix, niy):
    """Outer mesh (nz2, ny, nx) -> inner window (nplanes, niy, nix)."""
    ox, oy = (cfg.nx - nix) // 2, (cfg.ny - niy) // 2
    np_ = cfg.nplanes
    r = np.ascontiguousarray(re.reshape(cfg.nz2, cfg.ny, cfg.nx)[:np_, oy:oy + niy, ox:ox + nix])
    i = np.ascontiguousarray(im.reshape(cfg.nz2, cfg.ny, cfg.nx)[:np_, oy:oy + niy, ox:ox + nix])
    return r.reshape(-1), i.reshape(-1)


def inner_to_outer(cfg: Config, re, im, wr, wi, nix, niy):
    """Inner window -> outer mesh (in place); periodic tail plane mirrors plane 0."""
    ox, oy = (cfg.nx - nix) // 2, (cfg.ny - niy) // 2
    np_ = cfg.nplanes
    R = re.reshape(cfg.nz2, cfg.ny, cfg.nx)
    I = im.reshape(cfg.nz2, cfg.ny, cfg.nx)
    R[:np_, oy:oy + niy, ox:ox + nix] = wr.reshape(np_, niy, nix)
    I[:np_, oy:oy + niy, ox:ox + nix] = wi.reshape(np_, niy, nix)
    if cfg.mesh_type == MESH_PERIODIC:
        R[np_] = R[0]
        I[np_] = I[0]


# ---------------------------------------------------------------------------
# RK4 (C restatement)
# ---------------------------------------------------------------------------
@dataclass
class Beam:
    x: np.ndarray
    y: np.ndarray
    z2: np.ndarray
    px: np.ndarray
    py: np.ndarray   # stored as p_im = -py, as the reference's sElPY_G
    gam: np.ndarray
    chi: np.ndarray

    def copy(self):
        return Beam(*(np.array(getattr(self, k), dtype=np.float64, copy=True)
                      for k in ("x", "y", "z2", "px", "py", "gam", "chi")))

    def arrays(self):
        return [self.x, self.y, self.z2, self.px, self.py, self.gam]

    @property
    def n(self):
        return len(self.x)


@dataclass
class Taper:
    n2col: float
    n2col0: float
    undgrad: float
    profile_z: np.ndarray | None = None   # piecewise-linear alpha(z), if set
    profile_a: np.ndarray | None = None

    def c(self):
        if self.profile_z is None:
            return _Taper(self.n2col, self.n2col0, self.undgrad, 0, None, None)
        self._pz = np.ascontiguousarray(self.profile_z, dtype=np.float64)
        self._pa = np.ascontiguousarray(self.profile_a, dtype=np.float64)
        return _Taper(self.n2col, self.n2col0, self.undgrad, len(self._pz),
                      self._pz.ctypes.data, self._pa.ctypes.data)

    def update(self, t):
        self.n2col, self.n2col0, self.undgrad = t.n2col, t.n2col0, t.undgrad


def rk4_step(cfg: Config, taper: Taper, sz: float, h: float, beam: Beam,
             wr: np.ndarray, wi: np.ndarray, nix: int, niy: int) -> int:
    """One rk4par step in place on ``beam`` and the inner-window field."""
    p = cfg.cparams(nix, niy)
    t = taper.c()
    st = lib().or_rk4_step(ctypes.byref(p), ctypes.byref(t), float(sz), float(h),
                           beam.n, *(_ptr(a) for a in beam.arrays()), _ptr(beam.chi),
                           _ptr(wr), _ptr(wi))
    taper.update(t)
    return st


def stage_rhs(cfg: Config, sz: float, n2col: float, place: int, beam: Beam,
              wr, wi, nix, niy):
    """One getrhs evaluation; returns (status, derivs[6], dadz_r, dadz_i)."""
    p = cfg.cparams(nix, niy)
    st = _Stage(float(sz), float(n2col), int(place))
    d = [np.zeros(beam.n) for _ in range(6)]
    dr = np.zeros(len(wr))
    di = np.zeros(len(wi))
    s = lib().or_rhs(ctypes.byref(p), ctypes.byref(st), beam.n, _ptr(wr), _ptr(wi),
                     *(_ptr(a) for a in beam.arrays()), _ptr(beam.chi),
                     *(_ptr(a) for a in d), _ptr(dr), _ptr(di))
    return s, d, dr, di


def stage_setup(cfg: Config, taper: Taper, sz: float):
    p = cfg.cparams(1, 1)
    t = taper.c()
    st = _Stage()
    lib().or_stage_setup(ctypes.byref(p), ctypes.byref(t), float(sz), ctypes.byref(st))
    taper.update(t)
    return st.sz, st.n2col, st.place


def p2(gam, px, py, cfg: Config):
    """Vectorised getP2 (same operation order as the C restatement)."""
    a = 1.0 / ((cfg.gamma_r * cfg.gamma_r) * (gam * gam))
    b = 1.0 + (cfg.aw * cfg.aw) * ((px * px) + (py * py))
    return ((1.0 / np.sqrt(1.0 - a * b)) - 1.0) / cfg.eta


def wrap_z2(cfg: Config, z2: np.ndarray):
    p = cfg.cparams(1, 1)
    lib().or_wrap_z2(ctypes.byref(p), len(z2), _ptr(z2))


# ---------------------------------------------------------------------------
# Diffraction (numpy restatement)
# ---------------------------------------------------------------------------
def _linspace(a, b, n):
    """functions linspace (base_functions.f90:67-98): xstart + i*dx."""
    if n == 1:
        return np.array([a])
    d = (b - a) / float(n - 1)
    return a + np.arange(n) * d


def _mask1d2(x, dx, nx, nb):
    """masks.f90 Mask1D2 (:266-302); ranges applied in the reference's order,
    so overlapping ends keep the second (lower-end) assignment."""
    pi = PUFFIN_PI
    lb = (nb - 1) * dx
    x01, x02 = x[nx - 1], x[0]
    m = np.empty(nx)
    hi = slice(nx - nb, nx)
    m[hi] = np.cos(pi * (x[hi] - x01) / (2.0 * lb)) ** 2
    lo = slice(0, nb)
    m[lo] = np.cos(pi * (x[lo] - x02) / (2.0 * lb)) ** 2
    if nb < nx - nb:
        m[nb:nx - nb] = 0.0
    return m


def _maskf4(x, dx, nx, nb):
    """masks.f90 Maskf4 (:329-361)."""
    pi = PUFFIN_PI
    lb = (nb - 1) * dx
    x01, x02 = x[nx - nb], x[nb - 1]
    m = np.empty(nx)
    hi = slice(nx - nb, nx)
    m[hi] = np.cos(pi * (x[hi] - x01) / (2.0 * lb)) ** 2
    lo = slice(0, nb)
    m[lo] = np.cos(pi * (x[lo] - x02) / (2.0 * lb)) ** 2
    if nb < nx - nb:
        m[nb:nx - nb] = 1.0
    return m


def transverse_mask(cfg: Config):
    """getMask + Mask2D (masks.f90:50-189): mask(ix, iy) as a (ny, nx) array."""
    lenx = (cfg.nx - 1) * cfg.dx
    leny = (cfg.ny - 1) * cfg.dy
    x = _linspace(-lenx / 2, lenx / 2, cfg.nx)
    y = _linspace(-leny / 2, leny / 2, cfg.ny)
    maskx = _mask1d2(x, cfg.dx, cfg.nx, cfg.nbx)
    masky = _mask1d2(y, cfg.dy, cfg.ny, cfg.nby)
    maskx2 = _maskf4(x, cfg.dx, cfg.nx, cfg.nbx)
    masky2 = np.ones(cfg.ny)
    return masky2[:, None] * maskx[None, :] + maskx2[None, :] * masky[:, None]


def z2_mask(cfg: Config):
    """getZ2Mask (masks.f90:366-430), including its Lf = (nx - 1*dx) form;
    zero on the periodic mesh (diffraction.f90:447)."""
    n = cfg.nplanes
    if cfg.mesh_type == MESH_PERIODIC:
        return np.zeros(n)
    pi = PUFFIN_PI
    dx, nx, nb = cfg.dz2, cfg.nz2, cfg.nbz2
    x = _linspace(0.0 * dx, float(n - 1) * dx, n)
    lb = (nb - 1) * dx
    lf = (nx - 1 * dx)
    x0 = lf - lb / 2.0
    fbn = nx - nb + 1
    m = np.zeros(n)
    ind = np.arange(1, n + 1)
    sel = ind >= fbn
    m[sel] = np.cos(pi * (x[sel] - x0) / lb) ** 2
    return m


def k_values(cfg: Config):
    """GetKValues (transforms.f90:472-590); note the local full-precision pi."""
    pi = 4.0 * math.atan(1.0)
    lx = float(cfg.nx) * cfg.dx
    ly = float(cfg.ny) * cfg.dy
    n = cfg.nplanes
    lz = float(n) * cfg.dz2

    def idx(m):
        mx = math.ceil(float(m) / 2.0)
        i = np.arange(m)
        return np.where(i >= mx, i - m, i).astype(np.float64)

    kx = 2.0 * pi * idx(cfg.nx) / lx
    ky = 2.0 * pi * idx(cfg.ny) / ly
    kz = 2.0 * pi * idx(n) / lz
    return kx, ky, kz


def filter_cutoff(cfg: Config):
    """MultiplyExp cutoff (diffraction.f90:138-139) with sFilt from
    setup_calcs.f90:208-210 (Lenz2 = dz2 * NZ2, lambda_r = 4*pi*rho)."""
    lenz2 = cfg.dz2 * cfg.nz2
    sfilt = lenz2 / (4 * PUFFIN_PI * cfg.rho) * cfg.sfilt_frac
    cutoff = 2.0 * PUFFIN_PI * sfilt / (float(cfg.nz2) * cfg.dz2)
    if cfg.mesh_type == MESH_PERIODIC and cfg.sperwaves <= 1.1:
        cutoff = 0.0
    return cutoff


def ffact(cfg: Config):
    return float(cfg.nx) * float(cfg.ny) * float(cfg.nplanes)


def diffract(cfg: Config, re: np.ndarray, im: np.ndarray, h: float, fft=None):
    """DiffractionStep + AbsorptionStep on the outer mesh, in place.

    re/im are flat outer-mesh arrays of nx*ny*nz2 values, x fastest.  ``fft``
    may supply fftn/ifftn with numpy.fft's semantics (default numpy.fft)."""
    fft = np.fft if fft is None else fft
    n = cfg.nplanes
    R = re.reshape(cfg.nz2, cfg.ny, cfg.nx)
    I = im.reshape(cfg.nz2, cfg.ny, cfg.nx)
    A = R[:n] + 1j * I[:n]
    kx, ky, kz = k_values(cfg)
    ff = ffact(cfg)
    cutoff = filter_cutoff(cfg)
    # forward FFTW transform is the unnormalised e^{-i...} sum
    A = fft.fftn(A)
    k2 = (kx[None, None, :] ** 2 + ky[None, :, None] ** 2)
    pass_band = (kz > cutoff) | (kz < -cutoff)
    nz = kz != 0.0
    with np.errstate(divide="ignore", invalid="ignore"):
        theta = h * k2 / (2.0 * kz[:, None, None])
        prop = np.exp(1j * theta)
    use = (pass_band & nz)[:, None, None]
    A = np.where(use, prop * A, A)
    if cfg.qfilter:
        A = np.where((~pass_band)[:, None, None], 0.0, A)
    A = fft.ifftn(A) * (A.size) / ff      # unnormalised backward, then /ffact
    # AbsorptionStep
    mask = transverse_mask(cfg)[None, :, :]
    mz = z2_mask(cfg)[:, None, None]
    m = mask + mz * (1.0 - mask)
    anb = (1.0 - m) * A
    A = m * A
    A = fft.fftn(A)
    with np.errstate(divide="ignore", invalid="ignore"):
        damp = np.exp(-h * cfg.sbeta * (np.abs(kx)[None, None, :] + np.abs(ky)[None, :, None])
                      / np.sqrt(np.abs(2.0 * kz))[:, None, None])
    A = np.where(nz[:, None, None], damp * A, A)
    A = fft.ifftn(A) * (A.size) / ff
    A = A + anb
    R[:n] = A.real
    I[:n] = A.imag
    if cfg.mesh_type == MESH_PERIODIC:
        R[n] = R[0]
        I[n] = I[0]


# ---------------------------------------------------------------------------
# Split-step schedule (UndSection, undulator.f90:106-331), without writes.
# ---------------------------------------------------------------------------
@dataclass
class RunResult:
    steps: int
    status: int
    retries: int = 0
    power: list = field(default_factory=list)
    csteps: int = 0
    window: tuple = (0, 0)


def undulator_run(cfg: Config, beam: Beam, re: np.ndarray, im: np.ndarray,
                  h: float, nsteps: int, isteps4diff: int, qdiffraction: bool,
                  redist_every: int = 60, taper: Taper | None = None,
                  nix: int | None = None, niy: int | None = None,
                  on_step=None, csteps0: int = 0) -> RunResult:
    """Drive rk4_step + diffract like UndSection: a first half diffraction
    step, merged half steps between RK4 blocks, periodic z2 wraps whenever the
    cumulative step count (iCsteps, starting from ``csteps0``) is a multiple of
    ``redist_every`` (undulator.f90:325), and up to 3 retries with a
    recomputed inner window when a particle leaves it."""
    taper = taper or Taper(cfg.n2col0, cfg.n2col0, cfg.undgrad)
    if nix is None:
        nix, niy = get_in_node(cfg, beam.x, beam.y)
    szl = 0.0
    if qdiffraction:
        dzds = float(isteps4diff) * h / 2.0
        diffract(cfg, re, im, dzds)
    wr, wi = outer_to_inner(cfg, re, im, nix, niy)
    retries = 0
    for istep in range(1, nsteps + 1):
        for attempt in range(4):
            t_before = Taper(taper.n2col, taper.n2col0, taper.undgrad)
            st = rk4_step(cfg, taper, szl, h, beam, wr, wi, nix, niy)
            if st == 0:
                break
            if st & 2:
                return RunResult(istep - 1, st, retries)
            taper.n2col, taper.n2col0 = t_before.n2col, t_before.n2col0
            retries += 1
            inner_to_outer(cfg, re, im, wr, wi, nix, niy)
            nix, niy = get_in_node(cfg, beam.x, beam.y)
            wrap_z2(cfg, beam.z2)
            wr, wi = outer_to_inner(cfg, re, im, nix, niy)
        else:
            return RunResult(istep - 1, st, retries, csteps=csteps0 + istep - 1,
                             window=(nix, niy))
        szl = szl + h
        if qdiffraction and (istep % isteps4diff == 0 or istep == nsteps):
            inner_to_outer(cfg, re, im, wr, wi, nix, niy)
            dzdf = dzds
            if istep == nsteps:
                dzds = 0.0
            elif istep + isteps4diff <= nsteps:
                dzds = float(isteps4diff) * h / 2
            else:
                dzds = float(nsteps - istep) * h / 2
            diffract(cfg, re, im, dzdf + dzds)
            wr, wi = outer_to_inner(cfg, re, im, nix, niy)
        if on_step is not None:
            on_step(istep, beam, wr, wi, nix, niy)
        if (csteps0 + istep) % redist_every == 0:
            wrap_z2(cfg, beam.z2)
    inner_to_outer(cfg, re, im, wr, wi, nix, niy)
    return RunResult(nsteps, 0, retries, csteps=csteps0 + nsteps, window=(nix, niy))


# ---------------------------------------------------------------------------
# Undulator entry/exit matching (acc_lattice.f90:601-846, init_conds.f90:70-203)
# ---------------------------------------------------------------------------
def _x_offset(cfg: Config, gamma_j, px, py, n2col, sz0):
    """xOffSet_Array (init_conds.f90:70-102): nc = aw**2."""
    nc = cfg.aw ** 2
    return -(cfg.fy * 4.0 * cfg.kappa * cfg.rho ** 2 / math.sqrt(cfg.eta)
             * (cfg.gamma_r / np.sqrt(gamma_j * gamma_j - (1.0 + nc * (px * px + py * py))))
             * n2col * math.sin(sz0 / (2.0 * cfg.rho)))


def _y_offset(cfg: Config, gamma_j, px, py, n2col, sz0):
    """yOffSet_Array (init_conds.f90:149-183): nc = 2 aw**2 / (ux**2 + uy**2)."""
    nc = 2.0 * cfg.aw ** 2 / (cfg.fx ** 2 + cfg.fy ** 2)
    return (cfg.fx * 4.0 * cfg.kappa * cfg.rho ** 2 / math.sqrt(cfg.eta)
            * (cfg.gamma_r / np.sqrt(gamma_j * gamma_j - (1.0 + nc * (px * px + py * py))))
            * n2col * math.cos(sz0 / (2.0 * cfg.rho)))


def _p_offsets(cfg: Config, beam: Beam, sz, n2col):
    pxo = -(cfg.fy * n2col * math.cos(sz / (2.0 * cfg.rho)))
    pyo = -(cfg.fx * n2col * math.sin(sz / (2.0 * cfg.rho)))
    n = beam.n
    if cfg.und_type == UND_CURVED:
        kx, ky = cfg.kx_und, cfg.ky_und
        spx = pxo - 0.5 * kx ** 2 * beam.x ** 2 - 0.5 * ky ** 2 * beam.y ** 2
        spy = -1.0 * (pyo - kx ** 2 * beam.x * beam.y)
    elif cfg.und_type == UND_PLANEPOLE:
        spx = pxo - 0.5 * (cfg.eta / (4 * cfg.rho ** 2)) * beam.x ** 2
        spy = np.full(n, -1.0 * pyo)
    else:
        spx = np.full(n, pxo)
        spy = np.full(n, -1.0 * pyo)
    return spx, spy


def match_in(cfg: Config, beam: Beam, sz: float, n2col: float):
    """matchIn (acc_lattice.f90:743-846)."""
    spx, spy = _p_offsets(cfg, beam, sz, n2col)
    gj = cfg.gamma_r * beam.gam
    sxo = _x_offset(cfg, gj, spx, -spy, n2col, sz)
    syo = _y_offset(cfg, gj, spx, -spy, n2col, sz)
    beam.x[:] = beam.x + sxo
    beam.y[:] = beam.y + syo
    beam.px[:] = beam.px + spx
    beam.py[:] = beam.py + spy


def match_out(cfg: Config, beam: Beam, sz: float, n2col: float):
    """matchOut (acc_lattice.f90:638-741)."""
    spx, spy = _p_offsets(cfg, beam, sz, n2col)
    gj = cfg.gamma_r * beam.gam
    sxo = _x_offset(cfg, gj, spx, spy, n2col, sz)
    syo = _y_offset(cfg, gj, spx, spy, n2col, sz)
    beam.x[:] = beam.x - sxo
    beam.y[:] = beam.y - syo
    beam.px[:] = beam.px - spx
    beam.py[:] = beam.py - spy


def correct_trans(beam: Beam):
    """correctTrans (acc_lattice.f90:601-636): remove chi-weighted means."""
    w = beam.chi
    ws = np.sum(w)
    mpx = np.sum(w * beam.px) / ws
    mpy = np.sum(w * beam.py) / ws
    mx = np.sum(w * beam.x) / ws
    my = np.sum(w * beam.y) / ws
    beam.px[:] -= mpx
    beam.py[:] -= mpy
    beam.x[:] -= mx
    beam.y[:] -= my


# ---------------------------------------------------------------------------
# Diagnostics (puffin/lib/io/av_write.f90, write_adapter.f90:110-112,
# utilities/pyPlotting/plotSpecPow.py:58-110)
# ---------------------------------------------------------------------------
def _trapz_f32(x, y):
    """m_trapz: a default-real (single precision) accumulator updated with a
    double-precision term each step."""
    acc = np.float32(0.0)
    for i in range(len(x) - 1):
        acc = np.float32(float(acc) + (x[i + 1] - x[i]) * (y[i + 1] + y[i]) / 2.0)
    return float(acc)


def power(cfg: Config, re, im):
    """gPower: fPower_1D (|A|^2) or fPower_3D (2D trapezoid) per z2 plane."""
    R = re.reshape(cfg.nz2, cfg.ny, cfg.nx)
    I = im.reshape(cfg.nz2, cfg.ny, cfg.nx)
    inten = R * R + I * I
    if cfg.nx == 1 and cfg.ny == 1:
        return inten.reshape(cfg.nz2).copy()
    lx, ly = cfg.dx * (cfg.nx - 1), cfg.dy * (cfg.ny - 1)
    xa = _linspace(-lx / 2.0, lx / 2.0, cfg.nx)
    ya = _linspace(-ly / 2.0, ly / 2.0, cfg.ny)
    out = np.empty(cfg.nz2)
    for z in range(cfg.nz2):
        cul = np.array([_trapz_f32(xa, inten[z, iy]) for iy in range(cfg.ny)])
        out[z] = _trapz_f32(ya, cul)
    return out


def num_slices(cfg: Config):
    pi = PUFFIN_PI
    if cfg.mesh_type == MESH_TEMPORAL:
        return math.ceil((cfg.dz2 * cfg.nz2) / (4 * pi * cfg.rho))
    return math.ceil((cfg.dz2 * float(cfg.nz2 - 1)) / (4 * pi * cfg.rho))


def bunching(cfg: Config, z2, chi, harmonic=1):
    """|b_m| per slice as getSliceTwiss (av_write.f90:500-650, 700-770)."""
    ns = num_slices(cfg)
    S = 4 * PUFFIN_PI * cfg.rho
    br = np.zeros(ns + 1)
    bi = np.zeros(ns + 1)
    sd = np.zeros(ns + 1)
    periodic = cfg.mesh_type == MESH_PERIODIC
    for z, c in zip(z2, chi):
        s = math.ceil(z / S)
        if periodic:
            if s >= ns:
                s = s - math.floor(float(s) / float(ns)) * ns + 1
            if s < 1:
                raise ValueError("slice index out of bounds")
        elif s > ns or s < 1:
            raise ValueError("slice index out of bounds")
        ph = float(harmonic) * z / (2.0 * cfg.rho)
        w0 = (s * S - z) / S
        sd[s - 1] += c
        br[s - 1] += c * math.cos(ph) * w0
        bi[s - 1] += c * math.sin(ph) * w0
        if not periodic:
            w1 = -((s - 1) * S - z) / S
            br[s] += c * math.cos(ph) * w1
            bi[s] += c * math.sin(ph) * w1
    return np.where(sd[:ns] > 0, np.sqrt(br[:ns] ** 2 + bi[:ns] ** 2) / S, 0.0)


def spectrum(cfg: Config, re, im):
    """One-sided |FFT|^2 of the on-axis x (re) and y (im) field along z2."""
    R = re.reshape(cfg.nz2, cfg.ny, cfg.nx)[:, (cfg.ny - 1) // 2, (cfg.nx - 1) // 2]
    I = im.reshape(cfg.nz2, cfg.ny, cfg.nx)[:, (cfg.ny - 1) // 2, (cfg.nx - 1) // 2]
    n = cfg.nz2
    nu = int(np.ceil((n + 1) / 2))
    out = []
    for f in (R, I):
        p = np.abs(np.fft.fft(f, n=n)[:nu]) ** 2
        if n % 2 == 1:
            p[1:] *= 2
        else:
            p[1:-1] *= 2
        out.append(p)
    return out[0], out[1]


# ---------------------------------------------------------------------------
# Beam-line elements (puffin/lib/acc_lattice.f90) and the element loop
# (puffin/lib/puffin_module.f90:57-89)
# ---------------------------------------------------------------------------
def drift(cfg: Config, beam: Beam, dz: float):
    """driftSection (acc_lattice.f90:478-518), particle part."""
    sp2 = p2(beam.gam, beam.px, beam.py, cfg)
    beam.z2[:] = beam.z2 + dz * sp2
    if not cfg.one_d:
        c = 2 * cfg.rho * cfg.kappa / math.sqrt(cfg.eta)
        beam.x[:] = beam.x + (c * (1 + cfg.eta * sp2) / beam.gam * beam.px) * dz
        beam.y[:] = beam.y - (c * (1 + cfg.eta * sp2) / beam.gam * beam.py) * dz


def chicane(cfg: Config, beam: Beam, disp: float, slip: float):
    """disperse (acc_lattice.f90:420-463), particle part before the wrap."""
    beam.z2[:] = beam.z2 - 2.0 * disp * (beam.gam - 1.0) + slip


def quad(cfg: Config, beam: Beam, qfx: float, qfy: float):
    """Quad (acc_lattice.f90:531-561)."""
    if cfg.one_d:
        return
    c = math.sqrt(cfg.eta) / (2 * cfg.rho * cfg.kappa)
    beam.px[:] = beam.px + c * beam.x / qfx
    beam.py[:] = beam.py - c * beam.y / qfy


def modulation(beam: Beam, mag: float, k: float):
    """bModulation (acc_lattice.f90:575-585)."""
    beam.gam[:] = beam.gam + (mag * np.cos(k * beam.z2))


def init_undulator(cfg: Config, taper: Taper, und_type, fx, fy, kbxsf, kbysf, mf, grad,
                   nsteps, hstep, und_ends):
    """initUndulator (acc_lattice.f90:848-895)."""
    taper.n2col0 = mf
    taper.n2col = mf
    taper.undgrad = grad
    cfg.n2col0, cfg.undgrad = mf, grad
    cfg.und_type, cfg.fx, cfg.fy, cfg.kbxsf, cfg.kbysf = und_type, fx, fy, kbxsf, kbysf
    cfg.und_ends = bool(und_ends)
    if und_ends:
        cfg.szfs = 4.0 * PUFFIN_PI * cfg.rho * 2.0
        cfg.szfe = nsteps * hstep - 4.0 * PUFFIN_PI * cfg.rho * 2.0
    else:
        cfg.szfs = 0.0
        cfg.szfe = nsteps * hstep


def run_lattice(cfg: Config, beam: Beam, re, im, elements, qdiffraction=True,
                redist_every=60, sz=0.0):
    """The element loop of puffin_module.f90:57-89 over undulator, quad,
    chicane, drift and modulation elements (tuples as in
    puffin_gb300.lattice).  Returns (sz, csteps)."""
    taper = Taper(cfg.n2col0, cfg.n2col0, cfg.undgrad)
    csteps = 0
    # the inner window is set once (setup_calcs.f90:1292) and recomputed only
    # when a particle leaves it
    nix, niy = get_in_node(cfg, beam.x, beam.y)
    for el in elements:
        kind = el[0]
        if kind == "undulator":
            (_, und_type, fx, fy, kbxsf, kbysf, mf, grad, nsteps, h, isteps4diff) = el
            init_undulator(cfg, taper, und_type, fx, fy, kbxsf, kbysf, mf, grad, nsteps, h,
                           cfg.und_ends)
            sz0 = sz
            if not cfg.und_ends:
                match_in(cfg, beam, 0.0, taper.n2col)
            wrap_z2(cfg, beam.z2)     # getLocalFieldIndices (undulator.f90:102)
            r = undulator_run(cfg, beam, re, im, h, nsteps, isteps4diff, qdiffraction,
                              redist_every, taper, nix=nix, niy=niy, csteps0=csteps)
            if r.status:
                raise RuntimeError(f"undulator run failed with status {r.status}")
            csteps = r.csteps
            nix, niy = r.window
            szl = 0.0
            for _ in range(nsteps):
                szl = szl + h
            sz = sz0 + szl
            if not cfg.und_ends:
                match_out(cfg, beam, sz, taper.n2col)
            correct_trans(beam)
        elif kind == "quad":
            quad(cfg, beam, el[1], el[2])
        elif kind == "chicane":
            _, zbar, disp, slip = el
            chicane(cfg, beam, disp, slip)
            if qdiffraction and zbar > 0.0:
                diffract(cfg, re, im, zbar)
            sz = sz + zbar
            if cfg.mesh_type == MESH_PERIODIC:
                wrap_z2(cfg, beam.z2)
        elif kind == "drift":
            dz = el[1]
            drift(cfg, beam, dz)
            if qdiffraction:
                diffract(cfg, re, im, dz)
            sz = sz + dz
        elif kind == "modulation":
            modulation(beam, el[1], el[2])
        else:
            raise ValueError(kind)
    return sz, csteps


# ---------------------------------------------------------------------------
# Quiet-start beam (mp_sequences.f90:126-433, MPfDists.f90:406-620,
# noise.f90:25-80) with the library's seeded counter-based generator
# ---------------------------------------------------------------------------
def halton(ind: int, base: int) -> float:
    """halton (mp_sequences.f90:286-305)."""
    ft, y, it = 1.0, 0.0, ind
    while it > 0:
        ft = ft / float(base)
        y = y + ft * float(it % base)
        it = it // base
    return y


def project_gauss(seq):
    """projectRSeq + interp1 (mp_sequences.f90:318-433)."""
    n = 2000
    d = (4.0 - (-4.0)) / float(n - 1)
    yf = [-4.0 + i * d for i in range(n)]
    cdf = [0.5 * (1.0 + math.erf(v / math.sqrt(2.0))) for v in yf]
    out = []
    for v in seq:
        if cdf[0] < v < cdf[n - 1]:
            ic = 0
            while v > cdf[ic]:
                ic += 1
            ifl, ifu = ic, ic + 1
            dx = cdf[ifu] - cdf[ifl]
            locx = v - cdf[ifl]
            r = yf[ifl] * (1.0 - locx / dx)
            r = r + yf[ifu] * locx / dx
        elif v <= cdf[0]:
            r = yf[0]
        else:
            r = yf[n - 1]
        out.append(r)
    return np.array(out)


_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def _mix64(z):
    with np.errstate(over="ignore"):
        z = (z + np.uint64(0x9E3779B97F4A7C15)) & _M64
        z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & _M64
        z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & _M64
        return z ^ (z >> np.uint64(31))


def _uniform01(seed, i, d):
    with np.errstate(over="ignore"):
        k = (np.asarray(i, dtype=np.uint64) * np.uint64(64) + np.uint64(d)) & _M64
        r = _mix64(np.uint64(seed) ^ _mix64(k))
    return ((r >> np.uint64(11)).astype(np.float64) + 0.5) * (1.0 / 9007199254740992.0)


def generate_beam(z2m, ne, dz2, nseq, mean, sig, noise, seed, chi_per_electron):
    """Beamlets per slice from the Halton sequences of bases 2, 3, 5, 11, 7
    (Gaussian) and 13 (z2), with Poisson shot noise; returns a Beam."""
    z2m = np.asarray(z2m, dtype=np.float64)
    ne = np.asarray(ne, dtype=np.float64)
    ns = len(z2m)
    mean = np.broadcast_to(np.asarray(mean, dtype=np.float64), (ns, 5))
    sig = np.broadcast_to(np.asarray(sig, dtype=np.float64), (ns, 5))
    bases = (2, 3, 5, 11, 7, 13)
    seq = []
    for d, b in enumerate(bases):
        v = [halton(j + 1, b) for j in range(nseq)]
        seq.append(project_gauss(v) if d < 5 else (np.array(v) - 0.5) * dz2)
    n = ns * nseq
    i = np.arange(n)
    k = i // nseq
    j = i - k * nseq
    cols = [seq[d][j] * sig[k, d] + mean[k, d] for d in range(5)]
    z = seq[5][j] + z2m[k]
    nk = ne[k] / float(nseq)
    if noise:
        pk = np.empty(n)
        small = nk < 12.0
        # Knuth's product method below a mean of 12
        for t in np.nonzero(small)[0]:
            L = math.exp(-nk[t])
            p, c = 1.0, 0
            for it in range(60):
                p *= float(_uniform01(seed, t, 2 + it))
                if p <= L:
                    break
                c += 1
            pk[t] = c
        big = ~small
        u1 = _uniform01(seed, i[big], 0)
        u2 = _uniform01(seed, i[big], 1)
        g = np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * math.pi * u2)
        pk[big] = np.floor(nk[big] + np.sqrt(nk[big]) * g + 0.5)
        moved = pk > 0.0
        nk = np.where(moved, pk, nk)
        u = _uniform01(seed, i, 63)
        z = np.where(moved, z + (u - 0.5) * dz2 / np.sqrt(nk), z)
    return Beam(cols[0], cols[1], z, cols[2], cols[3], cols[4], nk * chi_per_electron)


# ---------------------------------------------------------------------------
# Known-answer formulas of the reference (puffin/lib/utilities/base_functions.f90),
# pinned by its own unit tests (test/testFFunctions.pf), and the linear FEL
# theory that the scaled units are built on.  The GPU tests compare a seed
# propagated through the diffraction step and the exponential gain of cold
# beams against them.
# ---------------------------------------------------------------------------
def gain_length(lam_w: float, rho: float) -> float:
    """GainLength (base_functions.f90:448-462): the gain length
    l_g = lambda_w / (4 pi rho) that scales zbar = z / l_g, with the
    module's single-precision pi (puffin_constants.f90:22)."""
    return lam_w / (4.0 * PUFFIN_PI * rho)


def raleigh_length(rho: float, sigma: float) -> float:
    """RaleighLength (base_functions.f90:514-525): sigma^2 / (2 rho), the
    Rayleigh range in zbar of a seed whose field amplitude is
    exp(-x^2 / (2 sigma^2)) (the gaussian() envelope of getSeed,
    setup_calcs.f90:1507-1514)."""
    return sigma ** 2 / (2.0 * rho)


def diffraction_length(z: float, zr: float, sigma: float) -> float:
    """DiffractionLength (base_functions.f90:489-507):
    sqrt(2 ((z / zR)^2 + 1)) 6 sigma, a transverse extent that grows with z as
    the width of a Gaussian beam, sqrt(1 + (z / zR)^2)."""
    return math.sqrt(2.0 * ((z / zr) ** 2 + 1.0)) * 6.0 * sigma


def cold_beam_power_growth(nodes_per_wavelength: int) -> float:
    """e-foldings of the radiated power per unit zbar of a cold, resonant beam
    in the exponential regime: sqrt(3) in the 1D high-gain theory (field
    amplitude exp(sqrt(3)/2 zbar); so the power gain length is
    gain_length / sqrt(3)), times the attenuation of linear (trilinear)
    interpolation on a mesh of n nodes per resonant wavelength: gather and
    deposit each multiply the coupling at the resonant wavenumber by
    sinc^2(pi / n), and the growth rate goes as the coupling to the 1/3."""
    x = math.pi / nodes_per_wavelength
    return math.sqrt(3.0) * (math.sin(x) / x) ** (4.0 / 3.0)
