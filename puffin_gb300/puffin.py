"""Host-side mirror of Puffin's hot-path interface over the puffgpu C ABI.

``Puffin`` holds one undulator module's particles and field on the GPU and
exposes the reference's operations under their own names:

* ``rk4par(szl, h)``        rk4par (puffin/lib/interaction/puffin_mpi_RK4.f90:38)
* ``diffractIM(dz)``         inner2Outer + diffractIM + outer2Inner
                             (puffin/lib/diffraction/diffraction.f90:46)
* ``redistribute()``         getInNode + getLocalFieldIndices
                             (puffin/lib/parallel/para_field.f90:1432, 83)
* ``und_section(...)``       the RK4/diffraction loop of UndSection
                             (puffin/lib/undulator.f90:182-333)

Error behaviour follows the reference: a particle leaving the inner window
makes ``rk4par`` return False with the state unchanged (qPArrOK_G = .false.),
and the conditions where the reference STOPs raise ``PuffinError``.
Arrays are numpy float64 on the host, or CUDA torch tensors (float64,
contiguous) which are used in place on the device.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import lib as L

PARTICLE_KEYS = ("x", "y", "z2", "px", "py", "gam", "chi")


class PuffinError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{L.STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


def _is_torch_cuda(a):
    return hasattr(a, "is_cuda") and a.is_cuda


def _host(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a, a.ctypes.data


def _dev(t):
    import torch
    if t.dtype != torch.float64 or not t.is_contiguous():
        raise ValueError("device arrays must be contiguous float64 CUDA tensors")
    return t, t.data_ptr()


class Puffin:
    def __init__(self, params: L.Params | None = None, **overrides):
        self._lib = L.load()
        p = L.default_params() if params is None else params
        for k, v in overrides.items():
            setattr(p, k, v)
        self.params = p
        h = ctypes.c_void_p()
        rc = self._lib.pf_create(ctypes.byref(p), ctypes.byref(h))
        if rc != L.PF_OK:
            raise PuffinError(rc, self._lib.pf_last_error(None).decode())
        self._h = h
        self.n_outer = p.nx * p.ny * p.nz2

    # -- life cycle -----------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None):
            self._lib.pf_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, rc, allow=()):
        if rc == L.PF_OK or rc in allow:
            return rc
        raise PuffinError(rc, self._lib.pf_last_error(self._h).decode())

    # -- particles --------------------------------------------------------------
    def set_particles(self, x, y, z2, px, py, gam, chi=None):
        """chi=None keeps the handle's chi (same macroparticle count)."""
        arrs = [x, y, z2, px, py, gam] + ([] if chi is None else [chi])
        if all(_is_torch_cuda(a) for a in arrs):
            keep = [_dev(a) for a in arrs]
            fn = self._lib.pf_set_particles_dev
        else:
            keep = [_host(a) for a in arrs]
            fn = self._lib.pf_set_particles
        n = len(keep[0][0])
        if any(len(k[0]) != n for k in keep):
            raise ValueError("particle arrays differ in length")
        ptrs = [k[1] for k in keep] + ([None] if chi is None else [])
        self._check(fn(self._h, n, *ptrs))

    @property
    def n_particles(self):
        return int(self._lib.pf_num_particles(self._h))

    def get_particles(self, out=None):
        n = self.n_particles
        if out is not None and all(_is_torch_cuda(out[k]) for k in PARTICLE_KEYS):
            self._check(self._lib.pf_get_particles_dev(
                self._h, *(_dev(out[k])[1] for k in PARTICLE_KEYS)))
            return out
        res = {k: np.empty(n) for k in PARTICLE_KEYS}
        self._check(self._lib.pf_get_particles(
            self._h, *(res[k].ctypes.data for k in PARTICLE_KEYS)))
        return res

    # -- field ----------------------------------------------------------------
    def set_field(self, re, im):
        if _is_torch_cuda(re) and _is_torch_cuda(im):
            (re, pr), (im, pi) = _dev(re), _dev(im)
            fn = self._lib.pf_set_field_dev
        else:
            (re, pr), (im, pi) = _host(re), _host(im)
            fn = self._lib.pf_set_field
        if re.size != self.n_outer or im.size != self.n_outer:
            raise ValueError(f"field arrays must hold nx*ny*nz2 = {self.n_outer} values")
        self._check(fn(self._h, pr, pi))

    def get_field(self, out=None):
        if out is not None and _is_torch_cuda(out[0]):
            self._check(self._lib.pf_get_field_dev(self._h, _dev(out[0])[1], _dev(out[1])[1]))
            return out
        re = np.empty(self.n_outer)
        im = np.empty(self.n_outer)
        self._check(self._lib.pf_get_field(self._h, re.ctypes.data, im.ctypes.data))
        return re, im

    @property
    def n_window(self) -> int:
        """Values per array of the inner-window field (nix * niy * planes)."""
        return int(self._lib.pf_window_nodes(self._h))

    def set_window_field(self, re, im):
        """Replace the inner-window field that the next rk4par advances
        (ac_rfield_in / ac_ifield_in; outer2Inner's layout, x fastest)."""
        if _is_torch_cuda(re) and _is_torch_cuda(im):
            (re, pr), (im, pi) = _dev(re), _dev(im)
            fn = self._lib.pf_set_window_field_dev
        else:
            (re, pr), (im, pi) = _host(re), _host(im)
            fn = self._lib.pf_set_window_field
        n = self.n_window
        if re.size != n or im.size != n:
            raise ValueError(f"window field arrays must hold nix*niy*planes = {n} values")
        self._check(fn(self._h, pr, pi))

    def get_window_field(self, out=None):
        if out is not None and _is_torch_cuda(out[0]):
            self._check(self._lib.pf_get_window_field_dev(self._h, _dev(out[0])[1],
                                                          _dev(out[1])[1]))
            return out
        n = self.n_window
        re = np.empty(n)
        im = np.empty(n)
        self._check(self._lib.pf_get_window_field(self._h, re.ctypes.data, im.ctypes.data))
        return re, im

    # -- taper / window ---------------------------------------------------------
    def set_taper(self, n2col, n2col0, undgrad):
        self._check(self._lib.pf_set_taper(self._h, n2col, n2col0, undgrad))

    def get_taper(self):
        a, b, c = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        self._check(self._lib.pf_get_taper(self._h, ctypes.byref(a), ctypes.byref(b),
                                           ctypes.byref(c)))
        return a.value, b.value, c.value

    @property
    def window(self):
        a, b = ctypes.c_int32(), ctypes.c_int32()
        self._check(self._lib.pf_get_window(self._h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    # -- the hot path -------------------------------------------------------------
    def rk4par(self, szl: float, h: float) -> bool:
        """One RK4 step; False (state unchanged) if a particle left the window."""
        rc = self._check(self._lib.pf_rk4_step(self._h, float(szl), float(h)),
                         allow=(L.PF_OUT_OF_WINDOW,))
        return rc == L.PF_OK

    rk4_step = rk4par

    def rk4par_host(self, szl: float, h: float, particles: dict, window: tuple) -> bool:
        """One RK4 step on the driver's host arrays (pf_rk4_step_host; FP64
        and mixed handles): the float64 arrays particles["x"] ..
        particles["gam"] and the window field (re, im), advanced in place,
        the copies overlapped with the step.
        False (arrays and state as they came in) if a particle left the
        window or the mesh."""
        arrs = [particles[k] for k in PARTICLE_KEYS[:6]] + list(window)
        for a in arrs:
            if not (isinstance(a, np.ndarray) and a.dtype == np.float64 and a.flags.c_contiguous):
                raise ValueError("rk4par_host takes C-contiguous float64 numpy arrays")
        if any(a.size != self.n_particles for a in arrs[:6]):
            raise ValueError("particle arrays must hold the handle's macroparticles")
        if any(a.size != self.n_window for a in arrs[6:]):
            raise ValueError(f"window field arrays must hold {self.n_window} values")
        rc = self._check(self._lib.pf_rk4_step_host(self._h, float(szl), float(h),
                                                    *[a.ctypes.data for a in arrs]),
                         allow=(L.PF_OUT_OF_WINDOW, L.PF_OUT_OF_Z2))
        return rc == L.PF_OK

    def diffractIM_host(self, dz: float, outer: tuple, window: tuple):
        """inner2Outer + diffractIM + outer2Inner on the driver's host arrays
        (pf_diffract_host; FP64 and mixed handles): the outer field (re, im)
        and the window field (re, im), C-contiguous float64, updated in
        place, their copies overlapped with the transforms by ranges of z2
        planes."""
        arrs = list(outer) + list(window)
        for a in arrs:
            if not (isinstance(a, np.ndarray) and a.dtype == np.float64 and a.flags.c_contiguous):
                raise ValueError("diffractIM_host takes C-contiguous float64 numpy arrays")
        if any(a.size != self.n_outer for a in arrs[:2]):
            raise ValueError(f"outer field arrays must hold {self.n_outer} values")
        if any(a.size != self.n_window for a in arrs[2:]):
            raise ValueError(f"window field arrays must hold {self.n_window} values")
        self._check(self._lib.pf_diffract_host(self._h, float(dz), *[a.ctypes.data for a in arrs]))

    def redistribute(self):
        self._check(self._lib.pf_redistribute(self._h))

    def wrap_z2(self):
        self._check(self._lib.pf_wrap_z2(self._h))

    def diffractIM(self, dz: float):
        self._check(self._lib.pf_diffract(self._h, float(dz)))

    diffract = diffractIM

    def und_section(self, nsteps: int, isteps4diff: int, qdiffraction: bool, h: float,
                    szl: float = 0.0):
        """UndSection's loop; returns the new local zbar."""
        z = ctypes.c_double(szl)
        done = ctypes.c_int32(0)
        self._check(self._lib.pf_run(self._h, int(nsteps), int(isteps4diff),
                                     int(bool(qdiffraction)), float(h), ctypes.byref(z),
                                     ctypes.byref(done)))
        return z.value

    def set_taper_profile(self, z=None, alpha=None):
        """Piecewise-linear alpha(z) through control points (None: the
        module's linear taper)."""
        if z is None:
            self._check(self._lib.pf_set_taper_profile(self._h, 0, None, None))
            return
        z = np.ascontiguousarray(z, dtype=np.float64)
        a = np.ascontiguousarray(alpha, dtype=np.float64)
        if z.shape != a.shape:
            raise ValueError("z and alpha need the same length")
        self._check(self._lib.pf_set_taper_profile(self._h, len(z), z.ctypes.data, a.ctypes.data))

    def set_fft_arithmetic(self, mode: int):
        """FP64 path: diffraction FFTs in FP64 (lib.FFT_FP64) or in paired
        FP32 arithmetic (lib.FFT_PAIRED_FP32; see pf_set_fft_arithmetic)."""
        self._check(self._lib.pf_set_fft_arithmetic(self._h, int(mode)))

    def set_launch_mode(self, mode: int):
        """0 step by step, 1 asynchronous step blocks, 2 blocks as CUDA graphs."""
        self._check(self._lib.pf_set_launch_mode(self._h, int(mode)))

    # -- Puffin dump files ----------------------------------------------------------
    def load_dump(self, particles_path=None, field_path=None):
        """Start from the reference's HDF5 dumps (particle and/or field file);
        returns the resume attributes of the particle file (iCsteps, zbarLocal,
        ...) and sets the cumulative step count from iCsteps."""
        from . import h5dump
        attrs = {}
        if particles_path is not None:
            beam, attrs = h5dump.read_particles(particles_path)
            self.set_particles(*(beam[k] for k in PARTICLE_KEYS))
            if "iCsteps" in attrs:
                self.step_count = int(attrs["iCsteps"])
        if field_path is not None:
            re, im, _, fattrs = h5dump.read_field(field_path)
            self.set_field(re, im)
            attrs = attrs or fattrs
        return attrs

    def save_dump(self, particles_path=None, field_path=None, attrs=None):
        """Write the particles and/or the field in the reference's dump layout."""
        from . import h5dump
        a = dict(attrs or {})
        a.setdefault("iCsteps", self.step_count)
        if particles_path is not None:
            h5dump.write_particles(particles_path, self.get_particles(), a)
        if field_path is not None:
            re, im = self.get_field()
            p = self.params
            h5dump.write_field(field_path, re, im, (p.nx, p.ny, p.nz2), a)

    # -- beam generation ------------------------------------------------------------
    def generate_beam(self, z2m, ne, dz2: float, nseq: int, mean, sig, noise: bool = True,
                      seed: int = 0x5EED, chi_per_electron: float = 1.0):
        """Quiet-start Halton beamlets per z2 slice with shot noise (see
        pf_generate_beam); mean and sig are (nslices, 5) arrays over x, y,
        px, py, gamma (or 5 values for every slice)."""
        z2m = np.ascontiguousarray(z2m, dtype=np.float64)
        ne = np.ascontiguousarray(ne, dtype=np.float64)
        ns = len(z2m)
        m = np.ascontiguousarray(np.broadcast_to(np.asarray(mean, dtype=np.float64), (ns, 5)))
        s = np.ascontiguousarray(np.broadcast_to(np.asarray(sig, dtype=np.float64), (ns, 5)))
        self._check(self._lib.pf_generate_beam(self._h, ns, z2m.ctypes.data, ne.ctypes.data,
                                               float(dz2), int(nseq), m.ctypes.data,
                                               s.ctypes.data, int(bool(noise)),
                                               int(seed) & (2 ** 64 - 1),
                                               float(chi_per_electron)))

    # -- adjoint (pulse-energy gradients) -------------------------------------------
    def adjoint_forward(self, nsteps: int, isteps4diff: int, qdiffraction: bool, h: float,
                        checkpoint_every: int, seed_re, seed_im, seed_amp: float,
                        chirp: float) -> float:
        """Pulse energy after nsteps (see pf_adjoint_forward); keeps the
        checkpoints for adjoint_backward."""
        sr = np.ascontiguousarray(seed_re, dtype=np.float64)
        si = np.ascontiguousarray(seed_im, dtype=np.float64)
        if sr.size != self.n_outer or si.size != self.n_outer:
            raise ValueError("the seed covers the outer mesh")
        e = ctypes.c_double()
        self._check(self._lib.pf_adjoint_forward(self._h, int(nsteps), int(isteps4diff),
                                                 int(bool(qdiffraction)), float(h),
                                                 int(checkpoint_every), sr.ctypes.data,
                                                 si.ctypes.data, float(seed_amp), float(chirp),
                                                 ctypes.byref(e)))
        return e.value

    def diffract_adjoint(self, dz: float, re, im):
        """Adjoint of one diffraction step applied to copies of (re, im)."""
        r = np.array(re, dtype=np.float64)
        i = np.array(im, dtype=np.float64)
        self._check(self._lib.pf_diffract_adjoint(self._h, float(dz), r.ctypes.data, i.ctypes.data))
        return r, i

    def adjoint_backward(self, ntaper: int, denergy: float = 1.0):
        """(dE/d taper profile values, dE/d seed_amp, dE/d chirp) times denergy."""
        g = np.zeros(int(ntaper))
        gs, gc = ctypes.c_double(), ctypes.c_double()
        self._check(self._lib.pf_adjoint_backward(self._h, float(denergy), g.ctypes.data,
                                                  int(ntaper), ctypes.byref(gs), ctypes.byref(gc)))
        return g, gs.value, gc.value

    # -- cumulative step count (iCsteps) -----------------------------------------
    @property
    def step_count(self) -> int:
        return int(self._lib.pf_step_count(self._h))

    @step_count.setter
    def step_count(self, n: int):
        self._check(self._lib.pf_set_step_count(self._h, int(n)))

    # -- beam-line elements (acc_lattice.f90) --------------------------------------
    def drift(self, dz: float, qdiffraction: bool = True):
        """driftSection (acc_lattice.f90:478-518)."""
        self._check(self._lib.pf_drift(self._h, float(dz), int(bool(qdiffraction))))

    def disperse(self, disp: float, slip: float, zbar: float, qdiffraction: bool = True):
        """disperse: a chicane (acc_lattice.f90:420-463)."""
        self._check(self._lib.pf_chicane(self._h, float(disp), float(slip), float(zbar),
                                         int(bool(qdiffraction))))

    def quad(self, qfx: float, qfy: float):
        """Quad point transform (acc_lattice.f90:531-561)."""
        self._check(self._lib.pf_quad(self._h, float(qfx), float(qfy)))

    def modulation(self, mag: float, wavenum: float):
        """bModulation (acc_lattice.f90:575-585)."""
        self._check(self._lib.pf_modulation(self._h, float(mag), float(wavenum)))

    def matchIn(self, sz: float):
        self._check(self._lib.pf_match_in(self._h, float(sz)))

    def matchOut(self, sz: float):
        self._check(self._lib.pf_match_out(self._h, float(sz)))

    def correctTrans(self):
        self._check(self._lib.pf_correct_trans(self._h))

    def init_undulator(self, und_type: int, fx: float, fy: float, kbxsf: float, kbysf: float,
                       mf: float, taper: float, nsteps: int, hstep: float, und_ends: bool):
        """initUndulator (acc_lattice.f90:848-895)."""
        self._check(self._lib.pf_init_undulator(self._h, int(und_type), float(fx), float(fy),
                                                float(kbxsf), float(kbysf), float(mf),
                                                float(taper), int(nsteps), float(hstep),
                                                int(bool(und_ends))))
        for k, v in (("und_type", und_type), ("fx", fx), ("fy", fy), ("kbxsf", kbxsf),
                     ("kbysf", kbysf), ("n2col0", mf), ("undgrad", taper),
                     ("und_ends", int(bool(und_ends)))):
            setattr(self.params, k, v)

    # -- diagnostics ------------------------------------------------------------
    def power(self):
        """Power per z2 plane (fPower_1D / fPower_3D)."""
        out = np.empty(self.params.nz2)
        self._check(self._lib.pf_power(self._h, out.ctypes.data, len(out)))
        return out

    def bunching(self, harmonic: int = 1):
        """|b_m| per resonant-wavelength slice (getSliceTwiss)."""
        n = int(self._lib.pf_num_slices(self._h))
        out = np.empty(n)
        self._check(self._lib.pf_bunching(self._h, int(harmonic), out.ctypes.data, n))
        return out

    def spectrum(self):
        """One-sided on-axis spectrum of the x (re) and y (im) field parts."""
        nu = (self.params.nz2 + 2) // 2
        sx, sy = np.empty(nu), np.empty(nu)
        self._check(self._lib.pf_spectrum(self._h, sx.ctypes.data, sy.ctypes.data, nu))
        return sx, sy

    def sync(self):
        self._check(self._lib.pf_sync(self._h))

    @property
    def kernel_launches(self) -> int:
        return int(self._lib.pf_kernel_launches(self._h))

    @property
    def stream_handle(self) -> int:
        """cudaStream_t of the handle (wrap with torch.cuda.ExternalStream)."""
        return int(self._lib.pf_get_stream(self._h) or 0)

    def profile(self, enable: bool = True):
        self._check(self._lib.pf_profile(self._h, int(enable)))

    def profile_read(self, kernel_class: int):
        ms = ctypes.c_double()
        n = ctypes.c_int64()
        self._check(self._lib.pf_profile_read(self._h, int(kernel_class), ctypes.byref(ms),
                                              ctypes.byref(n)))
        return ms.value, n.value


def rk4_step_noalloc(params, taper, szl, h, particles, wr, wi, nix, niy, stream=None):
    """One RK4 step through pf_rk4_step_noalloc, for callers that cannot
    allocate device memory (their device memory belongs to another allocator,
    or they must avoid cudaMalloc's implicit synchronisation): the caller's
    CUDA float64 tensors are updated in place and the library's temporaries
    come from its fixed-size static device array (at most
    NOALLOC_MAX_PARTICLES macroparticles and NOALLOC_MAX_NODES window nodes).
    ``taper`` is a two-element list [n2col, n2col0], updated in place.
    Returns True, or False (state unchanged) if a particle left the window."""
    lib = L.load()
    n2c = ctypes.c_double(taper[0])
    n2c0 = ctypes.c_double(taper[1])
    ptrs = [_dev(particles[k])[1] for k in PARTICLE_KEYS]
    np_ = len(particles["x"])
    rc = lib.pf_rk4_step_noalloc(ctypes.byref(params), ctypes.byref(n2c), ctypes.byref(n2c0),
                                 float(szl), float(h), np_, *ptrs, _dev(wr)[1], _dev(wi)[1],
                                 int(nix), int(niy), stream)
    taper[0], taper[1] = n2c.value, n2c0.value
    if rc == L.PF_OUT_OF_WINDOW:
        return False
    if rc != L.PF_OK:
        raise PuffinError(rc, "pf_rk4_step_noalloc failed")
    return True
