"""ctypes binding of libpuffgpu.so (the C ABI declared in include/puffgpu.h).

The library is the only compute path: there is no CPU fallback.  Loading
fails loudly when the shared library has not been built.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import _build

PF_OK, PF_OUT_OF_WINDOW, PF_OUT_OF_Z2, PF_BAD_ARG, PF_CUDA_ERR, PF_TIMEOUT, \
    PF_NO_DEVICE, PF_OVERFLOW, PF_STATE, PF_NOT_FINITE = range(10)
STATUS_NAMES = {
    PF_OK: "PF_OK", PF_OUT_OF_WINDOW: "PF_OUT_OF_WINDOW", PF_OUT_OF_Z2: "PF_OUT_OF_Z2",
    PF_BAD_ARG: "PF_BAD_ARG", PF_CUDA_ERR: "PF_CUDA_ERR", PF_TIMEOUT: "PF_TIMEOUT",
    PF_NO_DEVICE: "PF_NO_DEVICE", PF_OVERFLOW: "PF_OVERFLOW", PF_STATE: "PF_STATE",
    PF_NOT_FINITE: "PF_NOT_FINITE",
}
UND_PUFFIN, UND_HELICAL, UND_PLANEPOLE, UND_CURVED = 0, 1, 2, 3
MESH_TEMPORAL, MESH_PERIODIC = 0, 1
FP64, MIXED = 0, 1
FFT_FP64, FFT_PAIRED_FP32 = 0, 1

_DOUBLES = ("rho", "eta", "kappa", "aw", "gamma_r", "fx", "fy", "kx_und", "ky_und",
            "kbxsf", "kbysf", "szfs", "szfe", "n2col0", "undgrad", "dx", "dy", "dz2",
            "sbeta", "sfilt_frac", "sperwaves")
_INTS = ("und_type", "mesh_type", "nx", "ny", "nz2", "nix", "niy", "nbx", "nby", "nbz2",
         "one_d", "focusing", "und_ends", "field_evolve", "electrons_evolve", "coupling",
         "qfilter", "redist_every", "precision", "device")


class Params(ctypes.Structure):
    """Mirror of struct pf_params (include/puffgpu.h)."""
    _fields_ = [(k, ctypes.c_double) for k in _DOUBLES] + [(k, ctypes.c_int32) for k in _INTS]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None
SYMBOLS = (
    "pf_default_params", "pf_create", "pf_destroy", "pf_set_particles", "pf_get_particles",
    "pf_set_particles_dev", "pf_get_particles_dev", "pf_num_particles", "pf_set_field",
    "pf_get_field", "pf_set_field_dev", "pf_get_field_dev", "pf_set_taper", "pf_get_taper",
    "pf_get_window", "pf_rk4_step", "pf_rk4_step_host", "pf_diffract_host", "pf_redistribute", "pf_wrap_z2", "pf_diffract", "pf_run",
    "pf_sync", "pf_kernel_launches", "pf_last_error", "pf_abi_version", "pf_get_stream",
    "pf_profile", "pf_profile_read", "pf_rk4_step_noalloc", "pf_power", "pf_num_slices",
    "pf_bunching", "pf_spectrum", "pf_step_count", "pf_set_step_count", "pf_drift",
    "pf_chicane", "pf_quad", "pf_modulation", "pf_match_in", "pf_match_out",
    "pf_correct_trans", "pf_init_undulator", "pf_set_taper_profile", "pf_diffract_adjoint",
    "pf_adjoint_forward", "pf_generate_beam", "pf_set_launch_mode",
    "pf_adjoint_backward", "pf_batch_create", "pf_batch_destroy", "pf_batch_run",
    "pf_batch_tune", "pf_batch_get_shape", "pf_batch_set_shape", "pf_batch_use_graphs",
    "pf_batch_launches", "pf_batch_stream", "pf_batch_last_error", "pf_set_window_field",
    "pf_get_window_field", "pf_set_window_field_dev", "pf_get_window_field_dev",
    "pf_window_nodes", "pf_set_fft_arithmetic",
)
NOALLOC_MAX_PARTICLES = 32768
NOALLOC_MAX_NODES = 32768
PROF_STAGE, PROF_NODES, PROF_FFT, PROF_DIFF, PROF_OTHER = range(5)


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = False):
    """Load libpuffgpu.so and declare every entry point's prototype."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not os.path.exists(path):
        if build_if_missing:
            _build.build_library()
        else:
            raise RuntimeError(
                f"libpuffgpu.so not found at {path}: build it with "
                "`python -c 'import __graft_entry__ as g; g.build()'`")
    L = ctypes.CDLL(path)
    H = ctypes.c_void_p
    dp = ctypes.POINTER(ctypes.c_double)
    P = ctypes.POINTER(Params)
    i32, i64, f64 = ctypes.c_int32, ctypes.c_int64, ctypes.c_double
    proto = {
        "pf_default_params": (None, [P]),
        "pf_create": (ctypes.c_int, [P, ctypes.POINTER(H)]),
        "pf_destroy": (ctypes.c_int, [H]),
        "pf_set_particles": (ctypes.c_int, [H, i64] + [ctypes.c_void_p] * 7),
        "pf_get_particles": (ctypes.c_int, [H] + [ctypes.c_void_p] * 7),
        "pf_set_particles_dev": (ctypes.c_int, [H, i64] + [ctypes.c_void_p] * 7),
        "pf_get_particles_dev": (ctypes.c_int, [H] + [ctypes.c_void_p] * 7),
        "pf_num_particles": (i64, [H]),
        "pf_set_field": (ctypes.c_int, [H, ctypes.c_void_p, ctypes.c_void_p]),
        "pf_get_field": (ctypes.c_int, [H, ctypes.c_void_p, ctypes.c_void_p]),
        "pf_set_field_dev": (ctypes.c_int, [H, ctypes.c_void_p, ctypes.c_void_p]),
        "pf_get_field_dev": (ctypes.c_int, [H, ctypes.c_void_p, ctypes.c_void_p]),
        "pf_set_taper": (ctypes.c_int, [H, f64, f64, f64]),
        "pf_get_taper": (ctypes.c_int, [H, dp, dp, dp]),
        "pf_get_window": (ctypes.c_int, [H, ctypes.POINTER(i32), ctypes.POINTER(i32)]),
        "pf_set_window_field": (ctypes.c_int, [H, ctypes.c_void_p, ctypes.c_void_p]),
        "pf_get_window_field": (ctypes.c_int, [H, ctypes.c_void_p, ctypes.c_void_p]),
        "pf_set_window_field_dev": (ctypes.c_int, [H, ctypes.c_void_p, ctypes.c_void_p]),
        "pf_get_window_field_dev": (ctypes.c_int, [H, ctypes.c_void_p, ctypes.c_void_p]),
        "pf_window_nodes": (i64, [H]),
        "pf_rk4_step": (ctypes.c_int, [H, f64, f64]),
        "pf_rk4_step_host": (ctypes.c_int, [H, f64, f64] + [ctypes.c_void_p] * 8),
        "pf_diffract_host": (ctypes.c_int, [H, f64] + [ctypes.c_void_p] * 4),
        "pf_redistribute": (ctypes.c_int, [H]),
        "pf_wrap_z2": (ctypes.c_int, [H]),
        "pf_diffract": (ctypes.c_int, [H, f64]),
        "pf_run": (ctypes.c_int, [H, i32, i32, i32, f64, dp, ctypes.POINTER(i32)]),
        "pf_sync": (ctypes.c_int, [H]),
        "pf_kernel_launches": (i64, [H]),
        "pf_last_error": (ctypes.c_char_p, [H]),
        "pf_abi_version": (ctypes.c_int, []),
        "pf_get_stream": (ctypes.c_void_p, [H]),
        "pf_profile": (ctypes.c_int, [H, i32]),
        "pf_profile_read": (ctypes.c_int, [H, i32, dp, ctypes.POINTER(i64)]),
        "pf_power": (ctypes.c_int, [H, ctypes.c_void_p, i64]),
        "pf_num_slices": (i64, [H]),
        "pf_bunching": (ctypes.c_int, [H, i32, ctypes.c_void_p, i64]),
        "pf_spectrum": (ctypes.c_int, [H, ctypes.c_void_p, ctypes.c_void_p, i64]),
        "pf_step_count": (i64, [H]),
        "pf_set_taper_profile": (ctypes.c_int, [H, i32, ctypes.c_void_p, ctypes.c_void_p]),
        "pf_set_launch_mode": (ctypes.c_int, [H, i32]),
        "pf_set_fft_arithmetic": (ctypes.c_int, [H, i32]),
        "pf_generate_beam": (ctypes.c_int, [H, i64, ctypes.c_void_p, ctypes.c_void_p, f64, i32,
                                            ctypes.c_void_p, ctypes.c_void_p, i32,
                                            ctypes.c_uint64, f64]),
        "pf_diffract_adjoint": (ctypes.c_int, [H, f64, ctypes.c_void_p, ctypes.c_void_p]),
        "pf_adjoint_forward": (ctypes.c_int, [H, i32, i32, i32, f64, i32, ctypes.c_void_p,
                                              ctypes.c_void_p, f64, f64, dp]),
        "pf_adjoint_backward": (ctypes.c_int, [H, f64, ctypes.c_void_p, i32, dp, dp]),
        "pf_set_step_count": (ctypes.c_int, [H, i64]),
        "pf_drift": (ctypes.c_int, [H, f64, i32]),
        "pf_chicane": (ctypes.c_int, [H, f64, f64, f64, i32]),
        "pf_quad": (ctypes.c_int, [H, f64, f64]),
        "pf_modulation": (ctypes.c_int, [H, f64, f64]),
        "pf_match_in": (ctypes.c_int, [H, f64]),
        "pf_match_out": (ctypes.c_int, [H, f64]),
        "pf_correct_trans": (ctypes.c_int, [H]),
        "pf_init_undulator": (ctypes.c_int, [H, i32, f64, f64, f64, f64, f64, f64, i32, f64, i32]),
        "pf_batch_create": (ctypes.c_int, [ctypes.c_void_p, i32, ctypes.POINTER(H)]),
        "pf_batch_destroy": (ctypes.c_int, [H]),
        "pf_batch_run": (ctypes.c_int, [H, i32, i32, i32, ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.c_void_p]),
        "pf_batch_tune": (ctypes.c_int, [H, ctypes.c_void_p, ctypes.c_void_p, i32]),
        "pf_batch_get_shape": (ctypes.c_int, [H, ctypes.c_void_p, ctypes.c_void_p]),
        "pf_batch_set_shape": (ctypes.c_int, [H, ctypes.c_void_p, ctypes.c_void_p]),
        "pf_batch_use_graphs": (ctypes.c_int, [H, i32]),
        "pf_batch_launches": (i64, [H]),
        "pf_batch_stream": (ctypes.c_void_p, [H]),
        "pf_batch_last_error": (ctypes.c_char_p, [H]),
        "pf_rk4_step_noalloc": (ctypes.c_int, [P, dp, dp, f64, f64, i64] + [ctypes.c_void_p] * 9
                                + [i32, i32, ctypes.c_void_p]),
    }
    for name, (res, args) in proto.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


# The values pf_default_params writes (the reference's defaults; every other
# field is zero).  Held here as well so that a workload can be described
# without loading the CUDA library -- the CPU timing of the oracle does not
# load it.  tests/test_abi.py checks that the two agree field by field.
DEFAULTS = {
    "rho": 0.01, "aw": 1.0, "gamma_r": 100.0, "fx": 1.0, "fy": 1.0, "szfe": 1.0e30,
    "n2col0": 1.0, "dx": 1.0, "dy": 1.0, "dz2": 1.0, "sbeta": 1.0,
    "sfilt_frac": float(np.float32(0.3)), "sperwaves": -1.0,
    "und_type": UND_PUFFIN, "mesh_type": MESH_TEMPORAL, "nx": 1, "ny": 1, "nz2": 2,
    "nbx": 16, "nby": 16, "nbz2": 37, "field_evolve": 1, "electrons_evolve": 1,
    "coupling": 1, "qfilter": 1, "redist_every": 60, "precision": FP64,
}


def default_params(**overrides) -> Params:
    """pf_default_params' values (DEFAULTS) with the given overrides; does
    not load the library."""
    p = Params()
    for k, v in DEFAULTS.items():
        setattr(p, k, v)
    for k, v in overrides.items():
        if not hasattr(p, k):
            raise KeyError(k)
        setattr(p, k, v)
    return p
