"""puffin_gb300: GB300-native (sm_103a) CUDA library for Puffin's per-step hot
path (RK4 macroparticle push with trilinear gather/deposit, and the FFT
diffraction step), reached through the C ABI in include/puffgpu.h."""
from .lib import (FP64, MESH_PERIODIC, MESH_TEMPORAL, MIXED, UND_CURVED, UND_HELICAL,  # noqa: F401
                  UND_PLANEPOLE, UND_PUFFIN, Params, default_params, library_path, load)
from .puffin import PARTICLE_KEYS, Puffin, PuffinError, rk4_step_noalloc  # noqa: F401
from . import lattice  # noqa: F401
from . import adjoint  # noqa: F401
from . import h5dump  # noqa: F401
from .batch import Batch  # noqa: F401

__all__ = ["lattice", "adjoint", "h5dump", "Batch", "Puffin", "PuffinError", "rk4_step_noalloc", "Params", "default_params", "load", "library_path",
           "PARTICLE_KEYS", "FP64", "MIXED", "MESH_TEMPORAL", "MESH_PERIODIC",
           "UND_PUFFIN", "UND_HELICAL", "UND_PLANEPOLE", "UND_CURVED"]
