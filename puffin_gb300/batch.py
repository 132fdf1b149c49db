"""Batched runs of many independent instances over the puffgpu C ABI.

``Batch(sims)`` groups ``Puffin`` instances (one device, one precision, 3D,
particles and field set) and advances them together: ``run`` does what
``sim.und_section(nsteps, isteps4diff, qdiffraction, h[i], szl[i])`` does for
each instance (UndSection, puffin/lib/undulator.f90:33-358), with every RK4
stage of every instance in one launch and each block of steps between
diffraction calls replayed as one CUDA graph.  ``tune`` runs the autotuner
(deposit mode per instance; tile lengths, block size and grids for the
batch) on the instances' current state, which it leaves unchanged.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import lib as L
from .puffin import Puffin, PuffinError


class Batch:
    def __init__(self, sims: list[Puffin]):
        self._lib = L.load()
        self.sims = list(sims)
        arr = (ctypes.c_void_p * len(self.sims))(*[s._h.value for s in self.sims])
        b = ctypes.c_void_p()
        rc = self._lib.pf_batch_create(arr, len(self.sims), ctypes.byref(b))
        if rc != L.PF_OK:
            raise PuffinError(rc, "pf_batch_create: instances must share a device and a "
                                  "precision, be 3D and distinct")
        self._b = b

    @property
    def n(self) -> int:
        return len(self.sims)

    def close(self):
        if getattr(self, "_b", None):
            self._lib.pf_batch_destroy(self._b)
            self._b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, rc):
        if rc != L.PF_OK:
            raise PuffinError(rc, self._lib.pf_batch_last_error(self._b).decode())

    def _vec(self, v):
        a = np.ascontiguousarray(np.broadcast_to(np.asarray(v, dtype=np.float64), (self.n,)))
        return a

    def run(self, nsteps: int, isteps4diff: int, qdiffraction: bool, h, szl=0.0,
            raise_on_error: bool = True):
        """Advance every instance by nsteps; returns (szl, status) arrays."""
        hs = self._vec(h)
        z = self._vec(szl).copy()
        st = np.zeros(self.n, dtype=np.int32)
        rc = self._lib.pf_batch_run(self._b, int(nsteps), int(isteps4diff),
                                    int(bool(qdiffraction)), hs.ctypes.data, z.ctypes.data,
                                    st.ctypes.data)
        if raise_on_error:
            self._check(rc)
        return z, st

    def tune(self, h, szl=0.0, repeats: int = 3):
        hs = self._vec(h)
        z = self._vec(szl)
        self._check(self._lib.pf_batch_tune(self._b, hs.ctypes.data, z.ctypes.data, int(repeats)))
        return self.shape()

    def shape(self):
        """{stage_threads, stage_tile, node_tile, stage_grid, node_grid} and
        the per-instance deposit modes (0 direct, else the tile range)."""
        s = np.zeros(5, dtype=np.int64)
        m = np.zeros(self.n, dtype=np.int64)
        self._check(self._lib.pf_batch_get_shape(self._b, s.ctypes.data, m.ctypes.data))
        keys = ("stage_threads", "stage_tile", "node_tile", "stage_grid", "node_grid")
        return {**{k: int(v) for k, v in zip(keys, s)}, "modes": m}

    def set_shape(self, stage_threads=None, stage_tile=None, node_tile=None, stage_grid=None,
                  node_grid=None, modes=None):
        cur = self.shape()
        s = np.array([cur["stage_threads"] if stage_threads is None else stage_threads,
                      cur["stage_tile"] if stage_tile is None else stage_tile,
                      cur["node_tile"] if node_tile is None else node_tile,
                      cur["stage_grid"] if stage_grid is None else stage_grid,
                      cur["node_grid"] if node_grid is None else node_grid], dtype=np.int64)
        m = None if modes is None else np.ascontiguousarray(modes, dtype=np.int64)
        self._check(self._lib.pf_batch_set_shape(self._b, s.ctypes.data,
                                                 None if m is None else m.ctypes.data))

    def use_graphs(self, on: bool = True):
        self._check(self._lib.pf_batch_use_graphs(self._b, int(bool(on))))

    @property
    def kernel_launches(self) -> int:
        return int(self._lib.pf_batch_launches(self._b))

    @property
    def stream_handle(self) -> int:
        return self._lib.pf_batch_stream(self._b) or 0
