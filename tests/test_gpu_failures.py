"""Failures made on the host and reported through the C ABI.

The reference's error paths are the window retry of UndSection
(puffin/lib/undulator.f90:196-212), the STOP beyond the temporal mesh
(system_interpolation.f90:60-80) and nothing at all for a NaN or an
allocation failure.  Here every one of them returns a status and leaves the
handle usable:
* a NaN in one macroparticle coordinate, or in the inner-window field,
  gives PF_NOT_FINITE with the particles and the field unchanged (pf_run
  returns it as well: no retry loop);
* a source term beyond the FP64 deposit's fixed-point range gives
  PF_OVERFLOW with the state unchanged;
* a mesh or a beam too large to allocate gives PF_CUDA_ERR, after which the
  handle accepts a smaller beam, steps, and is destroyed normally.
No GPU fault is involved: the bad values are planted in the inputs, and the
failed allocations ask for more memory than the device has.
"""
import ctypes

import numpy as np
import pytest

import puffin_gb300 as P
from puffin_gb300 import configs
from puffin_gb300 import lib as L

pytestmark = pytest.mark.gpu


def _bits(a):
    return np.ascontiguousarray(a, dtype=np.float64).view(np.int64)


def _state(sim):
    parts = sim.get_particles()
    wr, wi = sim.get_window_field()
    return {k: _bits(v) for k, v in parts.items()}, _bits(wr), _bits(wi)


def _assert_same_state(a, b):
    for k in a[0]:
        assert np.array_equal(a[0][k], b[0][k]), k
    assert np.array_equal(a[1], b[1]) and np.array_equal(a[2], b[2])


def _sim(prec, np_=4096, seed=3):
    w = configs.config1(np_=np_, seed=seed)
    w.params.precision = prec
    sim = P.Puffin(w.params)
    sim.set_particles(*(w.beam[k] for k in P.PARTICLE_KEYS))
    rng = np.random.default_rng(seed)
    n = w.params.nx * w.params.ny * w.params.nz2
    sim.set_field(1e-3 * rng.standard_normal(n), 1e-3 * rng.standard_normal(n))
    return w, sim


@pytest.mark.parametrize("prec", [P.FP64, P.MIXED])
def test_nan_transverse_position_is_refused_by_set_particles(prec):
    """The inner window is computed from the transverse extremes when the
    particles are set (getInNode, para_field.f90:1432-1508): a NaN there is
    reported at once."""
    w, sim = _sim(prec)
    with sim:
        beam = {k: np.array(v) for k, v in w.beam.items()}
        beam["x"][777] = np.nan
        with pytest.raises(P.PuffinError) as e:
            sim.set_particles(*(beam[k] for k in P.PARTICLE_KEYS))
        assert e.value.code == L.PF_NOT_FINITE


@pytest.mark.parametrize("prec", [P.FP64, P.MIXED])
@pytest.mark.parametrize("key", ["z2", "px", "py", "gam"])
def test_nan_in_a_particle_coordinate(prec, key):
    w, sim = _sim(prec)
    with sim:
        beam = {k: np.array(v) for k, v in w.beam.items()}
        beam[key][777] = np.nan
        sim.set_particles(*(beam[k] for k in P.PARTICLE_KEYS))
        before = _state(sim)
        lib = L.load()
        assert lib.pf_rk4_step(sim._h, 0.0, w.h) == L.PF_NOT_FINITE
        _assert_same_state(before, _state(sim))
        z = ctypes.c_double(0.0)
        done = ctypes.c_int32(-1)
        assert lib.pf_run(sim._h, 8, 4, 1, w.h, ctypes.byref(z), ctypes.byref(done)) \
            == L.PF_NOT_FINITE
        assert done.value == 0


@pytest.mark.parametrize("prec", [P.FP64, P.MIXED])
def test_nan_in_the_seed_field(prec):
    w, sim = _sim(prec)
    with sim:
        p = w.params
        re, im = sim.get_field()
        centre = (p.nz2 // 2) * p.nx * p.ny + (p.ny // 2) * p.nx + p.nx // 2
        re[centre] = np.nan
        sim.set_field(re, im)
        before = _state(sim)
        assert L.load().pf_rk4_step(sim._h, 0.0, w.h) == L.PF_NOT_FINITE
        _assert_same_state(before, _state(sim))
        with pytest.raises(P.PuffinError) as e:
            sim.rk4par(0.0, w.h)
        assert e.value.code == L.PF_NOT_FINITE


def test_source_beyond_the_fixed_point_range():
    """The FP64 deposit's scale leaves 2^16 of headroom above max chi/dV3;
    one macroparticle with |p_perp| (1 + eta p2)/Gamma of about 1e6 (a beam
    of gamma_r = 1e6 with u = 0.49) exceeds it."""
    rho, aw, gr = 0.005, 1.0, 1.0e6
    eta, kappa, fx, fy = configs.calc_scaling(rho, aw, gr, P.UND_HELICAL)
    w = configs.config1(np_=4096, seed=9)
    p = w.params
    p.gamma_r, p.eta, p.kappa = gr, eta, kappa
    beam = {k: np.array(v) for k, v in w.beam.items()}
    beam["px"][100] = 0.7e6 / aw
    with P.Puffin(p) as sim:
        sim.set_particles(*(beam[k] for k in P.PARTICLE_KEYS))
        before = _state(sim)
        assert L.load().pf_rk4_step(sim._h, 0.0, w.h) == L.PF_OVERFLOW
        _assert_same_state(before, _state(sim))


def test_mesh_too_large_to_allocate():
    lib = L.load()
    p = P.default_params(nx=8192, ny=8192, nz2=65536, eta=1e-4)   # 35 TB per field array
    h = ctypes.c_void_p()
    assert lib.pf_create(ctypes.byref(p), ctypes.byref(h)) == L.PF_CUDA_ERR
    assert not h.value
    assert b"field" in lib.pf_last_error(None)
    assert lib.pf_destroy(None) == L.PF_OK
    # the device is still usable
    w, sim = _sim(P.FP64, np_=2048)
    with sim:
        assert sim.rk4par(0.0, w.h)


def test_beam_too_large_to_allocate_leaves_a_usable_handle():
    lib = L.load()
    w, sim = _sim(P.FP64, np_=2048)
    try:
        small = np.zeros(16)
        n_huge = 1 << 40                       # 8 TB per particle array
        rc = lib.pf_set_particles(sim._h, n_huge, *([small.ctypes.data] * 7))
        assert rc == L.PF_CUDA_ERR
        assert lib.pf_rk4_step(sim._h, 0.0, w.h) == L.PF_STATE
        sim.set_particles(*(w.beam[k] for k in P.PARTICLE_KEYS))
        assert sim.rk4par(0.0, w.h)
    finally:
        assert lib.pf_destroy(sim._h) == L.PF_OK
        sim._h = None
