"""pf_rk4_step_host and pf_diffract_host: rk4par and inner2Outer +
diffractIM + outer2Inner on the driver's host arrays, the copies in and out
overlapped with the kernels (the particles in chunks of 2^20 or more, the
outer field by ranges of z2 planes), against the device-resident sequences
they replace (set_window_field + set_particles with chi kept + rk4par +
get_particles + get_window_field; set_field + set_window_field + diffractIM
+ get_field + get_window_field): bit for bit in FP64; a macroparticle that
leaves the window leaves the host arrays and the handle's state as they
came in."""
import numpy as np
import pytest
import torch

import puffin_gb300 as P
from puffin_gb300 import configs
from puffin_gb300 import lib as L

pytestmark = pytest.mark.gpu
KEYS = P.PARTICLE_KEYS[:6]


def _pinned(a):
    t = torch.empty(a.size, dtype=torch.float64, pin_memory=True).numpy()
    t[:] = a
    return t


def _field(p, seed):
    rng = np.random.default_rng(seed)
    n = p.nx * p.ny * p.nz2
    return 1e-3 * rng.standard_normal(n), 1e-3 * rng.standard_normal(n)


# one chunk; three chunks; five chunks, the last of 4321 macroparticles
@pytest.mark.parametrize("np_", [3000, (1 << 21) + 12345, (1 << 22) + 4321])
def test_host_step_matches_resident_steps(np_):
    w = configs.config1(np_=np_, seed=5)
    field = _field(w.params, 5)
    with P.Puffin(w.params) as a, P.Puffin(w.params) as b:
        for sim in (a, b):
            sim.set_particles(*(w.beam[k] for k in P.PARTICLE_KEYS))
            sim.set_field(*field)
        parts = {k: _pinned(w.beam[k]) for k in KEYS}
        wre, wim = (_pinned(v) for v in a.get_window_field())
        szl = 0.0
        for _ in range(3):
            assert a.rk4par_host(szl, w.h, parts, (wre, wim))
            assert b.rk4par(szl, w.h)
            szl += w.h
        got_b = b.get_particles()
        wb = b.get_window_field()
        got_a = a.get_particles()
    for k in KEYS:
        np.testing.assert_array_equal(parts[k], got_b[k], err_msg=k)
        np.testing.assert_array_equal(got_a[k], got_b[k], err_msg=k)
    np.testing.assert_array_equal(wre, wb[0])
    np.testing.assert_array_equal(wim, wb[1])
    assert not np.array_equal(parts["z2"], w.beam["z2"])  # the steps moved the beam


def test_host_step_failure_leaves_arrays_and_state():
    w = configs.config1(np_=(1 << 21) + 7, seed=6)
    field = _field(w.params, 6)
    with P.Puffin(w.params) as sim:
        sim.set_particles(*(w.beam[k] for k in P.PARTICLE_KEYS))
        sim.set_field(*field)
        parts = {k: _pinned(w.beam[k]) for k in KEYS}
        wre, wim = (_pinned(v) for v in sim.get_window_field())
        # a macroparticle of a later chunk far outside the transverse window
        parts["x"][(1 << 20) + 5] = 1.0e3
        before = {k: v.copy() for k, v in parts.items()}
        w_before = (wre.copy(), wim.copy())
        assert not sim.rk4par_host(0.0, w.h, parts, (wre, wim))
        got = sim.get_particles()
    for k in KEYS:
        np.testing.assert_array_equal(parts[k], before[k], err_msg=k)
        np.testing.assert_array_equal(got[k], before[k], err_msg=k)
    np.testing.assert_array_equal(wre, w_before[0])
    np.testing.assert_array_equal(wim, w_before[1])


def test_host_step_after_z2_ordering_keeps_chi_with_the_caller_order():
    """After pf_run has z2-ordered the handle, host arrays in the caller's
    order take chi back to that order: the step equals a fresh handle's."""
    w = configs.config1(np_=1 << 16, seed=7)
    field = _field(w.params, 7)
    with P.Puffin(w.params) as a, P.Puffin(w.params) as b:
        for sim in (a, b):
            sim.set_particles(*(w.beam[k] for k in P.PARTICLE_KEYS))
            sim.set_field(*field)
        szl = a.und_section(120, 16, True, w.h, 0.0)   # z2-orders the beam at the wrap cadence
        state = a.get_particles()
        fr, fi = a.get_field()
        b.set_particles(*(state[k] for k in P.PARTICLE_KEYS))
        b.set_field(fr, fi)
        parts = {k: _pinned(state[k]) for k in KEYS}
        wre, wim = (_pinned(v) for v in a.get_window_field())
        assert a.rk4par_host(szl, w.h, parts, (wre, wim))
        assert b.rk4par(szl, w.h)
        got_b = b.get_particles()
    for k in KEYS:
        np.testing.assert_allclose(parts[k], got_b[k], rtol=0, atol=0, err_msg=k)


def test_host_step_mixed_matches_resident_steps():
    """The mixed form (window field converted to and from complex float on
    the device): the same steps as the five-call sequence, to the rounding
    of the FP32 float atomics (chunked launches cut the stage blocks, and
    so the split between shared tile and HBM deposits, differently)."""
    w = configs.config1(np_=(1 << 21) + 12345, seed=8)
    q = P.Params.from_buffer_copy(w.params)
    q.precision = P.MIXED
    field = _field(w.params, 8)
    with P.Puffin(q) as a, P.Puffin(q) as b:
        for sim in (a, b):
            sim.set_particles(*(w.beam[k] for k in P.PARTICLE_KEYS))
            sim.set_field(*field)
        parts = {k: _pinned(w.beam[k]) for k in KEYS}
        wre, wim = (_pinned(v) for v in a.get_window_field())
        szl = 0.0
        for _ in range(3):
            assert a.rk4par_host(szl, w.h, parts, (wre, wim))
            assert b.rk4par(szl, w.h)
            szl += w.h
        got_b = b.get_particles()
        wb = b.get_window_field()
    # the FP32 slopes of macroparticles whose deposits rounded differently
    # differ by FP32 roundings (3e-8 relative) times the step
    for k in KEYS:
        np.testing.assert_allclose(parts[k], got_b[k], rtol=1e-7, atol=1e-8, err_msg=k)
    scale = max(np.max(np.abs(wb[0])), np.max(np.abs(wb[1])))
    np.testing.assert_allclose(wre, wb[0], rtol=0, atol=1e-5 * scale)
    np.testing.assert_allclose(wim, wb[1], rtol=0, atol=1e-5 * scale)


@pytest.mark.parametrize("periodic", [False, True])
@pytest.mark.parametrize("arith", ["paired", "fp64"])
def test_host_diffraction_matches_set_diffract_get(periodic, arith):
    """pf_diffract_host (the outer field in and out by ranges of z2 planes,
    overlapped with the first and last x passes) against pf_set_field +
    pf_set_window_field + pf_diffract + pf_get_field + pf_get_window_field,
    bit for bit, on a 129 x 129 mesh (line kernels cut into plane ranges)."""
    w = configs.config2(np_=20000, nz2=65)
    p = P.Params.from_buffer_copy(w.params)
    if periodic:
        p.mesh_type = P.MESH_PERIODIC
    mode = {"paired": L.FFT_PAIRED_FP32, "fp64": L.FFT_FP64}[arith]
    rng = np.random.default_rng(11)
    n = p.nx * p.ny * p.nz2
    ore0, oim0 = 1e-3 * rng.standard_normal(n), 1e-3 * rng.standard_normal(n)
    with P.Puffin(p) as a, P.Puffin(p) as b:
        for sim in (a, b):
            sim.set_fft_arithmetic(mode)
            sim.set_particles(*(w.beam[k] for k in P.PARTICLE_KEYS))
            sim.set_field(ore0, oim0)
        wre0, wim0 = a.get_window_field()
        wre0 = wre0 + 1e-4 * rng.standard_normal(wre0.size)   # the driver's window differs
        wim0 = wim0 + 1e-4 * rng.standard_normal(wim0.size)
        ore, oim = _pinned(ore0), _pinned(oim0)
        wre, wim = _pinned(wre0), _pinned(wim0)
        a.diffractIM_host(8 * w.h, (ore, oim), (wre, wim))
        b.set_window_field(wre0, wim0)
        b.diffractIM(8 * w.h)
        fr, fi = b.get_field()
        gr, gi = b.get_window_field()
    np.testing.assert_array_equal(ore, fr)
    np.testing.assert_array_equal(oim, fi)
    np.testing.assert_array_equal(wre, gr)
    np.testing.assert_array_equal(wim, gi)
    assert not np.array_equal(ore, ore0)


@pytest.mark.parametrize("periodic", [False, True])
def test_host_diffraction_mixed_matches_set_diffract_get(periodic):
    """The mixed form (the FP64 arrays converted to and from the complex
    float field on the device, range by range): bit for bit as the
    five-call sequence, which converts with the same roundings."""
    w = configs.config2(np_=20000, nz2=65)
    p = P.Params.from_buffer_copy(w.params)
    p.precision = P.MIXED
    if periodic:
        p.mesh_type = P.MESH_PERIODIC
    rng = np.random.default_rng(13)
    n = p.nx * p.ny * p.nz2
    ore0, oim0 = 1e-3 * rng.standard_normal(n), 1e-3 * rng.standard_normal(n)
    with P.Puffin(p) as a, P.Puffin(p) as b:
        for sim in (a, b):
            sim.set_particles(*(w.beam[k] for k in P.PARTICLE_KEYS))
            sim.set_field(ore0, oim0)
        wre0, wim0 = a.get_window_field()
        wre0 = wre0 + 1e-4 * rng.standard_normal(wre0.size)
        wim0 = wim0 + 1e-4 * rng.standard_normal(wim0.size)
        ore, oim = _pinned(ore0), _pinned(oim0)
        wre, wim = _pinned(wre0), _pinned(wim0)
        for _ in range(2):  # the second call reuses the staging buffers
            a.diffractIM_host(8 * w.h, (ore, oim), (wre, wim))
        b.set_window_field(wre0, wim0)
        b.diffractIM(8 * w.h)
        b.set_field(*b.get_field())
        b.set_window_field(*b.get_window_field())
        b.diffractIM(8 * w.h)
        fr, fi = b.get_field()
        gr, gi = b.get_window_field()
    np.testing.assert_array_equal(ore, fr)
    np.testing.assert_array_equal(oim, fi)
    np.testing.assert_array_equal(wre, gr)
    np.testing.assert_array_equal(wim, gi)
    assert not np.array_equal(ore, ore0)


@pytest.mark.parametrize("mixed", [False, True])
def test_host_diffraction_without_a_window(mixed):
    """No particles, so no inner window: the call transforms the outer field
    alone (window arguments may be NULL), as pf_set_field + pf_diffract +
    pf_get_field do."""
    w = configs.config2(np_=20000, nz2=65)
    p = P.Params.from_buffer_copy(w.params)
    if mixed:
        p.precision = P.MIXED
    rng = np.random.default_rng(12)
    n = p.nx * p.ny * p.nz2
    ore0, oim0 = 1e-3 * rng.standard_normal(n), 1e-3 * rng.standard_normal(n)
    lib = L.load()
    with P.Puffin(p) as a, P.Puffin(p) as b:
        ore, oim = _pinned(ore0), _pinned(oim0)
        assert lib.pf_diffract_host(a._h, 8 * w.h, ore.ctypes.data, oim.ctypes.data, None,
                                    None) == 0
        b.set_field(ore0, oim0)
        b.diffractIM(8 * w.h)
        fr, fi = b.get_field()
    np.testing.assert_array_equal(ore, fr)
    np.testing.assert_array_equal(oim, fi)
