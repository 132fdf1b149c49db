"""The allocation-free RK4 step (pf_rk4_step_noalloc) against pf_rk4_step.

pf_rk4_step_noalloc exists for callers that cannot allocate device memory:
their device memory is owned by their own allocator, or they cannot take the
implicit synchronisation of cudaMalloc.  It runs the same kernels with its
temporaries in the library's fixed-size static device array, so on the same
inputs it must give the results of the handle-based pf_rk4_step.  Two calls
in a row check that contents left in the shared array by one call do not leak
into the next.  This file is collected last so that a stop at the first
failure has already run every other test.
"""
import numpy as np
import pytest

import puffin_gb300 as P
from puffin_gb300 import configs

pytestmark = pytest.mark.gpu


def test_noalloc_matches_handle_path_two_calls():
    torch = pytest.importorskip("torch")
    w = configs.config1(np_=5000, seed=17)
    rng = np.random.default_rng(4)
    n_out = w.params.nx * w.params.ny * w.params.nz2
    field = (1e-3 * rng.standard_normal(n_out), 1e-3 * rng.standard_normal(n_out))

    # reference: the handle-based entry point, two steps
    with P.Puffin(w.params) as sim:
        sim.set_particles(*(w.beam[k] for k in P.PARTICLE_KEYS))
        sim.set_field(*field)
        nix, niy = sim.window
        ref = []
        szl = 0.0
        for _ in range(2):
            assert sim.rk4par(szl, w.h)
            szl += w.h
            parts = sim.get_particles()
            fr, fi = sim.get_field()
            ref.append((parts, fr, fi))

    # allocation-free entry point on caller-owned device buffers
    p = w.params
    npl = p.nz2 - 1 if p.mesh_type == P.MESH_PERIODIC else p.nz2
    assert w.np <= P.lib.NOALLOC_MAX_PARTICLES and nix * niy * npl <= P.lib.NOALLOC_MAX_NODES
    ox, oy = (p.nx - nix) // 2, (p.ny - niy) // 2

    def window(a):
        return a.reshape(p.nz2, p.ny, p.nx)[:npl, oy:oy + niy, ox:ox + nix].reshape(-1)

    dev = {k: torch.tensor(w.beam[k], dtype=torch.float64, device="cuda") for k in P.PARTICLE_KEYS}
    wr = torch.tensor(np.ascontiguousarray(window(field[0])), dtype=torch.float64, device="cuda")
    wi = torch.tensor(np.ascontiguousarray(window(field[1])), dtype=torch.float64, device="cuda")
    taper = [p.n2col0, p.n2col0]
    szl = 0.0
    for step in range(2):
        torch.cuda.synchronize()
        assert P.rk4_step_noalloc(p, taper, szl, w.h, dev, wr, wi, nix, niy)
        szl += w.h
        torch.cuda.synchronize()
        parts, fr, fi = ref[step]
        for k in ("x", "y", "z2", "px", "py", "gam"):
            np.testing.assert_allclose(dev[k].cpu().numpy(), parts[k], rtol=1e-12, atol=1e-15,
                                       err_msg=f"step {step}: {k}")
        scale = max(np.abs(fr).max(), np.abs(fi).max())
        np.testing.assert_allclose(wr.cpu().numpy(), window(fr), rtol=0, atol=1e-12 * scale)
        np.testing.assert_allclose(wi.cpu().numpy(), window(fi), rtol=0, atol=1e-12 * scale)


def test_noalloc_rejects_sizes_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    w = configs.config1(np_=P.lib.NOALLOC_MAX_PARTICLES + 1, seed=2)
    p = w.params
    dev = {k: torch.tensor(w.beam[k], dtype=torch.float64, device="cuda") for k in P.PARTICLE_KEYS}
    npl = p.nz2 - 1
    wr = torch.zeros(21 * 21 * npl, dtype=torch.float64, device="cuda")
    wi = torch.zeros_like(wr)
    with pytest.raises(P.PuffinError) as e:
        P.rk4_step_noalloc(p, [1.0, 1.0], 0.0, w.h, dev, wr, wi, 21, 21)
    assert e.value.code == P.lib.PF_BAD_ARG
