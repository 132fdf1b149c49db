"""Batched runs against the same instances run one at a time.

Every instance of a batch follows pf_run's schedule, so in FP64 (integer
fixed-point deposit) the batch must give the same bits as und_section on
each instance alone, whatever the launch shapes (graphs or not, tuned or
not).  The mixed-precision batch deposits with float atomics whose order
varies: it is compared at rtol 1e-5 / atol 1e-8 on the particles and 1e-4
of the largest field value.

Instances: the batched form's recipe at small sizes (macroparticles
log-uniform in [2^10, 2^13], meshes {17, 33, 65}^2 x {32, 64, 128}), 40
steps with diffraction every 16 (two graph blocks and a short block), and a
wrap cadence of 12 steps on half of them so that wraps fall inside blocks.
"""
import numpy as np
import pytest

import puffin_gb300 as P
from puffin_gb300 import configs

pytestmark = pytest.mark.gpu
NSTEPS, EVERY = 40, 16


def _instances(n=6, seed=7, precision=P.FP64, np_range=(2 ** 10, 2 ** 13)):
    ws = configs.config5(n_inst=n, seed=seed, nsteps=NSTEPS, np_range=np_range)
    for k, w in enumerate(ws):
        w.params.precision = precision
        if k % 2:
            w.params.redist_every = 12
    return ws


def _make(w, field_scale=1e-3):
    sim = P.Puffin(w.params)
    sim.set_particles(*(w.beam[k] for k in P.PARTICLE_KEYS))
    rng = np.random.default_rng(int(w.np))
    n = len(w.field[0])
    sim.set_field(field_scale * rng.standard_normal(n), field_scale * rng.standard_normal(n))
    return sim


def _state(sim):
    return sim.get_particles(), sim.get_field(), sim.step_count


def _single(ws):
    out = []
    for w in ws:
        with _make(w) as sim:
            z = sim.und_section(NSTEPS, EVERY, True, w.h)
            out.append((_state(sim), z))
    return out


def _assert_same(got, want, exact, tag):
    (gp, gf, gc), gz = got
    (wp, wf, wc), wz = want
    assert gc == wc, tag
    assert gz == wz, tag
    for k in ("x", "y", "z2", "px", "py", "gam"):
        if exact:
            np.testing.assert_array_equal(gp[k], wp[k], err_msg=f"{tag} {k}")
        else:
            np.testing.assert_allclose(gp[k], wp[k], rtol=1e-5, atol=1e-8, err_msg=f"{tag} {k}")
    for a, b in zip(gf, wf):
        if exact:
            np.testing.assert_array_equal(a, b, err_msg=f"{tag} field")
        else:
            np.testing.assert_allclose(a, b, rtol=0, atol=1e-4 * np.max(np.abs(b)),
                                       err_msg=f"{tag} field")


def _batch_run(ws, graphs=True, tune=False, shape=None):
    sims = [_make(w) for w in ws]
    hs = np.array([w.h for w in ws])
    try:
        with P.Batch(sims) as b:
            b.use_graphs(graphs)
            if tune:
                b.tune(hs)
            if shape:
                b.set_shape(**shape)
            z, st = b.run(NSTEPS, EVERY, True, hs, raise_on_error=False)
            launches = b.kernel_launches
        res = [(_state(s), float(z[i])) for i, s in enumerate(sims)]
    finally:
        for s in sims:
            s.close()
    return res, st, launches


@pytest.mark.parametrize("graphs", [True, False])
def test_fp64_batch_matches_single_runs_bitwise(graphs):
    ws = _instances()
    want = _single(ws)
    got, st, launches = _batch_run(ws, graphs=graphs)
    assert np.all(st == 0)
    for i, (g, w) in enumerate(zip(got, want)):
        _assert_same(g, w, True, f"instance {i}")
    # one launch per stage kind and step (plus wraps), not per instance
    assert launches <= NSTEPS * (4 * 3 + 1)


def test_fp64_batch_shapes_keep_the_bits():
    ws = _instances(n=4, seed=11)
    want = _single(ws)
    for shape in ({"stage_tile": 256, "stage_grid": -1, "node_tile": 1024, "node_grid": -1},
                  {"stage_threads": 128, "stage_tile": 4096, "modes": [0, 0, 0, 0]},
                  {"modes": [2048, 0, 8192, 4096]}):
        if "modes" in shape and any(m > 0 for m in shape["modes"]):
            # shared-tile modes only where the instance's window fits the tile
            shape = dict(shape)
            shape["modes"] = [m if w.params.nx <= 17 else 0 for m, w in zip(shape["modes"], ws)]
        got, st, _ = _batch_run(ws, shape=shape)
        assert np.all(st == 0)
        for i, (g, w) in enumerate(zip(got, want)):
            _assert_same(g, w, True, f"{shape} instance {i}")


def test_fp64_batch_tuned():
    ws = _instances(n=5, seed=13)
    want = _single(ws)
    got, st, _ = _batch_run(ws, tune=True)
    assert np.all(st == 0)
    for i, (g, w) in enumerate(zip(got, want)):
        _assert_same(g, w, True, f"instance {i}")


def test_mixed_batch_matches_single_runs():
    ws = _instances(n=5, seed=17, precision=P.MIXED)
    want = _single(ws)
    got, st, _ = _batch_run(ws, tune=True)
    assert np.all(st == 0)
    for i, (g, w) in enumerate(zip(got, want)):
        _assert_same(g, w, False, f"instance {i}")


def test_window_replay_and_failure_isolation():
    """Instance 0 starts with a window smaller than its beam: its first block
    fails, is replayed step by step and redistributes (as pf_run does).
    Instance 1 has a macroparticle outside the mesh: it fails with
    PF_OUT_OF_WINDOW after the retries, and the others finish."""
    ws = _instances(n=4, seed=19)
    ws[0].params.nx = ws[0].params.ny = 65
    ws[0].params.dx = ws[0].params.dy = 0.2
    ws[0].params.nix = ws[0].params.niy = 9
    n1 = len(ws[1].field[0])
    ws[1].params.nix = ws[1].params.niy = 9
    ws[1].beam["x"][5] = 100.0
    for w in (ws[0], ws[1]):
        n = w.params.nx * w.params.ny * w.params.nz2
        w.field = (np.zeros(n), np.zeros(n))
    assert len(ws[1].field[0]) == n1
    with _make(ws[0]) as sim:
        assert sim.window == (9, 9)
        z = sim.und_section(NSTEPS, EVERY, True, ws[0].h)
        assert sim.window != (9, 9)
        want0 = (_state(sim), z)
    want = [want0, None] + _single(ws[2:])
    got, st, _ = _batch_run(ws)
    assert st[0] == 0 and st[2] == 0 and st[3] == 0
    assert st[1] == P.lib.PF_OUT_OF_WINDOW
    for i in (0, 2, 3):
        _assert_same(got[i], want[i], True, f"instance {i}")


def test_temporal_and_mixed_eager_batch():
    """A temporal-mesh instance (no wrap) beside periodic ones, FP64, and the
    mixed batch with direct launches instead of graphs."""
    ws = _instances(n=3, seed=23)
    t = ws[1]
    t.params.mesh_type = P.MESH_TEMPORAL
    # 128 planes (8 resonant wavelengths): the beam slips 1.25 wavelengths
    # forward in z2 over the 40 steps and must stay on the mesh
    t.params.nz2 = 129
    n = t.params.nx * t.params.ny * t.params.nz2
    t.field = (np.zeros(n), np.zeros(n))
    lz2 = (t.params.nz2 - 1) * t.params.dz2
    t.beam["z2"] = 0.1 * lz2 + 0.3 * lz2 * (t.beam["z2"] - t.beam["z2"].min()) / np.ptp(t.beam["z2"])
    want = _single(ws)
    got, st, _ = _batch_run(ws)
    assert np.all(st == 0)
    for i, (g, w) in enumerate(zip(got, want)):
        _assert_same(g, w, True, f"instance {i}")
    ws = _instances(n=4, seed=29, precision=P.MIXED)
    want = _single(ws)
    got, st, _ = _batch_run(ws, graphs=False)
    assert np.all(st == 0)
    for i, (g, w) in enumerate(zip(got, want)):
        _assert_same(g, w, False, f"instance {i}")


def _oracle_instances():
    """A sample of the batched form's own instance mixes: a 17^2 helical and a
    65^2 planepole periodic instance from the recipe, and a 33^2 instance of
    the recipe turned into a temporal mesh (its beam inside the mesh)."""
    ws = configs.config5(n_inst=48, seed=21, nsteps=NSTEPS, np_range=(2 ** 11, 2 ** 12))
    pick = {}
    for w in ws:
        key = (w.params.nx, w.params.und_type)
        if key == (33, P.UND_HELICAL) and w.params.nz2 - 1 != 128:
            continue   # the temporal one needs room for the 37-node z2 absorbing ends
        if key in ((17, P.UND_HELICAL), (65, P.UND_PLANEPOLE), (33, P.UND_HELICAL)) \
                and key not in pick:
            pick[key] = w
    assert len(pick) == 3
    t = pick[(33, P.UND_HELICAL)]
    p = t.params
    p.mesh_type = P.MESH_TEMPORAL
    p.nz2 = p.nz2 - 1
    lz2 = (p.nz2 - 1) * p.dz2
    t.beam["z2"] = 0.2 * lz2 + 0.6 * (t.beam["z2"] - t.beam["z2"].min()) / np.ptp(t.beam["z2"]) * lz2
    n = p.nx * p.ny * p.nz2
    t.field = (np.zeros(n), np.zeros(n))
    return [pick[(17, P.UND_HELICAL)], pick[(65, P.UND_PLANEPOLE)], t]


def test_batch_instances_match_the_oracle():
    """The batch against the oracle's UndSection (undulator.f90:106-331) on
    instances of the batched form's own mixes, at pf_run's single-instance
    tolerance (1e-9): the batch is checked against the restatement of the
    reference, not only against the library's own single-instance path."""
    from oracle import oracle as O
    from tests.oracle_bridge import assert_beam_close, oracle_beam, oracle_config
    ws = _oracle_instances()
    got, st, _ = _batch_run(ws)
    assert np.all(st == 0)
    for i, w in enumerate(ws):
        cfg = oracle_config(w.params)
        beam = oracle_beam(w.beam)
        rng = np.random.default_rng(int(w.np))
        n = len(w.field[0])
        re, im = 1e-3 * rng.standard_normal(n), 1e-3 * rng.standard_normal(n)   # as _make
        r = O.undulator_run(cfg, beam, re, im, w.h, NSTEPS, EVERY, True,
                            redist_every=w.params.redist_every)
        assert r.status == 0 and r.steps == NSTEPS, i
        (gp, (gfr, gfi), gc), gz = got[i]
        assert gc == r.csteps
        assert_beam_close(gp, beam, rtol=1e-9, atol=1e-12)
        scale = max(np.max(np.abs(re)), np.max(np.abs(im)))
        np.testing.assert_allclose(gfr, re, rtol=0, atol=1e-9 * scale, err_msg=f"instance {i}")
        np.testing.assert_allclose(gfi, im, rtol=0, atol=1e-9 * scale, err_msg=f"instance {i}")
