#!/usr/bin/env python
"""Benchmark of the Puffin hot path on GB300: macroparticle-RK4-steps/s.

Workload (default): the large FP64 drop-in configuration -- temporal mesh
129 x 129 x 4096 (complex FP64), planepole undulator, 2^23 macroparticles,
24 steps per period, diffraction every 8 steps.  One "step" is one RK4 step
over all macroparticles and the inner-window field, plus every 8th step the
merged diffraction call (dz = 8 h), exactly as UndSection schedules them.

* value  -- particle-steps/s with the state resident in HBM (CUDA events on
            the library's stream around K steps, after W warm-up steps);
* e2e    -- the same metric through the C ABI with host buffers, in the
            reference's data flow: every step copies the particles and the
            inner-window field (the arrays rk4par advances) in from pinned
            host memory and reads them back (pf_rk4_step_host, the copies
            overlapped with the step); around each diffraction call the
            outer field goes in and comes back as well (inner2Outer /
            diffractIM / outer2Inner);
* roofline -- the dominant kernel (the fused RK4 stage kernel) timed live
            with CUDA events; algorithmic bytes 104 B per particle per stage
            (416 B per particle-step over 4 stages);
* cpu_baseline -- the CPU restatement of the same step (oracle/), timed on the
            host cores on one diffraction block of the full workload (8 RK4
            steps and their diffraction call).

``--impl reference`` times the CPU implementation alone on the same workload
and schedule, W warm-up and K timed steps (the reference is Fortran + MPI +
FFTW-MPI + parallel HDF5 and cannot be built here, so the oracle
restatement stands in; the CUDA library is not loaded) and prints its own
line.

N > 1 (torchrun): the path does not shard here, so N independent
replicas run one per GPU ("replicas only"); value sums over ranks and the
time is the maximum over ranks.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "macroparticle-RK4-steps/s: mixed vs FP64 on GB300 at stated power error"
UNIT = "macroparticle-steps/s"
BYTES_PER_PARTICLE_STAGE = 104          # 56 B read + 48 B write (416 B per step)
# DRAM read + write of one FP64 stage launch per macroparticle, from one ncu
# capture of k_stage<3> on 2^22 macroparticles over 129 x 129 x 2048 planes
# (the config-2 density; the traffic grows with the macroparticles, the
# window field is mostly read from L2)
TRAFFIC_PER_PARTICLE_STAGE = 881.0e6 / 4194304
FLOPS_PER_PARTICLE_STAGE = 166          # ~664 FP64 flop per particle-step


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=48)
    ap.add_argument("--warmup", type=int, default=8)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--np", type=int, default=2 ** 23, help="macroparticles")
    ap.add_argument("--e2e-steps", type=int, default=48,
                    help="end-to-end steps (6 diffraction calls at the default cadence)")
    ap.add_argument("--nz2", type=int, default=4096,
                    help="z2 nodes of the mesh (smaller only for profiling captures)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-mixed", action="store_true", help="skip the mixed-precision leg")
    ap.add_argument("--np3", type=int, default=2 ** 24,
                    help="macroparticles of the mixed-vs-FP64 leg on the config-1 mesh (0: skip)")
    ap.add_argument("--steps3", type=int, default=32)
    ap.add_argument("--fidelity-np", type=int, default=2 ** 22,
                    help="macroparticles of the mixed-vs-FP64 run to saturation (0: skip)")
    ap.add_argument("--fidelity-steps", type=int, default=6000)
    ap.add_argument("--batch-n", type=int, default=128,
                    help="instances of the batched form (0: skip the leg)")
    ap.add_argument("--batch-steps", type=int, default=32)
    ap.add_argument("--batch-only", action="store_true",
                    help="run only the batched-form leg and print its record")
    ap.add_argument("--batch-precisions", default="fp64,mixed")
    ap.add_argument("--no-batch-single", action="store_true",
                    help="skip the one-at-a-time comparison of the batched form")
    ap.add_argument("--no-batch-tune", action="store_true",
                    help="batched form with the default shapes (persistent grids)")
    ap.add_argument("--no-dft-gemm", action="store_true",
                    help="skip the measurement of the transverse DFT as tensor-core GEMMs")
    ap.add_argument("--adjoint-steps", type=int, default=3000,
                    help="steps of the adjoint leg on the 33x33x128 periodic mesh (0: skip); "
                         "3000 is the adjoint form's full run")
    ap.add_argument("--adjoint-fd", default="3000:1e-6,3000:1e-7,1000:1e-6",
                    help="steps:step-size pairs of the adjoint's central-difference checks "
                         "('' : none)")
    return ap.parse_args()


# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(self.gpu)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)),
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# ---------------------------------------------------------------------------
def oracle_steps(w, steps, warmup):
    """The CPU restatement (oracle/) of the timed step on the whole workload,
    with the GPU arm's schedule: `warmup` untimed steps, then `steps` timed
    ones, each an rk4par step (the C + OpenMP restatement of rk4par/getrhs on
    every host core, with the reference's atomic deposit) and, every
    isteps4diff-th step, inner2Outer + the diffraction step (numpy
    restatement with scipy's threaded FFT) + outer2Inner over isteps4diff
    steps.  Wall-clock time around the timed steps; nothing is sampled or
    extrapolated.  A step whose macroparticle left the inner window is
    retried after the window is recomputed, as UndSection does."""
    from oracle import oracle as O
    from tests.oracle_bridge import oracle_beam, oracle_config

    cores = os.cpu_count() or 1
    O.set_threads(cores)
    fftmod = None
    try:
        import scipy.fft as sfft

        class _F:  # numpy.fft interface over scipy's threaded FFT
            @staticmethod
            def fftn(x):
                return sfft.fftn(x, workers=cores)

            @staticmethod
            def ifftn(x):
                return sfft.ifftn(x, workers=cores)
        fftmod = _F
    except Exception:
        pass
    p = w.params
    cfg = oracle_config(p)
    beam = oracle_beam(w.beam)
    re, im = (np.array(a, dtype=np.float64) for a in w.field)
    st = {"win": O.get_in_node(cfg, beam.x, beam.y), "szl": 0.0, "i": 0, "diff": 0,
          "retries": 0}
    st["w"] = O.outer_to_inner(cfg, re, im, *st["win"])
    taper = O.Taper(p.n2col0, p.n2col0, p.undgrad)

    def step():
        for _ in range(4):
            t = O.Taper(taper.n2col, taper.n2col0, taper.undgrad)
            rc = O.rk4_step(cfg, taper, st["szl"], w.h, beam, *st["w"], *st["win"])
            if rc == 0:
                break
            if rc & 2:
                raise RuntimeError("oracle: a macroparticle left the temporal mesh")
            taper.update(t)
            st["retries"] += 1
            O.inner_to_outer(cfg, re, im, *st["w"], *st["win"])
            st["win"] = O.get_in_node(cfg, beam.x, beam.y)
            st["w"] = O.outer_to_inner(cfg, re, im, *st["win"])
        else:
            raise RuntimeError("oracle: the window retries did not hold the beam")
        st["szl"] += w.h
        st["i"] += 1
        if w.qdiffraction and st["i"] % w.isteps4diff == 0:
            O.inner_to_outer(cfg, re, im, *st["w"], *st["win"])
            O.diffract(cfg, re, im, w.isteps4diff * w.h, fft=fftmod)
            st["w"] = O.outer_to_inner(cfg, re, im, *st["win"])
            st["diff"] += 1

    for _ in range(warmup):
        step()
    d0 = st["diff"]
    t0 = time.perf_counter()
    for _ in range(steps):
        step()
    sec = time.perf_counter() - t0
    return {"seconds": sec, "steps": steps, "warmup": warmup, "cores": cores,
            "diffraction_calls": st["diff"] - d0, "retries": st["retries"],
            "window": [int(v) for v in st["win"]], "value": w.np * steps / sec}


def cpu_baseline(w):
    """The oracle on one diffraction block of the workload (one warm-up step,
    then the next isteps4diff steps with their diffraction call) on the host
    cores: a bounded sample of the same work, timed as it is (no
    extrapolation)."""
    r = oracle_steps(w, w.isteps4diff, 1)
    return {
        "value": r["value"], "unit": UNIT, "cores": r["cores"], "kind": "port",
        "sample": (f"CPU restatement (oracle/: C+OpenMP RK4 on {r['cores']} threads, numpy "
                   f"diffraction with scipy's threaded FFT) on the full workload "
                   f"({w.np} macroparticles, full mesh): {r['steps']} RK4 steps and "
                   f"{r['diffraction_calls']} diffraction call after 1 warm-up step, "
                   f"{r['seconds']:.2f} s"),
    }


def workload_config(w, win, world):
    """The `config` of both arms' lines (the same keys and values)."""
    p = w.params
    return {
        "workload": w.name, "macroparticles": w.np, "mesh": [p.nx, p.ny, p.nz2],
        "inner_window": [int(v) for v in win], "steps_per_period": 24,
        "diffraction_every": w.isteps4diff,
        "precision": "fp64 (value); mixed in 'mixed'",
        "parallelism": f"replicas x{world}",
        "l2": "inputs larger than L2 (particle state 470 MB, field 1.09 GB per array pair)",
    }


# ---------------------------------------------------------------------------
def _time_path(args, dev, precision, world, workload="config2", steps=None, warmup=None,
               fft_arithmetic=None):
    """Run a workload on one precision path: W warm-up steps, then K timed
    steps (CUDA events on the library's stream).  Returns timings, the
    per-kernel-class device times, the final radiated power sum |A|^2 and the
    diagnostics (power per z2 plane, |b1| per slice, on-axis spectrum)."""
    import torch

    import puffin_gb300 as P
    from puffin_gb300 import configs
    from puffin_gb300 import lib as L

    steps = args.steps if steps is None else steps
    warmup = args.warmup if warmup is None else warmup
    if workload == "config2":
        w = configs.config2(np_=args.np, nz2=args.nz2)
    else:
        w = configs.config3(np_=args.np3)
    p = w.params
    p.device = dev
    p.precision = precision
    sim = P.Puffin(p)
    if fft_arithmetic is not None:
        sim.set_fft_arithmetic(fft_arithmetic)
    sim.set_particles(*(w.beam[k] for k in P.PARTICLE_KEYS))
    sim.set_field(*w.field)
    win = sim.window
    stream = torch.cuda.ExternalStream(sim.stream_handle, device=dev)
    every = w.isteps4diff
    state = {"szl": 0.0, "i": 0}

    def step():
        ok = sim.rk4par(state["szl"], w.h)
        if not ok:                      # reference behaviour: redistribute and retry
            sim.redistribute()
            ok = sim.rk4par(state["szl"], w.h)
            assert ok
        state["szl"] += w.h
        state["i"] += 1
        if state["i"] % every == 0:
            sim.diffractIM(every * w.h)   # merged end + start half steps

    for _ in range(warmup):
        step()
    sim.sync()
    if world > 1:
        torch.distributed.barrier()
    sim.profile(True)
    launches0 = sim.kernel_launches
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(dev) as clk:
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(steps):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
    ms = e0.elapsed_time(e1)
    out = {
        "w": w, "sim": sim, "step": step, "state": state, "stream": stream, "win": win, "ms": ms,
        "launches": sim.kernel_launches - launches0, "clocks": clk.summary(),
        "kernel": {name: sim.profile_read(cls) for name, cls in
                   (("stage", L.PROF_STAGE), ("nodes", L.PROF_NODES), ("fft", L.PROF_FFT),
                    ("diff_elementwise", L.PROF_DIFF))},
    }
    sim.profile(False)
    fr, fi = sim.get_field()
    out["power"] = float(np.sum(fr * fr + fi * fi))
    out["diag"] = {"power_z": sim.power(), "b1": sim.bunching(1), "spectrum": sim.spectrum()[0]}
    out["steps"], out["warmup"] = steps, warmup
    return out


def output_errors(r64, rmx):
    """Error of the mixed path against the FP64 path per output: power vs z
    (max |dP| over max P), |b1| per slice (max absolute difference) and the
    on-axis spectrum (relative L2 error)."""
    d64, dmx = r64["diag"], rmx["diag"]
    pz64, pzmx = d64["power_z"], dmx["power_z"]
    s64, smx = d64["spectrum"], dmx["spectrum"]
    return {
        "total_power_rel": abs(rmx["power"] - r64["power"]) / max(r64["power"], 1e-300),
        "power_vs_z_max_rel": float(np.max(np.abs(pzmx - pz64)) / max(np.max(pz64), 1e-300)),
        "b1_max_abs": float(np.max(np.abs(dmx["b1"] - d64["b1"]))),
        "b1_max_fp64": float(np.max(d64["b1"])),
        "spectrum_rel_l2": float(np.linalg.norm(smx - s64) / max(np.linalg.norm(s64), 1e-300)),
        "after_steps": r64["warmup"] + r64["steps"],
    }


def max_over_ranks(values, world, device=None):
    """Element-wise maximum over the ranks of a list of times (the slowest
    rank sets the job's time); with one process the values come back as
    they are.  The reduction runs on `device` (the GPU under NCCL; the host
    under gloo)."""
    if world <= 1:
        return [float(v) for v in values]
    import torch
    import torch.distributed as dist
    if device is None or dist.get_backend() == "gloo":
        device = "cpu"
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.cpu()]


def whole_job_rate(units_per_rank, steps, world, ms):
    """Whole-job throughput: the units every rank processed per step, times
    the ranks and the steps, over the (maximum) time."""
    return world * units_per_rank * steps / (ms * 1e-3)


def adjoint_leg(args, dev):
    """The adjoint form: periodic 33 x 33 x 128 mesh (129 nodes, 128 unique
    planes), 2^18 macroparticles, Gaussian seed of waist 1.0 on the resonant
    carrier at power 1e-3 of saturation (|A|^2 of about 1 in the scaled
    units), a 16-point taper profile, checkpoints every 64 steps; the forward
    run with checkpoints, then the backward pass (recompute + adjoint), timed
    with CUDA events on the library's stream.  Then the gradient against
    central finite differences with steps of 1e-6 (relative for the seed
    amplitude, absolute for the taper points and the chirp) on all 18
    components, at the horizons and step sizes of --adjoint-fd (two step
    sizes at one horizon show how far the differences themselves have
    converged)."""
    import torch

    import puffin_gb300 as P
    from puffin_gb300 import configs

    w = configs.config4(np_=2 ** 18, nsteps=args.adjoint_steps)
    p = w.params
    p.device = dev
    nx, ny, nz2 = p.nx, p.ny, p.nz2
    xs = (np.arange(nx) - (nx - 1) / 2) * p.dx
    ys = (np.arange(ny) - (ny - 1) / 2) * p.dy
    g = np.exp(-(xs[None, :] ** 2 + ys[:, None] ** 2) / 2.0).ravel()
    ph = np.arange(nz2) * p.dz2 / (2.0 * p.rho)
    seed = ((np.cos(ph)[:, None] * g[None, :]).ravel(), (np.sin(ph)[:, None] * g[None, :]).ravel())
    amp, chirp = math.sqrt(1e-3), 0.0
    out = {}
    with P.Puffin(p) as sim:
        sim.set_particles(*(w.beam[k] for k in P.PARTICLE_KEYS))
        stream = torch.cuda.ExternalStream(sim.stream_handle, device=dev)

        def energy(nsteps, alpha, a, c):
            sim.set_taper_profile(np.linspace(0.0, nsteps * w.h, 16), alpha)
            return sim.adjoint_forward(nsteps, w.isteps4diff, True, w.h, 64, seed[0], seed[1],
                                       a, c)

        alpha0 = np.ones(16)
        energy(w.nsteps, alpha0, amp, chirp)        # warm-up (plans, allocations)
        sim.adjoint_backward(16)
        e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        torch.cuda.synchronize()
        e[0].record(stream)
        e0 = energy(w.nsteps, alpha0, amp, chirp)
        e[1].record(stream)
        gt, gs, gc = sim.adjoint_backward(16)
        e[2].record(stream)
        torch.cuda.synchronize()
        fwd, bwd = e[0].elapsed_time(e[1]), e[1].elapsed_time(e[2])
        out = {
            "workload": w.name, "macroparticles": w.np, "mesh": [nx, ny, nz2],
            "steps": w.nsteps, "checkpoint_every": 64, "seed_amplitude": amp,
            "forward_ms": fwd, "backward_ms": bwd, "backward_over_forward": bwd / fwd,
            "energy": e0, "grad_seed_amp": gs, "grad_chirp": gc,
            "grad_taper_norm": float(np.linalg.norm(gt)),
        }
        def differences(nsteps, d):
            num = []
            for k in range(18):
                if k < 16:
                    ap, am = alpha0.copy(), alpha0.copy()
                    ap[k] += d
                    am[k] -= d
                    num.append((energy(nsteps, ap, amp, chirp) - energy(nsteps, am, amp, chirp))
                               / (2 * d))
                elif k == 16:
                    da = d * amp
                    num.append((energy(nsteps, alpha0, amp + da, chirp)
                                - energy(nsteps, alpha0, amp - da, chirp)) / (2 * da))
                else:
                    num.append((energy(nsteps, alpha0, amp, chirp + d)
                                - energy(nsteps, alpha0, amp, chirp - d)) / (2 * d))
            return np.array(num)

        checks = []
        for spec in [v for v in args.adjoint_fd.split(",") if v.strip()]:
            nsteps, d = (int(spec.split(":")[0]), float(spec.split(":")[1]))
            t0 = time.perf_counter()
            energy(nsteps, alpha0, amp, chirp)
            g_t, g_s, g_c = sim.adjoint_backward(16)
            adj = np.array(list(g_t) + [g_s, g_c])
            num = differences(nsteps, d)
            big = np.abs(num) >= 1e-3 * np.max(np.abs(num))
            rel = np.abs(adj - num) / np.maximum(np.abs(num), 1e-300)
            checks.append({
                "steps": nsteps, "zbar": nsteps * w.h, "fd_step": d,
                "max_rel_error": float(np.max(rel[big])),
                "within_1e-4": bool(np.max(rel[big]) <= 1e-4),
                "components_checked": int(np.count_nonzero(big)),
                "rel_error": [float(v) for v in rel],
                "adjoint": [float(v) for v in adj], "differences": [float(v) for v in num],
                "seconds": time.perf_counter() - t0,
            })
        # the differences' own convergence where two step sizes ran at one horizon
        for a in checks:
            for b in checks:
                if a["steps"] == b["steps"] and a["fd_step"] > b["fd_step"]:
                    na, nb = np.array(a["differences"]), np.array(b["differences"])
                    big = np.abs(nb) >= 1e-3 * np.max(np.abs(nb))
                    spread = np.abs(na - nb) / np.maximum(np.abs(nb), 1e-300)
                    a.setdefault("fd_spread_vs_smaller_step", float(np.max(spread[big])))
        out["finite_difference_checks"] = checks
        out["fd_note"] = ("central differences with the stated step (seed amplitude: relative "
                          "to the amplitude); components below 1e-3 of the largest are listed "
                          "but not counted; fd_spread_vs_smaller_step is the largest relative "
                          "change of the differences themselves between the two step sizes")

    # the same run on a mixed-precision handle: the recorded forward runs the
    # mixed stage kernels and the FP32 diffraction, the adjoint keeps their
    # precision split; its gradient is checked against the FP64 forward's
    # differences above (a step of 1e-6 of a taper value is below the FP32
    # resolution of the mixed coefficients)
    pm = P.Params.from_buffer_copy(p)
    pm.precision = P.MIXED
    with P.Puffin(pm) as sim:
        sim.set_particles(*(w.beam[k] for k in P.PARTICLE_KEYS))
        stream = torch.cuda.ExternalStream(sim.stream_handle, device=dev)

        def energy_m(nsteps, alpha, a, c):
            sim.set_taper_profile(np.linspace(0.0, nsteps * w.h, 16), alpha)
            return sim.adjoint_forward(nsteps, w.isteps4diff, True, w.h, 64, seed[0], seed[1],
                                       a, c)

        energy_m(w.nsteps, alpha0, amp, chirp)      # warm-up
        sim.adjoint_backward(16)
        e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        torch.cuda.synchronize()
        e[0].record(stream)
        em = energy_m(w.nsteps, alpha0, amp, chirp)
        e[1].record(stream)
        sim.adjoint_backward(16)
        e[2].record(stream)
        torch.cuda.synchronize()
        mfwd, mbwd = e[0].elapsed_time(e[1]), e[1].elapsed_time(e[2])
        mixed = {
            "forward_ms": mfwd, "backward_ms": mbwd, "backward_over_forward": mbwd / mfwd,
            "forward_speedup_vs_fp64": fwd / mfwd, "backward_speedup_vs_fp64": bwd / mbwd,
            "energy": em, "energy_rel_vs_fp64": abs(em - e0) / abs(e0),
        }
        vs = []
        for chk in checks:
            energy_m(chk["steps"], alpha0, amp, chirp)
            g_t, g_s, g_c = sim.adjoint_backward(16)
            adj = np.array(list(g_t) + [g_s, g_c])
            num = np.array(chk["differences"])
            a64 = np.array(chk["adjoint"])
            big = np.abs(num) >= 1e-3 * np.max(np.abs(num))
            rel = np.abs(adj - num) / np.maximum(np.abs(num), 1e-300)
            rel64 = np.abs(adj - a64) / np.maximum(np.abs(a64), 1e-300)
            vs.append({
                "steps": chk["steps"], "fd_step": chk["fd_step"],
                "max_rel_error_vs_fp64_differences": float(np.max(rel[big])),
                "within_1e-4": bool(np.max(rel[big]) <= 1e-4),
                "max_rel_diff_vs_fp64_adjoint": float(np.max(rel64[big])),
                "adjoint": [float(v) for v in adj],
            })
        mixed["finite_difference_checks"] = vs
    out["mixed"] = mixed
    return out


def fidelity_leg(args, dev):
    """The mixed form's physics targets: the config-1 mesh (periodic
    helical 21 x 21 x 64, rho 0.005, gamma_r 500) at args.fidelity_np
    macroparticles run to saturation in FP64 and in mixed precision from the
    same beam, the pulse energy sampled every 16 steps; the power gain length
    of the exponential regime (fit of ln E between 1e-3 and 1e-1 of the
    saturated energy) and the saturated energy (top of the first synchrotron
    oscillation) of the mixed run against the FP64 run."""
    import puffin_gb300 as P
    from puffin_gb300 import configs, fel

    curves = {}
    t = {}
    for name, prec in (("fp64", P.FP64), ("mixed", P.MIXED)):
        w = configs.config1(np_=args.fidelity_np, nsteps=args.fidelity_steps)
        w.params.precision = prec
        w.params.device = dev
        t0 = time.perf_counter()
        curves[name] = fel.power_curve(w.params, w.beam, w.field, w.h, args.fidelity_steps,
                                       timings=True)
        t[name] = time.perf_counter() - t0
    z = curves["fp64"][0]
    cmp = fel.compare(z, curves["fp64"][1], curves["mixed"][1])
    # time per step over the whole run and over its last 10 % (the
    # saturated, bunched beam), wall clock around each 16-step call
    nlast = max(1, len(z) // 10)
    per_step = {}
    for name in ("fp64", "mixed"):
        ts = curves[name][2]
        per_step[name] = {"all_ms": 1e3 * float(ts.sum()) / (16 * len(ts)),
                          "first_10pct_ms": 1e3 * float(ts[:nlast].sum()) / (16 * nlast),
                          "last_10pct_ms": 1e3 * float(ts[-nlast:].sum()) / (16 * nlast)}
    return {
        "workload": "config-1 mesh run to saturation (periodic helical 21x21x64, rho 0.005)",
        "macroparticles": args.fidelity_np, "steps": args.fidelity_steps,
        "zbar_end": float(z[-1]), "sample_every_steps": 16,
        "reference": "FP64 path (the oracle's GPU twin)",
        "gain_length": cmp["gain_length"], "saturated_energy": cmp["saturated_energy"],
        "max_energy": cmp["max_energy"],
        "targets": {"gain_length_rel": 5e-3, "saturated_power_rel": 1e-2},
        "within_targets": bool(abs(cmp["gain_length"]["rel_diff"]) <= 5e-3
                               and abs(cmp["saturated_energy"]["rel_diff"]) <= 1e-2),
        "ms_per_step": per_step,
        "speedup_mixed_vs_fp64": {
            "all": per_step["fp64"]["all_ms"] / per_step["mixed"]["all_ms"],
            "last_10pct": per_step["fp64"]["last_10pct_ms"] / per_step["mixed"]["last_10pct_ms"]},
        "macroparticle_steps_per_s_last_10pct": {
            k: args.fidelity_np / (1e-3 * v["last_10pct_ms"]) for k, v in per_step.items()},
        "wall_seconds": t,
    }


def dft_gemm_leg(args, dev, fft_call_ms):
    """The transverse 129-point DFT as a matrix product on the tensor cores,
    measured beside the butterfly kernels of the mixed path (a measurement,
    not a product path): the x transform of every row of the config-2
    complex-float mesh (129 * nz2 rows of 129 interleaved complex values,
    a real matrix of 258 columns) times the real form of the forward DFT
    matrix (258 x 258), in TF32 with the split-precision scheme that keeps
    FP32 accuracy (hi*hi + lo*hi + hi*lo, three products; hi keeps the
    operand's top 10 significand bits, lo the rest), through cuBLAS.
    Timed on the mesh's own layout (row stride 1032 bytes), on rows padded
    to 264 columns, and on a 64-plane slice that stays in L2 (the tensor
    rate for this shape); the error is against an FP64 product on sample
    rows.  A 2D transform is two such products (x and y, the same work)."""
    import torch

    d = f"cuda:{dev}"
    nx = 129
    n2 = 2 * nx
    nrow = nx * args.nz2
    gen = torch.Generator(device=d)
    gen.manual_seed(5)
    x = 1e-3 * torch.randn(nrow, n2, device=d, generator=gen)
    kk = torch.arange(nx, dtype=torch.float64)
    th = 2.0 * math.pi * torch.outer(kk, kk) / nx
    c, s = torch.cos(th), torch.sin(th)
    b64 = torch.empty(n2, n2, dtype=torch.float64)
    b64[0::2, 0::2] = c   # x_re -> y_re
    b64[1::2, 0::2] = s   # x_im -> y_re
    b64[0::2, 1::2] = -s  # x_re -> y_im
    b64[1::2, 1::2] = c   # x_im -> y_im
    b64 = b64.to(d)
    b32 = b64.to(torch.float32)

    def split(t):
        hi = (t.view(torch.int32) & -8192).view(torch.float32)  # low 13 bits cleared
        return hi, t - hi

    def three(xh, xl, bh, bl, y):
        torch.matmul(xh, bh, out=y)
        y.addmm_(xl, bh)
        y.addmm_(xh, bl)

    def timed(fn, reps):
        fn()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    old_tf32 = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = True
    try:
        out = {}
        bh, bl = split(b32)
        xh, xl = split(x)
        y = torch.empty(nrow, n2, device=d)
        flops = 3 * 2.0 * nrow * n2 * n2
        t = timed(lambda: three(xh, xl, bh, bl, y), 5)
        out["mesh_layout"] = {"ms": t, "tflops": flops / (t * 1e-3) / 1e12}
        # accuracy on sample rows against an FP64 product
        ns = 4096
        ref = x[:ns].double() @ b64
        scale = ref.abs().max().item()
        err3 = (y[:ns].double() - ref).abs().max().item() / scale
        err1 = ((x[:ns] @ b32).double() - ref).abs().max().item() / scale
        # padded rows (a 16-byte multiple stride): the library's best case
        pad = 264
        xp = torch.zeros(nrow, pad, device=d)
        xp[:, :n2] = x
        bp = torch.zeros(pad, pad, device=d)
        bp[:n2, :n2] = b32
        del xh, xl, y
        bph, bpl = split(bp)
        xph, xpl = split(xp)
        yp = torch.empty(nrow, pad, device=d)
        t = timed(lambda: three(xph, xpl, bph, bpl, yp), 5)
        out["padded_264"] = {"ms": t, "tflops": flops / (t * 1e-3) / 1e12}
        # 256 planes: 33,024 rows, 105 MB of operands and result, in L2
        m = nx * min(256, args.nz2)
        xs_h, xs_l, ys = xph[:m].contiguous(), xpl[:m].contiguous(), yp[:m].contiguous()
        t = timed(lambda: three(xs_h, xs_l, bph, bpl, ys), 50)
        fl = 3 * 2.0 * m * n2 * n2
        out["l2_resident_256_planes"] = {"ms": t, "tflops": fl / (t * 1e-3) / 1e12}
        del xp, xph, xpl, yp
    finally:
        torch.backends.cuda.matmul.allow_tf32 = old_tf32
    best = min(out["mesh_layout"]["ms"], out["padded_264"]["ms"])
    out.update({
        "what": "x transform of the 129x129x%d complex-float mesh as three TF32 GEMMs "
                "(%d x 258 by 258 x 258, split precision) in cuBLAS" % (args.nz2, nrow),
        "rel_error_three_products": err3,
        "rel_error_one_tf32_product": err1,
        "per_2d_transform_ms": 2 * best,
        "butterfly_fft_call_ms": fft_call_ms,
        "butterfly_note": "the mixed diffraction call runs four 2D transforms of this mesh "
                          "(three passes of the in-place plane kernel) and its z2 passes in "
                          "butterfly_fft_call_ms",
    })
    del x
    torch.cuda.empty_cache()
    return out


def batch_leg(args, dev):
    """The batched form: args.batch_n independent periodic single-slice
    instances (macroparticles log-uniform in [2^14, 2^20], meshes
    {17, 33, 65}^2 x {32, 64, 128}, rho, detuning, aw and undulator type drawn
    from the seed), 32 steps per period, diffraction every 16 steps.  Per
    precision: every instance alone through pf_run (its CUDA-graph blocks),
    then all of them as one batch (autotuned), each for args.batch_steps
    steps after a 16-step warm-up; wall-clock time around each, both ending
    with the device idle.  The state continues from one timing to the next
    (the rate does not depend on it)."""
    import torch

    import puffin_gb300 as P
    from puffin_gb300 import configs

    ws = configs.config5(n_inst=args.batch_n, nsteps=args.batch_steps)
    total = sum(w.np for w in ws)
    out = {"workload": f"{len(ws)} periodic single-slice instances (batched form)",
           "instances": len(ws), "macroparticles_total": total,
           "macroparticles_min": min(w.np for w in ws), "macroparticles_max": max(w.np for w in ws),
           "steps": args.batch_steps, "warmup_steps": 16, "diffraction_every": 16,
           "timing": "wall clock around the run calls (host and device)", "unit": UNIT}
    launches = 0
    precs = {"fp64": P.FP64, "mixed": P.MIXED}
    for name in args.batch_precisions.split(","):
        prec = precs[name]
        sims = []
        try:
            for w in ws:
                w.params.precision = prec
                w.params.device = dev
                sim = P.Puffin(w.params)
                sim.set_particles(*(w.beam[k] for k in P.PARTICLE_KEYS))
                sims.append(sim)
            hs = np.array([w.h for w in ws])
            z = np.zeros(len(ws))
            t_single = None
            if not args.no_batch_single:
                for i, sim in enumerate(sims):        # warm-up: plans, graphs
                    z[i] = sim.und_section(16, 16, True, ws[i].h, z[i])
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                for i, sim in enumerate(sims):
                    z[i] = sim.und_section(args.batch_steps, 16, True, ws[i].h, z[i])
                torch.cuda.synchronize()
                t_single = time.perf_counter() - t0
                launches += sum(s.kernel_launches for s in sims)
            with P.Batch(sims) as b:
                t0 = time.perf_counter()
                if args.no_batch_tune:
                    b.set_shape(stage_grid=-1, node_grid=-1)
                    shape = b.shape()
                else:
                    shape = b.tune(hs, z)
                t_tune = time.perf_counter() - t0
                z, _ = b.run(16, 16, True, hs, z)   # warm-up: graph capture
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                z, _ = b.run(args.batch_steps, 16, True, hs, z)
                torch.cuda.synchronize()
                t_batch = time.perf_counter() - t0
                launches += b.kernel_launches
            modes = shape.pop("modes")
            out[name] = {
                "one_at_a_time": None if t_single is None else {
                    "value": total * args.batch_steps / t_single,
                    "ms_per_step": 1e3 * t_single / args.batch_steps},
                "batched": {"value": total * args.batch_steps / t_batch,
                            "ms_per_step": 1e3 * t_batch / args.batch_steps},
                "speedup": None if t_single is None else t_single / t_batch,
                "tuned_shape": shape,
                "tuned_modes": {str(int(m)): int(c) for m, c in zip(*np.unique(modes, return_counts=True))},
                "tune_seconds": t_tune,
            }
        finally:
            for s in sims:
                s.close()
    out["gpu_launches"] = launches
    return out


def e2e_run(r, args, world):
    """The step loop end to end through the C ABI with host buffers, in
    UndSection's data flow, continuing the state of the timed leg r: every
    step hands in the six evolving particle arrays (chi, which rk4par never
    changes, stays the handle's) and the inner-window field (the arrays
    rk4par advances) from pinned host memory and takes them back, in one
    pf_rk4_step_host call that overlaps the copies with the step; every 8th
    step inner2Outer + diffractIM + outer2Inner take the outer field and the
    window in and back in one pf_diffract_host call, the outer field's copies
    overlapped with the transforms (a mixed handle converts the FP64 arrays
    to and from its complex-float field on the device).  CUDA events on the
    library's stream around args.e2e_steps steps, after one untimed block of
    steps with its diffraction call."""
    import torch

    import puffin_gb300 as P
    from puffin_gb300 import lib as L

    w, sim, state, stream = r["w"], r["sim"], r["state"], r["stream"]
    every = w.isteps4diff
    n = w.np
    pin = {k: torch.empty(n, dtype=torch.float64, pin_memory=True).numpy() for k in P.PARTICLE_KEYS}
    fre = torch.empty(sim.n_outer, dtype=torch.float64, pin_memory=True).numpy()
    fim = torch.empty(sim.n_outer, dtype=torch.float64, pin_memory=True).numpy()
    cur = sim.get_particles()
    for k in P.PARTICLE_KEYS:
        pin[k][:] = cur[k]
    r_, i_ = sim.get_field()
    fre[:] = r_
    fim[:] = i_
    lib = L.load()
    ptrs = [pin[k].ctypes.data for k in P.PARTICLE_KEYS]
    nw = sim.n_window
    wre = torch.empty(nw, dtype=torch.float64, pin_memory=True).numpy()
    wim = torch.empty(nw, dtype=torch.float64, pin_memory=True).numpy()
    assert lib.pf_get_window_field(sim._h, wre.ctypes.data, wim.ctypes.data) == 0
    n_diff = 0
    window_changes = 0
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    # wall time per call class (every call returns with its work done)
    parts = {"step_host": 0.0, "diffract": 0.0}
    # one block of steps with its diffraction call untimed first: the fresh
    # pinned host buffers' first copies and the calls' one-time work
    n_warm = every if args.e2e_steps > 0 else 0
    for it in range(n_warm + max(0, args.e2e_steps)):
        if it == n_warm:
            torch.cuda.synchronize()
            if world > 1:
                torch.distributed.barrier()
            n_diff = 0
            window_changes = 0
            parts = {k: 0.0 for k in parts}
            t0.record(stream)
        diff = (state["i"] + 1) % every == 0
        tq = time.perf_counter()
        rc = lib.pf_rk4_step_host(sim._h, state["szl"], w.h, *ptrs[:6], wre.ctypes.data,
                                  wim.ctypes.data)
        if rc == L.PF_OUT_OF_WINDOW:
            # the reference's retry: a new window from the particles (the
            # arrays came back as they went in), read back at its size
            assert lib.pf_redistribute(sim._h) == 0
            nw = lib.pf_window_nodes(sim._h)
            wre = torch.empty(nw, dtype=torch.float64, pin_memory=True).numpy()
            wim = torch.empty(nw, dtype=torch.float64, pin_memory=True).numpy()
            assert lib.pf_get_window_field(sim._h, wre.ctypes.data, wim.ctypes.data) == 0
            window_changes += 1
            rc = lib.pf_rk4_step_host(sim._h, state["szl"], w.h, *ptrs[:6], wre.ctypes.data,
                                      wim.ctypes.data)
        assert rc == 0, rc
        tr = time.perf_counter()
        parts["step_host"] += tr - tq
        state["szl"] += w.h
        state["i"] += 1
        if diff:
            assert lib.pf_diffract_host(sim._h, every * w.h, fre.ctypes.data, fim.ctypes.data,
                                        wre.ctypes.data, wim.ctypes.data) == 0
            n_diff += 1
        parts["diffract"] += time.perf_counter() - tr
    if args.e2e_steps <= 0:
        t0.record(stream)
    t1.record(stream)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    k_e2e = max(1, args.e2e_steps)
    h2d = (6 * 8 * n + 2 * 8 * nw) + (2 * 8 * sim.n_outer + 2 * 8 * nw) * n_diff / k_e2e
    d2h = (6 * 8 * n + 2 * 8 * nw) + (2 * 8 * sim.n_outer + 2 * 8 * nw) * n_diff / k_e2e
    return {"ms": max(t0.elapsed_time(t1), 1e-9), "h2d": h2d, "d2h": d2h, "n_diff": n_diff,
            "window_changes": window_changes, "nw": nw,
            "parts": {k: 1e3 * v / k_e2e for k, v in parts.items()}}


def run_gpu(args, rank, world):
    import torch

    import puffin_gb300 as P
    from puffin_gb300 import lib as L

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    r64 = _time_path(args, dev, P.FP64, world)
    w, sim, step, stream, win = r64["w"], r64["sim"], r64["step"], r64["stream"], r64["win"]
    p = w.params
    ms = r64["ms"]
    every = w.isteps4diff

    n = w.np
    e2e = e2e_run(r64, args, world)
    e2e_ms, h2d, d2h = e2e["ms"], e2e["h2d"], e2e["d2h"]
    e2e_diff_calls, window_changes, e2e_parts = e2e["n_diff"], e2e["window_changes"], e2e["parts"]
    nw = e2e["nw"]
    sim.close()

    # the same FP64 leg with the diffraction FFTs in FP64 arithmetic (the
    # default transforms in paired FP32, pf_set_fft_arithmetic)
    r64f = _time_path(args, dev, P.FP64, world, fft_arithmetic=L.FFT_FP64)
    r64f["sim"].close()
    (r64f_ms,) = max_over_ranks([r64f["ms"]], world, f"cuda:{dev}")

    rmx = None
    e2e_mx = None
    c3 = None
    if not args.no_mixed:
        rmx = _time_path(args, dev, P.MIXED, world)
        e2e_mx = e2e_run(rmx, args, world) if args.e2e_steps > 0 else None
        rmx["sim"].close()
        if args.np3 > 0:
            c3 = {}
            for name, prec in (("fp64", P.FP64), ("mixed", P.MIXED)):
                c3[name] = _time_path(args, dev, prec, world, "config3", args.steps3, args.warmup)
                c3[name]["sim"].close()

    dgemm = None
    if rmx and not args.no_dft_gemm:
        every_mx = rmx["w"].isteps4diff
        calls = sum(1 for i in range(args.warmup + 1, args.warmup + args.steps + 1)
                    if i % every_mx == 0)
        dgemm = dft_gemm_leg(args, dev, rmx["kernel"]["fft"][0] / max(1, calls))

    # the forms that hold many buffers run last
    fid = fidelity_leg(args, dev) if args.fidelity_np > 0 and not args.no_mixed else None
    adj = adjoint_leg(args, dev) if args.adjoint_steps > 0 else None
    bat = batch_leg(args, dev) if args.batch_n > 0 else None
    if rmx and e2e_mx:
        (e2e_mx["ms"],) = max_over_ranks([e2e_mx["ms"]], world, f"cuda:{dev}")
    ms, e2e_ms, mx_ms, c3_64_ms, c3_mx_ms = max_over_ranks(
        [ms, e2e_ms, rmx["ms"] if rmx else 0.0, c3["fp64"]["ms"] if c3 else 0.0,
         c3["mixed"]["ms"] if c3 else 0.0], world, f"cuda:{dev}")
    if rank != 0:
        return None

    value = whole_job_rate(n, args.steps, world, ms)
    e2e_value = whole_job_rate(n, args.e2e_steps, world, e2e_ms) if args.e2e_steps > 0 else None
    peak, peak_kind = measured_peaks()
    stage_ms, stage_n = r64["kernel"]["stage"]
    stage_avg = stage_ms / max(1, stage_n)
    achieved = n * BYTES_PER_PARTICLE_STAGE / (stage_avg * 1e-3) / 1e9
    # FP64 peak of this GPU, measured with a cuBLAS DGEMM
    a = torch.randn(4096, 4096, dtype=torch.float64, device=f"cuda:{dev}")
    torch.matmul(a, a)
    torch.cuda.synchronize()
    g0 = torch.cuda.Event(enable_timing=True)
    g1 = torch.cuda.Event(enable_timing=True)
    g0.record()
    for _ in range(3):
        torch.matmul(a, a)
    g1.record()
    torch.cuda.synchronize()
    dgemm_tflops = 3 * 2 * 4096 ** 3 / (g0.elapsed_time(g1) * 1e-3) / 1e12
    fp64_achieved = n * FLOPS_PER_PARTICLE_STAGE / (stage_avg * 1e-3) / 1e12
    kern = {k: v[0] for k, v in r64["kernel"].items()}
    kern.update({k + "_launches": v[1] for k, v in r64["kernel"].items()})
    rec = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded beam and zero seed field; no dataset)",
        "config": workload_config(w, win, world),
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "steps": args.e2e_steps,
                "diffraction_calls": e2e_diff_calls, "window_changes": window_changes,
                "per_step": "the six evolving particle arrays and the inner-window "
                            "field, in and out through pf_rk4_step_host (the copies "
                            "overlapped with the step; chi stays the handle's); the "
                            "outer field and the window in and out around each "
                            "diffraction call through pf_diffract_host",
                "api": "pf_rk4_step_host + pf_diffract_host",
                "ms_per_step_by_call": e2e_parts},
        "fft_arithmetic": {
            "value_leg": "paired FP32 (48-bit significands; the field stays FP64 in HBM)",
            "fp64_arithmetic": {"value": whole_job_rate(n, args.steps, world, r64f_ms),
                                "ms_per_step": r64f_ms / args.steps,
                                "fft_ms": r64f["kernel"]["fft"][0]},
            "paired_fp32_fft_ms": r64["kernel"]["fft"][0]},
        "gpu_launches": r64["launches"] + r64f["launches"] + (rmx["launches"] if rmx else 0)
        + (c3["fp64"]["launches"] + c3["mixed"]["launches"] if c3 else 0),
        "kernel_ms": kern,
        "roofline": {"kernel": "k_stage (fused FP64 RK4 stage)", "bound": "hbm",
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_kind": f"{peak_kind} copy bandwidth (burst)",
                     "traffic": n * TRAFFIC_PER_PARTICLE_STAGE,
                     "traffic_source": "ncu dram bytes of k_stage<3> at 2^22 macroparticles "
                                       "on 129x129x2048 planes, scaled to the launch's "
                                       "macroparticles",
                     "fp64": {"achieved_tflops": fp64_achieved, "peak_tflops": dgemm_tflops,
                              "peak_kind": "measured cuBLAS DGEMM 4096^3",
                              "frac": fp64_achieved / dgemm_tflops}},
        "clocks": r64["clocks"],
    }
    if rmx:
        mst, msn = rmx["kernel"]["stage"]
        mavg = mst / max(1, msn)
        m_ach = n * BYTES_PER_PARTICLE_STAGE / (mavg * 1e-3) / 1e9
        mk = {k: v[0] for k, v in rmx["kernel"].items()}
        rec["mixed"] = {
            "value": whole_job_rate(n, args.steps, world, mx_ms), "unit": UNIT,
            "ms_per_step": mx_ms / args.steps, "speedup_vs_fp64": ms / mx_ms,
            "dtype": "f32 field/weights/deposit/FFT, f64 state/p2/RK4 combination",
            "power_rel_error_vs_fp64": abs(rmx["power"] - r64["power"]) / max(r64["power"], 1e-300),
            "power_after_steps": {"fp64": r64["power"], "mixed": rmx["power"],
                                  "steps": args.warmup + args.steps},
            "errors_vs_fp64": output_errors(r64, rmx),
            "kernel_ms": mk,
            "roofline": {"kernel": "k_stage_mixed", "bound": "hbm", "achieved": m_ach,
                         "peak": peak, "unit": "GB/s", "frac": m_ach / peak},
            "clocks": rmx["clocks"],
        }
        if e2e_mx:
            rec["mixed"]["e2e"] = {
                "value": whole_job_rate(n, args.e2e_steps, world, e2e_mx["ms"]), "unit": UNIT,
                "h2d_bytes_per_step": e2e_mx["h2d"], "d2h_bytes_per_step": e2e_mx["d2h"],
                "steps": args.e2e_steps, "diffraction_calls": e2e_mx["n_diff"],
                "speedup_vs_fp64_e2e": e2e_ms / e2e_mx["ms"],
                "api": "pf_rk4_step_host + pf_diffract_host",
                "ms_per_step_by_call": e2e_mx["parts"]}
    if dgemm:
        rec["dft_as_tensor_core_gemm"] = dgemm
    if fid:
        rec["mixed_fidelity"] = fid
    if adj:
        rec["adjoint"] = adj
    if bat:
        rec["gpu_launches"] += bat.pop("gpu_launches")
        rec["batched"] = bat
    if c3:
        w3 = c3["fp64"]["w"]
        n3 = w3.np
        rec["mixed_config3"] = {
            "workload": w3.name, "macroparticles": n3,
            "mesh": [w3.params.nx, w3.params.ny, w3.params.nz2],
            "steps": args.steps3, "warmup": args.warmup,
            "fp64": {"value": whole_job_rate(n3, args.steps3, world, c3_64_ms),
                     "ms_per_step": c3_64_ms / args.steps3,
                     "kernel_ms": {k: v[0] for k, v in c3["fp64"]["kernel"].items()}},
            "mixed": {"value": whole_job_rate(n3, args.steps3, world, c3_mx_ms),
                      "ms_per_step": c3_mx_ms / args.steps3,
                      "kernel_ms": {k: v[0] for k, v in c3["mixed"]["kernel"].items()}},
            "speedup_vs_fp64": c3_64_ms / c3_mx_ms,
            "errors_vs_fp64": output_errors(c3["fp64"], c3["mixed"]),
            "unit": UNIT,
        }
    return rec


def run_reference(args, world):
    """The reference arm: the CPU implementation of the path on the host
    cores, on the GPU arm's workload, schedule, metric and config.  The
    reference is Fortran + MPI + FFTW-MPI + parallel HDF5 with no toolchain
    here or on the GPU host image, so its CPU restatement (oracle/) runs in
    its place: W warm-up and K timed steps on the full beam and mesh."""
    from puffin_gb300 import configs
    w = configs.config2(np_=args.np, nz2=args.nz2)
    r = oracle_steps(w, args.steps, args.warmup)
    v = r["value"]
    return {
        "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": 0,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * r["seconds"] / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded beam and zero seed field; no dataset)",
        "config": workload_config(w, r["window"], world),
        "impl": "reference",
        "cpu_baseline": {
            "value": v, "unit": UNIT, "cores": r["cores"], "kind": "port",
            "sample": (f"the whole timed run: {args.steps} RK4 steps with "
                       f"{r['diffraction_calls']} diffraction calls after {args.warmup} "
                       f"warm-up steps on the full workload ({r['seconds']:.1f} s)")},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "retries": r["retries"],
        "note": ("the reference is Fortran + MPI + FFTW-MPI + parallel HDF5 and no Fortran "
                 "toolchain exists here or on the GPU host image, so the CPU restatement "
                 "in oracle/ (C + OpenMP RK4 with the reference's atomic deposit, numpy "
                 "diffraction) is timed in its place; the CUDA library is not loaded"),
    }


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        if rank == 0:
            print(json.dumps(run_reference(args, world)), flush=True)
        return
    if args.batch_only:
        import torch
        dev = int(os.environ.get("LOCAL_RANK", "0"))
        torch.cuda.set_device(dev)
        if rank == 0:
            print(json.dumps({"metric": METRIC, "unit": UNIT, "batched": batch_leg(args, dev)}),
                  flush=True)
        return
    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl")
    rec = run_gpu(args, rank, world)
    if rank == 0:
        if not args.no_cpu_baseline:
            from puffin_gb300 import configs
            rec["cpu_baseline"] = cpu_baseline(configs.config2(np_=args.np, nz2=args.nz2))
        print(json.dumps(rec), flush=True)
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
