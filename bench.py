"""Benchmark of the Monte-Carlo forward walk on one GB300 (or N, one process per GPU).

Workload (the packed-substrate configuration): PackedCylinders on a periodic 16 x 16 square
lattice, volume fraction 0.6, lognormal radii (mean 2 um, sd 0.5 um, seed 0, clipped to 0.95 of
the half spacing), impermeable, D = 2e-9 m^2/s, 1,000,000 walkers per GPU, 64 measurements
(32 PGSE delta = 10 ms / DELTA = 40 ms at b = 0.5-3 ms/um^2 + 32 cosine OGSE 10-100 Hz snapped to
40/80 Hz, b = 1 ms/um^2), n_t = 1000 over 50 ms, walked as dmipy-sim's default engine does
(walk-once + replay semantics: step <= R_min/6, i.e. 27 sub-steps per sample).

One step = one complete walk of that workload (all walkers, all samples, all sub-steps, ensemble
reduction).  Metric: walker-steps/s, a walker-step being one walker advanced one physics sub-step
with every measurement's phase updated.

The roofline fraction is quoted against the FP32 FMA rate measured in the same process
(``dmsim_fp32_fma_peak``: FMA chains on every SM, CUDA-event timed).

The same JSON line carries, at N = 1:
  "legs"       every other configuration of the metric at its own size, inputs resident:
               free diffusion + PGSE (50,000 walkers), a cylinder with surface relaxivity and a
               permeable sphere (30 directions, 100,000 walkers), the lattice with permeable
               walls (kappa = 2e-5 m/s, 460 sub-steps per sample), the lattice as a 16-echo CPMG
               train (5 ms spacing) and the headline walk in the direct phase form (every
               measurement's phase accumulated separately); each with walker-steps/s, its
               roofline fraction and the oracle's CPU rate on a bounded sample;
  "batched"    signals/s of the batched walk on the 256-instance study (packed cylinders, packed
               spheres and a periodic mesh of 200 ellipsoid cells with ~500k triangles; radius,
               volume fraction, permeability, relaxivity, D, n_t and free waveforms of 8-96
               measurements drawn from seed 0), one graph-captured launch with every instance at
               --batched-walkers walkers (default 24,000, which keeps every signal's standard
               error below 0.005: the per-walker variance of w cos(phi) stays below 0.52),
               measured, with and without the host set-up;
  "surrogate"  signals/s of the trained MLP surrogate on 1,000,000 queries in one batch, its
               absolute error against the walk on held-out substrates, and its speed-up over
               the batched walk's signals/s.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

``--impl reference`` times the CPU restatement of the reference walk (oracle/, all host cores) on
a bounded walker sample of the same workload: dmipy-sim is pure Python/JAX and JAX is not
installed, so its own CPU path cannot run here.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

D = 2e-9
N_WALKERS = 1_000_000
N_T = 1000
METRIC = "walker-steps/s/GPU (plain MC); signals/s at <=0.005 err (batched+surrogate)"
UNIT = "walker-steps/s"
WORKLOAD = "PackedCylinders 16x16 square lattice f=0.6 lognormal r (2.0+-0.5 um), kappa=0"


def build_workload():
    import dmipy_sim_gb300 as d
    radii, centers, L = d.lattice_cylinders(16, 0.6, 2e-6, 0.5e-6, seed=0)
    geom = d.PackedCylinders(radii, centers, L)
    rng = np.random.default_rng(0)
    bv = rng.normal(size=(8, 3))
    bv /= np.linalg.norm(bv, axis=1, keepdims=True)
    pg = d.pgse(0.01, 0.04, 0.05, np.tile(bv, (4, 1)), N_T)
    pg = d.set_b(pg, np.repeat([0.5e9, 1e9, 2e9, 3e9], 8))
    import warnings
    Gs = [pg.G]
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        for f in (10.0, 40.0, 70.0, 100.0):
            og = d.set_b(d.ogse(f, 0.05, 0.05, bv, N_T), 1e9)
            Gs.append(og.G)
    wf = d.Waveform(G=np.concatenate(Gs, 0).astype(np.float32), dt=pg.dt, echo_idx=N_T - 1)
    return geom, wf


def _clock_sampler(stop, samples):
    cmd = ["nvidia-smi", "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,"
           "clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
           "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
           "clocks_event_reasons.sw_power_cap", "--format=csv,noheader,nounits", "-lms", "200"]
    try:
        p = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
    except OSError:
        return
    try:
        while not stop.is_set():
            line = p.stdout.readline()
            if not line:
                break
            samples.append([x.strip() for x in line.split(",")])
    finally:
        p.terminate()
        try:
            p.wait(timeout=5)
        except Exception:
            p.kill()


def _clock_summary(samples, dev_index):
    rows = [s for s in samples if s and s[0] == str(dev_index)]
    if not rows:
        return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["clock sampling unavailable"]}
    sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
    mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    reasons = sorted({names[i] for r in rows for i in range(4)
                      if len(r) > 5 + i and r[5 + i].lower().startswith("active")})
    return {"sm_mhz": statistics.median(sm) if sm else None,
            "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
            "samples": len(rows)}


def _dist():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def algorithmic_flops_per_walker_step(n_meas, sub_steps, k_alg=4):
    """FP32 FLOPs per walker-step of the walk: direction from two uniforms (20), the packed
    cylinder wall test (22 per candidate object, 4 objects within reach of a step) and the phase
    3 FMAs per measurement per waveform sample, spread over the sample's sub-steps."""
    return 20.0 + 22.0 * k_alg + 6.0 * n_meas / sub_steps


def cpu_baseline(geom, wf, S, threads, budget_s=15.0):
    """The CPU restatement of the reference walk (oracle/, FP32) on a bounded sample of walkers of
    the same workload, every host thread; returns (walker-steps/s, sample description)."""
    from dmipy_sim_gb300 import core
    from oracle import oracle as O
    G, _ = core._waveform_arrays(wf, geom)
    og = O.geom_from(geom)
    n = 64
    t0 = time.perf_counter()
    O.walk(og, n_walkers=n, G=G, dt=wf.dt, sub_steps=S, phase_per_substep=False, seed=1,
           n_threads=threads)
    dt1 = time.perf_counter() - t0
    n2 = int(max(threads, min(1_000_000, n * budget_s / max(dt1, 1e-3))))
    t0 = time.perf_counter()
    O.walk(og, n_walkers=n2, G=G, dt=wf.dt, sub_steps=S, phase_per_substep=False, seed=2,
           n_threads=threads)
    el = time.perf_counter() - t0
    steps = n2 * wf.G.shape[1] * S
    return steps / el, f"{n2} walkers x {wf.G.shape[1]} samples x {S} sub-steps in {el:.1f} s"


def fp32_peak_tflops(dev):
    """The measured FP32 FMA rate of this GPU (TFLOP/s): the library's FMA-chain kernel on 8
    blocks per SM x 256 threads, best of 5 launches timed with CUDA events."""
    import torch
    from dmipy_sim_gb300 import _lib
    lib = _lib.load()
    n_sm = torch.cuda.get_device_properties(dev).multi_processor_count
    blocks, threads, iters = 8 * n_sm, 256, 4096
    sink = torch.zeros(1, dtype=torch.float32, device=dev)
    best = None
    for _ in range(6):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        _lib.check(lib.dmsim_fp32_fma_peak(blocks, threads, iters, _lib.ptr(sink),
                                           _lib.stream_handle()), "dmsim_fp32_fma_peak")
        e1.record()
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        best = ms if best is None else min(best, ms)
    flops = float(blocks) * threads * iters * 16 * 8 * 2
    return flops / (best * 1e-3) / 1e12


def _pgse30():
    rng = np.random.default_rng(0)
    bv = rng.normal(size=(30, 3))
    return bv / np.linalg.norm(bv, axis=1, keepdims=True)


def leg_workloads():
    """The configurations of the metric besides the headline, as simulate() / simulate_cpmg()
    would walk them: name -> (geometry, waveform, api, walkers, T2, engine, timed steps)."""
    import warnings
    import dmipy_sim_gb300 as d
    radii, centers, L = d.lattice_cylinders(16, 0.6, 2e-6, 0.5e-6, seed=0)
    _, wf64 = build_workload()
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        c1 = d.set_b(d.pgse(0.01, 0.04, 0.05, [[1, 0, 0]] * 3, 300), [0.0, 1e9, 2e9])
        c2 = d.set_b(d.pgse(0.01, 0.04, 0.05, _pgse30(), 300), 1e9)
        cp = d.cpmg(16, 5e-3, 0.02, [[1, 0, 0], [0, 1, 0], [0, 0, 1], [0.6, 0.8, 0]],
                    n_t_per_echo=100)
    return {
        "c1_free_pgse": (d.FreeDiffusion(), c1, "simulate", 50_000, None, "auto", 20),
        "c2_cylinder_rho1e-6": (d.Cylinder(5e-6, (0, 0, 1), surface_relaxivity_t2=1e-6), c2,
                                "simulate", 100_000, None, "auto", 20),
        "c2_sphere_kappa1e-5": (d.Sphere(5e-6, permeability=1e-5), c2, "simulate", 100_000, None,
                                "auto", 5),
        "c3_lattice_kappa2e-5": (d.PackedCylinders(radii, centers, L, permeability=2e-5), wf64,
                                 "simulate", N_WALKERS, None, "auto", 1),
        "c3_lattice_cpmg16": (d.PackedCylinders(radii, centers, L), cp, "cpmg", N_WALKERS, 0.08,
                              "auto", 5),
        "c3_lattice_direct_form": (d.PackedCylinders(radii, centers, L), wf64, "simulate",
                                   N_WALKERS, None, "direct", 2),
    }


def _leg_plan(geom, wf, api, engine):
    """(G, chi, sub_steps, phase_per_substep, echo_idx) as simulate() / simulate_cpmg() pick
    them."""
    from dmipy_sim_gb300 import core
    G, chi = core._waveform_arrays(wf, geom)
    if api == "cpmg":
        return G, chi, core.fused_sub_steps(geom, D, wf.dt), True, \
            np.unique(np.asarray(wf.echo_indices, int))
    gap = core._replay_gap(geom, return_positions=False, return_compartments=False,
                           return_walker_signals=False, diffusivity=D)
    rep = gap is None and core._replay_auto_allowed(geom)
    S = core.replay_sub_steps(geom, D, wf.dt) if rep else core.fused_sub_steps(geom, D, wf.dt)
    return G, chi, S, not rep, None


def _leg_flops(geom, n_meas, S, fused):
    """Algorithmic FP32 FLOPs per walker-step: direction 20, the geometry's wall test (free 0,
    cylinder 18, sphere 20, packed cylinders 22 per object within reach x 4), +10 with surface
    relaxivity or permeability, the phase 6 M per waveform sample (G is constant over a sample's
    sub-steps, so sum_s g.r_s = g.sum_s r_s) spread over its S sub-steps, +3 for the position sum
    of the fused engine."""
    kind = type(geom).__name__
    f_geom = {"FreeDiffusion": 0.0, "Cylinder": 18.0, "Sphere": 20.0,
              "PackedCylinders": 88.0, "PackedSpheres": 176.0}.get(kind, 0.0)
    if getattr(geom, "surface_relaxivity_t2", None) or getattr(geom, "permeability", None):
        f_geom += 10.0
    return 20.0 + f_geom + 6.0 * n_meas / S + (3.0 if fused else 0.0)


def _leg_cpu(geom, G, wf, S, fused, chi, T2, echo, threads, budget_s=4.0):
    """The oracle (CPU restatement, every host thread) on a bounded walker sample of a leg."""
    from oracle import oracle as O
    og = O.geom_from(geom)
    rho = getattr(geom, "surface_relaxivity_t2", None)
    kappa = getattr(geom, "permeability", None)
    wall = O.PERMEATE if kappa is not None else (O.RELAX if rho is not None else O.REFLECT)
    kw = dict(G=G, dt=wf.dt, sub_steps=S, phase_per_substep=fused, wall=wall, chi=chi, T2=T2,
              rho_over_D=0.0 if rho is None else rho / D,
              kappa_over_D=0.0 if kappa is None else kappa / D, D=D, echo_idx=echo,
              n_threads=threads)
    n = max(threads, 16)
    O.walk(og, n_walkers=threads, seed=0, **kw)          # loads the oracle library
    t0 = time.perf_counter()
    O.walk(og, n_walkers=n, seed=1, **kw)
    dt1 = time.perf_counter() - t0
    n2 = int(max(threads, min(200_000, n * budget_s / max(dt1, 1e-3))))
    t0 = time.perf_counter()
    O.walk(og, n_walkers=n2, seed=2, **kw)
    el = time.perf_counter() - t0
    steps = float(n2) * G.shape[1] * S
    return {"value": steps / el, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{n2} walkers x {G.shape[1]} samples x {S} sub-steps in {el:.1f} s"}


def legs_measure(dev, peak_tflops, cpu=True):
    """walker-steps/s of every other configuration of the metric at its own size, inputs
    resident, timed with CUDA events (a 512 MB L2 flush between launches), with its roofline
    fraction against the measured FP32 rate and the oracle's CPU rate beside it."""
    import torch
    from dmipy_sim_gb300 import core
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    out = {}
    for name, (geom, wf, api, n, T2, engine, steps) in leg_workloads().items():
        G, chi, S, fused, echo = _leg_plan(geom, wf, api, engine)
        walk = core.PreparedWalk(geom, n_walkers=n, diffusivity=D, G=G, dt=wf.dt, sub_steps=S,
                                 phase_per_substep=fused, seed=77, chi=chi, T2=T2,
                                 echo_idx=echo, use_basis=engine != "direct")
        walk.launch()
        torch.cuda.synchronize(dev)
        ms = []
        for k in range(steps):
            flush.fill_(float(k))
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            walk.launch()
            e1.record()
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
        res = walk.result()
        sec = float(np.mean(ms)) * 1e-3
        ws = float(n) * G.shape[1] * S
        F = _leg_flops(geom, G.shape[0], S, fused)
        ach = ws * F / sec / 1e12
        leg = {"walker_steps_per_s": ws / sec, "ms_per_walk": sec * 1e3, "walkers": n,
               "n_t": int(G.shape[1]), "n_meas": int(G.shape[0]), "sub_steps": int(S),
               "engine": ("fused" if fused else "replay semantics") +
                         (", direct phase form" if engine == "direct" else ""),
               "roofline": {"bound": "fp32", "achieved": ach, "peak": peak_tflops,
                            "unit": "TFLOP/s", "frac": ach / peak_tflops,
                            "flops_per_walker_step": F},
               "gpu_launches_per_walk": walk.launches_per_call, "timed_walks": steps,
               "signal_first": float(res.signal.ravel()[0]), "status": res.status}
        if cpu:
            leg["cpu_baseline"] = _leg_cpu(geom, G, wf, S, fused, chi, T2, echo,
                                           os.cpu_count() or 1)
        out[name] = leg
        del walk
    del flush
    return out


# walkers per instance for a standard error of at most 0.005 on every signal: the per-walker
# variance of w cos(phi) measured over the study stays below 0.52 (0.5 for uniformly spread
# phases), so 24,000 walkers give <= 0.0047; the line reports the largest standard error seen
N_SE_005 = 24_000
SURROGATE = ROOT / "dmipy_sim_gb300" / "data" / "surrogate_packed_cylinders.npz"
SURROGATE_REPORT = ROOT / "dmipy_sim_gb300" / "data" / "surrogate_packed_cylinders.json"


def batched_measure(dev, walkers=2000):
    """The 256-instance study as one captured batched launch at ``walkers`` walkers per
    instance; also the signals/s at <= 0.005 error (24,000 walkers per instance)."""
    import dataclasses
    import torch
    from dmipy_sim_gb300 import substrates as S
    from dmipy_sim_gb300.batched import PreparedBatch, Tuning
    t_host = time.perf_counter()
    mesh = S.ellipsoid_cell_mesh()
    insts, params = S.instance_mix(256, seed=0, mesh=mesh)
    full = [dataclasses.replace(i, n_walkers=int(walkers)) for i in insts]
    warm = PreparedBatch([dataclasses.replace(i, n_walkers=640) for i in insts], Tuning())
    warm.launch()
    torch.cuda.synchronize(dev)
    warm.close()
    b = PreparedBatch(full, Tuning())
    host_s = time.perf_counter() - t_host
    b.capture()
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    b.replay()
    e1.record()
    e1.synchronize()
    sec = e0.elapsed_time(e1) * 1e-3
    res = b.results()
    n_sig = sum(int(r.sums.shape[1]) for r in res)
    max_se = max(float(np.max(r.stderr)) for r in res)
    info = b.info()
    kinds = {k: sum(1 for p in params if p["kind"] == k) for k in ("PackedCylinders",
                                                                   "PackedSpheres", "Mesh")}
    out = {"signals_per_s": n_sig / sec, "signals": n_sig, "seconds": sec,
           "signals_per_s_incl_host_setup": n_sig / (sec + host_s),
           "walker_steps_per_s": b.walker_steps() / sec, "instances": len(full),
           "walkers_per_instance": int(walkers), "max_stderr": max_se,
           "signals_per_s_at_0.005_err": n_sig / sec * (int(walkers) / N_SE_005),
           "at_0.005_err": ("measured" if max_se <= 0.005 else
                            f"measured at {int(walkers)} walkers (largest standard error "
                            f"{max_se:.4f})") if int(walkers) >= N_SE_005 else
                           f"measured rate x {int(walkers)}/{N_SE_005} (cost linear in walkers)",
           "kinds": kinds,
           "mesh_triangles": int(len(mesh[0].faces)), "groups": info["groups"],
           "gpu_launches": info["kernels"], "graph": True, "host_setup_s": host_s}
    b.close()
    return out, params


def surrogate_measure(dev, mc_signals_per_s):
    """The trained surrogate: 1M queries in one batch, and its error against the walk on a few
    held-out substrates (2e5 walkers each)."""
    import torch
    from dmipy_sim_gb300 import surrogate as SG
    if not SURROGATE.exists():
        return {"unavailable": "no trained surrogate weights in dmipy_sim_gb300/data"}
    sur = SG.Surrogate.load(SURROGATE)
    insts, hp = SG.draw_instances(4, 424242, n_meas=64, n_walkers=200_000)
    X = np.concatenate([SG.features(p, i.waveform, sur.form) for p, i in zip(hp, insts)])
    ref, ref_se, _ = SG.monte_carlo(insts)
    ref = np.concatenate(ref)
    err = np.abs(sur.predict(X) - ref)
    q = torch.as_tensor(np.resize(X, (1_000_000, X.shape[1])), device=dev)
    sur.net.predict(q)                   # warm-up at the timed size (buffers, tensor maps)
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    y = sur.net.predict(q)
    e1.record()
    e1.synchronize()
    sec = e0.elapsed_time(e1) * 1e-3
    out = {"signals_per_s": 1e6 / sec, "queries": 1_000_000, "seconds": sec,
           "live_mae_vs_mc_2e5": float(err.mean()), "live_max_err": float(err.max()),
           "live_mc_median_se": float(np.median(np.concatenate(ref_se))),
           "speedup_vs_batched_mc": (1e6 / sec) / mc_signals_per_s if mc_signals_per_s else None,
           "forward": "fused (one launch)" if sur.net.fused() else "layer by layer",
           "gpu_launches_per_query_batch": 1 if sur.net.fused() else sur.net.depth + 2}
    keys = ("held_out_instances", "held_out_signals", "judge_walkers", "mae", "p95_abs_err",
            "max_abs_err", "signals")
    if SURROGATE_REPORT.exists():
        rep = json.loads(SURROGATE_REPORT.read_text())
        out["held_out"] = {k: rep.get(k) for k in keys}
    sph = SURROGATE.parent / "surrogate_packed_spheres.json"
    if sph.exists():   # the packed-sphere surrogate's training report (same network and judge)
        rep = json.loads(sph.read_text())
        out["packed_spheres_held_out"] = {k: rep.get(k) for k in keys}
    return out


def profile_case(a):
    """Small single-kernel cases for profiler captures (not bench values):
    mesh      the permeable walk through the 200-cell ellipsoid mesh (~500k triangles),
              8192 walkers x 64 samples;
    mlp       the surrogate's forward pass on 262,144 queries (4 tensor-core GEMMs + head);
    batched   a 32-instance slice of the batched study at 4096 walkers per instance;
    bloch     the vector-Bloch walk of a diffusion-weighted spin echo (2 measurements, 201
              samples) in a 4 um cylinder with surface relaxivity, 1,048,576 walkers; also
              times the scalar walk of the same gradient, geometry and walk;
    mt        the magnetisation-transfer walk of a CW saturation (200 Hz, 1 kHz off, 25 ms at
              dt 20 us) in a 2 um sphere, 131,072 walkers x 1251 samples x 38 sub-steps, FP64
              magnetisation, no burn-in (times the sequence walk alone);
    rbloch    the vector-Bloch replay of a stored float16 walk, 262,144 walkers x 500 samples,
              4 measurements, a spin echo with T2 and T1 (FP64);
    free_flight / lockstep   the permeable 16x16 lattice (kappa = 2e-5 m/s, 461 sub-steps per
              sample, 64 measurements) at 20,000 walkers in either packed-cylinder schedule."""
    import dataclasses
    import torch
    import dmipy_sim_gb300 as d
    from dmipy_sim_gb300 import core
    from dmipy_sim_gb300 import substrates as S
    dev = torch.device("cuda", 0)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    extra = {}
    if a.profile_case == "bloch":
        from dmipy_sim_gb300 import bloch as B
        n_w = 1 << 20
        seq = d.spin_echo(20e-3, 1e-4, n_meas=2)
        seq.G[0, 20:60, 0] = seq.G[0, 110:150, 0] = 0.1
        seq.G[1, 20:60, 2] = seq.G[1, 110:150, 2] = 0.1
        cyl = d.Cylinder(4e-6, (0, 0, 1))
        bw, _u, _i = B._prepare(n_w, D, seq, cyl, seq.rf_events, T2=0.08, T1=1.0, M0=1.0,
                                off_resonance_hz=20.0, seed=7, echo_steps=None, return_mz=True,
                                crusher=None, surface_relaxivity=2e-5)
        sw = core.PreparedWalk(d.Cylinder(4e-6, (0, 0, 1), surface_relaxivity_t2=2e-5),
                               n_walkers=n_w, diffusivity=D, G=seq.G, dt=seq.dt, sub_steps=1,
                               phase_per_substep=True, seed=7, T2=0.08)
        for _ in range(2):
            sw.launch()
        s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize(dev)
        s0.record()
        for _ in range(max(1, a.steps)):
            sw.launch()
        s1.record()
        torch.cuda.synchronize(dev)
        ms = s0.elapsed_time(s1) / max(1, a.steps)
        extra = {"walker_steps_per_launch": n_w * seq.n_t,
                 "scalar_walk_ms": ms,
                 "scalar_walker_steps_per_s": n_w * seq.n_t / (ms * 1e-3)}
    if a.profile_case in ("mt", "rbloch"):
        import time
        if a.profile_case == "mt":
            from dmipy_sim_gb300 import bloch as B
            n_w, n_t, n_sub, dt = 1 << 17, 1251, 38, 2e-5
            sph = d.Sphere(2e-6)
            rf = [{'t_s': 0.0125, 'flip_deg': 360.0 * 200.0 * 0.025, 'axis_deg': 0.0,
                   'duration_s': 0.025, 'offset_hz': 1000.0}]
            r0 = torch.from_numpy(np.asarray(sph.init_positions(n_w, 3), np.float32))
            kw = dict(T2=0.08, T1=1.0, M0=1.0, off_resonance_hz=0.0, off_resonance_bound=0.0,
                      T2_bound=1e-5, T1_bound=1.0, echo_steps=None, return_mz=True,
                      crusher=None, return_bound_frac=False)

            def run():
                w = B.MTWalk(sph, n_w, D, dt, n_sub, 3, kappa_MT=40.0 * 2e-6 / 3.0,
                             dwell_time=1.0 / 80.0, surface_relaxivity=0.0)
                w.r.copy_(r0)
                B._mt_run(w, np.zeros((1, n_t, 3)), dt, rf, **kw)
            units, unit = n_w * n_t * n_sub, "walker_substeps"
        else:
            from dmipy_sim_gb300.trajectories import replay_bloch
            n_w, n_t, dt = 1 << 18, 500, 1e-4
            g = torch.Generator(device=dev).manual_seed(0)
            traj = (torch.randn((n_w, n_t, 3), generator=g, device=dev) * 2e-6).half()
            G = np.zeros((4, n_t, 3))
            for m in range(4):
                G[m, 50:150, m % 3] = G[m, 300:400, m % 3] = 0.04
            rf = [{'t_s': 0.0, 'flip_deg': 90.0, 'axis_deg': 90.0},
                  {'t_s': 0.0225, 'flip_deg': 180.0}]

            def run():
                replay_bloch(traj, dt, G, dt, rf, T2=0.08, T1=1.0)
            units, unit = n_w * n_t, "walker_samples"
        for _ in range(max(1, a.warmup)):
            run()
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        for _ in range(max(1, a.steps)):
            run()
        torch.cuda.synchronize(dev)
        ms = (time.perf_counter() - t0) * 1e3 / max(1, a.steps)
        print(json.dumps({"profile_case": a.profile_case, "ok": True, "ms_per_call": ms,
                          unit + "_per_call": units, unit + "_per_s": units / (ms * 1e-3),
                          "timing": "host clock around synchronised calls (incl. host setup)"}))
        return
    for _ in range(max(1, a.warmup) + a.steps):
        if _ == max(1, a.warmup):
            torch.cuda.synchronize(dev)
            e0.record()
        if a.profile_case == "mesh":
            if _ == 0:
                mesh, _f = S.ellipsoid_cell_mesh()
                g = mesh.with_walls(None, 1e-5)
                rng = np.random.default_rng(0)
                wf, _i, _dd, _b = S.free_waveform_set(16, 64, 0.02, rng)
                G, chi = core._waveform_arrays(wf, g)
                Sm = core.fused_sub_steps(g, D, wf.dt)
                walk = core.PreparedWalk(g, n_walkers=8192, diffusivity=D, G=G, dt=wf.dt,
                                         sub_steps=Sm, phase_per_substep=True, seed=5)
            walk.launch()
        elif a.profile_case in ("free_flight", "lockstep"):
            if _ == 0:
                geom, wf, api, _n, T2, engine, _st = leg_workloads()["c3_lattice_kappa2e-5"]
                G, chi, Sk, fused, echo = _leg_plan(geom, wf, api, engine)
                walk = core.PreparedWalk(geom, n_walkers=20_000, diffusivity=D, G=G, dt=wf.dt,
                                         sub_steps=Sk, phase_per_substep=fused, seed=77,
                                         chi=chi, schedule=a.profile_case)
                extra = {"walker_steps_per_launch": 20_000 * G.shape[1] * Sk}
            walk.launch()
        elif a.profile_case == "mlp":
            if _ == 0:
                from dmipy_sim_gb300.mlp import MLP
                net = MLP(69, 256, 4, seed=0)
                x = torch.randn(262_144, 69, device=dev)
            net.predict(x)
        elif a.profile_case == "bloch":
            bw.launch()
        else:
            if _ == 0:
                from dmipy_sim_gb300.batched import PreparedBatch
                insts, _p = S.instance_mix(32, seed=0, kinds=("PackedCylinders",
                                                              "PackedSpheres"))
                b = PreparedBatch([dataclasses.replace(i, n_walkers=4096) for i in insts])
            b.launch()
    e1.record()
    torch.cuda.synchronize(dev)
    ms = e0.elapsed_time(e1) / max(1, a.steps)
    if a.profile_case == "bloch":
        extra["bloch_walker_steps_per_s"] = extra["walker_steps_per_launch"] / (ms * 1e-3)
    if a.profile_case in ("free_flight", "lockstep"):
        extra["walker_steps_per_s"] = extra["walker_steps_per_launch"] / (ms * 1e-3)
    print(json.dumps(dict({"profile_case": a.profile_case, "ok": True, "ms_per_step": ms},
                          **extra)))


def gpu_arm(a):
    import torch
    import dmipy_sim_gb300 as d
    from dmipy_sim_gb300 import core
    world, rank, local = _dist()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    geom, wf = build_workload()
    G, chi = core._waveform_arrays(wf, geom)
    S = core.replay_sub_steps(geom, D, wf.dt)
    n = a.walkers
    walk = core.PreparedWalk(geom, n_walkers=n, diffusivity=D, G=G, dt=wf.dt, sub_steps=S,
                             phase_per_substep=False, seed=1234, walker_offset=rank * n)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize(dev)

    for _ in range(a.warmup):
        walk.launch()
    barrier()
    stop, samples = threading.Event(), []
    th = threading.Thread(target=_clock_sampler, args=(stop, samples), daemon=True)
    th.start()
    time.sleep(0.3)
    barrier()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(a.steps)]
    t_wall = time.perf_counter()
    for k in range(a.steps):
        flush.fill_(float(k))                       # evict L2 between timed walks
        ev[k][0].record()
        walk.launch()
        ev[k][1].record()
    barrier()
    t_wall = time.perf_counter() - t_wall
    ms = [s.elapsed_time(e) for s, e in ev]
    kernel_s = sum(ms) / 1e3
    t = torch.tensor([kernel_s], dtype=torch.float64, device=dev)
    if world > 1:
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    kernel_s = float(t.item())
    res = walk.result()

    # end to end through the public API: host waveform in, host signals out, every step
    e2e_s = None
    e2e_steps = max(2, min(a.steps, 5))
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        sig = d.simulate(n, D, wf, geom, seed=1234)
    torch.cuda.synchronize(dev)
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    te = torch.tensor([e2e_s], dtype=torch.float64, device=dev)
    if world > 1:
        torch.distributed.all_reduce(te, op=torch.distributed.ReduceOp.MAX)
    e2e_s = float(te.item())
    stop.set()
    th.join(timeout=5)
    clocks = _clock_summary(samples, local)

    walker_steps = float(n) * wf.G.shape[1] * S
    value = walker_steps * world * a.steps / kernel_s
    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return
    m = wf.G.shape[0]
    F = algorithmic_flops_per_walker_step(m, S)
    per_launch_s = kernel_s / a.steps
    achieved = walker_steps * F / per_launch_s / 1e12
    sm_max = clocks.get("sm_max_mhz") or 2070.0
    nominal = 152 * 128 * 2 * sm_max * 1e6 / 1e12       # FP32 FMA pipes at the max SM clock
    peak = fp32_peak_tflops(dev)                         # measured: FMA-chain kernel, this GPU
    traffic = None
    tpath = ROOT / "profiles" / "walk_packed_cylinders_traffic.txt"
    if tpath.exists():
        for line in tpath.read_text().splitlines():
            if line.startswith("dram_bytes_per_launch:"):
                traffic = float(line.split(":")[1])
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": 1e3 * kernel_s / a.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp32",
        "data": "synthetic substrate and waveforms (seeded), no dataset",
        "config": {"workload": WORKLOAD, "n_walkers_per_gpu": n, "n_t": int(wf.G.shape[1]),
                   "n_meas": int(m), "sub_steps": int(S), "engine": "replay semantics (auto)",
                   "walker_steps_per_step": walker_steps * world,
                   "l2": "512 MB buffer written between timed walks",
                   "parallelism": f"walker shards x{world}"},
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "flops_per_walker_step": F,
                     "peak_source": "measured: FP32 FMA-chain kernel (dmsim_fp32_fma_peak) "
                                    "timed with CUDA events in this process (MEASURED_PEAKS.json "
                                    "has no FP32 figure)",
                     "nominal_peak": nominal},
        "e2e": {"value": walker_steps * world / e2e_s, "unit": UNIT,
                "h2d_bytes_per_step": int(wf.G.nbytes + 4 * wf.G.shape[1]),
                "d2h_bytes_per_step": int(8 * 3 * m + 4 * 8)},
        "gpu_launches": walk.launches_per_call * a.steps,
        "clocks": clocks,
        "signal_b1_pgse_x": float(res.signal[0, 8]),
        "status": res.status,
    }
    if world == 1 and not a.no_cpu_baseline:
        v, sample = cpu_baseline(geom, wf, S, os.cpu_count() or 1)
        out["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                               "sample": sample}
    if world == 1 and not a.no_legs:
        out["legs"] = legs_measure(dev, peak, cpu=not a.no_cpu_baseline)
    if world == 1 and not a.no_batched:
        try:
            out["batched"], _ = batched_measure(dev, a.batched_walkers)
        except Exception as e:          # reported, never silently dropped
            out["batched"] = {"error": f"{type(e).__name__}: {e}"}
        try:
            out["surrogate"] = surrogate_measure(
                dev, out["batched"].get("signals_per_s_at_0.005_err"))
        except Exception as e:
            out["surrogate"] = {"error": f"{type(e).__name__}: {e}"}
    print(json.dumps(out), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def reference_arm(a):
    world, rank, local = _dist()
    if rank != 0:
        return
    from dmipy_sim_gb300 import core
    from oracle import oracle as O
    geom, wf = build_workload()
    G, _ = core._waveform_arrays(wf, geom)
    S = core.replay_sub_steps(geom, D, wf.dt)
    og = O.geom_from(geom)
    threads = os.cpu_count() or 1
    n = max(threads, 16 * threads)
    for _ in range(a.warmup):
        O.walk(og, n_walkers=n, G=G, dt=wf.dt, sub_steps=S, phase_per_substep=False, seed=7,
               n_threads=threads)
    t0 = time.perf_counter()
    for k in range(a.steps):
        O.walk(og, n_walkers=n, G=G, dt=wf.dt, sub_steps=S, phase_per_substep=False, seed=8 + k,
               n_threads=threads)
    el = time.perf_counter() - t0
    walker_steps = float(n) * wf.G.shape[1] * S
    v = walker_steps * a.steps / el
    sample = f"{n} walkers x {wf.G.shape[1]} samples x {S} sub-steps per step"
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": 1e3 * el / a.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp32",
        "data": "synthetic substrate and waveforms (seeded), no dataset",
        "config": {"workload": WORKLOAD, "n_walkers_per_step": n, "n_t": int(wf.G.shape[1]),
                   "n_meas": int(wf.G.shape[0]), "sub_steps": int(S),
                   "engine": "CPU restatement of the reference walk (dmipy-sim is Python+JAX; "
                             "JAX is not installed)"},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-legs", action="store_true",
                    help="skip the other configurations (free, cylinder, sphere, permeable "
                         "lattice, CPMG, direct phase form)")
    ap.add_argument("--no-batched", action="store_true",
                    help="skip the batched-walk and surrogate measurements")
    ap.add_argument("--batched-walkers", type=int, default=N_SE_005,
                    help="walkers per instance of the batched study (the default 24000 keeps "
                         "every signal's standard error below 0.005)")
    ap.add_argument("--walkers", type=int, default=N_WALKERS,
                    help="walkers per GPU (smaller only for profiling captures)")
    ap.add_argument("--profile-case", choices=["mesh", "mlp", "batched", "bloch", "mt", "rbloch",
                                               "free_flight", "lockstep"],
                    default=None,
                    help="run one small kernel case for a profiler capture and exit")
    a = ap.parse_args()
    if a.profile_case:
        profile_case(a)
    elif a.impl == "reference":
        reference_arm(a)
    else:
        gpu_arm(a)


if __name__ == "__main__":
    main()
