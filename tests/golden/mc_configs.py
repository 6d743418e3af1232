"""The reference's own Monte-Carlo signals on the benchmark configurations (mc_configs.json).

The benchmark walks (free PGSE; a cylinder with surface relaxivity and a permeable sphere with
30 directions; the 16 x 16 packed-cylinder lattice at f = 0.6 walked by the default engine, with
permeable walls, and as a 16-echo CPMG train) are run through dmipy-sim's own ``core.simulate`` /
``core.simulate_cpmg``, unmodified, under ``jaxbatch.py`` (a batching numpy stand-in for JAX, which
is not installed where the fixtures are made), in independent walker chunks across processes.
``mc_configs.json`` keeps, per configuration, the pooled mean signal, the walker count and the
chunk-spread standard error.  The GPU test (tests/test_gpu_reference_configs.py) builds the same
substrate and waveform with this module and this package's constructors.

The permeable-lattice fixture runs 80 samples (4 ms) at the benchmark's sample spacing
(50.05 us), so it takes the same 460 permeable sub-steps per sample as the full 1000-sample walk;
the others run the benchmark's configuration as specified.

Usage:  python tests/golden/mc_configs.py [--only NAME ...] [--procs P] [--ref SRC]
"""
import argparse
import json
import multiprocessing as mp
import os
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
D = 2e-9
BENCH_NT = 1000
BENCH_DT = 0.05 / (BENCH_NT - 1)

# name -> walk; n = total reference walkers, chunk = walkers per independent run
CONFIGS = {
    "c1_free_pgse": dict(geom=("free",), wf=("c1_pgse",), api="simulate", engine="auto",
                         n=50_000, chunk=6_250),
    "c2_cyl_rho": dict(geom=("c2_cyl",), wf=("c2_pgse30",), api="simulate", engine="auto",
                       n=48_000, chunk=4_000),
    "c2_sph_kappa": dict(geom=("c2_sph",), wf=("c2_pgse30",), api="simulate", engine="auto",
                         n=48_000, chunk=4_000),
    "c3_lattice_auto": dict(geom=("lattice16", None), wf=("bench64",), api="simulate",
                            engine="auto", n=80_000, chunk=2_000),
    "c3_lattice_kappa": dict(geom=("lattice16", 2e-5), wf=("lat_short",), api="simulate",
                             engine="auto", n=42_000, chunk=2_000),
    "c3_lattice_cpmg": dict(geom=("lattice16", None), wf=("cpmg16",), api="cpmg", T2=0.08,
                            n=48_000, chunk=4_000),
}


def lattice16():
    """The benchmark substrate: 16 x 16 square lattice, f = 0.6, lognormal radii 2 +- 0.5 um."""
    if str(ROOT) not in sys.path:
        sys.path.insert(0, str(ROOT))
    from dmipy_sim_gb300.geometries import lattice_cylinders
    return lattice_cylinders(16, 0.6, 2e-6, 0.5e-6, seed=0)


def _dirs30():
    rng = np.random.default_rng(0)
    bv = rng.normal(size=(30, 3))
    return bv / np.linalg.norm(bv, axis=1, keepdims=True)


def waveform(wfm, spec):
    """The waveform ``spec`` built with the waveform module ``wfm`` (reference's or this
    package's: the same constructors)."""
    import warnings
    name = spec[0]
    if name == "c1_pgse":
        return wfm.set_b(wfm.pgse(0.01, 0.04, 0.05, [[1, 0, 0]] * 3, 300), [0.0, 1e9, 2e9])
    if name == "c2_pgse30":
        return wfm.set_b(wfm.pgse(0.01, 0.04, 0.05, _dirs30(), 300), 1e9)
    if name == "bench64":
        rng = np.random.default_rng(0)
        bv = rng.normal(size=(8, 3))
        bv /= np.linalg.norm(bv, axis=1, keepdims=True)
        pg = wfm.pgse(0.01, 0.04, 0.05, np.tile(bv, (4, 1)), BENCH_NT)
        pg = wfm.set_b(pg, np.repeat([0.5e9, 1e9, 2e9, 3e9], 8))
        Gs = [np.asarray(pg.G)]
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            for f in (10.0, 40.0, 70.0, 100.0):
                Gs.append(np.asarray(wfm.set_b(wfm.ogse(f, 0.05, 0.05, bv, BENCH_NT), 1e9).G))
        return wfm.Waveform(G=np.concatenate(Gs, 0).astype(np.float32), dt=pg.dt,
                            echo_idx=BENCH_NT - 1)
    if name == "lat_short":
        n_t = 80
        T = (n_t - 1) * BENCH_DT
        bv = [[1, 0, 0], [0, 1, 0], [0.6, 0.8, 0]]
        pg = wfm.pgse(T / 3, 2 * T / 3, 0.05, bv * 2, n_t)
        return wfm.set_b(pg, [0.25e9] * 3 + [0.5e9] * 3)
    if name == "cpmg16":
        return wfm.cpmg(16, 5e-3, 0.02, [[1, 0, 0], [0, 1, 0], [0, 0, 1], [0.6, 0.8, 0]],
                        n_t_per_echo=100)
    raise KeyError(name)


def geometry(geo, spec):
    """The geometry ``spec`` built with the geometry module ``geo``."""
    kind = spec[0]
    if kind == "free":
        return geo.FreeDiffusion()
    if kind == "c2_cyl":
        return geo.Cylinder(5e-6, (0, 0, 1), surface_relaxivity_t2=1e-6)
    if kind == "c2_sph":
        return geo.Sphere(5e-6, permeability=1e-5)
    if kind == "lattice16":
        radii, centers, L = lattice16()
        return geo.PackedCylinders(radii, centers, L, permeability=spec[1])
    raise KeyError(kind)


def _worker(args):
    ref, name, cfg, seed, n = args
    import contextlib
    import io
    sys.path.insert(0, str(HERE))
    import jaxbatch
    m = jaxbatch.load_reference(ref)
    wf = waveform(m["waveforms"], cfg["wf"])
    g = geometry(m["geometries"], cfg["geom"])
    t0 = time.time()
    with contextlib.redirect_stdout(io.StringIO()):
        if cfg["api"] == "cpmg":
            s = m["core"].simulate_cpmg(n, D, wf, g, T2=cfg.get("T2"), seed=seed,
                                        require_gpu=False)
        else:
            s = m["core"].simulate(n, D, wf, g, seed=seed, T2=cfg.get("T2"), require_gpu=False,
                                   engine=cfg.get("engine", "auto"))
    return name, seed, n, np.asarray(s, np.float64).tolist(), time.time() - t0


def make(ref, procs, only=None, partial=None):
    jobs = []
    for name, cfg in CONFIGS.items():
        if only and name not in only:
            continue
        for k in range(cfg["n"] // cfg["chunk"]):
            jobs.append((ref, name, cfg, 7000 + 31 * k, cfg["chunk"]))
    partial = Path(partial or "/tmp/mc_configs.partial.jsonl")
    done = {}
    if partial.exists():
        for line in partial.read_text().splitlines():
            r = json.loads(line)
            done[(r["name"], r["seed"])] = r
    todo = [j for j in jobs if (j[1], j[3]) not in done]
    # longest walks first, so the pool drains evenly
    todo.sort(key=lambda j: -(j[2]["chunk"] * (1 + ("lattice" in j[1]) * 50)))
    print(f"{len(jobs)} chunks, {len(todo)} to run on {procs} processes", flush=True)
    t0 = time.time()
    with mp.get_context("spawn").Pool(procs) as pool:
        for name, seed, n, s, dt in pool.imap_unordered(_worker, todo):
            r = dict(name=name, seed=seed, n=n, signal=s, seconds=dt)
            done[(name, seed)] = r
            with partial.open("a") as f:
                f.write(json.dumps(r) + "\n")
            print(f"  {name} seed {seed}: {n} walkers in {dt:.0f} s "
                  f"({time.time() - t0:.0f} s)", flush=True)
    path = HERE / "mc_configs.json"
    out = json.loads(path.read_text()) if path.exists() else {}
    for name, cfg in CONFIGS.items():
        rows = [r for (nm, _), r in done.items() if nm == name]
        if not rows or (only and name not in only):
            continue
        arr = np.array([r["signal"] for r in rows], np.float64)
        ns = np.array([r["n"] for r in rows], np.float64)
        mean = np.tensordot(ns, arr, axes=1) / ns.sum()
        flat = arr.reshape(len(ns), -1)
        se = np.sqrt(np.sum(ns[:, None] * (flat - mean.reshape(1, -1)) ** 2, axis=0)
                     / ns.sum() / max(len(ns) - 1, 1)).reshape(mean.shape)
        out[name] = dict(config={k: (list(v) if isinstance(v, tuple) else v)
                                 for k, v in cfg.items()},
                         n_walkers=int(ns.sum()), chunks=len(ns), signal=mean.tolist(),
                         stderr=se.tolist(),
                         cpu_seconds=float(sum(r["seconds"] for r in rows)))
    path.write_text(json.dumps(out, indent=1))
    print(f"mc_configs.json: {sorted(out)}")


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("DMIPY_SIM_SRC", "/root/reference"))
    ap.add_argument("--only", nargs="*")
    ap.add_argument("--procs", type=int, default=max(1, (os.cpu_count() or 4) - 2))
    ap.add_argument("--partial", default=None)
    a = ap.parse_args()
    make(a.ref, a.procs, a.only, a.partial)
