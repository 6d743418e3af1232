"""Learned surrogate of the Monte-Carlo signal, trained on signals the batched walk generates.

The surrogate maps 5 substrate parameters -- mean radius, volume fraction, permeability, surface
relaxivity, diffusivity -- plus a 64-number waveform encoding (the dephasing q(t) at 32 absolute
times, along and across the cylinder axis; :func:`substrates.q_encoding`) to one signal, with the
tensor-core MLP of :mod:`mlp` (4 x 256 GELU, bf16 weights, fp32 accumulation, AdamW).

Scope: one surrogate per substrate kind -- packed parallel cylinders (the axis is the encoding's
reference axis) and packed spheres -- with the parameters inside the hull it was trained on
(:data:`HULLS`) and echo times up to ``t_max``.  Every query
outside the hull -- another substrate kind, a parameter out of range, a longer waveform -- is
answered by the batched Monte-Carlo walk (:meth:`Surrogate.signals` does the routing), and the
same walk at 1e6 walkers is what the surrogate's error on held-out substrates is measured against.
"""
import dataclasses
import time

import numpy as np
import torch

from . import substrates as S
from .batched import Instance, PreparedBatch, Tuning
from .mlp import MLP

N_Q = 32
T_MAX = 0.08
# the training hull of each substrate kind a surrogate exists for (the batched study's ranges;
# random sequential addition of a few spheres jams near f = 0.38)
HULLS = {
    "PackedCylinders": {"radius": (0.5e-6, 5e-6), "f": (0.3, 0.70), "kappa": (0.0, 1e-4),
                        "rho": (0.0, 5e-6), "D": (1e-9, 3e-9), "TE": (0.03, 0.08),
                        "b": (0.0, 3e9)},
    "PackedSpheres": {"radius": (0.5e-6, 5e-6), "f": (0.2, 0.38), "kappa": (0.0, 1e-4),
                      "rho": (0.0, 5e-6), "D": (1e-9, 3e-9), "TE": (0.03, 0.08),
                      "b": (0.0, 3e9)},
}
HULL = HULLS["PackedCylinders"]
# objects per training substrate: enough that one packing's signal is close to the mean over
# packings of the same radius and volume fraction
N_OBJECTS = {"PackedCylinders": 64, "PackedSpheres": 27}
# substrate inputs in natural units (um, 1, 1e-5 m/s, 1e-6 m/s, 1e-9 m^2/s)
_UNITS = np.array([1e6, 1.0, 1e5, 1e6, 1e9])


def substrate_features(radius, f, kappa, rho, D, form="dimensionless"):
    """The 5 substrate inputs.  ``raw``: radius (um), f, kappa (1e-5 m/s), rho (1e-6 m/s),
    D (1e-9 m^2/s).  ``dimensionless``: log(radius / 1 um), f, kappa R / D, rho R / D,
    log(D / 1e-9) -- the groups the walk's physics depends on."""
    if form == "raw":
        return np.array([radius, f, kappa, rho, D], np.float64) * _UNITS
    return np.array([np.log(radius * 1e6), f, kappa * radius / D, rho * radius / D,
                     np.log(D * 1e9)], np.float64)


def features(params, wf, form="dimensionless"):
    """(M, 69) inputs of the M measurements of one instance.  In the dimensionless form the
    dephasing samples are scaled by sqrt(D t_max / N_Q), so that their sum of squares is the
    attenuation exponent b D of free diffusion."""
    sub = substrate_features(params["radius"], params["f"], params["kappa"], params["rho"],
                             params["D"], form)
    q = S.q_encoding(wf, N_Q, T_MAX)
    if form != "raw":
        q = q * 1e6 * np.sqrt(params["D"] * T_MAX / N_Q)
    return np.concatenate([np.repeat(sub[None, :], len(q), 0), q], axis=1).astype(np.float32)


def in_hull(params, wf=None, kind="PackedCylinders"):
    if params.get("kind", "PackedCylinders") != kind or kind not in HULLS:
        return False
    hull = HULLS[kind]
    for k in ("radius", "f", "kappa", "rho", "D"):
        lo, hi = hull[k]
        if not (lo <= params[k] <= hi):
            return False
    if wf is not None and (np.asarray(wf.G).shape[1] - 1) * wf.dt > T_MAX:
        return False
    return True


def draw_instances(n, seed, n_meas=256, n_t=200, n_walkers=8192, n_objects=None,
                   radius_sampling="uniform", kind="PackedCylinders"):
    """``n`` packed instances of ``kind`` with parameters uniform in its hull and free waveform
    sets of ``n_meas`` measurements; returns (instances, params).  Each substrate holds
    ``n_objects`` objects (default :data:`N_OBJECTS`), enough that one packing's signal is close
    to the mean over packings of the same radius and volume fraction (the 5 substrate inputs do
    not name the packing).  ``radius_sampling="mixture"`` draws half the radii log-uniformly
    instead, putting more substrates at small radii, where the signal changes fastest with the
    parameters."""
    rng = np.random.default_rng(int(seed))
    insts, params = [], []
    hull = HULLS[kind]
    n_objects = N_OBJECTS[kind] if n_objects is None else int(n_objects)
    lo, hi = hull["radius"]
    for i in range(n):
        if radius_sampling == "mixture" and rng.uniform() < 0.5:
            r = float(np.exp(rng.uniform(np.log(lo), np.log(hi))))
        else:
            r = rng.uniform(lo, hi)
        f = rng.uniform(*hull["f"])
        kappa = rng.uniform(*hull["kappa"])
        rho = rng.uniform(*hull["rho"])
        D = rng.uniform(*hull["D"])
        te = rng.uniform(*hull["TE"])
        wf, _, _, _ = S.free_waveform_set(n_meas, n_t, te, rng, b_max=hull["b"][1])
        geom, fa = S.packed_substrate(kind, r, f, rng, n_objects=n_objects, rho=rho, kappa=kappa)
        radius = float(np.mean(geom._radii_np))
        insts.append(Instance(int(n_walkers), D, wf, geom, seed=int(rng.integers(1, 2 ** 62))))
        params.append(dict(kind=kind, radius=radius, f=fa, kappa=kappa, rho=rho, D=D, TE=te))
    return insts, params


def monte_carlo(insts, tuning=None, chunk=256, log=None):
    """Signals and standard errors of ``insts`` from the batched walk, ``chunk`` instances per
    launch; also returns the GPU seconds spent."""
    sig, se, gpu_s = [], [], 0.0
    for c0 in range(0, len(insts), chunk):
        part = insts[c0:c0 + chunk]
        b = PreparedBatch(part, tuning or Tuning())
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        b.launch()
        e1.record()
        res = b.results()
        gpu_s += e0.elapsed_time(e1) * 1e-3
        for r in res:
            sig.append(r.signal[0].astype(np.float32))
            se.append(r.stderr[0].astype(np.float32))
        b.close()
        if log is not None:
            log(f"  MC {c0 + len(part)}/{len(insts)} instances, {gpu_s:.1f} GPU s")
    return sig, se, gpu_s


class Surrogate:
    def __init__(self, width=256, depth=4, seed=0, lr=1e-3, weight_decay=1e-5,
                 form="dimensionless", kind="PackedCylinders"):
        if kind not in HULLS:
            raise ValueError(f"no surrogate hull for {kind!r}")
        self.net = MLP(5 + 2 * N_Q, width=width, depth=depth, seed=seed, lr=lr,
                       weight_decay=weight_decay)
        self.lr0 = lr
        self.form = form
        self.kind = kind

    # ---- training -----------------------------------------------------------------------------
    def fit(self, X, y, epochs=40, batch=8192, val=None, log=None, seed=0):
        """AdamW on (X, y) with a cosine learning-rate decay; the training step is a captured
        CUDA graph.  Returns the per-epoch history (train loss, validation MAE)."""
        X = np.asarray(X, np.float32)
        y = np.asarray(y, np.float32)
        mu, sd = X.mean(0), X.std(0)
        sd[sd < 1e-12] = 1.0
        self.net.set_normalisation(mu, 1.0 / sd)
        dev = self.net.dev
        Xd = torch.as_tensor(X, device=dev)
        yd = torch.as_tensor(y, device=dev)
        n = (len(X) // batch) * batch
        steps = epochs * (n // batch)
        self.net.capture_step(batch)
        g = torch.Generator(device=dev).manual_seed(int(seed))
        hist, step = [], 0
        t_ep = time.time()
        for ep in range(epochs):
            perm = torch.randperm(len(X), device=dev, generator=g)[:n]
            tot = torch.zeros(1, device=dev)
            for s0 in range(0, n, batch):
                self.net.set_lr(self.lr0 * 0.5 * (1 + np.cos(np.pi * step / steps)))
                idx = perm[s0:s0 + batch]
                tot += self.net.train_step(Xd[idx], yd[idx])
                step += 1
            train = float(tot.item()) / (n // batch)
            v = None
            if val is not None:
                v = float(np.mean(np.abs(self.predict(val[0]) - val[1])))
            hist.append((train, v))
            if log is not None:
                log(f"  epoch {ep + 1}/{epochs}: train mse {train:.3e}" +
                    ("" if v is None else f", val mae {v:.4f}") +
                    f" ({time.time() - t_ep:.1f} s)")
        self.net.check_errors()
        return hist

    # ---- inference ----------------------------------------------------------------------------
    def predict(self, X):
        return self.net.predict(X).cpu().numpy()

    def signals(self, instances, params, tuning=None):
        """Signals of every instance: the surrogate inside the hull, the batched Monte-Carlo
        walk outside it.  Returns (signals, used_surrogate flags)."""
        out, flags, mc_idx = [None] * len(instances), [], []
        feats, owners = [], []
        for i, (inst, p) in enumerate(zip(instances, params)):
            wf = inst.waveform.waveform if hasattr(inst.waveform, "waveform") else inst.waveform
            ok = in_hull(p, wf, self.kind)
            flags.append(ok)
            if ok:
                feats.append(features(p, wf, self.form))
                owners.append(i)
            else:
                mc_idx.append(i)
        if feats:
            y = self.predict(np.concatenate(feats))
            o = 0
            for i, fb in zip(owners, feats):
                out[i] = y[o:o + len(fb)].astype(np.float32)
                o += len(fb)
        if mc_idx:
            sig, _, _ = monte_carlo([instances[i] for i in mc_idx], tuning)
            for i, s in zip(mc_idx, sig):
                out[i] = s
        return out, flags

    def save(self, path):
        sd = self.net.state_dict()
        np.savez_compressed(path, **{f"W{l}": w.numpy() for l, w in enumerate(sd["W"])},
                            **{f"b{l}": b.numpy() for l, b in enumerate(sd["b"])},
                            w_head=sd["w_head"].numpy(), b_head=sd["b_head"].numpy(),
                            shift=sd["shift"].numpy(), scale=sd["scale"].numpy(),
                            shape=np.array(sd["shape"]), form=np.array(self.form),
                            kind=np.array(self.kind))

    @classmethod
    def load(cls, path):
        z = np.load(path)
        n_in, width, depth = (int(x) for x in z["shape"])
        s = cls(width=width, depth=depth, form=str(z["form"]) if "form" in z else "raw",
                kind=str(z["kind"]) if "kind" in z else "PackedCylinders")
        sd = {"W": [torch.as_tensor(z[f"W{l}"]) for l in range(depth)],
              "b": [torch.as_tensor(z[f"b{l}"]) for l in range(depth)],
              "w_head": torch.as_tensor(z["w_head"]), "b_head": torch.as_tensor(z["b_head"]),
              "shift": torch.as_tensor(z["shift"]), "scale": torch.as_tensor(z["scale"])}
        s.net.load_state_dict(sd)
        return s


def build_training_set(n_instances, seed=0, n_meas=256, n_t=200, n_walkers=8192, log=None,
                       tuning=None, form="dimensionless", radius_sampling="uniform",
                       kind="PackedCylinders"):
    """(X, y, se, params, GPU seconds) from ``n_instances`` batched-walk instances."""
    t0 = time.time()
    insts, params = draw_instances(n_instances, seed, n_meas, n_t, n_walkers,
                                   radius_sampling=radius_sampling, kind=kind)
    if log is not None:
        log(f"  drew {n_instances} instances in {time.time() - t0:.1f} s")
    sig, se, gpu_s = monte_carlo(insts, tuning, log=log)
    X = np.concatenate([features(p, i.waveform, form) for p, i in zip(params, insts)])
    return X, np.concatenate(sig), np.concatenate(se), params, gpu_s


__all__ = ["Surrogate", "HULL", "HULLS", "N_OBJECTS", "features", "in_hull", "draw_instances",
           "monte_carlo", "build_training_set"]
