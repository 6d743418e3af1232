"""Train a packed-substrate surrogate (``--kind``: cylinders or spheres) from batched Monte-Carlo
signals and judge it against the walk at high walker counts on held-out substrates.

    python -m dmipy_sim_gb300.train_surrogate --instances 20000 --out surrogate.npz

Steps: draw ``instances`` substrates in the hull (256 free measurements each; radii half uniform,
half log-uniform), walk
them with the batched kernel at ``walkers`` walkers, fit the MLP (graph-captured AdamW steps on
the tensor cores), then draw ``held_out`` new substrates, walk them at ``judge_walkers`` and
report the surrogate's absolute error against them, with the throughput of both methods.
"""
import argparse
import json
import sys
import time

import numpy as np
import torch

from . import surrogate as SG


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--instances", type=int, default=20000)
    ap.add_argument("--meas", type=int, default=256)
    ap.add_argument("--walkers", type=int, default=4096)
    ap.add_argument("--epochs", type=int, default=80)
    ap.add_argument("--batch", type=int, default=8192)
    ap.add_argument("--held-out", type=int, default=24)
    ap.add_argument("--judge-walkers", type=int, default=1_000_000)
    ap.add_argument("--judge-meas", type=int, default=64)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--form", default="dimensionless", choices=["dimensionless", "raw"])
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--radius-sampling", default="mixture", choices=["uniform", "mixture"])
    ap.add_argument("--kind", default="PackedCylinders", choices=sorted(SG.HULLS))
    ap.add_argument("--out", default="surrogate.npz")
    ap.add_argument("--report", default=None)
    a = ap.parse_args(argv)

    def log(msg):
        print(msg, flush=True)

    t0 = time.time()
    log(f"training set: {a.instances} instances x {a.meas} measurements, {a.walkers} walkers")
    X, y, se, params, gpu_train_mc = SG.build_training_set(a.instances, a.seed, a.meas,
                                                           n_walkers=a.walkers, log=log,
                                                           form=a.form,
                                                           radius_sampling=a.radius_sampling,
                                                           kind=a.kind)
    log(f"  {len(y)} signals, median SE {np.median(se):.4f}, MC {gpu_train_mc:.1f} GPU s")
    # validation split: the last 5 % of instances
    n_val = max(1, a.instances // 20) * a.meas
    Xtr, ytr, Xva, yva = X[:-n_val], y[:-n_val], X[-n_val:], y[-n_val:]
    sur = SG.Surrogate(seed=a.seed, lr=a.lr, form=a.form, kind=a.kind)
    t1 = time.time()
    hist = sur.fit(Xtr, ytr, epochs=a.epochs, batch=a.batch, val=(Xva, yva), log=log)
    torch.cuda.synchronize()
    train_s = time.time() - t1
    sur.save(a.out)
    log(f"  trained in {train_s:.1f} s; saved {a.out}")

    # judge: held-out substrates at high walker counts
    insts, hp = SG.draw_instances(a.held_out, a.seed + 10_000, a.judge_meas,
                                  n_walkers=a.judge_walkers, kind=a.kind)
    ref, ref_se, gpu_judge = SG.monte_carlo(insts, chunk=8, log=log)
    Xh = np.concatenate([SG.features(p, i.waveform, a.form) for p, i in zip(hp, insts)])
    pred = sur.predict(Xh)
    ref = np.concatenate(ref)
    ref_se = np.concatenate(ref_se)
    err = np.abs(pred - ref)
    # throughput: the surrogate on 1M queries in one batch, against the walk's signals/s
    q = np.repeat(Xh, int(np.ceil(1_000_000 / len(Xh))), axis=0)[:1_000_000]
    qd = torch.as_tensor(q, device=sur.net.dev)
    sur.net.predict(qd)                  # warm-up at the timed size (buffers, tensor maps)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    sur.net.predict(qd)
    e1.record()
    e1.synchronize()
    sur_s = e0.elapsed_time(e1) * 1e-3
    rep = {
        "kind": a.kind, "instances": a.instances, "signals": int(len(y)), "walkers": a.walkers,
        "form": a.form,
        "radius_sampling": a.radius_sampling,
        "train_mc_gpu_s": gpu_train_mc, "train_s": train_s, "epochs": a.epochs,
        "final_train_mse": hist[-1][0], "val_mae_vs_training_mc": hist[-1][1],
        "held_out_instances": a.held_out, "held_out_signals": int(len(ref)),
        "judge_walkers": a.judge_walkers, "judge_median_se": float(np.median(ref_se)),
        "mae": float(err.mean()), "rmse": float(np.sqrt(np.mean(err ** 2))),
        "p95_abs_err": float(np.percentile(err, 95)), "max_abs_err": float(err.max()),
        "surrogate_signals_per_s": 1_000_000 / sur_s,
        "judge_mc_signals_per_s": len(ref) / gpu_judge,
        "judge_mc_gpu_s": gpu_judge, "wall_s": time.time() - t0,
    }
    log(json.dumps(rep, indent=1))
    if a.report:
        with open(a.report, "w") as f:
            json.dump(rep, f, indent=1)
        # the held-out queries, predictions and judge signals, for error analysis
        np.savez_compressed(a.report.rsplit(".", 1)[0] + "_held_out.npz", X=Xh, pred=pred,
                            ref=ref, ref_se=ref_se,
                            params=np.array([[p[k] for k in ("radius", "f", "kappa", "rho",
                                                             "D", "TE")] for p in hp]))
    return rep


if __name__ == "__main__":
    sys.exit(0 if main() else 1)
