"""Generate training data for, train, and evaluate the preconditioner-choice
network on the GPU.

    python -m gempy_gb300.train_precond --systems 90 --large 6 --out DIR

1. Systems of ``synthetic.training_system`` are built, solved by the dense
   FP64 LU (the reference solution) and by FGMRES with a random subset of the candidate
   two-level configurations; each run's wall time, status and field error
   against the LU solution become one labelled sample.
2. The cost model is trained with the library's own forward / backward /
   AdamW kernels.
3. On held-out systems the network's pick is compared with the fixed default
   configuration and with the best configuration found by trying them all.

Writes DIR/precond_cost.npz (weights, optimizer state, normalisation),
DIR/dataset.npz, DIR/records.json and DIR/summary.json.  ``--resume`` continues
training from a saved model (weights and optimizer state).
"""
import argparse
import json
import os
import time

import numpy as np
import torch

from . import learned, synthetic


def evaluate(model, n_systems, base_seed, n_min, n_max, log=print):
    out = []
    for i in range(n_systems):
        m = synthetic.training_system(i, base_seed, n_min, n_max)
        s = learned.series_of(m)
        N = s.N
        cands = learned.candidates_for(N)
        pick = model.choose(s, N)
        rows, t_lu = learned.label_system(s, cands)
        by = {learned.PrecondConfig(**r["config"]): r for r in rows}
        best = min(rows, key=lambda r: r["cost_s"])
        rec = dict(N=N, lu_seconds=t_lu, pick=by[pick], default=by[learned.DEFAULT_CONFIG], best=best,
                   rank_of_pick=int(sorted(r["cost_s"] for r in rows).index(by[pick]["cost_s"])), runs=rows,
                   sys_feats=learned.system_features(s).cpu().numpy().tolist())
        out.append(rec)
        log(f"held-out {i}: N={N} lu={t_lu:.3f}s pick={by[pick]['cost_s']:.3f}s (ok={by[pick]['ok']}) "
            f"default={rec['default']['cost_s']:.3f}s best={best['cost_s']:.3f}s")
    return out


def rescore(model, summary_path):
    """The new model's picks on an earlier run's held-out systems, every
    candidate of which was run and checked there (no new solves)."""
    with open(summary_path) as f:
        old = json.load(f)["heldout"]
    out = []
    for h in old:
        rows = h["runs"]
        cands = [learned.PrecondConfig(**r["config"]) for r in rows]
        k = int(np.argmin(model.expected_cost(np.asarray(h["sys_feats"], np.float32), cands)))
        rec = dict(h)
        rec["pick"] = rows[k]
        rec["rank_of_pick"] = int(sorted(r["cost_s"] for r in rows).index(rows[k]["cost_s"]))
        out.append(rec)
    return out


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--systems", type=int, default=90)
    ap.add_argument("--large", type=int, default=6, help="extra systems with 12k-20k surface points")
    ap.add_argument("--configs", type=int, default=12)
    ap.add_argument("--large-configs", type=int, default=16)
    ap.add_argument("--epochs", type=int, default=300)
    ap.add_argument("--heldout", type=int, default=6)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--out", default="precond_training")
    ap.add_argument("--resume", default=None, help="model .npz to continue training from")
    ap.add_argument("--lu-weight-alpha", type=float, default=0.0,
                    help="weight each sample's loss by (LU seconds of its system)^alpha")
    ap.add_argument("--heldout-json", default=None,
                    help="summary.json of an earlier run: re-score its held-out runs instead of running new ones")
    ap.add_argument("--dataset", default=None, help="reuse a dataset .npz instead of generating one")
    ap.add_argument("--extra-dataset", action="append", default=[],
                    help="dataset .npz of an earlier run to train on together with the new one (repeatable)")
    a = ap.parse_args(argv)
    os.makedirs(a.out, exist_ok=True)
    summary = dict(args=vars(a))
    t0 = time.perf_counter()
    if a.dataset:
        z = np.load(a.dataset)
        ds = {k: z[k] for k in z.files}
        records = []
    else:
        ds1, rec1 = learned.generate(a.systems, base_seed=a.seed, configs_per_system=a.configs, n_min=1000,
                                     n_max=8000, seed=a.seed, log=print)
        ds2, rec2 = learned.generate(a.large, base_seed=a.seed + 50, configs_per_system=a.large_configs, n_min=12000,
                                     n_max=20000, seed=a.seed + 1, log=print)
        ds = {k: np.concatenate([ds1[k], ds2[k]]) for k in ds1}
        records = rec1 + rec2
        with open(os.path.join(a.out, "records.json"), "w") as f:
            json.dump(records, f)
    summary["generate_seconds"] = time.perf_counter() - t0
    summary["systems"] = len(records)
    summary["new_samples"] = int(len(ds["cost_s"]))
    for path in a.extra_dataset:
        z = np.load(path)
        ds = {k: np.concatenate([ds[k], z[k]]) for k in ds}
    summary["samples"] = int(len(ds["cost_s"]))
    np.savez(os.path.join(a.out, "dataset.npz"), **ds)  # everything the model was trained on

    model = learned.CostModel.load(a.resume) if a.resume else None
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    model, hist = learned.train(ds, epochs=a.epochs, batch=256, lr=2e-3, weight_decay=1e-3, seed=a.seed, model=model,
                                log_every=50, lu_weight_alpha=a.lu_weight_alpha)
    torch.cuda.synchronize()
    summary["train_seconds"] = time.perf_counter() - t1
    summary["train_steps"] = int(model.mlp.step)
    summary["loss_first_last"] = [hist[0], hist[-1]]
    model.meta.update(dict(samples=summary["samples"], systems=summary["systems"], epochs=a.epochs,
                           steps=int(model.mlp.step), final_loss=hist[-1]))
    model.save(os.path.join(a.out, "precond_cost.npz"))

    if a.heldout_json:
        ev = rescore(model, a.heldout_json)
    else:
        ev = evaluate(model, a.heldout, base_seed=99, n_min=4000, n_max=12000)
    summary["heldout"] = ev
    tp = sum(r["pick"]["cost_s"] for r in ev)
    td = sum(r["default"]["cost_s"] for r in ev)
    tb = sum(r["best"]["cost_s"] for r in ev)
    tl = sum(r["lu_seconds"] for r in ev)
    summary["heldout_totals"] = dict(pick=tp, default=td, best=tb, lu=tl,
                                     picks_ok=sum(r["pick"]["ok"] for r in ev))
    print(json.dumps(summary["heldout_totals"]))
    with open(os.path.join(a.out, "summary.json"), "w") as f:
        json.dump(summary, f, indent=1, default=float)


if __name__ == "__main__":
    main()
