"""Train the hybrid's smoothness classifier on the GPU with libfst's own
kernels and write fiesta_gb300/classifier_params.json.

Data: every face of 4 states of each of `--runs` seeded runs (expanding
high-pressure bubbles, planar shock tubes, Gaussian pressure-kernel mixing,
smooth random fields; the benchmark's five-species gas) at `--n`^3, labelled
by WENO5 smoothness-indicator ratios (> `--ratio` means the face needs WENO).
Measured on the 256^3 benchmark case over 9 steps against the FP64 path: the
default 1.1 routes 53 % of faces to WENO5 and keeps every conserved field
within 1.6e-6 (rel-L2); 1.5 routes 4.6 % and reaches 1.1e-4 on the momentum
increments; 1.03 routes 77 % and gives 4.6e-8.
The last run of each kind is held out for validation.

    python -m fiesta_gb300.train_classifier [--runs 50] [--n 48] [--epochs 6]
"""
import argparse
import json
import os
import time

import numpy as np

from . import hybrid as H

HERE = os.path.dirname(os.path.abspath(__file__))
PARAMS_JSON = os.path.join(HERE, "classifier_params.json")


def load_params(path=PARAMS_JSON):
    if not os.path.exists(path):
        return None
    d = json.load(open(path))
    return np.asarray(d["params"], dtype=np.float32), d


def main():
    import torch
    ap = argparse.ArgumentParser()
    ap.add_argument("--runs", type=int, default=50)
    ap.add_argument("--n", type=int, default=48)
    ap.add_argument("--snapshots", type=int, default=4)
    ap.add_argument("--epochs", type=int, default=6)
    ap.add_argument("--ratio", type=float, default=1.1)
    ap.add_argument("--pos-weight", type=float, default=3.0)
    ap.add_argument("--threshold", type=float, default=0.35)
    ap.add_argument("--out", default=PARAMS_JSON)
    a = ap.parse_args()
    t0 = time.time()
    X, Y = H.generate_training_data(n_runs=a.runs, n=a.n, snapshots=a.snapshots,
                                    label_ratio=a.ratio)
    per_run = X.shape[0] // a.runs
    nval = 4 * per_run
    Xt, Yt, Xv, Yv = X[:-nval], Y[:-nval], X[-nval:], Y[-nval:]
    t1 = time.time()
    params, losses = H.train(Xt, Yt, epochs=a.epochs, lr=3e-3, batch=16384,
                             pos_weight=a.pos_weight, seed=0)
    t2 = time.time()
    prob = H.forward(Xv, params, tensor_cores=True)
    yv = Yv.cpu().numpy().astype(bool)
    weno = prob > a.threshold
    meta = {
        "params": [float(x) for x in params],
        "threshold": a.threshold, "label_ratio": a.ratio, "pos_weight": a.pos_weight,
        "train_faces": int(Xt.shape[0]), "val_faces": int(Xv.shape[0]),
        "label_positive_fraction": float(Y.float().mean().item()),
        "epoch_losses": losses,
        "val_weno_fraction": float(weno.mean()),
        "val_miss_rate": float((yv & ~weno).sum() / max(1, yv.sum())),
        "val_accuracy": float(((prob > 0.5) == yv).mean()),
        "runs": a.runs, "n": a.n, "snapshots": a.snapshots,
        "data_seconds": t1 - t0, "train_seconds": t2 - t1,
        "trained_on": torch.cuda.get_device_name(0),
    }
    with open(a.out, "w") as f:
        json.dump(meta, f)
    print(json.dumps({k: v for k, v in meta.items() if k != "params"}))


if __name__ == "__main__":
    main()
