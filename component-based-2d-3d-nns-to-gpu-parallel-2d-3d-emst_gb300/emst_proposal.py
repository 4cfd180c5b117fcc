"""Learned search proposal: traces, training and the weights file.

The plain component search (search_mode 0) writes training traces: for a
sample of first-pass queries, the 8 features the fused inference sees, and
after the round the d2 of the shortest edge the query's component got and
whether the query's lower bound allowed it to hold that edge.  Training runs
on the GPU in the library's own BF16 tensor-core forward/backward kernels
with Adam (emst_proposal_train).  The trained weights live in
proposal_weights.json beside this file, with how they were made.

Training set: 64 clouds of 10^6 3D points from the clustered-Gaussian
generator with 256 clusters (seeds 1000..1063), disjoint from the seeds of
the benchmark workloads.

    python emst_proposal.py [--clouds 64] [--n 1000000] [--out proposal_weights.json]
"""
import argparse
import json
import os
import time

import numpy as np

import emst_gb300 as E
import emst_workloads as W

HERE = os.path.dirname(os.path.abspath(__file__))
WEIGHTS_PATH = os.path.join(HERE, "proposal_weights.json")
DEFAULT_MARGIN = 4.0     # log2 factor on the predicted radius (d2)
DEFAULT_THRESHOLD = 1.0  # class logit at or above which a point searches first


def training_clouds(n_clouds=64, n=1_000_000, first_seed=1000, clusters=256):
    for s in range(first_seed, first_seed + n_clouds):
        yield s, W.gauss_mixture(n, 3, clusters, s)


def fit(n_clouds=64, n=1_000_000, sample_shift=4, epochs=4, batch=4096, lr=2e-3, reg_weight=1.0, seed=0,
        device=0, capacity=None):
    """Traces from the plain method on the training clouds, then training.
    -> (weights, info dict)."""
    if capacity is None:
        capacity = max(1 << 16, int(n_clouds * n * 6 / (1 << sample_shift)))
    t0 = time.perf_counter()
    with E.Emst(device=device) as e:
        e.trace_enable(capacity, sample_shift)
        for _, pts in training_clouds(n_clouds, n):
            e.solve(pts)
        ptr, count = e.trace_device()
        t1 = time.perf_counter()
        w0 = E.proposal_init(seed)
        w, curve = E.proposal_train(None, w0, epochs=epochs, batch=batch, lr=lr, reg_weight=reg_weight, seed=seed,
                                    device=device, records_on_device=ptr, n_records=count)
    t2 = time.perf_counter()
    info = {"records": int(count), "clouds": n_clouds, "points_per_cloud": n, "sample_shift": sample_shift,
            "generator": "gauss_mixture(n, 3, 256 clusters, seed), seeds %d..%d" % (1000, 1000 + n_clouds - 1),
            "epochs": epochs, "batch": batch, "lr": lr, "reg_weight": reg_weight, "seed": seed,
            "loss_curve": [float(v) for v in curve], "trace_s": t1 - t0, "train_s": t2 - t1,
            "margin": DEFAULT_MARGIN, "threshold": DEFAULT_THRESHOLD}
    return w, info


def save(weights, info, path=WEIGHTS_PATH):
    with open(path, "w") as f:
        json.dump({"info": info, "weights": [float(v) for v in np.asarray(weights, np.float32)]}, f, indent=0)


def load(path=WEIGHTS_PATH):
    """-> (weights float32[1410], info) or (None, None) when there is no file."""
    if not os.path.exists(path):
        return None, None
    with open(path) as f:
        d = json.load(f)
    w = np.asarray(d["weights"], np.float32)
    assert w.size == E.PROPOSAL_WEIGHTS
    return w, d["info"]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--clouds", type=int, default=64)
    ap.add_argument("--n", type=int, default=1_000_000)
    ap.add_argument("--shift", type=int, default=4)
    ap.add_argument("--epochs", type=int, default=4)
    ap.add_argument("--batch", type=int, default=4096)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--out", default=WEIGHTS_PATH)
    a = ap.parse_args()
    w, info = fit(a.clouds, a.n, a.shift, a.epochs, a.batch, a.lr)
    save(w, info, a.out)
    print(json.dumps(info))


if __name__ == "__main__":
    main()
