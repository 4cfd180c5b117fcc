"""Learned search proposal: traces, training, calibration and the weights file.

The proposal steers the round-1 neighbour-list build, the dominant step of a
solve: for each query it predicts how far below the own leaf's certified
bound its K-th nearest distance lies (and a gate: whether the bound can be
tightened at all), and the walk starts from that radius (include/emst.h,
emst_set_proposal).  The plain method writes the training traces: for a
sample of round-1 queries, the 8 features the fused inference sees and,
once the query's list is complete, the targets.  Training runs on the GPU in
the library's own BF16 tensor-core forward/backward kernels with Adam
(emst_proposal_train).  The margin on the predicted radius is then chosen on
held-out records (the quantile of the log2 shortfall between prediction and
truth) and confirmed by timing solves of a training cloud.  The trained
weights live in proposal_weights.json beside this file, with how they were
made.

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
DEFAULT_MARGIN = 1.0      # log2 factor on the predicted radius (d2)
DEFAULT_THRESHOLD = 0.0   # gate logit at or above which a query starts from the predicted radius
QUANTILES = (0.98, 0.99, 0.995, 0.999)


def training_clouds(n_clouds=64, n=1_000_000, first_seed=1000, clusters=256):
    for s in range(first_seed, first_seed + n_clouds):
        yield s, W.gauss_mixture(n, 3, clusters, s)


def predict(weights, feats):
    """The network's two outputs for rows of 8 features (FP32, numpy): used
    to calibrate the margin on held-out records."""
    w = np.asarray(weights, np.float32)
    o = 0
    W1 = w[o:o + 256].reshape(8, 32); o += 256
    b1 = w[o:o + 32]; o += 32
    W2 = w[o:o + 1024].reshape(32, 32); o += 1024
    b2 = w[o:o + 32]; o += 32
    W3 = w[o:o + 64].reshape(32, 2); o += 64
    b3 = w[o:o + 2]
    h = np.maximum(np.asarray(feats, np.float32) @ W1 + b1, 0)
    h = np.maximum(h @ W2 + b2, 0)
    out = h @ W3 + b3
    return out[:, 0], out[:, 1]


def margin_for(weights, records, quantile, threshold=DEFAULT_THRESHOLD):
    """Smallest margin (log2, in d2) that covers `quantile` of the held-out
    queries the gate lets through: below it their radius would hold fewer
    than K points and they would be searched again."""
    r = np.asarray(records, np.float32)
    r = r[r[:, 10] > 0]
    o0, o1 = predict(weights, r[:, :8])
    use = o1 >= threshold
    if not use.any():
        return 0.0
    short = 8.0 * (r[use, 8] - o0[use])  # log2 factor the prediction falls short by
    return float(max(0.0, np.quantile(short, quantile) + 0.05))


def time_margins(weights, pts, margins, threshold=DEFAULT_THRESHOLD, device=0, reps=3):
    """Best-of-reps solve time (s, host clock, points on the host) per margin."""
    out = []
    with E.Emst(device=device) as e:
        e.solve(pts)
        for m in margins:
            e.set_proposal(weights, m, threshold)
            e.solve(pts)
            best = float("inf")
            for _ in range(reps):
                t0 = time.perf_counter()
                e.solve(pts)
                best = min(best, time.perf_counter() - t0)
            out.append(best)
    return out


def fit(n_clouds=64, n=1_000_000, sample_shift=4, epochs=4, batch=4096, lr=2e-3, reg_weight=1.0, seed=0,
        device=0, capacity=None, holdout=0.1):
    """Traces from the plain method on the training clouds, training, margin
    calibration.  -> (weights, info dict)."""
    if capacity is None:
        capacity = max(1 << 16, int(n_clouds * n / (1 << sample_shift) * 1.05))
    t0 = time.perf_counter()
    last = None
    with E.Emst(device=device) as e:
        e.trace_enable(capacity, sample_shift)
        for _, pts in training_clouds(n_clouds, n):
            e.solve(pts)
            last = pts
        rec = e.trace()
    t1 = time.perf_counter()
    rng = np.random.default_rng(seed)
    idx = rng.permutation(len(rec))
    n_hold = int(len(rec) * holdout)
    hold, train = rec[idx[:n_hold]], np.ascontiguousarray(rec[idx[n_hold:]])
    w0 = E.proposal_init(seed)
    w, curve = E.proposal_train(train, w0, epochs=epochs, batch=batch, lr=lr, reg_weight=reg_weight, seed=seed,
                                device=device)
    t2 = time.perf_counter()
    margins = [margin_for(w, hold, q) for q in QUANTILES]
    times = time_margins(w, last, margins, device=device)
    best = int(np.argmin(times))
    info = {"records": int(len(rec)), "train_records": int(len(train)), "holdout_records": int(n_hold),
            "clouds": n_clouds, "points_per_cloud": n, "sample_shift": sample_shift,
            "generator": "gauss_mixture(n, 3, 256 clusters, seed), seeds %d..%d" % (1000, 1000 + n_clouds - 1),
            "epochs": epochs, "batch": batch, "lr": lr, "reg_weight": reg_weight, "seed": seed,
            "loss_curve": [float(v) for v in curve], "trace_s": t1 - t0, "train_s": t2 - t1,
            "margin_quantiles": list(QUANTILES), "margin_candidates": margins,
            "margin_solve_s": times, "margin": margins[best], "threshold": DEFAULT_THRESHOLD}
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
