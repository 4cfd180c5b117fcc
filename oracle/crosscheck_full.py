"""Cross-check of the two CPU restatements at full benchmark sizes.

TEST INFRASTRUCTURE ONLY (runs the oracle, no GPU): solves a named workload
with the faithful ring-search restatement (emst_oracle.c) and the kd-tree
restatement (emst_kd_oracle.c) on all host cores and reports both times,
whether edges (in order) and labels are identical, and the canonical edge
hash (SHA-256 of the sorted (min id << 32 | max id) pairs, first 16 hex
digits) to compare with a GPU solve of the same workload.  The faithful
search is slow on clustered sets (its cells are overfull): minutes at 10^6
points, 51 minutes on 8 x86 threads for gauss3d_1e7.

    python oracle/crosscheck_full.py gauss3d_1e6 bezier2d_1e7
"""
import hashlib
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "component-based-2d-3d-nns-to-gpu-parallel-2d-3d-emst_gb300"))

import numpy as np  # noqa: E402

import emst_workloads as W  # noqa: E402
import pyoracle as O  # noqa: E402


def main(names):
    O.set_threads(os.cpu_count() or 1)
    for name in names:
        pts = W.make(name)
        sp, _, _, _ = O.rescale(pts)
        t0 = time.perf_counter()
        a = O.emst(sp, "faithful")
        t1 = time.perf_counter()
        b = O.emst_kd(sp)
        t2 = time.perf_counter()
        same = np.array_equal(a.edges, b.edges) and np.array_equal(a.labels, b.labels)
        print("%s n=%d threads=%d faithful %.1f s kd %.1f s identical=%s edge_hash=%s" % (
            name, len(pts), os.cpu_count(), t1 - t0, t2 - t1, same, edge_hash(a.edges)), flush=True)


def edge_hash(edges):
    """Canonical edge hash: SHA-256 of the sorted (min id << 32 | max id)
    pairs as int64, first 16 hex digits."""
    e = np.asarray(edges, dtype=np.int64).reshape(-1, 2)
    key = np.sort(np.minimum(e[:, 0], e[:, 1]) << 32 | np.maximum(e[:, 0], e[:, 1]))
    return hashlib.sha256(key.tobytes()).hexdigest()[:16]


if __name__ == "__main__":
    main(sys.argv[1:] or ["uniform2d_1e4"])
