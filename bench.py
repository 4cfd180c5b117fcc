"""EMST throughput benchmark (one JSON line on stdout).

Default workload: gauss3d_1e7 -- 10,000,000 3D points, 90% from 256 anisotropic
Gaussian clusters + 10% uniform background (seed 5), the plain Boruvka EMST.
  value   Mpoints/s with the points already in HBM (emst_solve_device), device
          time by CUDA events on the library's stream, L2 flushed between steps
  e2e     Mpoints/s through emst_solve with pinned host points in and host
          edges + length out (H2D and D2H inside the timed region)
  roofline  the static-pruning region-table kernel (k_nns): algorithmic bytes
          N*(4*D + 8*K) per launch / its CUDA-event time, against the measured
          HBM copy bandwidth
  cpu_baseline  the oracle (CPU restatement of the reference's algorithm)
          on a bounded sample of the same workload, 1 thread

--impl reference: the CPU restatement of the reference's path (oracle port,
OpenMP over all host cores), each step a bounded sample of the same workload.
Under torchrun (N > 1) every rank solves its own replica ("replicas only").
"""
import argparse
import hashlib
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "component-based-2d-3d-nns-to-gpu-parallel-2d-3d-emst_gb300")
sys.path.insert(0, PKG)

METRIC = "EMST Mpoints/s at 1e7 pts (learned vs plain, same edge set); % HBM roofline"
L2_FLUSH_BYTES = 512 << 20


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            f = [x.strip() for x in line.split(",")]
            if len(f) >= 8:
                self.rows.append(f)

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for f in self.rows:
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if f[4 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def nns_bytes(n, dim):
    """Algorithmic bytes of one static region-table launch (k_nns): read the
    sorted points once (4*D per point) and write K (id, d2) pairs (8*K per point)."""
    K = 8 if dim == 2 else 24
    return n * (4 * dim + 8 * K)


CNNS_BYTES_PER_QUERY = 16 + 4 + 12 + 8
"""Algorithmic bytes per query of the component search (k_cnns_t): read the
query point (float4) and its label, write partner + key, one 8-byte atomicMin."""

KNN_LIST = 6  # EMST_ROUND1_NEIGHBOURS
KNN_BYTES_PER_POINT = (16 + 4 + 4 + 4) + (8 * KNN_LIST + 1) + (4 + 4 + 8) + 8
"""Algorithmic bytes per point of the round-1 neighbour-list kernel (k_knn_first):
read the query point (float4), its input id, label and list slot; write its
6 list entries (8 B each) and list cursor (1 B), its lower bound, partner and
key; one 8-byte atomicMin.  Candidates are other queries' points: each point is
read once."""

PHASES = ["ms_grid", "ms_octants", "ms_select", "ms_resolve", "ms_hook", "ms_flatten"]


def profile_value(name, key):
    """A figure from a committed ncu summary profiles/<name>.md: the line
    '<key>: <value>' (null if absent)."""
    path = os.path.join(ROOT, "profiles", "%s.md" % name)
    try:
        for line in open(path):
            if line.startswith(key + ":"):
                return float(line.split(":")[1])
    except OSError:
        pass
    return None


def traffic_from_profile(name):
    """Mean DRAM bytes (read + write) per launch of the dominant kernel, from the
    committed ncu summary profiles/<kernel>_<workload>.md (null if absent)."""
    return profile_value(name, "traffic_bytes_per_launch")


def issue_from_profile(kernel):
    """What bounds an instruction-bound search kernel, from its committed full
    ncu section set (profiles/<kernel>_gauss3d_4e6.md): issue-slot use, warp
    instructions per 32 queries and active lanes per instruction."""
    name = "%s_gauss3d_4e6" % kernel
    busy = profile_value(name, "issue_slots_busy")
    if busy is None:
        return None
    return {"bound": "instruction issue", "issue_slots_busy": busy,
            "warp_instructions_per_32_queries": profile_value(name, "warp_instructions_per_32_queries"),
            "active_lanes_per_instruction": profile_value(name, "active_lanes_per_instruction"),
            "source": "ncu --set full of the same kernel on 4e6 points of the same generator (profiles/%s.md)" % name}


def cpu_baseline(pts, threads, sample_n, seed=0, with_edges=False):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as O
    rng = np.random.default_rng(seed)
    idx = rng.choice(len(pts), min(sample_n, len(pts)), replace=False)
    sub = np.ascontiguousarray(pts[np.sort(idx)])
    O.set_threads(threads)
    # timed from the raw points, as the GPU solve is (rescale included)
    t0 = time.perf_counter()
    sp, _, _, _ = O.rescale(sub)
    r = O.emst(sp, "faithful")
    dt = time.perf_counter() - t0
    assert len(r.edges) == len(sub) - 1
    if with_edges:
        return len(sub) / dt / 1e6, dt, len(sub), sub, np.asarray(r.edges).reshape(-1, 2)
    return len(sub) / dt / 1e6, dt, len(sub)


def cpu_model():
    """The host CPU's model name (lscpu, else /proc/cpuinfo)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return None


def canon_edges(uv):
    a = np.sort(np.asarray(uv, np.int64).reshape(-1, 2), axis=1)
    return a[np.lexsort((a[:, 1], a[:, 0]))]


def batch_bench(E, device, reps=3, rank=0, world=1, dist=None):
    """512-cloud workload (sizes log-uniform 1e3..1e5, half 2D half 3D, uniform
    or 8-cluster): clouds/s of one batched solve (emst_solve_batch) vs the plain
    solver launched once per cloud (emst_solve), host buffers in and out.  With
    several ranks the cloud list is sharded by cumulative size, each rank solves
    its share on its GPU and rank 0 gathers every cloud's edges (emst_shard)."""
    import emst_workloads as W
    clouds = W.batch_clouds()
    total = sum(len(c) for c in clouds)
    if world > 1:
        import emst_shard
        with E.Emst(device=device) as e:
            emst_shard.solve_sharded(clouds, rank, world, e.solve_batch, dist)  # warm-up
            dt = []
            for _ in range(reps):
                dist.barrier()
                t0 = time.perf_counter()
                uvs, _ = emst_shard.solve_sharded(clouds, rank, world, e.solve_batch, dist)
                dt.append(time.perf_counter() - t0)
        import torch
        t = torch.tensor([sum(dt) / reps], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        tb = float(t.item())
        return {"clouds": len(clouds), "points": total, "ranks": world, "batched_clouds_per_s": len(clouds) / tb,
                "batched_ms": 1e3 * tb,
                "note": "cloud list sharded by cumulative size over the ranks, one batched solve per rank, edges "
                        "gathered to rank 0; wall clock, max over ranks"}
    with E.Emst(device=device) as e:
        e.solve_batch(clouds)
        t0 = time.perf_counter()
        for _ in range(reps):
            uvs, _ = e.solve_batch(clouds)
        tb = (time.perf_counter() - t0) / reps
        for c in clouds[:8]:
            e.solve(c)
        t0 = time.perf_counter()
        for c in clouds:
            e.solve(c)
        tl = time.perf_counter() - t0
    return {"clouds": len(clouds), "points": total, "batched_clouds_per_s": len(clouds) / tb,
            "per_cloud_clouds_per_s": len(clouds) / tl, "speedup": tl / tb,
            "batched_ms": 1e3 * tb, "per_cloud_ms": 1e3 * tl,
            "note": "wall clock, host points in / host edges + lengths out, same edge sets"}


def edge_hash(d_uv):
    """Canonical hash of an edge list on the device: pairs (min, max), sorted."""
    a = np.sort(d_uv.cpu().numpy().astype(np.int64), axis=1)
    key = np.sort(a[:, 0] * (1 << 32) + a[:, 1])
    return hashlib.sha1(key.tobytes()).hexdigest()


def learned_leg(E, args, local, stream, settings, flush, dev_pts, d_uv, d_len, n, dim):
    """Learned-vs-plain comparison on the benchmark workload: the same steps
    with and without the trained proposal, both on the autotuned search
    settings with the list length the network is trained for, interleaved;
    edge-set identity and the proposal's counters."""
    import torch
    import emst_proposal as PR
    w, info = PR.load()
    if w is None:
        return {"unavailable": "no trained weights (run emst_proposal.py)"}
    margin = float(info.get("margin", PR.DEFAULT_MARGIN))
    thr = float(info.get("threshold", PR.DEFAULT_THRESHOLD))
    cfg = dict(settings)
    cfg["round1_neighbours"] = E.ROUND1_NEIGHBOURS  # the network's list length
    ctxs = {"plain": E.Emst(device=local, **cfg), "learned": E.Emst(device=local, **cfg)}
    ctxs["learned"].set_proposal(w, margin, thr)
    hashes, ms = {}, {"plain": [], "learned": []}
    for name, c in ctxs.items():
        c.set_stream(stream.cuda_stream)
        for _ in range(args.warmup):
            c.solve_device(dev_pts.data_ptr(), n, dim, d_uv.data_ptr(), d_len.data_ptr())
        hashes[name] = edge_hash(d_uv)
    torch.cuda.synchronize()
    for _ in range(args.steps):
        for name, c in ctxs.items():
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            c.solve_device(dev_pts.data_ptr(), n, dim, d_uv.data_ptr(), d_len.data_ptr())
            e1.record(stream)
            e1.synchronize()
            ms[name].append(e0.elapsed_time(e1))
    for c in ctxs.values():
        c.close()
    same = hashes["learned"] == hashes["plain"]

    def counters(weights):
        with E.Emst(device=local, profile=True, **cfg) as pc:
            pc.set_stream(stream.cuda_stream)
            if weights is not None:
                pc.set_proposal(weights, margin, thr)
            pc.solve_device(dev_pts.data_ptr(), n, dim, d_uv.data_ptr(), d_len.data_ptr())
            return pc.profile()

    pp, pl = counters(None), counters(w)
    K = args.steps

    def per(p):
        q = max(p["search_queries"], 1)
        return {"searches_per_point": p["search_queries"] / n, "cells_visited_per_query": p["leaf_visits"] / q,
                "cells_visited_per_point": p["leaf_visits"] / n, "node_tests_per_query": p["node_tests"] / q,
                "knn_candidates_marked_per_point": p["knn_marked"] / n,
                "knn_insert_steps_per_warp": p["knn_insert_steps"] / max(n / 32, 1),
                "knn_learned_queries": p["knn_learned"], "knn_resumed_queries": p["knn_resumed"],
                "ms_knn": p["ms_knn"] / max(p["knn_launches"], 1)}
    mp, ml = sum(ms["plain"]) / K, sum(ms["learned"]) / K
    return {"value": n / (ml / 1e3) / 1e6, "unit": "Mpoints/s", "ms_per_step": ml,
            "plain_value": n / (mp / 1e3) / 1e6, "plain_ms_per_step": mp, "vs_plain": mp / ml,
            "same_edge_set": same, "margin": margin, "threshold": thr, "settings": cfg,
            "mispredict_rate": pl["knn_resumed"] / max(pl["knn_learned"], 1),
            "plain": per(pp), "learned": per(pl),
            "weights": {k: info.get(k) for k in ("records", "clouds", "points_per_cloud", "generator", "epochs",
                                                  "loss_curve")},
            "note": "plain and learned timed interleaved on the same settings (list length of the trained "
                    "network); the top-level value is the autotuned plain form (the library default)"}


def workload_config(workload, n, dim):
    """The benchmark configuration, the same dict in both arms."""
    return {"workload": workload, "n": n, "dim": dim,
            "l2": "GPU arm: 512 MB buffer written between timed steps; working set > 129 MB L2"}


def run_reference(args, pts, dim):
    """The CPU restatement of the reference's path, all host threads."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as O
    threads = os.cpu_count() or 1
    sample_n = args.ref_sample
    for _ in range(args.warmup):
        cpu_baseline(pts, threads, min(sample_n, 20000), seed=1)
    times, npts = [], 0
    for s in range(args.steps):
        v, dt, m = cpu_baseline(pts, threads, sample_n, seed=100 + s)
        times.append(dt)
        npts += m
    total = sum(times)
    value = npts / total / 1e6
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "Mpoints/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": workload_config(args.workload, len(pts), dim),
            "cpu_baseline": {"value": value, "unit": "Mpoints/s", "cores": threads, "kind": "port",
                             "cpu_model": cpu_model(),
                             "sample": "%d random points of %s per step (CPU restatement of the reference's "
                                       "ring-search static pruning + Boruvka, OpenMP)" % (sample_n, args.workload)},
            "e2e": {"value": value, "unit": "Mpoints/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="gauss3d_1e7")
    ap.add_argument("--n", type=int, default=None, help="override the workload size")
    ap.add_argument("--cpu-sample", type=int, default=100_000)
    ap.add_argument("--ref-sample", type=int, default=400_000)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--mode", type=int, default=0, help="0: component search, 1: static region table")
    ap.add_argument("--no-static", action="store_true", help="skip the one-step static-table comparison")
    ap.add_argument("--no-batch", action="store_true", help="skip the 512-cloud batch comparison")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default launch shape")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned-proposal leg")
    args = ap.parse_args()

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    import emst_workloads as W
    pts = W.make(args.workload, args.n)
    n, dim = pts.shape

    if args.impl == "reference":
        if rank == 0:
            run_reference(args, pts, dim)
        return

    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    import emst_gb300 as E

    dev_pts = torch.from_numpy(pts).cuda()
    d_uv = torch.empty((max(n - 1, 1), 2), dtype=torch.int32, device="cuda")
    d_len = torch.empty(1, dtype=torch.float64, device="cuda")
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    # one dedicated stream for torch's work (inputs, the L2 flush, events) and the
    # library's, so that every step is ordered after the previous one
    stream = torch.cuda.Stream()
    torch.cuda.synchronize()  # inputs above were made on the default stream
    torch.cuda.set_stream(stream)
    # timed context: the default path (the component search runs its round loop
    # as one CUDA graph); a separate profiled context (host-driven rounds with
    # per-phase CUDA events) gives the phase split and the kernel times
    ctx = E.Emst(device=local, search_mode=args.mode)
    ctx.set_stream(stream.cuda_stream)
    # search settings of the component search: the autotuner times the
    # round-1 list length, the list-length thresholds of the search kernels and
    # the thread-per-query launch shape on this workload (before the timed
    # region) and keeps the fastest of each; the other contexts take them over
    shape, shape_ms = 0, None
    tuning = None
    if args.mode == 0 and not args.no_autotune:
        shape, shape_ms = ctx.autotune(pts)
        tuning = ctx.tuning()
    settings = {} if tuning is None else {"search_shape": tuning["search_shape"], "round1_neighbours": tuning["knn_k"],
                                          "wide_max_list": tuning["wide_max"], "coop_min_list": tuning["coop_min"]}
    _, sh_threads, sh_blocks = E.search_shapes()
    sh = shape if shape else 2  # library default: entry 2 of the table
    launch_shape = {"threads": int(sh_threads[sh - 1]), "min_blocks_per_sm": int(sh_blocks[sh - 1]),
                    "search_shape": sh, "autotuned_ms": None if shape_ms is None else [round(float(v), 3) for v in shape_ms]}
    if tuning is not None:
        r3 = lambda v: [round(float(x), 3) for x in v]
        launch_shape["autotune"] = {
            "round1_list_length": {"chosen": tuning["knn_k"], "candidates": tuning["knn_k_values"],
                                   "ms": r3(tuning["ms_knn_k"])},
            "coop_min_list": {"chosen": tuning["coop_min"], "candidates": tuning["coop_min_values"],
                              "ms": r3(tuning["ms_coop_min"])},
            "wide_max_list": {"chosen": tuning["wide_max"], "candidates": tuning["wide_max_values"],
                              "ms": r3(tuning["ms_wide_max"])},
            "search_shape": {"chosen": tuning["search_shape"], "ms": r3(tuning["ms_shape"])}}
        every = [v for k in ("ms_knn_k", "ms_coop_min", "ms_wide_max", "ms_shape") for v in tuning[k] if v > 0]
        launch_shape["autotune"]["spread"] = {"best_ms": round(min(every), 3), "worst_ms": round(max(every), 3)}
    pctx = E.Emst(device=local, profile=True, search_mode=args.mode, **settings)
    pctx.set_stream(stream.cuda_stream)

    def step():
        return ctx.solve_device(dev_pts.data_ptr(), n, dim, d_uv.data_ptr(), d_len.data_ptr())

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()

    def barrier():
        if dist is not None:
            dist.barrier()

    sampler = ClockSampler(local)
    sampler.start()
    barrier()
    torch.cuda.synchronize()
    dev_ms, launches, rounds = [], 0, 0
    phase = {k: 0.0 for k in PHASES}
    stat = {"leaf_visits": 0, "node_tests": 0, "candidates": 0, "search_warps": 0, "search_queries": 0,
            "octant_launches": 0, "ms_knn": 0.0, "ms_search": 0.0, "knn_launches": 0, "search_launches": 0}
    for _ in range(args.steps):
        flush.zero_()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        ne = step()
        ev1.record(stream)
        ev1.synchronize()
        dev_ms.append(ev0.elapsed_time(ev1))
        prof = ctx.profile()
        launches += prof["launches"]
        rounds = prof["rounds"]
        assert ne == n - 1
    torch.cuda.synchronize()
    barrier()
    clocks = sampler.stop()
    total_ms = sum(dev_ms)
    if dist is not None:
        t = torch.tensor([total_ms], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    value = world * n * args.steps / (total_ms / 1e3) / 1e6

    # learned proposal: the same steps with the trained network steering the
    # first search pass; its edge set must equal the plain one
    learned = None
    if args.mode == 0 and not args.no_learned and rank == 0:
        learned = learned_leg(E, args, local, stream, settings, flush, dev_pts, d_uv, d_len, n, dim)

    # profiled run(s): phase split, search counters and the dominant kernel's time
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        pctx.solve_device(dev_pts.data_ptr(), n, dim, d_uv.data_ptr(), d_len.data_ptr())
        prof = pctx.profile()
        for k in PHASES:
            phase[k] += prof[k]
        for k in stat:
            stat[k] += prof[k]
    pctx.close()

    # e2e through the public host API: pinned points in, host edges + length out
    host_pts = torch.from_numpy(pts).pin_memory().numpy()
    host_uv = torch.empty((max(n - 1, 1), 2), dtype=torch.int32).pin_memory().numpy()
    for _ in range(max(1, args.warmup // 2)):
        ctx.solve_into(host_pts, host_uv)
    e2e_s = 0.0
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ne, length = ctx.solve_into(host_pts, host_uv)
        e2e_s += time.perf_counter() - t0
    e2e = world * n * args.steps / e2e_s / 1e6

    peak, peak_kind = peaks()
    K = args.steps
    if args.mode == 0:
        # the dominant search kernel, timed by CUDA events around its own
        # launches on the library's stream (profile contexts run host-driven
        # rounds): the round-1 neighbour-list kernel or the component search
        if stat["ms_knn"] >= stat["ms_search"] and stat["knn_launches"] > 0:
            kernel = "k_knn_first"
            n_launch = stat["knn_launches"]
            per_launch_ms = stat["ms_knn"] / n_launch
            alg = KNN_BYTES_PER_POINT * n
        else:
            kernel = "k_cnns_t"
            n_launch = max(stat["search_launches"], 1)
            per_launch_ms = stat["ms_search"] / n_launch
            later = stat["search_queries"] - (n * K if stat["knn_launches"] else 0)
            alg = CNNS_BYTES_PER_QUERY * later / n_launch
    elif args.mode == 2:
        kernel = "k_cnns"
        n_launch = max(stat["octant_launches"], 1)
        per_launch_ms = phase["ms_select"] / n_launch
        alg = CNNS_BYTES_PER_QUERY * stat["search_queries"] / n_launch
    else:
        kernel = "k_nns"
        n_launch = max(stat["octant_launches"], 1)
        per_launch_ms = phase["ms_octants"] / n_launch
        alg = nns_bytes(n, dim) * K / n_launch
    achieved = alg / (per_launch_ms / 1e3) / 1e9
    traffic = traffic_from_profile("%s_%s" % (kernel, args.workload)) if args.n is None else None
    issue = issue_from_profile(kernel) if args.workload.startswith("gauss3d") else None
    search = {"leaf_visits_per_warp": stat["leaf_visits"] / max(stat["search_warps"], 1),
              "node_tests_per_warp": stat["node_tests"] / max(stat["search_warps"], 1),
              "candidates_per_point": stat["candidates"] / (n * K),
              "searches_per_point": stat["search_queries"] / (n * K) if args.mode != 1 else 1.0}
    phase_ms = {k[3:]: round(v / K, 3) for k, v in phase.items()}

    static = None
    if args.mode != 1 and not args.no_static:
        with E.Emst(device=local, search_mode=1) as cs:
            cs.set_stream(stream.cuda_stream)
            cs.solve_device(dev_pts.data_ptr(), n, dim, d_uv.data_ptr(), d_len.data_ptr())
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            cs.solve_device(dev_pts.data_ptr(), n, dim, d_uv.data_ptr(), d_len.data_ptr())
            e1.record(stream)
            e1.synchronize()
            static = {"value": n / (e0.elapsed_time(e1) / 1e3) / 1e6, "unit": "Mpoints/s", "steps": 1,
                      "note": "static-pruning region table (the reference's computeOctants), same edge set"}

    batch = None
    if not args.no_batch and (rank == 0 or world > 1):
        batch = batch_bench(E, local, rank=rank, world=world, dist=dist)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        v, dt, m, sub, cedges = cpu_baseline(pts, 1, args.cpu_sample, with_edges=True)
        with E.Emst(device=local) as ce:  # the same sample on the GPU: same edge set
            guv, _ = ce.solve(sub)
        cpu = {"value": v, "unit": "Mpoints/s", "cores": 1, "kind": "port", "cpu_model": cpu_model(),
               "host_threads": os.cpu_count(),
               "edge_set_match": bool(np.array_equal(canon_edges(guv), canon_edges(cedges))),
               "sample": "%d random points of %s (%.1f s), CPU restatement of the reference's ring-search static "
                         "pruning + Boruvka, single thread" % (m, args.workload, dt)}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "Mpoints/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": workload_config(args.workload, n, dim),
                "settings": {"rounds": rounds,
                             "search": {0: "component: round-1 neighbour lists (warp per 32 queries); later "
                                           "rounds by query-list length: warp per query, thread per query, "
                                           "warp per 32 queries", 1: "static region table",
                                        2: "component, warp per 32 queries"}[args.mode],
                             "launch_shape": launch_shape,
                             "parallelism": "replicas" if world > 1 else "single"},
                "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                             "frac": achieved / peak, "traffic": traffic, "kernel": kernel,
                             "alg_bytes_per_launch": alg, "ms_per_launch": per_launch_ms,
                             "peak_kind": peak_kind, "issue": issue},
                "phase_ms": phase_ms, "learned": learned, "static_table_mode": static, "batch512": batch,
                "cpu_baseline": cpu,
                "e2e": {"value": e2e, "unit": "Mpoints/s", "h2d_bytes_per_step": int(pts.nbytes),
                        "d2h_bytes_per_step": int(8 * (n - 1) + 8)},
                "gpu_launches": launches, "clocks": clocks, "search": search}
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()
    ctx.close()


if __name__ == "__main__":
    main()
