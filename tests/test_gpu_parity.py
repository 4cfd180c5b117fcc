"""GPU parity: the CUDA path (through the C ABI) against the oracle.

Bit-exact for everything integer (edge sets, per-round edge counts, labels,
region-table ids) and for the float values the reference computes in float
(rescaled coordinates, region-table squared distances).  Tree lengths are
doubles summed in a different order: relative tolerance 1e-9 against the
oracle, and 6 significant digits against the reference's recorded traces.
"""
import numpy as np
import pytest

import emst_workloads as W
import pyoracle as O
from families import KINDS, family

pytestmark = pytest.mark.gpu

TRACED = [("pts2d_1000", 2), ("pts2d_3000", 2), ("pts2d_4000", 2), ("pts3d_1000", 3), ("pts3d_2000", 3),
          ("pts3d_10000", 3)]


def _canon(e):
    return O.canon(np.asarray(e, np.int64))


def _is_spanning_tree(n, edges):
    if len(edges) != n - 1:
        return False
    par = np.arange(n)

    def find(x):
        while par[x] != x:
            par[x] = par[par[x]]
            x = par[x]
        return x

    for u, v in edges:
        a, b = find(u), find(v)
        if a == b:
            return False
        par[a] = b
    return True


MODES = [0, 1, 2, 3]  # 0: component search (default), 1: static region table (reference's computeOctants),
#                       2: component search, warp per 32 queries, 3: dynamic pruning (ring search over cells)


@pytest.mark.parametrize("mode", MODES)
def test_golden_3000_edges_labels_length(gpu_lib, fixtures, mode):
    pts = fixtures["pts2d_3000"]
    with gpu_lib.Emst(search_mode=mode) as e:
        e.initialize(pts)
        e.run()
        uv = e.edges()
        ne, length = e.evaluate()
        labels = e.labels()
        stats = e.round_stats()
    assert ne == 2999
    assert np.array_equal(_canon(uv), _canon(fixtures["outypu_edges"]))
    assert np.array_equal(labels, fixtures["outypu_labels"])
    assert list(stats) == [2058, 2724, 2931, 2983, 2996, 2999]
    assert float("%.6g" % length) == 359222.0
    assert length == pytest.approx(O.length(pts, uv.astype(np.int64)), rel=1e-9)


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("key,dim", TRACED)
def test_golden_round_traces(gpu_lib, fixtures, traces, key, dim, mode):
    pts = fixtures[key]
    n = len(pts)
    trace = traces["%dd" % dim]["%drandomCity.%dd" % (n, dim)][0]
    with gpu_lib.Emst(search_mode=mode) as e:
        e.initialize(pts)
        e.run()
        uv, rounds = e.edges(with_rounds=True)
        stats = e.round_stats()
    assert list(stats) == [row[1] for row in trace]
    uv = uv.astype(np.int64)
    for k, row in enumerate(trace):
        sel = uv[rounds <= k + 1]
        assert len(sel) == row[1]
        assert float("%.6g" % O.length(pts, sel)) == pytest.approx(row[2], rel=1e-6)
    sp, _, _, _ = O.rescale(pts)
    r = O.emst(sp, "faithful")
    assert np.array_equal(_canon(uv), _canon(r.edges))
    # same edges added in the same rounds as the reference's algorithm
    for k in range(1, r.rounds + 1):
        assert np.array_equal(_canon(uv[rounds == k]), _canon(r.edges[r.edge_round == k]))


@pytest.mark.parametrize("dim", [2, 3])
def test_rescale_bit_exact(gpu_lib, dim):
    pts = family("cluster", 5000, dim, 11) * np.float32(123.25) - np.float32(7.5)
    with gpu_lib.Emst() as e:
        e.initialize(pts)
        got, ux = e.rescaled()
    ref, rux, _, _ = O.rescale(pts)
    assert ux == rux
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("kind", KINDS)
def test_region_table_bit_exact(gpu_lib, kind, dim):
    pts = family(kind, 4000, dim, 21)
    with gpu_lib.Emst(keep_region_table=True) as e:
        e.initialize(pts)
        e.flatten()
        e.compute_octants()
        ids, d2 = e.region_table()
    sp, _, _, _ = O.rescale(pts)
    ti, td = O.region_table(sp, "brute")
    assert np.array_equal(ids.astype(np.int64), ti)
    assert np.array_equal(d2.view(np.uint32), td.view(np.uint32))


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("n", [2, 3, 17, 33, 1000, 6000])
@pytest.mark.parametrize("mode", MODES)
def test_edge_set_and_rounds_vs_oracle(gpu_lib, kind, dim, n, mode):
    pts = family(kind, n, dim, 1000 + n)
    with gpu_lib.Emst(search_mode=mode) as e:
        e.initialize(pts)
        e.run()
        uv, rounds = e.edges(with_rounds=True)
        stats = e.round_stats()
    sp, _, _, _ = O.rescale(pts)
    r = O.emst(sp, "faithful")
    assert np.array_equal(_canon(uv), _canon(r.edges))
    assert list(stats) == [int(x) for x in r.round_edges]
    if n <= 2000:
        assert np.array_equal(_canon(uv), _canon(O.prim(sp)))


@pytest.mark.parametrize("mode", MODES)
def test_operator_sequence_equals_run(gpu_lib, mode):
    pts = family("cluster", 20000, 3, 5)
    with gpu_lib.Emst(search_mode=mode) as e:
        e.initialize(pts)
        e.run()
        ref_edges = _canon(e.edges())
    with gpu_lib.Emst(search_mode=mode) as e:
        e.initialize(pts)
        others = []
        for _ in range(100):
            e.flatten()
            k = e.test_termination()
            others.append(k)
            if k == 0:
                break
            e.compute_octants()
            e.find_next_closest()
            e.find_min_pair()
            e.connect_union()
        assert others[-1] == 0 and all(o > 0 for o in others[:-1])
        assert np.array_equal(_canon(e.edges()), ref_edges)
        assert len(set(e.labels().tolist())) == 1


@pytest.mark.parametrize("kind,dim,n", [("cluster", 3, 50000), ("uniform", 2, 30000), ("dups", 3, 5000),
                                        ("uniform", 2, 2)])
def test_graph_loop_matches_host_loop(gpu_lib, kind, dim, n):
    """emst_run in the component mode runs the round loop as one CUDA graph with
    device-side termination; a profiled context runs it from the host.  Same
    edges, same rounds, same per-round counts."""
    pts = family(kind, n, dim, 77)
    out = []
    for prof in (False, True):
        with gpu_lib.Emst(profile=prof) as e:
            e.initialize(pts)
            e.run()
            uv, rounds = e.edges(with_rounds=True)
            out.append((_canon(uv), e.round_stats(), rounds, e.labels()))
    assert np.array_equal(out[0][0], out[1][0])
    assert list(out[0][1]) == list(out[1][1])
    assert np.array_equal(np.sort(out[0][2]), np.sort(out[1][2]))
    assert np.array_equal(out[0][3], out[1][3])


def test_batch_equals_per_cloud_solves(gpu_lib):
    """One batched solve of mixed 2D/3D clouds (sizes 0, 1, 2, small and large,
    duplicates and clusters) gives, cloud by cloud, the edge set and length of
    solving that cloud alone."""
    rng = np.random.default_rng(5)
    clouds = []
    for i in range(40):
        n = int(rng.choice([0, 1, 2, 3, 50, 500, 3000, 20000]))
        dim = int(rng.choice([2, 3]))
        kind = KINDS[i % len(KINDS)]
        clouds.append(family(kind, n, dim, 300 + i) if n > 0 else np.zeros((0, dim), np.float32))
    with gpu_lib.Emst() as e:
        uvs, lens = e.solve_batch(clouds)
    for pts, uv, ln in zip(clouds, uvs, lens):
        if len(pts) < 2:
            assert len(uv) == 0 and ln == 0.0
            continue
        with gpu_lib.Emst() as e:
            ref_uv, ref_len = e.solve(pts)
        assert np.array_equal(_canon(uv), _canon(ref_uv))
        assert ln == pytest.approx(ref_len, rel=1e-9)


def test_batch_workload_512_clouds_vs_oracle(gpu_lib):
    """The 512-cloud workload (sizes log-uniform 1e3..1e5, half 2D half 3D,
    uniform or 8-cluster): every cloud against the oracle on a sample, all
    against per-cloud solves."""
    clouds = W.batch_clouds()
    with gpu_lib.Emst() as e:
        uvs, lens = e.solve_batch(clouds)
    assert len(uvs) == 512
    for i in range(0, 512, 37):
        if len(clouds[i]) > 30000:
            continue
        sp, _, _, _ = O.rescale(clouds[i])
        ref = O.emst(sp, "faithful")
        assert np.array_equal(_canon(uvs[i]), _canon(ref.edges))
        assert lens[i] == pytest.approx(O.length(clouds[i], ref.edges), rel=1e-9)
    with gpu_lib.Emst() as e:
        for i in range(1, 512, 29):
            ref_uv, _ = e.solve(clouds[i])
            assert np.array_equal(_canon(uvs[i]), _canon(ref_uv))


@pytest.mark.parametrize("kind,dim,n", [("cluster", 3, 20000), ("uniform", 2, 20000), ("dups", 3, 3000)])
def test_every_search_shape_same_edges(gpu_lib, kind, dim, n):
    """Every launch shape of the component search gives the same edge set,
    single clouds and batches alike."""
    pts = family(kind, n, dim, 41)
    with gpu_lib.Emst() as e:
        ref, ref_len = e.solve(pts)
    count, threads, min_blocks = gpu_lib.search_shapes()
    assert count >= 2 and all(t % 32 == 0 for t in threads) and all(m >= 1 for m in min_blocks)
    for k in range(1, count + 1):
        # thread per query for every list, so each shape of k_cnns_t runs
        with gpu_lib.Emst(search_shape=k, wide_search=-1) as e:
            assert e.search_shape() == k
            uv, ln = e.solve(pts)
            assert np.array_equal(_canon(uv), _canon(ref)), k
            assert ln == pytest.approx(ref_len, rel=1e-12)
            uvs, _ = e.solve_batch([pts, pts[: n // 3]])
            assert np.array_equal(_canon(uvs[0]), _canon(ref)), k


def test_autotune_picks_a_shape_and_keeps_edges(gpu_lib):
    """emst_autotune times every list length, list-length threshold and
    launch shape, keeps the fastest of each stage, and later solves with them
    give the default settings' edge set."""
    pts = family("cluster", 30000, 3, 42)
    with gpu_lib.Emst() as e:
        ref, _ = e.solve(pts)
        assert e.search_shape() == 0
        t0 = e.tuning()
        assert t0["knn_k"] == gpu_lib.ROUND1_NEIGHBOURS and t0["coop_min"] == 150000 and t0["wide_max"] == 65536
        best, ms = e.autotune(pts)
        count, _, _ = gpu_lib.search_shapes()
        assert 1 <= best <= count and e.search_shape() == best
        assert np.all(np.isfinite(ms)) and np.all(ms > 0) and ms[best - 1] == ms.min()
        t = e.tuning()
        assert t["search_shape"] == best
        assert t["knn_k_values"] == [4, 5, 6, 8] and all(v > 0 for v in t["ms_knn_k"])
        assert t["knn_k"] == t["knn_k_values"][int(np.argmin(t["ms_knn_k"]))]
        assert t["coop_min"] == t["coop_min_values"][int(np.argmin(t["ms_coop_min"]))]
        assert t["wide_max"] == t["wide_max_values"][int(np.argmin(t["ms_wide_max"]))]
        uv, _ = e.solve(pts)
        assert np.array_equal(_canon(uv), _canon(ref))
        other = family("uniform", 5000, 2, 43)
        uv2, _ = e.solve(other)
    with gpu_lib.Emst() as e:
        ref2, _ = e.solve(other)
    assert np.array_equal(_canon(uv2), _canon(ref2))


def test_autotune_rejects_static_mode(gpu_lib):
    with gpu_lib.Emst(search_mode=1) as e:
        with pytest.raises(gpu_lib.EmstError):
            e.autotune(family("uniform", 1000, 2, 44))


@pytest.mark.parametrize("which", ["default", "side"])
def test_device_outputs_ordered_on_caller_stream(gpu_lib, which):
    """Device outputs are ready for work the caller queues next on the stream
    it bound (the legacy default stream, or a stream of its own), with no
    extra synchronisation -- also right after another context freed its
    buffers, whose stale contents must never show through."""
    torch = pytest.importorskip("torch")
    pts = family("cluster", 60000, 3, 91)
    n = len(pts)
    with gpu_lib.Emst() as e:
        ref, ref_len = e.solve(pts)
    ref = _canon(ref)
    stream = torch.cuda.Stream() if which == "side" else torch.cuda.default_stream()
    with torch.cuda.stream(stream):
        dev = torch.from_numpy(pts).cuda()
        uv = torch.full((n - 1, 2), -1, dtype=torch.int32, device="cuda")
        ln = torch.zeros(1, dtype=torch.float64, device="cuda")
        for rep in range(6):
            with gpu_lib.Emst() as e:
                e.set_stream(stream.cuda_stream)
                uv.fill_(-1)
                e.solve_device(dev.data_ptr(), n, 3, uv.data_ptr(), ln.data_ptr())
                got = uv.cpu().numpy()  # queued on the same stream: must see the solve's output
                assert np.array_equal(_canon(got), ref), rep
                assert ln.item() == pytest.approx(ref_len, rel=1e-12)
            with gpu_lib.Emst(host_rounds=True) as e2:  # frees buffers between the timed contexts
                e2.solve(pts)


@pytest.mark.parametrize("kw", [dict(first_pass_factor=1.0001), dict(first_pass_factor=4.0),
                                dict(first_pass_factor=1.5, first_pass_ordered=True),
                                dict(first_pass_factor=float("inf"), first_pass_ordered=True)])
@pytest.mark.parametrize("kind,dim", [("cluster", 3), ("dups", 2), ("lattice", 3)])
@pytest.mark.parametrize("wide", [0, -1])
def test_first_pass_rules_keep_edges(gpu_lib, kw, kind, dim, wide):
    """The first-pass rule (who searches first, in one launch or two) only
    changes the order of the searches, never the edge set -- with short
    lists searched warp per query or thread per query."""
    pts = family(kind, 20000, dim, 71)
    with gpu_lib.Emst() as e:
        ref, ref_len = e.solve(pts)
        ref_rounds = e.round_stats()
    with gpu_lib.Emst(wide_search=wide, **kw) as e:
        uv, ln = e.solve(pts)
        assert np.array_equal(_canon(uv), _canon(ref))
        assert ln == pytest.approx(ref_len, rel=1e-12)
        assert np.array_equal(e.round_stats(), ref_rounds)


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("n", [2, 7, 33, 20000])
def test_round1_neighbour_lists_exact(gpu_lib, kind, dim, n):
    """Every round-1 list is the exact k nearest other points under (d2, id),
    for every list length: ids and squared distances bit-exact against the
    kd-tree oracle (sets of fewer than k + 1 points end in -1 / inf), in the
    graph loop and the host loop."""
    pts = family(kind, n, dim, 97 + n)
    sp, _, _, _ = O.rescale(pts)
    for k in (4, 5, 6, 8):
        rid, rd2 = O.knn(sp, k)
        for host in (False, True):
            with gpu_lib.Emst(round1_neighbours=0 if k == 6 else k, host_rounds=host) as e:
                e.solve(pts)
                ids, d2 = e.neighbour_lists()
            assert ids.shape == (n, k)
            assert np.array_equal(ids.astype(np.int64), rid), (k, host)
            assert np.array_equal(d2, rd2), (k, host)


def test_neighbour_lists_need_the_list_search(gpu_lib):
    pts = family("uniform", 500, 2, 5)
    for kw in ({"round1_neighbours": -1}, {"search_mode": 1}, {"search_mode": 2}, {"search_mode": 3}):
        with gpu_lib.Emst(**kw) as e:
            e.solve(pts)
            with pytest.raises(gpu_lib.EmstError):
                e.neighbour_lists()


@pytest.mark.parametrize("kind,dim,n", [("cluster", 3, 30000), ("uniform", 2, 30000), ("dups", 3, 8000),
                                        ("lattice", 2, 5000), ("line", 3, 3000), ("dups", 2, 9)])
def test_round1_neighbour_lists_keep_edges(gpu_lib, kind, dim, n):
    """Round-1 neighbour lists (default) answer later rounds without changing
    any edge or round, in the graph loop and the host loop."""
    pts = family(kind, n, dim, 83)
    out = []
    for k in (-1, 0, 4, 5, 8):  # off, default (6), every other list length
        for host in (False, True):
            with gpu_lib.Emst(round1_neighbours=k, host_rounds=host) as e:
                uv, ln = e.solve(pts)
                out.append((_canon(uv), ln, e.round_stats()))
    for uv, ln, rs in out[1:]:
        assert np.array_equal(uv, out[0][0]) and ln == pytest.approx(out[0][1], rel=1e-12)
        assert np.array_equal(rs, out[0][2])


def test_operator_order_is_checked(gpu_lib):
    with gpu_lib.Emst() as e:
        e.initialize(family("uniform", 100, 2, 1))
        with pytest.raises(gpu_lib.EmstError) as ex:
            e.find_next_closest()
        assert ex.value.status == 6


def test_single_point_and_pairs(gpu_lib):
    with gpu_lib.Emst() as e:
        uv, length = e.solve(np.array([[0.5, 0.5]], np.float32))
        assert len(uv) == 0 and length == 0.0
        uv, length = e.solve(np.array([[0.0, 0.0, 0.0], [1.0, 2.0, 2.0]], np.float32))
        assert _canon(uv).tolist() == [[0, 1]] and length == pytest.approx(3.0)


@pytest.mark.parametrize("mode", MODES)
def test_all_identical_points(gpu_lib, mode):
    pts = np.full((777, 3), 0.25, np.float32)
    with gpu_lib.Emst(search_mode=mode) as e:
        e.initialize(pts)
        e.run()
        uv = e.edges()
        _, length = e.evaluate()
    sp, _, _, _ = O.rescale(pts)
    assert np.array_equal(_canon(uv), _canon(O.emst(sp, "faithful").edges))
    assert length == 0.0


@pytest.mark.parametrize("bad", [np.nan, np.inf])
def test_non_finite_input_is_rejected(gpu_lib, bad):
    pts = family("uniform", 1000, 2, 3)
    pts[17, 1] = bad
    with gpu_lib.Emst() as e:
        with pytest.raises(gpu_lib.EmstError) as ex:
            e.solve(pts)
        assert ex.value.status == 1


def test_bad_dim_is_rejected(gpu_lib):
    with gpu_lib.Emst() as e:
        with pytest.raises(gpu_lib.EmstError) as ex:
            e.solve(np.zeros((10, 4), np.float32))
        assert ex.value.status == 1


def test_device_entry_point_matches_host(gpu_lib):
    torch = pytest.importorskip("torch")
    pts = family("cluster", 50000, 3, 9)
    with gpu_lib.Emst() as e:
        uv_h, len_h = e.solve(pts)
    d_pts = torch.from_numpy(pts).cuda()
    d_uv = torch.zeros((len(pts) - 1, 2), dtype=torch.int32, device="cuda")
    d_len = torch.zeros(1, dtype=torch.float64, device="cuda")
    with gpu_lib.Emst() as e:
        e.set_stream(torch.cuda.current_stream().cuda_stream)
        ne = e.solve_device(d_pts.data_ptr(), len(pts), 3, d_uv.data_ptr(), d_len.data_ptr())
        torch.cuda.synchronize()
    assert ne == len(pts) - 1
    assert np.array_equal(_canon(d_uv.cpu().numpy()), _canon(uv_h))
    assert d_len.item() == pytest.approx(len_h, rel=1e-12)


@pytest.mark.parametrize("mode", MODES)
def test_repeat_runs_are_identical(gpu_lib, mode):
    """Union-find compression and the searches run concurrently; repeated
    solves in one context (buffers holding the previous solve's data) must
    agree exactly."""
    pts = family("cluster", 6000, 3, 7000)
    ref = None
    with gpu_lib.Emst(search_mode=mode) as e:
        for _ in range(200):
            uv, length = e.solve(pts)
            if ref is None:
                ref = _canon(uv)
            assert np.array_equal(_canon(uv), ref)
    pts = family("dups", 30000, 2, 4)
    outs = []
    with gpu_lib.Emst() as e:
        for _ in range(3):
            uv, length = e.solve(pts)
            outs.append((_canon(uv), length))
    for uv, length in outs[1:]:
        assert np.array_equal(uv, outs[0][0])
        assert length == pytest.approx(outs[0][1], rel=1e-12)


@pytest.mark.parametrize("name,n", [("gauss3d_1e6", 1_000_000), ("bezier2d_1e7", 1_000_000)])
def test_full_size_structure(gpu_lib, name, n):
    """Size-independent checks at workload scale: the GPU's region table rows
    equal the oracle's exact rows on a random sample, and the GPU edge set is
    the MST of the GPU's own candidate graph (Kruskal under the same order),
    which is a spanning tree."""
    pts = W.make(name, n)
    with gpu_lib.Emst(keep_region_table=True) as e:
        e.initialize(pts)
        e.run()
        uv = e.edges()
        ids, d2 = e.region_table()
        scaled, _ = e.rescaled()
    assert _is_spanning_tree(len(pts), uv)
    rows = np.random.default_rng(0).choice(len(pts), 1500, replace=False)
    ti, td = O.region_rows(scaled, rows)
    assert np.array_equal(ids[rows].astype(np.int64), ti)
    assert np.array_equal(d2[rows].view(np.uint32), td.view(np.uint32))
    mst = O.kruskal_table(ids, d2)
    assert np.array_equal(_canon(mst), _canon(uv))
    # the component search reaches the same tree, round by round
    with gpu_lib.Emst(search_mode=1) as e:
        e.initialize(pts)
        e.run()
        uv1, r1 = e.edges(with_rounds=True)
    with gpu_lib.Emst(search_mode=0) as e:
        e.initialize(pts)
        e.run()
        uv0, r0 = e.edges(with_rounds=True)
    assert np.array_equal(_canon(uv0), _canon(uv))
    for k in range(1, int(r1.max()) + 1):
        assert np.array_equal(_canon(uv0[r0 == k]), _canon(uv1[r1 == k]))


@pytest.mark.parametrize("kind,dim,n", [("cluster", 3, 40000), ("uniform", 2, 40000), ("dups", 3, 8000),
                                        ("lattice", 2, 6000), ("line", 3, 3000), ("dups", 2, 9),
                                        ("cluster", 2, 150000)])
@pytest.mark.parametrize("mode", [0, 1, 2])
def test_search_kernels_keep_edges(gpu_lib, kind, dim, n, mode):
    """Every search kernel gives the thread-per-query search's edges, lengths
    and per-round edge counts, in the graph loop, the host loop and batches,
    without neighbour lists too: the default split by list length (0), warp
    per query for every list (1, k_cnns_w), warp per 32 queries walking the
    tree together for every list (2, k_cnns_c)."""
    pts = family(kind, n, dim, 97)
    with gpu_lib.Emst(wide_search=-1) as e:
        ref, ref_len = e.solve(pts)
        ref_rounds = e.round_stats()
    # the first-pass rules send a second list (two passes) or a second list
    # segment (one ordered launch) through the same kernels
    for kw in (dict(), dict(host_rounds=True), dict(round1_neighbours=-1), dict(first_pass_factor=1.5),
               dict(first_pass_factor=1.5, first_pass_ordered=True)):
        with gpu_lib.Emst(wide_search=mode, **kw) as e:
            uv, ln = e.solve(pts)
            assert np.array_equal(_canon(uv), _canon(ref)), kw
            assert ln == pytest.approx(ref_len, rel=1e-12)
            assert np.array_equal(e.round_stats(), ref_rounds), kw
    other = family("uniform", max(n // 3, 2), dim, 98)
    with gpu_lib.Emst(wide_search=-1) as e:
        ref_b, _ = e.solve_batch([pts, other])
    with gpu_lib.Emst(wide_search=mode) as e:
        got_b, _ = e.solve_batch([pts, other])
    for a, b in zip(ref_b, got_b):
        assert np.array_equal(_canon(a), _canon(b))


def test_search_split_rejects_unknown_values(gpu_lib):
    for bad in (-2, 3):
        with pytest.raises(gpu_lib.EmstError):
            gpu_lib.Emst(wide_search=bad)


@pytest.mark.parametrize("coop,wide", [(1, 1), (50000, 16384), (0xffffffff, 150000), (10, 0xffffffff)])
def test_list_thresholds_keep_edges(gpu_lib, coop, wide):
    """The list-length thresholds that pick the search kernel of a round (set
    by hand or by the autotuner) never change the edges or the rounds."""
    pts = W.gauss_mixture(60000, 3, 16, 91)
    with gpu_lib.Emst() as e:
        ref, ref_len = e.solve(pts)
        ref_rounds = e.round_stats()
    with gpu_lib.Emst(coop_min_list=coop, wide_max_list=wide) as e:
        uv, ln = e.solve(pts)
        assert np.array_equal(_canon(uv), _canon(ref))
        assert ln == pytest.approx(ref_len, rel=1e-12)
        assert np.array_equal(e.round_stats(), ref_rounds)


def test_bad_list_length_is_rejected(gpu_lib):
    for k in (1, 3, 7, 9, -2):
        with pytest.raises(gpu_lib.EmstError):
            gpu_lib.Emst(round1_neighbours=k)


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("n", [2, 17, 1000, 6000])
def test_dynamic_pruning_with_diffusion_min_find(gpu_lib, kind, dim, n):
    """search_mode 3 with the diffusion min-find (every component's minimum
    taken over its forest instead of one atomic slot): the oracle's edges,
    per-round counts and labels."""
    pts = family(kind, n, dim, 2000 + n)
    with gpu_lib.Emst(search_mode=3, min_find=1) as e:
        e.initialize(pts)
        e.run()
        uv = e.edges()
        stats = e.round_stats()
        labels = e.labels()
    sp, _, _, _ = O.rescale(pts)
    r = O.emst(sp, "faithful")
    assert np.array_equal(_canon(uv), _canon(r.edges))
    assert list(stats) == [int(x) for x in r.round_edges]
    assert np.array_equal(labels.astype(np.int64), r.labels)


def test_dynamic_pruning_full_config_1e6(gpu_lib):
    """search_mode 3 on the full gauss3d_1e6 configuration (10^6 clustered 3D
    points, cells of any occupancy) against the default mode: same edges,
    per-round counts and labels."""
    pts = W.make("gauss3d_1e6")
    out = []
    for mode in (0, 3):
        with gpu_lib.Emst(search_mode=mode) as e:
            e.initialize(pts)
            e.run()
            out.append((_canon(e.edges()), list(e.round_stats()), e.labels()))
    assert np.array_equal(out[0][0], out[1][0])
    assert out[0][1] == out[1][1]
    assert np.array_equal(out[0][2], out[1][2])


def test_min_find_needs_dynamic_mode(gpu_lib):
    for mode in (0, 1, 2):
        with pytest.raises(gpu_lib.EmstError):
            gpu_lib.Emst(search_mode=mode, min_find=1)
    with pytest.raises(gpu_lib.EmstError):
        gpu_lib.Emst(search_mode=4)
