"""The CPU oracle against the reference's own golden outputs (no GPU needed).

Pins oracle/emst_oracle.c to:
  * test_2D_2/outypu.links    -- the 3000-point EMST edge set;
  * test_2D_2/outypu.points   -- the rescaled coordinates (6 significant digits);
  * test_2D_2/outypu.disjointSetMap -- the final root of every point;
  * test_2D_2/output, test_3D_2/output -- per-round cumulative edge counts and
    tree lengths recorded by the reference for 1000/3000/4000 (2D) and
    1000/2000/10000 (3D) points.
"""
import numpy as np
import pytest

import pyoracle as O
from families import KINDS, family

TRACED = [("pts2d_1000", 2), ("pts2d_3000", 2), ("pts2d_4000", 2), ("pts3d_1000", 3), ("pts3d_2000", 3),
          ("pts3d_10000", 3)]


def test_rescale_matches_reference_points(fixtures):
    sp, ux, _, _ = O.rescale(fixtures["pts2d_3000"])
    gold = fixtures["outypu_points"]
    rel = np.abs(sp - gold) / np.maximum(np.abs(gold), 1e-3)
    assert rel.max() < 1e-5  # the .points file carries 6 significant digits


def test_golden_edge_set_3000(fixtures):
    sp, _, _, _ = O.rescale(fixtures["pts2d_3000"])
    r = O.emst(sp, "faithful")
    gold = O.canon(fixtures["outypu_edges"])
    assert len(gold) == 2999
    assert np.array_equal(O.canon(r.edges), gold)


def test_golden_labels_3000(fixtures):
    sp, _, _, _ = O.rescale(fixtures["pts2d_3000"])
    r = O.emst(sp, "faithful")
    assert np.array_equal(r.labels, fixtures["outypu_labels"].astype(np.int64))


@pytest.mark.parametrize("key,dim", TRACED)
@pytest.mark.parametrize("mode", ["faithful", "exact"])
def test_golden_round_traces(fixtures, traces, key, dim, mode):
    pts = fixtures[key]
    n = len(pts)
    trace = traces["%dd" % dim]["%drandomCity.%dd" % (n, dim)][0]
    sp, _, _, _ = O.rescale(pts)
    r = O.emst(sp, mode)
    assert [int(x) for x in r.round_edges] == [row[1] for row in trace]
    for k, row in enumerate(trace):
        length = O.length(pts, r.edges[: r.round_edges[k]])
        assert float("%.6g" % length) == pytest.approx(row[2], rel=1e-6)


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("kind", KINDS)
def test_three_oracles_agree(kind, dim):
    for seed in range(3):
        pts = family(kind, 300 + 211 * seed, dim, 100 + seed)
        sp, _, _, _ = O.rescale(pts)
        a = O.canon(O.emst(sp, "faithful").edges)
        b = O.canon(O.emst(sp, "exact").edges)
        c = O.canon(O.prim(sp))
        assert np.array_equal(a, c) and np.array_equal(b, c)


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("kind", KINDS)
def test_exact_table_is_brute_force_table(kind, dim):
    pts = family(kind, 700, dim, 7)
    sp, _, _, _ = O.rescale(pts)
    ti, td = O.region_table(sp, "exact")
    bi, bd = O.region_table(sp, "brute")
    assert np.array_equal(ti, bi)
    assert np.array_equal(td.view(np.uint32), bd.view(np.uint32))


def test_kruskal_over_table_is_emst(fixtures):
    sp, _, _, _ = O.rescale(fixtures["pts3d_2000"])
    ti, td = O.region_table(sp, "exact")
    mst = O.kruskal_table(ti.astype(np.int32), td)
    assert np.array_equal(O.canon(mst), O.canon(O.prim(sp)))


def test_region_mask_rules():
    # ties and zeros belong to several regions (NodeEMST.h:1212-1232)
    m = O.lib().oracle_region_mask
    f = lambda *d: m(np.array(d, np.float32).ctypes.data_as(O.ctypes.c_void_p), len(d))
    assert f(1.0, 0.5) == 1 << 0          # +x face, y >= 0 slab
    assert f(1.0, -0.5) == 1 << 1         # +x face, y <= 0 slab
    assert f(1.0, 0.0) == 0b11            # zero: both slabs
    assert bin(f(1.0, 1.0)).count("1") == 2  # tie: +x and +y faces
    # duplicate: every dominant axis, '+' face only (d >= 0), every slab
    assert f(0.0, 0.0) == 0b00110011
    assert f(0.0, 0.0, 0.0) == 0xF0F0F


@pytest.mark.parametrize("key,dim", TRACED)
def test_kd_oracle_golden_round_traces(fixtures, traces, key, dim):
    """The kd-tree restatement reproduces the reference's recorded per-round
    edge counts and lengths, and the 3000-point golden edges and labels."""
    pts = fixtures[key]
    n = len(pts)
    trace = traces["%dd" % dim]["%drandomCity.%dd" % (n, dim)][0]
    sp, _, _, _ = O.rescale(pts)
    r = O.emst_kd(sp)
    assert [int(x) for x in r.round_edges] == [row[1] for row in trace]
    for k, row in enumerate(trace):
        length = O.length(pts, r.edges[: r.round_edges[k]])
        assert float("%.6g" % length) == pytest.approx(row[2], rel=1e-6)
    if key == "pts2d_3000":
        assert np.array_equal(O.canon(r.edges), O.canon(fixtures["outypu_edges"]))
        assert np.array_equal(r.labels, fixtures["outypu_labels"].astype(np.int64))


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("n", [2, 3, 17, 33, 1000, 5000])
def test_kd_oracle_equals_faithful(kind, dim, n):
    """Same edges in the same order, same rounds, same labels as the faithful
    ring-search restatement (ties on lattices, exact duplicates, lines)."""
    pts = family(kind, n, dim, 1000 + n)
    sp, _, _, _ = O.rescale(pts)
    a, b = O.emst(sp, "faithful"), O.emst_kd(sp)
    assert np.array_equal(a.edges, b.edges)
    assert np.array_equal(a.edge_round, b.edge_round)
    assert list(a.round_edges) == list(b.round_edges)
    assert np.array_equal(a.labels, b.labels)


def test_full_size_golden_hash_is_the_faithful_oracles():
    """The full-size golden hashes (tests/golden/full_size_edge_hashes.json)
    hold while the seeded generator and the faithful restatement stay as they
    were: bezier2d_1e7, the one the oracle solves in well under a minute on the
    host cores, is solved again here and must hash the same."""
    import json
    import os

    import emst_workloads as W
    from crosscheck_full import edge_hash

    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "full_size_edge_hashes.json")
    golden = json.load(open(path))["hashes"]["bezier2d_1e7"]["edge_hash"]
    O.set_threads(os.cpu_count() or 1)
    pts = W.make("bezier2d_1e7")
    sp, _, _, _ = O.rescale(pts)
    ref = O.emst(sp, "faithful")
    assert edge_hash(ref.edges) == golden
