"""The learned proposal on the GPU: training kernels against the CPU oracle,
traces, and -- the bar for any proposal -- edge sets identical to the plain
method's whatever the network predicts."""
import numpy as np
import pytest

import emst_workloads as W
import mlp_oracle as M
import pyoracle as O
from families import KINDS, family

pytestmark = pytest.mark.gpu


def _canon(e):
    e = np.sort(np.asarray(e, np.int64).reshape(-1, 2), axis=1)
    return e[np.lexsort((e[:, 1], e[:, 0]))]


def _records(n, seed):
    rng = np.random.default_rng(seed)
    r = np.zeros((n, M.REC), np.float32)
    r[:, :8] = rng.normal(0, 0.6, (n, 8))
    r[:, 8] = rng.normal(-0.2, 0.4, n)
    r[:, 9] = rng.random(n) < 0.4
    r[:, 10] = rng.random(n) < 0.9
    return r


@pytest.mark.parametrize("n,seed", [(64, 1), (1000, 2), (4097, 3)])
def test_gradient_matches_oracle(gpu_lib, n, seed):
    """BF16 tensor-core forward/backward vs the oracle: tight against the
    oracle that rounds the same operands to BF16, looser against pure FP64."""
    rec = _records(n, seed)
    w = gpu_lib.proposal_init(seed) + np.float32(0.05)  # non-zero biases too
    g, loss = gpu_lib.proposal_grad(w, rec, reg_weight=0.8)
    lb, gb, _ = M.forward_backward(w, rec, reg=0.8, emulate_bf16=True)
    l64, g64, _ = M.forward_backward(w, rec, reg=0.8, emulate_bf16=False)
    assert loss == pytest.approx(lb, rel=1e-4)
    assert loss == pytest.approx(l64, rel=2e-2)
    parts = [(M.OFF_W1, M.OFF_B1), (M.OFF_B1, M.OFF_W2), (M.OFF_W2, M.OFF_B2), (M.OFF_B2, M.OFF_W3),
             (M.OFF_W3, M.OFF_B3), (M.OFF_B3, M.N_WEIGHTS)]
    for a, b in parts:
        ref = np.linalg.norm(gb[a:b]) + 1e-12
        assert np.linalg.norm(g[a:b] - gb[a:b]) / ref < 1e-2, (a, b)
        assert np.linalg.norm(g[a:b] - g64[a:b]) / (np.linalg.norm(g64[a:b]) + 1e-12) < 6e-2, (a, b)


def _traces(gpu_lib, clouds, shift=2):
    with gpu_lib.Emst() as e:
        e.trace_enable(1 << 22, shift)
        for p in clouds:
            e.solve(p)
        return e.trace()


def test_traces_are_well_formed(gpu_lib):
    """Round-1 records: finite features, the round and component size of
    round 1, a target radius at or below the own leaf's bound, 0/1 labels."""
    clouds = [W.gauss_mixture(50_000, 3, 64, 7), family("uniform", 30_000, 2, 8)]
    rec = _traces(gpu_lib, clouds, shift=1)
    assert 20_000 < len(rec) < 60_000  # about half of the 80,000 queries
    assert np.all(np.isfinite(rec))
    assert set(np.unique(rec[:, 9])) <= {0.0, 1.0} and set(np.unique(rec[:, 10])) <= {0.0, 1.0}
    assert rec[:, 10].mean() > 0.99  # every query of a big cloud has K neighbours
    assert np.all(rec[:, 6] == 0.125) and np.all(rec[:, 7] == 0.0)  # round 1, components of one point
    assert np.all((rec[:, 5] > 0) & (rec[:, 5] <= 1))  # leaf occupancy
    full = rec[:, 10] > 0
    assert np.all(rec[full, 8] <= 0.0)  # the K-th nearest is never beyond the own leaf's bound
    tight = rec[full, 9] > 0
    assert np.all(rec[full][tight, 8] < 0.0) and np.all(rec[full][~tight, 8] == 0.0)
    assert 0.2 < tight.mean() < 0.999
    # sampling: shift 2 keeps about half as many records as shift 1
    rec2 = _traces(gpu_lib, clouds, shift=2)
    assert 0.35 < len(rec2) / len(rec) < 0.65


def test_training_reduces_loss(gpu_lib):
    rec = _traces(gpu_lib, [W.gauss_mixture(100_000, 3, 64, s) for s in (11, 12)], shift=1)
    w0 = gpu_lib.proposal_init(5)
    l0 = M.forward_backward(w0, rec[:20000], emulate_bf16=False)[0]
    w, curve = gpu_lib.proposal_train(rec, w0, epochs=3, batch=2048, lr=3e-3, seed=1)
    assert np.all(np.isfinite(w)) and np.all(np.isfinite(curve))
    assert curve[-1] < curve[0] < l0
    l1 = M.forward_backward(w, rec[:20000], emulate_bf16=False)[0]
    assert l1 < 0.7 * l0


def _weight_sets(gpu_lib):
    z = np.zeros(gpu_lib.PROPOSAL_WEIGHTS, np.float32)
    gate_off = z.copy()
    gate_off[M.OFF_B3 + 1] = -5.0  # gate logit < 0: every query keeps the certified bound
    tiny = z.copy()
    tiny[M.OFF_B3] = -4.0  # radius 2^-32 of the bound: every query is searched again
    return [("random", gpu_lib.proposal_init(3), 1.0), ("random_m0", gpu_lib.proposal_init(4), 0.0),
            ("gate_off", gate_off, 1.0), ("tiny_radius", tiny, 0.0), ("zero", z, 0.0),
            ("huge_margin", gpu_lib.proposal_init(6), 40.0)]


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("n", [2, 33, 1000, 6000])
def test_learned_radius_keeps_edges_and_rounds(gpu_lib, kind, dim, n):
    """Whatever the network predicts -- random, gated off, a radius that holds
    no neighbour at all, no tightening, a loose margin -- edges, per-round
    edge counts and the length are the plain method's, and every round-1
    list is the exact 6 nearest (the kd-tree oracle's ids and d2)."""
    pts = family(kind, n, dim, 60 + n)
    with gpu_lib.Emst() as e:
        ref, ref_len = e.solve(pts)
        ref_rounds = e.round_stats()
    rid, rd2 = O.knn(O.rescale(pts)[0], 6)
    for name, w, margin in _weight_sets(gpu_lib):
        with gpu_lib.Emst() as e:
            e.set_proposal(w, margin)
            uv, ln = e.solve(pts)
            assert np.array_equal(_canon(uv), _canon(ref)), name
            assert ln == pytest.approx(ref_len, rel=1e-12), name
            assert np.array_equal(e.round_stats(), ref_rounds), name
            # and the lists themselves stay the exact 6 nearest
            ids, d2 = e.neighbour_lists()
            assert np.array_equal(ids.astype(np.int64), rid) and np.array_equal(d2, rd2), name


def test_learned_graph_and_host_loops_agree(gpu_lib):
    pts = W.gauss_mixture(200_000, 3, 64, 21)
    w = gpu_lib.proposal_init(9)
    out = []
    for host in (False, True):
        with gpu_lib.Emst(host_rounds=host) as e:
            e.set_proposal(w, 1.0)
            out.append(_canon(e.solve(pts)[0]))
    with gpu_lib.Emst() as e:
        ref = _canon(e.solve(pts)[0])
    for got in out:
        assert np.array_equal(got, ref)


def test_learned_counters(gpu_lib):
    """Mispredictions are counted and searched again: a radius that holds
    nothing sends every query it steers back; a closed gate steers none."""
    pts = W.gauss_mixture(100_000, 3, 64, 22)
    sets = {name: (w, m) for name, w, m in _weight_sets(gpu_lib)}
    prof = {}
    for name in ("plain", "tiny_radius", "gate_off", "zero"):
        with gpu_lib.Emst(profile=True) as e:
            if name != "plain":
                e.set_proposal(*sets[name])
            e.solve(pts)
            prof[name] = e.profile()
    assert prof["plain"]["knn_learned"] == 0 and prof["plain"]["knn_resumed"] == 0
    assert prof["gate_off"]["knn_learned"] == 0
    assert prof["tiny_radius"]["knn_learned"] > 0.9 * len(pts)
    assert prof["tiny_radius"]["knn_resumed"] == prof["tiny_radius"]["knn_learned"]
    # the zero network predicts the certified bound itself: nothing changes
    assert prof["zero"]["knn_resumed"] == 0
    assert prof["zero"]["knn_marked"] == prof["plain"]["knn_marked"]


def test_trained_proposal_ablation(gpu_lib):
    """On a fixed 10^6-point clustered set (not a training cloud): trained
    network, untrained network and no network give the same edge set; the
    trained network starts a large share of the queries from a radius below
    the own leaf's bound, marks fewer candidates than the plain search, and
    mispredicts rarely (each misprediction is searched again)."""
    import emst_proposal as PR
    w, info = PR.load()
    assert w is not None, "no trained weights"
    pts = W.gauss_mixture(1_000_000, 3, 256, 77)
    out = {}
    for name, weights, margin in (("plain", None, 0.0), ("untrained", gpu_lib.proposal_init(11), info["margin"]),
                                  ("trained", w, info["margin"])):
        with gpu_lib.Emst(profile=True) as e:
            if weights is not None:
                e.set_proposal(weights, margin, info["threshold"])
            uv, _ = e.solve(pts)
            out[name] = (_canon(uv), e.profile())
    for name in ("untrained", "trained"):
        assert np.array_equal(out[name][0], out["plain"][0]), name
    plain, trained = out["plain"][1], out["trained"][1]
    assert trained["knn_learned"] > 0.05 * len(pts)
    assert trained["knn_marked"] < plain["knn_marked"]
    assert trained["knn_resumed"] < 0.05 * trained["knn_learned"]


def test_set_proposal_rejects_bad_input(gpu_lib):
    with gpu_lib.Emst(search_mode=1) as e:
        with pytest.raises(gpu_lib.EmstError):
            e.set_proposal(gpu_lib.proposal_init(0))
    with gpu_lib.Emst() as e:
        w = gpu_lib.proposal_init(0)
        w[5] = np.nan
        with pytest.raises(gpu_lib.EmstError):
            e.set_proposal(w)
        with pytest.raises(gpu_lib.EmstError):
            e.set_proposal(gpu_lib.proposal_init(0), margin=-1.0)
        e.set_proposal(None)  # off again
