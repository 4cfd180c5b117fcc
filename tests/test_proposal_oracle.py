"""CPU checks of the proposal's oracle (oracle/mlp_oracle.py) and of the
sizes the header declares.  The oracle is the checker of the GPU training
kernels; it is pinned here by finite differences of its FP64 loss."""
import os
import re

import numpy as np
import pytest

import mlp_oracle as M

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def random_records(n, seed):
    rng = np.random.default_rng(seed)
    r = np.zeros((n, M.REC), np.float32)
    r[:, :8] = rng.normal(0, 0.6, (n, 8))
    r[:, 8] = rng.normal(-0.2, 0.4, n)
    r[:, 9] = rng.random(n) < 0.4
    r[:, 10] = rng.random(n) < 0.9
    return r


def random_weights(seed, scale=0.4):
    rng = np.random.default_rng(seed)
    return (rng.normal(0, scale, M.N_WEIGHTS)).astype(np.float32)


def test_header_sizes_match_oracle():
    h = open(os.path.join(ROOT, "include", "emst.h")).read()
    assert int(re.search(r"#define EMST_PROPOSAL_WEIGHTS (\d+)", h).group(1)) == M.N_WEIGHTS == 1410
    assert int(re.search(r"#define EMST_TRACE_RECORD (\d+)", h).group(1)) == M.REC


def test_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.005859375, 1.0078125, -3.14159, 0.0, 65504.0], np.float32)
    b = M.bf16(x)
    # 1 + 2^-8 is a tie between 1 and 1 + 2^-7 -> even (1.0); 1 + 1.5 * 2^-8 rounds up
    assert b[0] == 1.0 and b[1] == 1.0 and b[2] == 1.0078125 and b[3] == 1.0078125
    assert abs(b[4] - (-3.140625)) < 1e-12 and b[5] == 0.0
    assert np.all(np.abs(b - x) <= np.abs(x) * 2.0 ** -8)


def test_fp64_gradient_matches_finite_differences():
    rec = random_records(64, 1)
    w = random_weights(2).astype(np.float64)
    loss, g, _ = M.forward_backward(w, rec, reg=0.7, emulate_bf16=False)
    rng = np.random.default_rng(3)
    for i in rng.choice(M.N_WEIGHTS, 60, replace=False):
        h = 1e-6
        wp, wm = w.copy(), w.copy()
        wp[i] += h
        wm[i] -= h
        fd = (M.forward_backward(wp, rec, 0.7, False)[0] - M.forward_backward(wm, rec, 0.7, False)[0]) / (2 * h)
        assert fd == pytest.approx(g[i], rel=1e-4, abs=1e-8), i


def test_bf16_emulation_stays_close_to_fp64():
    rec = random_records(256, 4)
    w = random_weights(5)
    l64, g64, _ = M.forward_backward(w, rec, emulate_bf16=False)
    lb, gb, _ = M.forward_backward(w, rec, emulate_bf16=True)
    assert lb == pytest.approx(l64, rel=2e-2)
    assert np.linalg.norm(gb - g64) / np.linalg.norm(g64) < 5e-2


def test_predict_matches_forward():
    rec = random_records(50, 6)
    w = random_weights(7)
    _, _, O = M.forward_backward(w, rec, emulate_bf16=False)
    assert np.allclose(M.predict(w, rec[:, :8]), O)
