"""Result files on the GPU path: the golden 3000-point set written the way the
reference writes it, compared with the reference's own files, and the
command-line driver end to end."""
import hashlib
import json
import os
import subprocess

import numpy as np
import pytest

import emst_gb300 as E

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _canon(uv):
    a = np.sort(np.asarray(uv, np.int64), axis=1)
    return a[np.lexsort((a[:, 1], a[:, 0]))]


def _sha(path):
    return hashlib.sha256(open(path, "rb").read()).hexdigest()


def test_results_match_reference_files(gpu_lib, fixtures, tmp_path):
    ref = json.load(open(os.path.join(GOLDEN, "reference_files.json")))
    pts = fixtures["pts2d_3000"]
    base = str(tmp_path / "outypu")
    with gpu_lib.Emst() as e:
        e.solve(pts)
        e.write_results(base)
    uv, npts = gpu_lib.read_links(base + ".links")
    assert npts == 3000
    assert np.array_equal(_canon(uv), _canon(fixtures["outypu_edges"]))
    # final roots as byte offsets: the reference's file, byte for byte
    assert _sha(base + ".disjointSetMap") == ref["outypu.disjointSetMap"]["sha256"]
    # rescaled coordinates at 6 significant digits
    toks = open(base + ".points").read().split()
    assert toks[:6] == ["Width", "=", "3000", "Height", "=", "1"]
    got = np.array([float(t) for t in toks[6:]]).reshape(3000, 3)
    assert np.allclose(got[:, :2], fixtures["outypu_points"], rtol=1e-5, atol=1e-4) and np.all(got[:, 2] == 0)
    # every point has a record; degrees sum to 2 (n - 1)
    txt = open(base + ".links").read()
    assert txt.count("NodeP =") == 3000


def test_points_file_bytes(gpu_lib, fixtures, tmp_path):
    """The .points file reproduces the reference's byte for byte when every
    rescaled float prints the same at 6 significant digits."""
    ref = json.load(open(os.path.join(GOLDEN, "reference_files.json")))
    base = str(tmp_path / "outypu")
    with gpu_lib.Emst() as e:
        e.solve(fixtures["pts2d_3000"])
        e.write_results(base)
    data = open(base + ".points", "rb").read()
    assert len(data) == ref["outypu.points"]["bytes"]
    assert hashlib.sha256(data).hexdigest() == ref["outypu.points"]["sha256"]


def test_cli_end_to_end(gpu_lib, fixtures, tmp_path):
    exe = os.path.join(os.path.dirname(gpu_lib.LIB_PATH), "emst_run")
    assert os.path.exists(exe), "emst_run is built with the library"
    data = tmp_path / "1000randomCity.2d"
    data.write_bytes(bytes(fixtures["raw_2d_1000"]))
    sol, stats = tmp_path / "run1.svg", tmp_path / "run1.stats"
    r = subprocess.run([exe, str(data), str(sol), str(stats)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    uv, npts = gpu_lib.read_links(str(tmp_path / "run1.links"))
    with gpu_lib.Emst() as e:
        ref, length = e.solve(fixtures["pts2d_1000"])
    assert npts == 1000 and np.array_equal(_canon(uv), _canon(ref))
    f = open(stats).read().split()
    assert int(f[0]) == 1000 and int(f[1]) == 2 and int(f[2]) == 999
    assert float(f[3]) == pytest.approx(length, rel=1e-6)
    assert os.path.exists(tmp_path / "run1.disjointSetMap") and os.path.exists(tmp_path / "run1.points")


@pytest.mark.parametrize("host", [False, True])
@pytest.mark.parametrize("case", ["golden2d", "cluster3d", "dups2d"])
def test_round_forests_and_labels(gpu_lib, fixtures, case, host):
    """Hierarchical EMSF: after every round, the kept roots are constant on each
    tree of the forest of edges up to that round and differ between trees,
    every root is a point of its own tree, roots only disappear, and the last
    round's roots are the final labels (pinned to the reference's
    disjointSetMap for the golden set)."""
    from families import family
    pts = {"golden2d": fixtures["pts2d_3000"], "cluster3d": family("cluster", 20000, 3, 5),
           "dups2d": family("dups", 5000, 2, 6)}[case]
    n = len(pts)
    with gpu_lib.Emst(host_rounds=host) as e:
        e.keep_round_labels(32)
        e.solve(pts)
        uv, rd = e.edges(with_rounds=True)
        final = e.labels()
        cum = e.round_stats()
        R = len(cum)
        snaps = [e.round_labels(r) for r in range(1, R + 1)]
        with pytest.raises(gpu_lib.EmstError):
            e.round_labels(R + 1)
    if case == "golden2d":
        assert np.array_equal(final, fixtures["outypu_labels"])
    assert np.array_equal(snaps[-1], final)
    prev_roots = None
    for r in range(1, R + 1):
        lab = snaps[r - 1]
        sel = rd <= r
        assert int(sel.sum()) == int(cum[r - 1])
        # union-find over the forest up to round r
        par = np.arange(n)

        def find(a):
            while par[a] != a:
                par[a] = par[par[a]]
                a = par[a]
            return a
        for u, v in uv[sel]:
            ru, rv = find(u), find(v)
            if ru != rv:
                par[max(ru, rv)] = min(ru, rv)
        comp = np.array([find(i) for i in range(n)])
        # same tree <=> same label, and the label is a member of the tree
        assert len(np.unique(comp)) == len(np.unique(lab)) == n - int(cum[r - 1])
        pairs = np.unique(np.stack([comp, lab], 1), axis=0)
        assert len(pairs) == len(np.unique(comp))
        assert np.array_equal(comp[lab], comp)
        roots = set(np.unique(lab).tolist())
        if prev_roots is not None:
            assert roots <= prev_roots
        prev_roots = roots
