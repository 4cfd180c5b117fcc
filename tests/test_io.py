"""The reference's file formats on the host (no GPU): point readers against the
reference's own input files and their parsed values, the .links reader
against the golden edge set, and the command-line driver's argument handling."""
import os
import subprocess

import numpy as np
import pytest

import emst_gb300 as E


def _write(tmp_path, name, data):
    p = tmp_path / name
    p.write_bytes(bytes(data))
    return str(p)


def test_reads_reference_2d_and_3d_files(fixtures, tmp_path):
    p2 = _write(tmp_path, "1000randomCity.2d", fixtures["raw_2d_1000"])
    p3 = _write(tmp_path, "1000randomCity.3d", fixtures["raw_3d_1000"])
    a = E.read_points(p2)
    b = E.read_points(p3)
    assert a.shape == (1000, 2) and b.shape == (1000, 3)
    assert np.array_equal(a, fixtures["pts2d_1000"])  # parsed as float, bit for bit
    assert np.array_equal(b, fixtures["pts3d_1000"])


def test_suffix_is_taken_from_the_file_name(fixtures, tmp_path):
    d = tmp_path / "run.v1_data"
    d.mkdir()
    p = _write(d, "cities.2d", fixtures["raw_2d_1000"])
    assert E.read_points(p).shape == (1000, 2)


def test_reads_tsplib_layout(tmp_path):
    rng = np.random.default_rng(3)
    xy = (rng.random((57, 2)) * 1e4).astype(np.float32)
    lines = ["NAME : synthetic57", "COMMENT : generated for the reader test", "TYPE : TSP", "DIMENSION : 57",
             "EDGE_WEIGHT_TYPE : EUC_2D", "NODE_COORD_SECTION"]
    lines += ["%d %.6f %.6f" % (i + 1, x, y) for i, (x, y) in enumerate(xy)]
    lines += ["EOF"]
    p = tmp_path / "synthetic57.tsp"
    p.write_text("\n".join(lines) + "\n")
    got = E.read_points(str(p))
    want = np.array([[np.float32("%.6f" % x), np.float32("%.6f" % y)] for x, y in xy], np.float32)
    assert np.array_equal(got, want)


def test_reads_points_grid_file(tmp_path):
    pts = np.array([[1.5, 2.25, 0.0], [110.713, 103.486, 7.0], [-3.0, 4.0, 5.0]], np.float32)
    body = "Width = 3 Height = 1 \n" + "".join("%g %g %g  " % tuple(p) for p in pts) + "\n\n"
    p = tmp_path / "three.points"
    p.write_text(body)
    got = E.read_points(str(p))
    assert got.shape == (3, 3) and np.array_equal(got, pts)


def test_bad_files_are_rejected(tmp_path):
    with pytest.raises(E.EmstError):
        E.read_points(str(tmp_path / "missing.2d"))
    p = tmp_path / "short.3d"
    p.write_text("5\n1 2 3\n")
    with pytest.raises(E.EmstError):
        E.read_points(str(p))


def test_reads_links_in_the_reference_layout(fixtures, tmp_path):
    edges = fixtures["outypu_edges"]
    n = int(edges.max()) + 1
    adj = [[] for _ in range(n)]
    for u, v in edges:
        adj[u].append(v)
        adj[v].append(u)
    out = ["Width = %d Height = 1 " % n]
    for i in range(n):
        out.append("")
        out.append("NodeP = %d 0 NumLinks = %d %s" % (i, len(adj[i]), "".join("%d 0 " % j for j in adj[i])))
    p = tmp_path / "golden.links"
    p.write_text("\n".join(out) + "\n")
    uv, npts = E.read_links(str(p))
    assert npts == n
    got = np.sort(uv, axis=1)
    got = got[np.lexsort((got[:, 1], got[:, 0]))]
    assert np.array_equal(got, edges)


def test_cli_reports_unreadable_data(tmp_path):
    exe = os.path.join(os.path.dirname(E.LIB_PATH), "emst_run")
    if not os.path.exists(exe):
        pytest.skip("emst_run not built")
    r = subprocess.run([exe, str(tmp_path / "nothing.2d"), str(tmp_path / "out.svg")], capture_output=True, text=True)
    assert r.returncode == 1 and "reading" in r.stderr
