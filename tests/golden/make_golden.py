"""Generate the golden fixtures in tests/golden/ from the reference's own test data.

Run once in a container that has the reference checkout (read-only):
    python tests/golden/make_golden.py <reference checkout>
It reads the reference's uniform point sets ({1000..6000}randomCity.2d,
{1000,2000,10000}randomCity.3d), its golden 3000-point edge set
(test_2D_2/outypu.links, Appendix format "NodeP = i 0 NumLinks = k j 0 ..."),
its rescaled coordinates (test_2D_2/outypu.points), its final disjoint-set
labels (test_2D_2/outypu.disjointSetMap) and the per-round traces
its runs recorded (test_2D_2/output, test_3D_2/output: iteration, edges so
far, tree length).  It writes compact binary / JSON fixtures so that the
tests never need the reference checkout.  No TSPLIB instance is copied.
For the file-format tests it also keeps the raw bytes of the two 1000-point
input files (1000randomCity.2d / .3d) and the SHA-256 and size of the golden
outypu.points / outypu.disjointSetMap files (reference_files.json).
"""
import ctypes
import hashlib
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_libc = ctypes.CDLL(None)
_libc.strtof.restype = ctypes.c_float
_libc.strtof.argtypes = [ctypes.c_char_p, ctypes.c_void_p]


def strtof(tok):
    return _libc.strtof(tok.encode(), None)


def read_points(path, dim):
    """InputRW::readUniform (emst_coalition/include/InputRW.h:516-565): N then coords, parsed as float."""
    toks = open(path).read().split()
    n = int(toks[0])
    vals = [strtof(t) for t in toks[1:1 + n * dim]]
    return np.array(vals, dtype=np.float32).reshape(n, dim)


def read_links(path):
    """NeuralNetEMST::writeLinks / BufferLink operator<< (.links adjacency)."""
    txt = open(path).read()
    edges = set()
    for m in re.finditer(r"NodeP\s*=\s*(\d+)\s+0\s+NumLinks\s*=\s*(\d+)((?:\s+-?\d+\s+-?\d+)*)", txt):
        i = int(m.group(1))
        k = int(m.group(2))
        nums = [int(x) for x in m.group(3).split()]
        for j in range(k):
            q = nums[2 * j]
            edges.add((min(i, q), max(i, q)))
    return np.array(sorted(edges), dtype=np.int32)


def read_points_file(path):
    """.points writer output: header then x y z triplets per point."""
    toks = open(path).read().split()
    # header "Width = N Height = 1"
    n = int(toks[2])
    vals = [float(t) for t in toks[6:6 + 3 * n]]
    return np.array(vals, dtype=np.float64).reshape(n, 3)


def read_traces(path):
    """Stats rows (SolutionEMSTRW.cu:100-165): iteration, objective, durations, benchmark, size, length, ..."""
    runs = {}
    cur = None
    for line in open(path):
        f = line.split()
        if len(f) < 8 or not f[0].isdigit():
            continue
        it, bench, size, length = int(f[0]), f[5], int(float(f[6])), float(f[7])
        if cur is None or cur["bench"] != bench or it < cur["rows"][-1][0] or (it == cur["rows"][-1][0] and size != cur["rows"][-1][1]):
            cur = {"bench": bench, "rows": []}
            runs.setdefault(bench, []).append(cur)
        if cur["rows"] and it == cur["rows"][-1][0]:
            continue  # final repeated row
        cur["rows"].append((it, size, length))
    out = {}
    for bench, lst in runs.items():
        seen = []
        for r in lst:
            rows = r["rows"]
            if not rows or rows[-1][1] <= 0:
                continue
            if rows[0][0] != 1:
                continue
            key = json.dumps(rows)
            if key not in [json.dumps(s) for s in seen]:
                seen.append(rows)
        if seen:
            out[bench] = seen
    return out


def main(ref):
    t2 = os.path.join(ref, "emst_coalition", "test_emst", "test_2D_2")
    t3 = os.path.join(ref, "emst_coalition", "test_emst", "test_3D_2")
    arrays = {}
    for n in (1000, 2000, 3000, 4000, 5000, 6000):
        arrays["pts2d_%d" % n] = read_points(os.path.join(t2, "%drandomCity.2d" % n), 2)
    for n in (1000, 2000, 10000):
        arrays["pts3d_%d" % n] = read_points(os.path.join(t3, "%drandomCity.3d" % n), 3)
    arrays["outypu_edges"] = read_links(os.path.join(t2, "outypu.links"))
    arrays["outypu_points"] = read_points_file(os.path.join(t2, "outypu.points"))[:, :2].astype(np.float32)
    # disjointSetMap holds byte offsets of 4-byte labels (GridOfNodes.h:454-464)
    dsm = open(os.path.join(t2, "outypu.disjointSetMap")).read().split()[6:]
    arrays["outypu_labels"] = (np.array([int(v) for v in dsm], dtype=np.int64) // 4).astype(np.int32)
    arrays["raw_2d_1000"] = np.frombuffer(open(os.path.join(t2, "1000randomCity.2d"), "rb").read(), np.uint8)
    arrays["raw_3d_1000"] = np.frombuffer(open(os.path.join(t3, "1000randomCity.3d"), "rb").read(), np.uint8)
    files = {}
    for name in ("outypu.points", "outypu.disjointSetMap"):
        data = open(os.path.join(t2, name), "rb").read()
        files[name] = {"sha256": hashlib.sha256(data).hexdigest(), "bytes": len(data)}
    with open(os.path.join(HERE, "reference_files.json"), "w") as fo:
        json.dump(files, fo, indent=1)
    np.savez_compressed(os.path.join(HERE, "reference_fixtures.npz"), **arrays)
    traces = {"2d": read_traces(os.path.join(t2, "output")), "3d": read_traces(os.path.join(t3, "output"))}
    with open(os.path.join(HERE, "reference_traces.json"), "w") as fo:
        json.dump(traces, fo, indent=1)
    print("wrote", sorted(arrays), "traces for", {k: sorted(v) for k, v in traces.items()})


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <path of the reference checkout>")
    main(sys.argv[1])
