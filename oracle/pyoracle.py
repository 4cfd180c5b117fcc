"""ctypes binding of the CPU oracle (oracle/emst_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, always as the checker or the timed CPU baseline.
The product library never imports this module.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libemst_oracle.so")
_lib = None

K_OF_DIM = {2: 8, 3: 24}


def build():
    """Compile the oracle with the committed Makefile (gcc, -ffp-contract=off)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        srcs = [os.path.join(_HERE, f) for f in ("emst_oracle.c", "emst_kd_oracle.c")]
        if not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < max(os.path.getmtime(s) for s in srcs):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        P = ctypes.c_void_p
        i64 = ctypes.c_int64
        L.oracle_rescale.argtypes = [P, i64, ctypes.c_int, P, P, P, P]
        L.oracle_rescale.restype = ctypes.c_int
        L.oracle_emst.argtypes = [P, i64, ctypes.c_int, ctypes.c_int, ctypes.c_int, P, P, P, P, P, P, P]
        L.oracle_emst.restype = i64
        L.oracle_region_table.argtypes = [P, i64, ctypes.c_int, ctypes.c_int, ctypes.c_int, P, P]
        L.oracle_region_table.restype = ctypes.c_int
        L.oracle_region_table_brute.argtypes = [P, i64, ctypes.c_int, P, P]
        L.oracle_region_table_brute.restype = ctypes.c_int
        L.oracle_prim.argtypes = [P, i64, ctypes.c_int, P]
        L.oracle_prim.restype = ctypes.c_int
        L.oracle_length.argtypes = [P, ctypes.c_int, P, i64]
        L.oracle_length.restype = ctypes.c_double
        L.oracle_set_metric_variant.argtypes = [ctypes.c_int]
        L.oracle_d2.argtypes = [P, P, ctypes.c_int]
        L.oracle_d2.restype = ctypes.c_float
        L.oracle_region_mask.argtypes = [P, ctypes.c_int]
        L.oracle_region_mask.restype = ctypes.c_uint32
        L.oracle_region_rows.argtypes = [P, i64, ctypes.c_int, ctypes.c_int, P, i64, P, P]
        L.oracle_region_rows.restype = ctypes.c_int
        L.oracle_kruskal_table.argtypes = [i64, ctypes.c_int, P, P, P]
        L.oracle_kruskal_table.restype = i64
        L.oracle_emst_kd.argtypes = [P, i64, ctypes.c_int, P, P, P, P]
        L.oracle_emst_kd.restype = i64
        L.oracle_knn_kd.argtypes = [P, i64, ctypes.c_int, ctypes.c_int, P, P]
        L.oracle_knn_kd.restype = ctypes.c_int
        L.oracle_set_threads.argtypes = [ctypes.c_int]
        L.oracle_max_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def set_threads(t):
    """OpenMP threads for the per-point loops (1 = the scalar restatement)."""
    lib().oracle_set_threads(int(t))


def max_threads():
    return lib().oracle_max_threads()


def set_metric_variant(v):
    lib().oracle_set_metric_variant(int(v))


def rescale(pts):
    """SolutionEMST::initialize normalisation; returns (scaled, unitX, pmin, pmax)."""
    pts = np.ascontiguousarray(pts, dtype=np.float32)
    n, dim = pts.shape
    out = np.empty_like(pts)
    ux = ctypes.c_double()
    pmin = np.empty(3, np.float32)
    pmax = np.empty(3, np.float32)
    rc = lib().oracle_rescale(_ptr(pts), n, dim, _ptr(out), ctypes.byref(ux), _ptr(pmin), _ptr(pmax))
    if rc != 0:
        raise ValueError("oracle_rescale failed")
    return out, ux.value, pmin[:dim].copy(), pmax[:dim].copy()


class EmstResult:
    def __init__(self, edges, edge_round, round_edges, labels, table_id, table_d2, rounds, max_occ):
        self.edges = edges
        self.edge_round = edge_round
        self.round_edges = round_edges
        self.labels = labels
        self.table_id = table_id
        self.table_d2 = table_d2
        self.rounds = rounds
        self.max_occ = max_occ


def emst(scaled, mode="faithful", level_radius=1, want_table=False):
    """Boruvka EMST on rescaled points.  mode: 'faithful' (reference ring
    search) or 'exact' (certified exact region nearest neighbours)."""
    sp = np.ascontiguousarray(scaled, dtype=np.float32)
    n, dim = sp.shape
    K = K_OF_DIM[dim]
    edges = np.zeros((max(n - 1, 1), 2), np.int64)
    eround = np.zeros(max(n - 1, 1), np.int32)
    rounds_e = np.zeros(101, np.int64)
    labels = np.zeros(n, np.int64)
    max_occ = ctypes.c_int()
    tid = np.zeros((n, K), np.int64) if want_table else None
    td2 = np.zeros((n, K), np.float32) if want_table else None
    r = lib().oracle_emst(_ptr(sp), n, dim, 0 if mode == "faithful" else 1, int(level_radius), _ptr(edges),
                          _ptr(eround), _ptr(rounds_e), _ptr(labels),
                          _ptr(tid) if want_table else None, _ptr(td2) if want_table else None,
                          ctypes.byref(max_occ))
    if r < 0:
        raise ValueError("oracle_emst failed (%d)" % r)
    ne = int(rounds_e[r - 1]) if r > 0 else 0
    return EmstResult(edges[:ne].copy(), eround[:ne].copy(), rounds_e[:r].copy(), labels, tid, td2, int(r),
                      max_occ.value)


def emst_kd(scaled):
    """Exact EMST by kd-tree Boruvka (emst_kd_oracle.c): the same rounds,
    edges, per-round counts and labels as emst(), fast enough for 10^7 points."""
    sp = np.ascontiguousarray(scaled, dtype=np.float32)
    n, dim = sp.shape
    edges = np.zeros((max(n - 1, 1), 2), np.int64)
    eround = np.zeros(max(n - 1, 1), np.int32)
    rounds_e = np.zeros(101, np.int64)
    labels = np.zeros(n, np.int64)
    r = lib().oracle_emst_kd(_ptr(sp), n, dim, _ptr(edges), _ptr(eround), _ptr(rounds_e), _ptr(labels))
    if r < 0:
        raise ValueError("oracle_emst_kd failed (%d)" % r)
    ne = int(rounds_e[r - 1]) if r > 0 else 0
    return EmstResult(edges[:ne].copy(), eround[:ne].copy(), rounds_e[:r].copy(), labels, None, None, int(r), 0)


def knn(scaled, k):
    """Every point's k nearest other points under (d2, id) by kd-tree
    (emst_kd_oracle.c): ids (n, k) int64 and d2 (n, k) float32, ascending;
    -1 / inf past the end when fewer than k other points exist."""
    sp = np.ascontiguousarray(scaled, dtype=np.float32)
    n, dim = sp.shape
    ids = np.zeros((n, k), np.int64)
    d2 = np.zeros((n, k), np.float32)
    rc = lib().oracle_knn_kd(_ptr(sp), n, dim, int(k), _ptr(ids), _ptr(d2))
    if rc != 0:
        raise ValueError("oracle_knn_kd failed (%d)" % rc)
    return ids, d2


def region_table(scaled, mode="exact", level_radius=1):
    sp = np.ascontiguousarray(scaled, dtype=np.float32)
    n, dim = sp.shape
    K = K_OF_DIM[dim]
    tid = np.zeros((n, K), np.int64)
    td2 = np.zeros((n, K), np.float32)
    if mode == "brute":
        rc = lib().oracle_region_table_brute(_ptr(sp), n, dim, _ptr(tid), _ptr(td2))
    else:
        rc = lib().oracle_region_table(_ptr(sp), n, dim, 0 if mode == "faithful" else 1, int(level_radius),
                                       _ptr(tid), _ptr(td2))
    if rc != 0:
        raise ValueError("oracle_region_table failed (%d)" % rc)
    return tid, td2


def prim(scaled):
    sp = np.ascontiguousarray(scaled, dtype=np.float32)
    n, dim = sp.shape
    edges = np.zeros((max(n - 1, 1), 2), np.int64)
    lib().oracle_prim(_ptr(sp), n, dim, _ptr(edges))
    return edges[: n - 1].copy()


def length(orig, edges):
    orig = np.ascontiguousarray(orig, dtype=np.float32)
    e = np.ascontiguousarray(edges, dtype=np.int64)
    return lib().oracle_length(_ptr(orig), orig.shape[1], _ptr(e), len(e))


def canon(edges):
    """Canonical edge set: (min, max) rows sorted lexicographically."""
    e = np.asarray(edges, dtype=np.int64).reshape(-1, 2)
    e = np.sort(e, axis=1)
    order = np.lexsort((e[:, 1], e[:, 0]))
    return e[order]


def region_rows(scaled, rows, level_radius=1):
    """Exact round-1 region table rows for the selected query points."""
    sp = np.ascontiguousarray(scaled, dtype=np.float32)
    n, dim = sp.shape
    K = K_OF_DIM[dim]
    rows = np.ascontiguousarray(rows, dtype=np.int64)
    tid = np.zeros((len(rows), K), np.int64)
    td2 = np.zeros((len(rows), K), np.float32)
    rc = lib().oracle_region_rows(_ptr(sp), n, dim, int(level_radius), _ptr(rows), len(rows), _ptr(tid), _ptr(td2))
    if rc != 0:
        raise ValueError("oracle_region_rows failed (%d)" % rc)
    return tid, td2


def kruskal_table(ids, d2):
    """MST of the candidate graph given by a region table (n, K) under the reference order."""
    ids = np.ascontiguousarray(ids, dtype=np.int32)
    d2 = np.ascontiguousarray(d2, dtype=np.float32)
    n, K = ids.shape
    out = np.zeros((max(n - 1, 1), 2), np.int64)
    ne = lib().oracle_kruskal_table(n, K, _ptr(ids), _ptr(d2), _ptr(out))
    return out[:ne].copy()
