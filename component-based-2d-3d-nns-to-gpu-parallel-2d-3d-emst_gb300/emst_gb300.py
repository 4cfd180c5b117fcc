"""Python binding of libemst_gb300.so (the C ABI in include/emst.h).

Mirrors the reference's operator surface (emst_coalition/include/EMSTOperators.h,
driven by SolutionEMST::activate / run in emst_coalition/src/SolutionEMSTOperators.cu):
    initialize -> [flatten, test_termination, compute_octants, find_next_closest,
                   find_min_pair, connect_union]* -> evaluate / edges / labels
plus the one-shot solve() / solve_device().  There is no CPU fallback: if the
CUDA library is missing or no GPU is present, the calls raise.
"""
import ctypes
import os
import re
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libemst_gb300.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "emst.h")

STATUS = {0: "EMST_OK", 1: "EMST_EINVAL", 2: "EMST_ENOMEM", 3: "EMST_EOVERFLOW", 4: "EMST_ENOCONVERGE",
          5: "EMST_ECUDA", 6: "EMST_ESTATE"}
K_OF_DIM = {2: 8, 3: 24}


class EmstError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s: %s" % (STATUS.get(status, status), msg))
        self.status = status


class Config(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("max_rounds", ctypes.c_int), ("warps_per_block", ctypes.c_int),
                ("keep_region_table", ctypes.c_int), ("profile", ctypes.c_int), ("search_mode", ctypes.c_int),
                ("host_rounds", ctypes.c_int), ("search_shape", ctypes.c_int),
                ("first_pass_factor", ctypes.c_float), ("first_pass_ordered", ctypes.c_int),
                ("round1_neighbours", ctypes.c_int), ("wide_search", ctypes.c_int),
                ("wide_max_list", ctypes.c_uint32), ("coop_min_list", ctypes.c_uint32), ("min_find", ctypes.c_int)]


class Tuning(ctypes.Structure):
    _fields_ = [("knn_k", ctypes.c_int), ("coop_min", ctypes.c_uint32), ("wide_max", ctypes.c_uint32),
                ("search_shape", ctypes.c_int), ("knn_k_values", ctypes.c_int * 4), ("ms_knn_k", ctypes.c_double * 4),
                ("coop_min_values", ctypes.c_uint32 * 4), ("ms_coop_min", ctypes.c_double * 4),
                ("wide_max_values", ctypes.c_uint32 * 3), ("ms_wide_max", ctypes.c_double * 3),
                ("ms_shape", ctypes.c_double * 6)]


class Profile(ctypes.Structure):
    _fields_ = [("ms_grid", ctypes.c_double), ("ms_octants", ctypes.c_double), ("ms_select", ctypes.c_double),
                ("ms_resolve", ctypes.c_double), ("ms_hook", ctypes.c_double), ("ms_flatten", ctypes.c_double),
                ("launches", ctypes.c_int64), ("octant_launches", ctypes.c_int64), ("rounds", ctypes.c_int64),
                ("leaf_visits", ctypes.c_int64), ("node_tests", ctypes.c_int64), ("candidates", ctypes.c_int64),
                ("search_warps", ctypes.c_int64), ("search_queries", ctypes.c_int64),
                ("first_pass_searches", ctypes.c_int64), ("first_pass_resumed", ctypes.c_int64),
                ("first_pass_deferred", ctypes.c_int64), ("ms_knn", ctypes.c_double), ("ms_search", ctypes.c_double),
                ("knn_launches", ctypes.c_int64), ("search_launches", ctypes.c_int64),
                ("knn_marked", ctypes.c_int64), ("knn_insert_steps", ctypes.c_int64),
                ("knn_learned", ctypes.c_int64), ("knn_resumed", ctypes.c_int64)]


class TrainConfig(ctypes.Structure):
    _fields_ = [("epochs", ctypes.c_int), ("batch", ctypes.c_int), ("lr", ctypes.c_float),
                ("reg_weight", ctypes.c_float), ("seed", ctypes.c_uint64), ("device", ctypes.c_int)]


ROUND1_NEIGHBOURS = 6  # EMST_ROUND1_NEIGHBOURS
PROPOSAL_WEIGHTS = 1410
TRACE_RECORD = 12


def build(jobs=4):
    """Compile the CUDA library in-tree for sm_103a (make -C <package>)."""
    subprocess.run(["make", "-s", "-j%d" % jobs, "-C", HERE], check=True)
    return LIB_PATH


def declared_symbols():
    """Entry points declared in include/emst.h."""
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:emst_status|const char\*)\s+(emst_\w+)\s*\(", txt, re.M)))


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise OSError("libemst_gb300.so is not built (run build() / __graft_entry__.build())")
        L = ctypes.CDLL(LIB_PATH)
        P, i64, I = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int
        sig = {
            "emst_create": [P, P], "emst_destroy": [P], "emst_set_stream": [P, P],
            "emst_initialize": [P, P, i64, I, I], "emst_compute_octants": [P], "emst_find_next_closest": [P],
            "emst_find_min_pair": [P], "emst_connect_union": [P], "emst_flatten": [P],
            "emst_test_termination": [P, P], "emst_activate": [P, P], "emst_run": [P],
            "emst_evaluate": [P, P, P], "emst_get_edges": [P, P, P, i64, P], "emst_get_labels": [P, P, i64],
            "emst_get_round_stats": [P, P, P, i64], "emst_get_region_table": [P, P, P, i64],
            "emst_get_neighbour_lists": [P, P, P, i64, P],
            "emst_get_rescaled": [P, P, P, i64], "emst_solve": [P, P, i64, I, P, P, P],
            "emst_solve_device": [P, P, i64, I, P, P, P], "emst_get_profile": [P, P],
            "emst_region_table_noalloc": [P, i64, I, P, P, P], "emst_solve_batch": [P, P, P, P, I, P, P, P],
            "emst_search_shape_info": [P, P, P, I], "emst_autotune": [P, P, i64, I, P, P, I],
            "emst_get_search_shape": [P, P], "emst_get_tuning": [P, P],
            "emst_set_proposal": [P, P, ctypes.c_float, ctypes.c_float], "emst_trace_enable": [P, i64, I],
            "emst_get_trace": [P, P, i64, P], "emst_get_trace_device": [P, P, P],
            "emst_proposal_init": [ctypes.c_uint64, P], "emst_proposal_train": [P, i64, I, P, P, P],
            "emst_proposal_grad": [P, P, i64, ctypes.c_float, P, P],
            "emst_read_points": [ctypes.c_char_p, P, i64, P, P], "emst_write_results": [P, ctypes.c_char_p],
            "emst_read_links": [ctypes.c_char_p, P, i64, P, P], "emst_get_size": [P, P, P],
            "emst_keep_round_labels": [P, I], "emst_get_round_labels": [P, I, P, i64],
        }
        for name, args in sig.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = ctypes.c_int
        L.emst_last_error.argtypes = [P]
        L.emst_last_error.restype = ctypes.c_char_p
        _lib = L
    return _lib


def search_shapes():
    """Launch shapes of the component search: (count, threads per block, min blocks per SM)."""
    cnt = ctypes.c_int()
    lib().emst_search_shape_info(ctypes.byref(cnt), None, None, 0)
    t = np.zeros(cnt.value, np.int32)
    m = np.zeros(cnt.value, np.int32)
    lib().emst_search_shape_info(ctypes.byref(cnt), _p(t), _p(m), cnt.value)
    return cnt.value, t, m


def read_points(path):
    """A point file of the reference's formats -> (n, dim) float32."""
    n, d = ctypes.c_int64(), ctypes.c_int()
    st = lib().emst_read_points(str(path).encode(), None, 0, ctypes.byref(n), ctypes.byref(d))
    if st != 0:
        raise EmstError(st, "cannot read points from %s" % path)
    out = np.zeros((n.value, d.value), np.float32)
    if n.value:
        st = lib().emst_read_points(str(path).encode(), _p(out), n.value, ctypes.byref(n), ctypes.byref(d))
        if st != 0:
            raise EmstError(st, "cannot read points from %s" % path)
    return out


def read_links(path):
    """A .links file -> ((m, 2) int32 edges u < v, number of points)."""
    m, npts = ctypes.c_int64(), ctypes.c_int64()
    st = lib().emst_read_links(str(path).encode(), None, 0, ctypes.byref(m), ctypes.byref(npts))
    if st != 0:
        raise EmstError(st, "cannot read links from %s" % path)
    uv = np.zeros((max(m.value, 1), 2), np.int32)
    st = lib().emst_read_links(str(path).encode(), _p(uv), m.value, ctypes.byref(m), ctypes.byref(npts))
    if st != 0:
        raise EmstError(st, "cannot read links from %s" % path)
    return uv[: m.value], npts.value


def proposal_init(seed=0):
    w = np.zeros(PROPOSAL_WEIGHTS, np.float32)
    lib().emst_proposal_init(ctypes.c_uint64(seed), _p(w))
    return w


def proposal_train(records, weights, epochs=4, batch=4096, lr=2e-3, reg_weight=1.0, seed=0, device=0,
                   records_on_device=None, n_records=None):
    """Trains on trace records (host array, or device pointer + n_records) with the
    library's tensor-core kernels. -> (trained weights, mean loss per epoch)."""
    w = np.ascontiguousarray(weights, np.float32).copy()
    cfg = TrainConfig(int(epochs), int(batch), float(lr), float(reg_weight), int(seed), int(device))
    curve = np.zeros(max(int(epochs), 1), np.float32)
    if records_on_device is not None:
        st = lib().emst_proposal_train(ctypes.c_void_p(records_on_device), int(n_records), 1, ctypes.byref(cfg),
                                       _p(w), _p(curve))
    else:
        r = np.ascontiguousarray(records, np.float32)
        st = lib().emst_proposal_train(_p(r), len(r), 0, ctypes.byref(cfg), _p(w), _p(curve))
    if st != 0:
        raise EmstError(st, "emst_proposal_train failed")
    return w, curve


def proposal_grad(weights, records, reg_weight=1.0):
    """One GPU forward/backward: (gradient of the mean loss, loss)."""
    w = np.ascontiguousarray(weights, np.float32)
    r = np.ascontiguousarray(records, np.float32)
    g = np.zeros(PROPOSAL_WEIGHTS, np.float32)
    loss = ctypes.c_float()
    st = lib().emst_proposal_grad(_p(w), _p(r), len(r), float(reg_weight), _p(g), ctypes.byref(loss))
    if st != 0:
        raise EmstError(st, "emst_proposal_grad failed")
    return g, loss.value


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class Emst:
    """One context = one CUDA stream on one device."""

    def __init__(self, device=0, max_rounds=0, keep_region_table=False, warps_per_block=0, profile=False,
                 search_mode=0, host_rounds=False, search_shape=0, first_pass_factor=0.0,
                 first_pass_ordered=False, round1_neighbours=0, wide_search=0, wide_max_list=0, coop_min_list=0,
                 min_find=0):
        cfg = Config(device, max_rounds, warps_per_block, 1 if keep_region_table else 0, 1 if profile else 0,
                     int(search_mode), 1 if host_rounds else 0, int(search_shape), float(first_pass_factor),
                     1 if first_pass_ordered else 0, int(round1_neighbours), int(wide_search), int(wide_max_list),
                     int(coop_min_list), int(min_find))
        h = ctypes.c_void_p()
        st = lib().emst_create(ctypes.byref(cfg), ctypes.byref(h))
        if st != 0:
            raise EmstError(st, "emst_create failed")
        self.h = h
        self.n = 0
        self.dim = 0

    def _chk(self, st):
        if st != 0:
            raise EmstError(st, lib().emst_last_error(self.h).decode())

    def close(self):
        if self.h:
            lib().emst_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream_ptr):
        """A cudaStream_t as an integer (0: the legacy default stream), or None for
        the context's own stream."""
        p = ctypes.c_void_p(-1 if stream_ptr is None else stream_ptr)
        self._chk(lib().emst_set_stream(self.h, p))

    # --- operators -------------------------------------------------------
    def initialize(self, pts=None, device_ptr=None, n=None, dim=None):
        if device_ptr is not None:
            self._chk(lib().emst_initialize(self.h, ctypes.c_void_p(device_ptr), int(n), int(dim), 1))
            self.n, self.dim = int(n), int(dim)
        else:
            pts = np.ascontiguousarray(pts, dtype=np.float32)
            self._keep = pts
            self._chk(lib().emst_initialize(self.h, _p(pts), pts.shape[0], pts.shape[1], 0))
            self.n, self.dim = pts.shape
        return self

    def flatten(self):
        self._chk(lib().emst_flatten(self.h))

    def test_termination(self):
        v = ctypes.c_int64()
        self._chk(lib().emst_test_termination(self.h, ctypes.byref(v)))
        return v.value

    def compute_octants(self):
        self._chk(lib().emst_compute_octants(self.h))

    def find_next_closest(self):
        self._chk(lib().emst_find_next_closest(self.h))

    def find_min_pair(self):
        self._chk(lib().emst_find_min_pair(self.h))

    def connect_union(self):
        self._chk(lib().emst_connect_union(self.h))

    def activate(self):
        m = ctypes.c_int()
        self._chk(lib().emst_activate(self.h, ctypes.byref(m)))
        return bool(m.value)

    def run(self):
        self._chk(lib().emst_run(self.h))

    # --- results ---------------------------------------------------------
    def evaluate(self):
        ne, ln = ctypes.c_int64(), ctypes.c_double()
        self._chk(lib().emst_evaluate(self.h, ctypes.byref(ne), ctypes.byref(ln)))
        return ne.value, ln.value

    def edges(self, with_rounds=False):
        cap = max(self.n - 1, 1)
        uv = np.zeros((cap, 2), np.int32)
        rd = np.zeros(cap, np.int32)
        ne = ctypes.c_int64()
        self._chk(lib().emst_get_edges(self.h, _p(uv), _p(rd), cap, ctypes.byref(ne)))
        if with_rounds:
            return uv[: ne.value].copy(), rd[: ne.value].copy()
        return uv[: ne.value].copy()

    def labels(self):
        out = np.zeros(self.n, np.int32)
        self._chk(lib().emst_get_labels(self.h, _p(out), self.n))
        return out

    def round_stats(self):
        r = ctypes.c_int64()
        cum = np.zeros(128, np.int64)
        self._chk(lib().emst_get_round_stats(self.h, ctypes.byref(r), _p(cum), 128))
        return cum[: r.value].copy()

    def region_table(self):
        K = K_OF_DIM[self.dim]
        ids = np.zeros((self.n, K), np.int32)
        d2 = np.zeros((self.n, K), np.float32)
        self._chk(lib().emst_get_region_table(self.h, _p(ids), _p(d2), self.n * K))
        return ids, d2

    def neighbour_lists(self):
        """Round-1 neighbour lists of the last solve: ids (n, k) int32 and d2
        (n, k) float32 in the rescaled frame, ascending by (d2, id); -1 / inf
        past the end."""
        k = ctypes.c_int()
        self._chk(lib().emst_get_neighbour_lists(self.h, None, None, 0, ctypes.byref(k)))
        ids = np.zeros((self.n, k.value), np.int32)
        d2 = np.zeros((self.n, k.value), np.float32)
        self._chk(lib().emst_get_neighbour_lists(self.h, _p(ids), _p(d2), ids.size, None))
        return ids, d2

    def profile(self):
        p = Profile()
        self._chk(lib().emst_get_profile(self.h, ctypes.byref(p)))
        return {k: getattr(p, k) for k, _ in Profile._fields_ if k != "reserved"}

    def rescaled(self):
        out = np.zeros((self.n, self.dim), np.float32)
        ux = ctypes.c_double()
        self._chk(lib().emst_get_rescaled(self.h, _p(out), ctypes.byref(ux), self.n * self.dim))
        return out, ux.value

    # --- one-shot --------------------------------------------------------
    def solve(self, pts):
        pts = np.ascontiguousarray(pts, dtype=np.float32)
        n, dim = pts.shape
        uv = np.zeros((max(n - 1, 1), 2), np.int32)
        ne, ln = ctypes.c_int64(), ctypes.c_double()
        self._chk(lib().emst_solve(self.h, _p(pts), n, dim, _p(uv), ctypes.byref(ne), ctypes.byref(ln)))
        self.n, self.dim = n, dim
        return uv[: ne.value].copy(), ln.value

    def solve_into(self, pts, uv_out):
        """Host arrays in and out, no allocation: pts (n, dim) float32, uv_out (n-1, 2) int32."""
        ne, ln = ctypes.c_int64(), ctypes.c_double()
        self._chk(lib().emst_solve(self.h, _p(pts), pts.shape[0], pts.shape[1], _p(uv_out), ctypes.byref(ne),
                                   ctypes.byref(ln)))
        self.n, self.dim = pts.shape
        return ne.value, ln.value

    def solve_batch(self, clouds):
        """clouds: list of (n_i, dim_i) float32 arrays -> (list of (n_i-1, 2) int32 edges, lengths)."""
        sizes = np.array([len(c) for c in clouds], np.int64)
        dims = np.array([c.shape[1] for c in clouds], np.int32)
        offs = np.zeros(len(clouds) + 1, np.int64)
        offs[1:] = np.cumsum(sizes)
        flat = np.ascontiguousarray(np.concatenate([np.ascontiguousarray(c, np.float32).ravel() for c in clouds]))
        rows = int(np.maximum(sizes - 1, 0).sum())
        uv = np.zeros((max(rows, 1), 2), np.int32)
        lens = np.zeros(len(clouds), np.float64)
        ne = ctypes.c_int64()
        self._chk(lib().emst_solve_batch(self.h, _p(flat), _p(offs), _p(dims), len(clouds), _p(uv), _p(lens),
                                         ctypes.byref(ne)))
        eo = np.concatenate([[0], np.cumsum(np.maximum(sizes - 1, 0))])
        return [uv[eo[i]:eo[i + 1]].copy() for i in range(len(clouds))], lens

    def autotune(self, pts):
        """Times every launch shape on pts; keeps the fastest. -> (search_shape, ms per shape)."""
        pts = np.ascontiguousarray(pts, np.float32)
        cnt, _, _ = search_shapes()
        ms = np.zeros(cnt, np.float64)
        best = ctypes.c_int()
        self._chk(lib().emst_autotune(self.h, _p(pts), len(pts), pts.shape[1], ctypes.byref(best), _p(ms), cnt))
        self.n, self.dim = len(pts), pts.shape[1]
        return best.value, ms

    def search_shape(self):
        v = ctypes.c_int()
        self._chk(lib().emst_get_search_shape(self.h, ctypes.byref(v)))
        return v.value

    def tuning(self):
        """The search settings in use and the last autotune's stage tables (dict)."""
        t = Tuning()
        self._chk(lib().emst_get_tuning(self.h, ctypes.byref(t)))
        return {"knn_k": t.knn_k, "coop_min": t.coop_min, "wide_max": t.wide_max, "search_shape": t.search_shape,
                "knn_k_values": list(t.knn_k_values), "ms_knn_k": list(t.ms_knn_k),
                "coop_min_values": list(t.coop_min_values), "ms_coop_min": list(t.ms_coop_min),
                "wide_max_values": list(t.wide_max_values), "ms_wide_max": list(t.ms_wide_max),
                "ms_shape": list(t.ms_shape)}

    # --- learned proposal ------------------------------------------------
    def set_proposal(self, weights, margin=1.0, threshold=0.0):
        """weights: PROPOSAL_WEIGHTS floats (learned first pass on) or None (off)."""
        if weights is None:
            self._chk(lib().emst_set_proposal(self.h, None, 0.0, 0.0))
            return
        w = np.ascontiguousarray(weights, np.float32).ravel()
        assert w.size == PROPOSAL_WEIGHTS
        self._chk(lib().emst_set_proposal(self.h, _p(w), float(margin), float(threshold)))

    def trace_enable(self, capacity, sample_shift=0):
        self._chk(lib().emst_trace_enable(self.h, int(capacity), int(sample_shift)))

    def trace(self):
        """Trace records so far, (count, TRACE_RECORD) float32."""
        cnt = ctypes.c_int64()
        self._chk(lib().emst_get_trace(self.h, None, 0, ctypes.byref(cnt)))
        out = np.zeros((cnt.value, TRACE_RECORD), np.float32)
        if cnt.value:
            self._chk(lib().emst_get_trace(self.h, _p(out), cnt.value, ctypes.byref(cnt)))
        return out

    def trace_device(self):
        """(device pointer, count) of the trace records."""
        ptr, cnt = ctypes.c_void_p(), ctypes.c_int64()
        self._chk(lib().emst_get_trace_device(self.h, ctypes.byref(ptr), ctypes.byref(cnt)))
        return ptr.value, cnt.value

    def keep_round_labels(self, rounds):
        """Keep each point's root after each of the first `rounds` rounds (next solve on)."""
        self._chk(lib().emst_keep_round_labels(self.h, int(rounds)))

    def round_labels(self, r):
        """Roots (input ids) after round r of the last solve."""
        out = np.zeros(self.n, np.int32)
        self._chk(lib().emst_get_round_labels(self.h, int(r), _p(out), self.n))
        return out

    def write_results(self, base):
        """<base>.links, <base>.disjointSetMap, <base>.points of the finished solve."""
        self._chk(lib().emst_write_results(self.h, str(base).encode()))

    def solve_device(self, d_points, n, dim, d_uv, d_length):
        ne = ctypes.c_int64()
        self._chk(lib().emst_solve_device(self.h, ctypes.c_void_p(d_points), int(n), int(dim), ctypes.c_void_p(d_uv),
                                          ctypes.c_void_p(d_length), ctypes.byref(ne)))
        self.n, self.dim = int(n), int(dim)
        return ne.value


def solve(pts, device=0):
    with Emst(device=device) as e:
        return e.solve(pts)
