"""emst_region_table_noalloc: the allocation-free region table.

Some callers cannot allocate device memory once running (their device memory
is owned by their own allocator, or a mid-run cudaMalloc / cudaFree could
stall or fail, or their callback forbids allocation).  This entry point takes
device buffers for the points and both outputs and works inside one fixed
device array of the library, up to EMST_NOALLOC_MAX_POINTS points.

Called through the C ABI, twice in a row, and checked against the regular
entry point (emst_compute_octants + emst_get_region_table): both outputs must
be identical bit for bit, the same tolerance the other region-table tests use.
The file is named so that pytest collects it last.
"""
import ctypes
import re

import numpy as np
import pytest

from families import family

pytestmark = pytest.mark.gpu


def _limits(gpu_lib):
    txt = open(gpu_lib.HEADER).read()
    max_pts = int(re.search(r"#define EMST_NOALLOC_MAX_POINTS (\d+)", txt).group(1))
    return max_pts


def _noalloc(gpu_lib, torch, pts):
    n, dim = pts.shape
    K = gpu_lib.K_OF_DIM[dim]
    d_pts = torch.from_numpy(np.ascontiguousarray(pts)).cuda()
    d_ids = torch.full((n, K), 7, dtype=torch.int32, device="cuda")
    d_d2 = torch.full((n, K), 7.0, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    st = gpu_lib.lib().emst_region_table_noalloc(ctypes.c_void_p(d_pts.data_ptr()), n, dim,
                                                 ctypes.c_void_p(d_ids.data_ptr()),
                                                 ctypes.c_void_p(d_d2.data_ptr()), ctypes.c_void_p(stream))
    torch.cuda.synchronize()
    return st, d_ids.cpu().numpy(), d_d2.cpu().numpy()


def _regular(gpu_lib, pts):
    with gpu_lib.Emst(keep_region_table=True) as e:
        e.initialize(pts)
        e.flatten()
        e.compute_octants()
        return e.region_table()


def test_noalloc_matches_regular_entry_point_twice(gpu_lib):
    torch = pytest.importorskip("torch")
    max_pts = _limits(gpu_lib)
    # 3D at the limit carves the most scratch (24 regions per point)
    cases = [family("cluster", 20000, 3, 31), family("dups", max_pts, 2, 32), family("uniform", max_pts, 3, 34)]
    for pts in cases:
        ref_ids, ref_d2 = _regular(gpu_lib, pts)
        st, ids, d2 = _noalloc(gpu_lib, torch, pts)
        assert st == 0
        assert np.array_equal(ids, ref_ids)
        assert np.array_equal(d2.view(np.uint32), ref_d2.view(np.uint32))
    # a later call on the same data leaves device memory use unchanged (the
    # first call on a device may place the library's static array there)
    free_before = torch.cuda.mem_get_info()[0]
    st, ids, d2 = _noalloc(gpu_lib, torch, cases[0])
    free_after = torch.cuda.mem_get_info()[0]
    assert st == 0 and free_after == free_before
    ref_ids, ref_d2 = _regular(gpu_lib, cases[0])
    assert np.array_equal(ids, ref_ids)
    assert np.array_equal(d2.view(np.uint32), ref_d2.view(np.uint32))


def test_noalloc_rejects_sizes_beyond_its_limit(gpu_lib):
    torch = pytest.importorskip("torch")
    max_pts = _limits(gpu_lib)
    st, _, _ = _noalloc(gpu_lib, torch, family("uniform", max_pts + 1, 2, 33))
    assert st == 3  # EMST_EOVERFLOW, nothing launched
