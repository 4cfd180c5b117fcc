// noalloc.cu -- emst_region_table_noalloc: the static-pruning region table
// for callers that cannot allocate device memory.
//
// Every intermediate buffer of the region-table computation (rescaled and
// sorted points, cell keys, radix-sort temporary storage, the leaf tree,
// per-point lists and counters) is carved from one file-scope device array,
// g_noalloc_scratch, of EMST_NOALLOC_SCRATCH_BYTES.  The caller passes the
// points and the two output arrays.  No cudaMalloc / cudaFree (or any
// allocating library routine) is called.
//
// The array's host-side name is only a stand-in for the symbol, not a device
// address: the device address is fetched once per device with
// cudaGetSymbolAddress, with that device current, on the first call made on
// that device, and cached.  That first call should therefore come before any
// stream capture.  Under CUDA's lazy module loading (the default) the array
// itself is placed on a device when this file's module is first used there,
// which is that first call's address lookup, not the loading of the library:
// a caller that must not see that reservation mid-run makes one call at
// start-up.
//
// All calls share the array and it keeps the previous call's contents, so the
// counters and sort scratch that must start at zero are cleared on every
// call; two calls whose work overlaps on the GPU (different streams, or
// different host threads) race on the array and must be serialised by the
// caller.
//
// The slices are sized with the same helpers the allocating path uses
// (grid_reduce_blocks, radix_scratch_bytes), and the context is built with
// Ctx::no_alloc set: if a slice were ever smaller than what a kernel step
// asks for, that step fails (EMST_ENOMEM) instead of allocating.
#include <cstring>
#include <mutex>

#include "../../include/emst.h"
#include "emst_ctx.h"
#include "emst_device.cuh"
#include "radix.cuh"

namespace {

constexpr size_t kScratchBytes = EMST_NOALLOC_SCRATCH_BYTES;
constexpr int64_t kMaxPoints = EMST_NOALLOC_MAX_POINTS;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_setup_mutex;
unsigned char* g_scratch_addr[kMaxDevices] = {nullptr};

// Carves aligned slices off the scratch array.
struct Carver {
    unsigned char* base;
    size_t off = 0;
    bool ok = true;
    template <typename T>
    void take(emst::DevBuf<T>& b, size_t count)
    {
        size_t bytes = count * sizeof(T);
        size_t start = (off + 255) & ~size_t(255);
        if (start + bytes > kScratchBytes) {
            ok = false;
            return;
        }
        b.p = reinterpret_cast<T*>(base + start);
        b.cap = count;
        off = start + bytes;
    }
};

}  // namespace

extern "C" emst_status emst_region_table_noalloc(const float* d_points, int64_t n, int dim, int32_t* d_ids,
                                                 float* d_d2, void* stream)
{
    if (!d_points || !d_ids || !d_d2) return EMST_EINVAL;
    if (dim != 2 && dim != 3) return EMST_EINVAL;
    if (n < 1) return EMST_EINVAL;
    if (n > kMaxPoints) return EMST_EOVERFLOW;
    // A launch error left pending by the caller's earlier, unrelated work is
    // reported here, before anything is queued, rather than blamed on this
    // call's kernels afterwards.
    if (cudaGetLastError() != cudaSuccess) return EMST_ECUDA;

    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return EMST_ECUDA;
    unsigned char* base = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_setup_mutex);
        if (!g_scratch_addr[dev]) {
            void* p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess || !p) {
                cudaGetLastError();
                return EMST_ECUDA;
            }
            g_scratch_addr[dev] = static_cast<unsigned char*>(p);
        }
        base = g_scratch_addr[dev];
    }

    emst::Ctx c;  // no allocation: every DevBuf below points into the scratch array
    c.no_alloc = true;
    c.device = dev;
    c.stream = static_cast<cudaStream_t>(stream);
    c.n = n;
    c.dim = dim;
    c.K = dim == 2 ? 8 : 24;
    c.in = d_points;
    c.nchunk = (n + emst::kLeaf - 1) / emst::kLeaf;
    int64_t L = 1;
    while (L < c.nchunk) L <<= 1;
    const int nblk = emst::grid_reduce_blocks(n);
    const size_t sort_bytes = emst::radix_scratch_bytes(n, emst::grid_sort_end_bit(dim));
    Carver cv{base};
    cv.take(c.ctr, 1);
    cv.take(c.part, (size_t)nblk * 6);
    cv.take(c.norm, 1);
    cv.take(c.scaled, (size_t)n * dim);
    cv.take(c.mkey, (size_t)n);
    cv.take(c.mkey_alt, (size_t)n);
    cv.take(c.perm, (size_t)n);
    cv.take(c.perm_alt, (size_t)n);
    cv.take(c.sp, (size_t)n);
    cv.take(c.sort_tmp, sort_bytes);
    cv.take(c.nlo, (size_t)2 * L);
    cv.take(c.nhi, (size_t)2 * L);
    cv.take(c.nid, (size_t)2 * L);
    cv.take(c.cand, (size_t)n * c.K);
    cv.take(c.cnt, (size_t)n);
    cv.take(c.cur, (size_t)n);
    cv.take(c.zflag, (size_t)n);
    cv.take(c.zero, (size_t)n);
    cv.take(c.zero2, (size_t)n);
    if (!cv.ok) return EMST_EOVERFLOW;
    c.tab_id.p = d_ids;
    c.tab_id.cap = (size_t)n * c.K;
    c.tab_d2.p = d_d2;
    c.tab_d2.cap = (size_t)n * c.K;
    c.keep_table = true;

    // The array keeps the previous call's data: clear the counters.
    if (cudaMemsetAsync(c.ctr.p, 0, sizeof(emst::DevCounters), c.stream) != cudaSuccess) return EMST_ECUDA;
    cudaError_t e = emst::grid_build(c);
    if (e == cudaSuccess) e = emst::nns_full(c);
    if (e == cudaErrorMemoryAllocation) return EMST_ENOMEM;  // a slice too small: nothing was allocated
    if (e != cudaSuccess) return EMST_ECUDA;
    uint32_t err = 0;
    if (cudaMemcpyAsync(&err, &c.ctr.p->err, sizeof(err), cudaMemcpyDeviceToHost, c.stream) != cudaSuccess)
        return EMST_ECUDA;
    if (cudaStreamSynchronize(c.stream) != cudaSuccess) return EMST_ECUDA;
    return err ? EMST_EINVAL : EMST_OK;
}
