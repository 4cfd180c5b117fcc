// radix.cu -- stable LSD radix sort of (64-bit key, 32-bit value) pairs in
// 8-bit digits, one launch per digit (see radix.cuh for its role).
//
//   k_radix_hist     one read of the keys: the digit histogram of every pass
//   k_radix_offsets  each pass's histogram -> the first output position of
//                    every digit (exclusive scan, one block)
//   k_radix_pass     per pass: a block takes the next tile of kRadixTile keys
//                    (a ticket keeps tiles in launch order), ranks its keys
//                    by digit in input order (digit-bit ballots + per-warp counts),
//                    publishes its per-digit counts and looks back over the
//                    earlier tiles' counts for its output offsets (decoupled
//                    look-back, one thread per digit), then writes keys and
//                    values through shared memory so that each digit's run
//                    is written contiguously.
//
// Bytes per pair and pass: 12 read + 12 written (8 + 8 for keys alone); the
// histogram reads the keys once more.  A block waits only on tiles whose tickets came before its own,
// so every block it waits on is already running; each wait is still bounded
// and reports through *err instead of spinning on.
#include "radix.cuh"

#include <algorithm>

namespace emst {

namespace {

constexpr unsigned kFullMask = 0xffffffffu;
constexpr int kRadixWarps = kRadixThreads / 32;
constexpr unsigned long long kStAgg = 1ull << 62;   // tile count published
constexpr unsigned long long kStIncl = 2ull << 62;  // inclusive prefix published
constexpr uint32_t kSpinLimit = 1u << 20;
constexpr uint32_t kErrSortWait = 1u << 16;

// Exclusive scan over the block of one value per thread (blockDim = kRadixThreads).
__device__ __forceinline__ uint32_t block_scan_excl(uint32_t v, uint32_t* s_tmp)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(kFullMask, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) s_tmp[w] = incl;
    __syncthreads();
    if (w == 0) {
        const uint32_t x = lane < kRadixWarps ? s_tmp[lane] : 0u;
        uint32_t in = x;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(kFullMask, in, o);
            if (lane >= o) in += t;
        }
        if (lane < kRadixWarps) s_tmp[lane] = in - x;
    }
    __syncthreads();
    const uint32_t ex = s_tmp[w] + incl - v;
    __syncthreads();
    return ex;
}

__global__ void __launch_bounds__(kRadixThreads)
    k_radix_hist(const uint64_t* __restrict__ keys, uint32_t n, int begin_bit, int passes, uint32_t* __restrict__ hist)
{
    __shared__ uint32_t s_h[kRadixMaxPasses][kRadixBins];
    for (int i = threadIdx.x; i < kRadixMaxPasses * kRadixBins; i += blockDim.x) (&s_h[0][0])[i] = 0;
    __syncthreads();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint64_t k = keys[i];
        for (int p = 0; p < passes; ++p)
            atomicAdd(&s_h[p][(uint32_t)(k >> (begin_bit + kRadixBits * p)) & 0xffu], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < passes * kRadixBins; i += blockDim.x) {
        const uint32_t v = (&s_h[0][0])[i];
        if (v) atomicAdd(&hist[i], v);
    }
}

__global__ void __launch_bounds__(kRadixThreads) k_radix_offsets(int passes, uint32_t* __restrict__ hist)
{
    __shared__ uint32_t s_tmp[kRadixWarps];
    for (int p = 0; p < passes; ++p) {
        const uint32_t v = hist[p * kRadixBins + threadIdx.x];
        hist[p * kRadixBins + threadIdx.x] = block_scan_excl(v, s_tmp);
    }
}

template <bool VALUES>
__global__ void __launch_bounds__(kRadixThreads, VALUES ? 2 : 3)
    k_radix_pass(const uint64_t* __restrict__ kin, const uint32_t* __restrict__ vin, uint64_t* __restrict__ kout,
                 uint32_t* __restrict__ vout, uint32_t n, int shift, const uint32_t* __restrict__ goff,
                 unsigned long long* __restrict__ status, uint32_t* __restrict__ ticket, uint32_t* __restrict__ err)
{
    __shared__ uint32_t s_tile;
    __shared__ uint32_t s_wcnt[kRadixWarps][kRadixBins];  // per warp: running digit counts, then prefixes
    __shared__ uint32_t s_dstart[kRadixBins];             // first tile-local position of each digit
    __shared__ uint32_t s_gbase[kRadixBins];              // output position minus tile-local position
    __shared__ uint32_t s_tmp[kRadixWarps];
    __shared__ uint64_t s_buf[kRadixTile];                // keys, then values, in sorted tile order
    __shared__ unsigned char s_dig[kRadixTile];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (threadIdx.x == 0) s_tile = atomicAdd(ticket, 1u);
    for (int i = threadIdx.x; i < kRadixWarps * kRadixBins; i += blockDim.x) (&s_wcnt[0][0])[i] = 0;
    __syncthreads();
    const uint32_t tile = s_tile;
    const uint32_t base = tile * (uint32_t)kRadixTile;
    const uint32_t tile_n = min((uint32_t)kRadixTile, n - base);
    const uint32_t lt = (1u << lane) - 1u;

    // 1. rank every key among the tile's keys of its digit, in input order:
    // warp w holds elements [w * 32 * items, (w + 1) * 32 * items), item i of
    // lane l being element i * 32 + l of that range
    uint64_t k[kRadixItems];
    uint32_t v[kRadixItems];  // the values, loaded with the keys so that both reads overlap the ranking
    uint32_t pos[kRadixItems];
    const uint32_t wbase = base + (uint32_t)w * 32u * kRadixItems;
#pragma unroll
    for (int i = 0; i < kRadixItems; ++i) {
        const uint32_t idx = wbase + (uint32_t)i * 32u + (uint32_t)lane;
        k[i] = idx < n ? kin[idx] : 0ull;
        if constexpr (VALUES) v[i] = idx < n ? vin[idx] : 0u;
    }
#pragma unroll
    for (int i = 0; i < kRadixItems; ++i) {
        const uint32_t idx = wbase + (uint32_t)i * 32u + (uint32_t)lane;
        const bool valid = idx < n;
        const uint32_t d = (uint32_t)(k[i] >> shift) & 0xffu;
        // lanes of this item holding the same digit: one ballot per digit bit
        uint32_t peers = __ballot_sync(kFullMask, valid);
        peers = valid ? peers : (1u << lane);
#pragma unroll
        for (int b = 0; b < kRadixBits; ++b) {
            const uint32_t m = __ballot_sync(kFullMask, (d >> b) & 1u);
            peers &= ((d >> b) & 1u) ? m : ~m;
        }
        uint32_t c0 = 0;
        if (valid) c0 = s_wcnt[w][d];
        __syncwarp();
        if (valid) {
            pos[i] = c0 + __popc(peers & lt);
            if ((peers & lt) == 0) s_wcnt[w][d] = c0 + __popc(peers);
        }
        __syncwarp();
    }
    __syncthreads();

    // 2. per digit (one thread each): the tile's count, the per-warp prefixes
    const uint32_t dg = threadIdx.x;
    uint32_t tot = 0;
#pragma unroll
    for (int ww = 0; ww < kRadixWarps; ++ww) {
        const uint32_t c = s_wcnt[ww][dg];
        s_wcnt[ww][dg] = tot;
        tot += c;
    }
    volatile unsigned long long* st = status + (size_t)tile * kRadixBins + dg;
    *st = (tile == 0 ? kStIncl : kStAgg) | tot;
    const uint32_t dstart = block_scan_excl(tot, s_tmp);
    s_dstart[dg] = dstart;

    // 3. look back: the counts of this digit in all earlier tiles
    uint32_t prefix = 0;
    if (tile > 0) {
        bool stuck = false;
        for (uint32_t t = tile - 1;; --t) {
            volatile const unsigned long long* ps = status + (size_t)t * kRadixBins + dg;
            unsigned long long v = *ps;
            for (uint32_t it = 0; (v >> 62) == 0; ++it) {
                if (it >= kSpinLimit) {
                    stuck = true;
                    break;
                }
                v = *ps;
            }
            if (stuck) break;
            prefix += (uint32_t)v;
            if ((v >> 62) == 2ull || t == 0) break;
        }
        if (stuck) atomicOr(err, kErrSortWait);
        *st = kStIncl | (prefix + tot);
    }
    s_gbase[dg] = goff[dg] + prefix - dstart;
    __syncthreads();

    // 4. keys to their sorted tile positions, then out in runs per digit
#pragma unroll
    for (int i = 0; i < kRadixItems; ++i) {
        const uint32_t idx = wbase + (uint32_t)i * 32u + (uint32_t)lane;
        if (idx < n) {
            const uint32_t d = (uint32_t)(k[i] >> shift) & 0xffu;
            pos[i] += s_dstart[d] + s_wcnt[w][d];
            s_buf[pos[i]] = k[i];
            s_dig[pos[i]] = (unsigned char)d;
        }
    }
    __syncthreads();
    for (uint32_t j = threadIdx.x; j < tile_n; j += kRadixThreads) kout[s_gbase[s_dig[j]] + j] = s_buf[j];
    if constexpr (!VALUES) return;
    __syncthreads();
    // 5. the values the same way
    uint32_t* const s_val = reinterpret_cast<uint32_t*>(s_buf);
#pragma unroll
    for (int i = 0; i < kRadixItems; ++i) {
        const uint32_t idx = wbase + (uint32_t)i * 32u + (uint32_t)lane;
        if (idx < n) s_val[pos[i]] = v[i];
    }
    __syncthreads();
    for (uint32_t j = threadIdx.x; j < tile_n; j += kRadixThreads) vout[s_gbase[s_dig[j]] + j] = s_val[j];
}

struct Layout {
    size_t hist, tickets, status, total;
};

Layout layout(int64_t n, int end_bit)
{
    const int passes = radix_passes(end_bit);
    const size_t tiles = (size_t)((n + kRadixTile - 1) / kRadixTile);
    Layout l;
    l.hist = 0;
    l.tickets = l.hist + sizeof(uint32_t) * kRadixMaxPasses * kRadixBins;
    l.status = l.tickets + 256;
    l.total = l.status + sizeof(unsigned long long) * (size_t)passes * tiles * kRadixBins;
    return l;
}

}  // namespace

size_t radix_scratch_bytes(int64_t n, int end_bit) { return layout(n, end_bit).total; }

namespace {

cudaError_t radix_sort(uint64_t* keys, uint64_t* keys_alt, uint32_t* vals, uint32_t* vals_alt, int64_t n,
                       int begin_bit, int nbits, void* scratch, size_t scratch_bytes, uint32_t* err, bool* in_alt,
                       cudaStream_t s)
{
    *in_alt = false;
    if (n <= 1 || nbits <= 0) return cudaSuccess;
    if (begin_bit < 0 || begin_bit + nbits > 64 || n > (int64_t)0x7fffffff) return cudaErrorInvalidValue;
    const Layout l = layout(n, nbits);
    if (!scratch || scratch_bytes < l.total) return cudaErrorInvalidValue;
    const int passes = radix_passes(nbits);
    const uint32_t tiles = (uint32_t)((n + kRadixTile - 1) / kRadixTile);
    unsigned char* base = static_cast<unsigned char*>(scratch);
    uint32_t* hist = reinterpret_cast<uint32_t*>(base + l.hist);
    uint32_t* tickets = reinterpret_cast<uint32_t*>(base + l.tickets);
    unsigned long long* status = reinterpret_cast<unsigned long long*>(base + l.status);
    cudaError_t e = cudaMemsetAsync(scratch, 0, l.total, s);
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const uint64_t hblocks = std::min<uint64_t>(((uint64_t)n + kRadixThreads - 1) / kRadixThreads,
                                                (uint64_t)std::max(sms, 1) * 4);
    k_radix_hist<<<(unsigned)hblocks, kRadixThreads, 0, s>>>(keys, (uint32_t)n, begin_bit, passes, hist);
    k_radix_offsets<<<1, kRadixThreads, 0, s>>>(passes, hist);
    uint64_t* ki = keys;
    uint64_t* ko = keys_alt;
    uint32_t* vi = vals;
    uint32_t* vo = vals_alt;
    for (int p = 0; p < passes; ++p) {
        const int shift = begin_bit + kRadixBits * p;
        if (vals)
            k_radix_pass<true><<<tiles, kRadixThreads, 0, s>>>(ki, vi, ko, vo, (uint32_t)n, shift, hist + p * kRadixBins,
                                                               status + (size_t)p * tiles * kRadixBins, tickets + p,
                                                               err);
        else
            k_radix_pass<false><<<tiles, kRadixThreads, 0, s>>>(ki, nullptr, ko, nullptr, (uint32_t)n, shift,
                                                                hist + p * kRadixBins,
                                                                status + (size_t)p * tiles * kRadixBins, tickets + p,
                                                                err);
        std::swap(ki, ko);
        std::swap(vi, vo);
    }
    *in_alt = (passes & 1) != 0;
    return cudaGetLastError();
}

}  // namespace

cudaError_t radix_sort_pairs(uint64_t* keys, uint64_t* keys_alt, uint32_t* vals, uint32_t* vals_alt, int64_t n,
                             int end_bit, void* scratch, size_t scratch_bytes, uint32_t* err, bool* in_alt,
                             cudaStream_t s)
{
    if (!vals || !vals_alt) return cudaErrorInvalidValue;
    return radix_sort(keys, keys_alt, vals, vals_alt, n, 0, end_bit, scratch, scratch_bytes, err, in_alt, s);
}

cudaError_t radix_sort_keys(uint64_t* keys, uint64_t* keys_alt, int64_t n, int begin_bit, int nbits, void* scratch,
                            size_t scratch_bytes, uint32_t* err, bool* in_alt, cudaStream_t s)
{
    return radix_sort(keys, keys_alt, nullptr, nullptr, n, begin_bit, nbits, scratch, scratch_bytes, err, in_alt, s);
}

}  // namespace emst
