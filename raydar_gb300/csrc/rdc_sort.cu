// rdc_sort.cu -- the device sort and prefix sum the LBVH build uses (sm_103a).
//
// radix_sort_pairs: stable least-significant-digit radix sort of (key, value)
// pairs of 32-bit words, 10 bits of key per pass (3 passes for the 30-bit
// Morton codes).  Each pass is three launches over tiles of 2048 pairs:
//   1. per tile, a histogram of the pass's digit (shared-memory atomics),
//      stored digit-major: counts[digit * ntiles + tile];
//   2. an exclusive prefix sum of that array (exclusive_scan below), which
//      gives every (digit, tile) its first output position: all smaller
//      digits of every tile, then this digit in earlier tiles;
//   3. per tile, the stable rank of every pair among the tile's pairs with
//      the same digit, and the scatter.  A warp owns 256 consecutive pairs
//      and walks them 32 at a time in order: __match_any_sync groups the
//      lanes holding the same digit, a lane's rank in its group is the count
//      of lower lanes in it, and per-warp digit counters in shared memory
//      carry the ranks from one group of 32 to the next; a prefix over the
//      warps' counters then orders the warps.  Pairs with equal keys keep
//      their input order, as the Karras construction's tie-break (by
//      position) expects of the sort it follows.
//
// exclusive_scan: out[i] = in[0] + ... + in[i - 1] over uint32_t, in
// chunks of 4096 (a block of 1024 threads, 4 values each): each chunk is
// scanned in shared memory and its total kept; the totals (at most 4096 of
// them, so n <= 2^24) are scanned by one block; each chunk then adds its
// total's prefix.  In place (out == in) is allowed.
#include <cstdint>

#include "rdc_internal.hpp"

namespace rdc {

namespace {

constexpr int kSortThreads = 256;
constexpr int kSortWarps = kSortThreads / 32;
constexpr int kSortPerWarp = 256;  // consecutive pairs a warp ranks, 32 at a time
constexpr int kSortTile = kSortWarps * kSortPerWarp;  // 2048
constexpr int kRadixBits = 10;
constexpr int kRadixDigits = 1 << kRadixBits;

constexpr int kScanThreads = 1024;
constexpr int kScanChunk = 4 * kScanThreads;  // 4096

__global__ void __launch_bounds__(kSortThreads) radix_hist_kernel(const uint32_t* __restrict__ keys, uint32_t n,
                                                                  int shift, uint32_t ntiles,
                                                                  uint32_t* __restrict__ counts) {
    __shared__ uint32_t h[kRadixDigits];
    for (int d = threadIdx.x; d < kRadixDigits; d += kSortThreads) h[d] = 0u;
    __syncthreads();
    const uint32_t base = blockIdx.x * kSortTile;
    for (uint32_t i = threadIdx.x; i < kSortTile; i += kSortThreads) {
        const uint32_t idx = base + i;
        if (idx < n) atomicAdd(&h[(keys[idx] >> shift) & (kRadixDigits - 1)], 1u);
    }
    __syncthreads();
    for (int d = threadIdx.x; d < kRadixDigits; d += kSortThreads) counts[(size_t)d * ntiles + blockIdx.x] = h[d];
}

__global__ void __launch_bounds__(kSortThreads) radix_scatter_kernel(const uint32_t* __restrict__ keys,
                                                                     const uint32_t* __restrict__ vals, uint32_t n,
                                                                     int shift, uint32_t ntiles,
                                                                     const uint32_t* __restrict__ offsets,
                                                                     uint32_t* __restrict__ keys_out,
                                                                     uint32_t* __restrict__ vals_out) {
    __shared__ uint32_t wc[kSortWarps][kRadixDigits];  // per-warp digit counts, then the warp's prefix
    __shared__ uint32_t gbase[kRadixDigits];            // this tile's first output position per digit
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < kSortWarps * kRadixDigits; i += kSortThreads) (&wc[0][0])[i] = 0u;
    __syncthreads();
    constexpr int R = kSortPerWarp / 32;
    const uint32_t base = blockIdx.x * kSortTile + warp * kSortPerWarp;
    uint32_t key[R], val[R], rank[R];
#pragma unroll
    for (int k = 0; k < R; ++k) {
        const uint32_t idx = base + k * 32 + lane;
        const bool ok = idx < n;
        key[k] = ok ? keys[idx] : 0u;
        val[k] = ok ? vals[idx] : 0u;
        // a digit outside 0..1023 for the lanes past the end: they form their own group
        const uint32_t d = (key[k] >> shift) & (kRadixDigits - 1);
        const unsigned peers = __match_any_sync(FULL, ok ? d : (uint32_t)kRadixDigits);
        const unsigned below = peers & ((1u << lane) - 1u);
        rank[k] = ok ? wc[warp][d] + (uint32_t)__popc(below) : 0u;
        __syncwarp();
        if (ok && below == 0u) wc[warp][d] += (uint32_t)__popc(peers);
        __syncwarp();
    }
    __syncthreads();
    for (int d = threadIdx.x; d < kRadixDigits; d += kSortThreads) {
        uint32_t s = 0;
#pragma unroll
        for (int w = 0; w < kSortWarps; ++w) {
            const uint32_t c = wc[w][d];
            wc[w][d] = s;
            s += c;
        }
        gbase[d] = offsets[(size_t)d * ntiles + blockIdx.x];
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < R; ++k) {
        const uint32_t idx = base + k * 32 + lane;
        if (idx < n) {
            const uint32_t d = (key[k] >> shift) & (kRadixDigits - 1);
            const uint32_t pos = gbase[d] + wc[warp][d] + rank[k];
            keys_out[pos] = key[k];
            vals_out[pos] = val[k];
        }
    }
}

// Exclusive prefix of the block's 1024 values v (one per thread); returns the
// block total through *total (thread 0's view of shared memory).
__device__ __forceinline__ uint32_t block_exclusive(uint32_t v, uint32_t* s_warp, uint32_t* total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t inc = v;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const uint32_t o = __shfl_up_sync(0xffffffffu, inc, off);
        if (lane >= off) inc += o;
    }
    if (lane == 31) s_warp[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = s_warp[lane];
        uint32_t wi = w;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const uint32_t o = __shfl_up_sync(0xffffffffu, wi, off);
            if (lane >= off) wi += o;
        }
        s_warp[lane] = wi - w;  // exclusive prefix of the warp totals
        if (lane == 31) *total = wi;
    }
    __syncthreads();
    return s_warp[warp] + inc - v;
}

__global__ void __launch_bounds__(kScanThreads) scan_chunks_kernel(const uint32_t* in, uint32_t* out, uint32_t n,
                                                                   uint32_t* chunk_totals) {
    __shared__ uint32_t s_warp[32];
    __shared__ uint32_t s_total;
    const uint32_t i0 = blockIdx.x * kScanChunk + 4 * threadIdx.x;
    uint32_t v[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) v[j] = i0 + j < n ? in[i0 + j] : 0u;
    const uint32_t sum = (v[0] + v[1]) + (v[2] + v[3]);
    uint32_t run = block_exclusive(sum, s_warp, &s_total);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        if (i0 + j < n) out[i0 + j] = run;
        run += v[j];
    }
    if (threadIdx.x == 0) chunk_totals[blockIdx.x] = s_total;
}

// One block: exclusive scan of m <= 4096 chunk totals, in place.
__global__ void __launch_bounds__(kScanThreads) scan_totals_kernel(uint32_t* t, uint32_t m) {
    __shared__ uint32_t s_warp[32];
    __shared__ uint32_t s_total;
    const uint32_t i0 = 4 * threadIdx.x;
    uint32_t v[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) v[j] = i0 + j < m ? t[i0 + j] : 0u;
    uint32_t run = block_exclusive((v[0] + v[1]) + (v[2] + v[3]), s_warp, &s_total);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        if (i0 + j < m) t[i0 + j] = run;
        run += v[j];
    }
}

__global__ void scan_add_kernel(uint32_t* out, uint32_t n, const uint32_t* __restrict__ chunk_prefix) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] += chunk_prefix[i / kScanChunk];
}

}  // namespace

size_t exclusive_scan_scratch_bytes(uint32_t n) {
    const size_t chunks = ((size_t)n + kScanChunk - 1) / kScanChunk;
    return (chunks > 0 ? chunks : 1) * sizeof(uint32_t);
}

cudaError_t exclusive_scan(const uint32_t* in, uint32_t* out, uint32_t n, void* scratch, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    const uint32_t chunks = (n + kScanChunk - 1) / kScanChunk;
    if (chunks > (uint32_t)kScanChunk) return cudaErrorInvalidValue;  // more than 2^24 values
    uint32_t* totals = static_cast<uint32_t*>(scratch);
    scan_chunks_kernel<<<chunks, kScanThreads, 0, s>>>(in, out, n, totals);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || chunks == 1) return e;
    scan_totals_kernel<<<1, kScanThreads, 0, s>>>(totals, chunks);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    const uint32_t B = 256;
    scan_add_kernel<<<(n + B - 1) / B, B, 0, s>>>(out, n, totals);
    return cudaGetLastError();
}

size_t radix_sort_scratch_bytes(uint32_t n) {
    const size_t ntiles = ((size_t)n + kSortTile - 1) / kSortTile;
    const size_t counts = (ntiles > 0 ? ntiles : 1) * kRadixDigits;
    auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
    return up(counts * sizeof(uint32_t)) + up(exclusive_scan_scratch_bytes((uint32_t)counts));
}

cudaError_t radix_sort_pairs(uint32_t* keys, uint32_t* vals, uint32_t* keys_alt, uint32_t* vals_alt, uint32_t n,
                             int key_bits, void* scratch, cudaStream_t s, uint32_t** keys_sorted,
                             uint32_t** vals_sorted) {
    *keys_sorted = keys;
    *vals_sorted = vals;
    if (n <= 1) return cudaSuccess;
    const uint32_t ntiles = (n + kSortTile - 1) / kSortTile;
    if ((size_t)ntiles * kRadixDigits > (size_t)kScanChunk * kScanChunk) return cudaErrorInvalidValue;
    uint32_t* counts = static_cast<uint32_t*>(scratch);
    const size_t counts_b = ((size_t)ntiles * kRadixDigits * sizeof(uint32_t) + 255) & ~(size_t)255;
    void* scan_scratch = static_cast<char*>(scratch) + counts_b;
    uint32_t *ka = keys, *va = vals, *kb = keys_alt, *vb = vals_alt;
    for (int shift = 0; shift < key_bits; shift += kRadixBits) {
        radix_hist_kernel<<<ntiles, kSortThreads, 0, s>>>(ka, n, shift, ntiles, counts);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        e = exclusive_scan(counts, counts, ntiles * (uint32_t)kRadixDigits, scan_scratch, s);
        if (e != cudaSuccess) return e;
        radix_scatter_kernel<<<ntiles, kSortThreads, 0, s>>>(ka, va, n, shift, ntiles, counts, kb, vb);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        uint32_t* t = ka;
        ka = kb;
        kb = t;
        t = va;
        va = vb;
        vb = t;
    }
    *keys_sorted = ka;
    *vals_sorted = va;
    return cudaSuccess;
}

}  // namespace rdc
