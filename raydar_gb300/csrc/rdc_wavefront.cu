// rdc_wavefront.cu -- wavefront form of the render (sm_103a), the other side of
// the megakernel-vs-wavefront comparison.
//
// The megakernel (render_kernel) keeps each path in one lane's registers from
// its primary ray to its end.  Here a path's state lives in HBM (one 64-byte
// record per path) and every bounce is two launches over queues:
//   wf_intersect  one thread per queued ray: the brute-force closest hit over
//                 the scene staged in shared memory (the megakernel's
//                 intersect_all), then the ray's queue entry is appended to
//                 one of four class queues -- diffuse/specular mix, metal,
//                 glass, miss -- with one warp-aggregated atomic per class;
//   wf_shade      over the four class queues back to back, so a warp shades
//                 one material class at a time (no divergence between the
//                 glass, metal and rough branches of the scatter); survivors
//                 are compacted into the next ray queue.
// A wave is W consecutive sample indices of every pixel (W <= 16 and at most
// 2^25 paths): generate, max_bounces x (intersect, shade), accumulate.
// Accumulation must add a pixel's samples in sample order (the reference
// sums sequentially, src/renderer/cpu.rs:198-210), so the accumulate kernel
// adds each pixel's W radiances in order.  The wave is captured once as a
// CUDA graph and replayed; the first sample index and the number of samples
// in the wave (W, or the remainder in the last wave) are read from device
// memory, and the accumulate kernel advances the first.  The records
// (WfPath) are indexed by path = pixel * n + sub, n the wave's sample count
// and sub the sample's place in the wave, and the first ray queue lists them
// in that order: a warp's lanes start on a few pixels' samples, whose primary
// rays are the same (the reference samples the pixel corner), and the first
// bounces' rays start close together.  A queue entry is (sub << 28) | pixel
// (RDC_MAX_RESOLUTION^2 = 2^28 pixels).  Results are bit-identical to
// render_kernel.
#include <cstdint>

#include "rdc_bvh.cuh"
#include "rdc_device.cuh"

namespace rdc {

namespace {

__device__ __forceinline__ int material_class(const MatDev& m) {
    if (m.c.x > 0.0f) return 2;     // transmission: the glass branch
    if (m.b.w >= 1.0f) return 1;    // metallic 1: always the specular lobe
    return 0;                        // the diffuse / specular draw
}

// Queue entries: the path's place in the wave (its sample's offset from the
// wave's first) above kWfPixBits, its pixel below.
__device__ __forceinline__ uint32_t wf_entry(uint32_t sub, uint32_t pix) { return (sub << kWfPixBits) | pix; }
__device__ __forceinline__ uint32_t wf_pix(uint32_t e) { return e & ((1u << kWfPixBits) - 1u); }
__device__ __forceinline__ uint32_t wf_sub(uint32_t e) { return e >> kWfPixBits; }

// The pixel and the path (record index) a queue entry names; wn: the
// wave's sample count.
__device__ __forceinline__ void wf_decode(const WfParams& P, uint32_t wn, uint32_t e, uint32_t& pix,
                                          uint32_t& path) {
    pix = (uint32_t)checked_index(P.sc.oob, wf_pix(e), P.npix);
    path = (uint32_t)checked_index(P.sc.oob, (long long)pix * wn + wf_sub(e), P.npath);
}

// One thread per record, in record order (a warp writes 32 consecutive
// records: whole sectors; one thread per pixel writing its wn records, or
// blocks per sample index, measured slower).
__global__ void wf_generate(const WfParams P) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t wn = *P.wave_n;
    if (k == 0) {
        P.counts[0] = P.max_bounces > 0 ? P.npix * wn : 0u;
    }
    if (k >= P.npix * wn) return;
    const uint32_t i = k / wn, sub = k - i * wn;
    V3 o, d;
    primary_ray(P.sc, i % P.sc.width, i / P.sc.width, o, d);
    WfPath& w = P.path[checked_index(P.sc.oob, k, P.npath)];
    w.ot = make_float4(o.x, o.y, o.z, 0.0f);
    w.dh = make_float4(d.x, d.y, d.z, __int_as_float(-1));
    w.atten = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
    w.light = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    P.queue0[k] = wf_entry(sub, i);
}

// Append the lanes with cls >= 0 (their queue entry e) to the class queues,
// one warp-aggregated atomic per class present.  Called by a full warp.
__device__ __forceinline__ void wf_append_class(const WfParams& P, int cls, uint32_t e) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        const unsigned m = __ballot_sync(FULL, cls == c);
        if (m == 0u) continue;
        const int leader = __ffs(m) - 1;
        uint32_t b = 0;
        if (lane == leader) b = atomicAdd(&P.counts[2 + c], (uint32_t)__popc(m));
        b = __shfl_sync(FULL, b, leader);
        if (cls == c)
            P.cls[(size_t)c * P.npath + checked_index(P.sc.oob, b + __popc(m & ((1u << lane) - 1u)), P.npath)] = e;
    }
}

__global__ void __launch_bounds__(256) wf_intersect(const WfParams P, const uint32_t* __restrict__ q_in,
                                                     const uint32_t* __restrict__ n_in) {
    extern __shared__ float4 smem[];
    __shared__ __align__(8) uint64_t s_bar;
    float4* s_rec = smem;
    int4* s_runs = reinterpret_cast<int4*>(smem + P.sc.nrec);
    if (threadIdx.x == 0) bulk_init(&s_bar);
    __syncthreads();
    if (!stage_scene(&s_bar, 0u, s_rec, P.sc.rec, P.sc.nrec, s_runs, P.sc.runs, P.sc.nruns, P.errors)) return;
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const uint32_t n = *n_in;
    const uint32_t wn = *P.wave_n;
    const bool scene_fast = P.sc.fast_div != 0u;
    uint32_t segs = 0;
    // warp-uniform trip count so the ballots below see whole warps
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t base0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31u);
    for (uint32_t wbase = base0; wbase < n; wbase += stride) {
        const uint32_t k = wbase + lane;
        int cls = -1;
        uint32_t e = 0;
        if (k < n) {
            e = q_in[checked_index(P.sc.oob, k, P.npath)];
            uint32_t pix, path;  // pix: unused here
            wf_decode(P, wn, e, pix, path);
            const float4 ot = P.path[path].ot, dh = P.path[path].dh;
            const RayPre r = ray_pre(mk(ot.x, ot.y, ot.z), mk(dh.x, dh.y, dh.z), P.sc.neg_zero);
            float t;
            int idx;
            intersect_all(s_rec, s_runs, (int)P.sc.nruns, scene_fast, r, t, idx);
            P.path[path].ot.w = t;
            P.path[path].dh.w = __int_as_float(idx);
            ++segs;
            cls = idx < 0 ? 3 : material_class(P.sc.mat[checked_index(P.sc.oob, idx, P.sc.nobj)]);
        }
        wf_append_class(P, cls, e);
    }
    unsigned long long s = segs;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(FULL, s, off);
    if (lane == 0 && s != 0ull) atomicAdd(P.segments, s);
}

// LBVH scenes: the closest hit of every queued ray through the device LBVH,
// by a persistent grid whose lanes fetch rays from the queue as they finish
// (one warp-aggregated atomic per refill).  Each lane runs render_bvh_kernel's
// traversal state machine; a loop iteration is a node visit (up to two) or a
// deferred leaf test, whichever more lanes wait for, until min_idle lanes are
// done; then the finished lanes store their hit, append their pixel to a
// class queue and take the next rays.  There is no shading in this kernel, so
// a refill costs only the ray set-up, and a lane holds only traversal state.
__global__ void __launch_bounds__(kWfBvhBlock, kWfBvhMinBlocks)
    wf_intersect_bvh(const WfParams P, const uint32_t* __restrict__ q_in, const uint32_t* __restrict__ n_in,
                     uint32_t* __restrict__ fetch) {
    extern __shared__ uint2 s_stack[];  // kShortStack entries per thread
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    uint2 deep[kBvhStack - kShortStack];
    SplitStack stack{s_stack + threadIdx.x, blockDim.x, deep};
    const uint32_t n = *n_in;
    const uint32_t wn = *P.wave_n;
    const bool scene_fast = P.sc.fast_div != 0u;
    BvhCounters cnt;
    BvhTrav T;
    T.cur = -1;
    T.lmask = 0u;
    T.best = 0.0f;
    T.bidx = -1;
    RayPre r;
    bool rfast = false, busy = false, pool_open = true;
    uint32_t e = 0, path = 0, segs = 0;
    for (;;) {
        // lanes whose traversal is over: store the hit, queue the pixel by class
        const bool done = busy && T.cur < 0 && T.lmask == 0u;
        int cls = -1;
        if (done) {
            P.path[path].ot.w = T.best;
            P.path[path].dh.w = __int_as_float(T.bidx);
            if (T.bidx < 0) {
                cls = 3;
            } else {
                const MatDev* mp = P.sc.mat + checked_index(P.sc.oob, T.bidx, P.sc.nobj);
                const float metallic = __ldg(&mp->b.w), transmission = __ldg(&mp->c.x);
                cls = transmission > 0.0f ? 2 : (metallic >= 1.0f ? 1 : 0);  // material_class
            }
            busy = false;
        }
        if (__ballot_sync(FULL, done) != 0u) wf_append_class(P, cls, e);
        // refill the idle lanes from the ray queue
        const unsigned idle = __ballot_sync(FULL, !busy);
        if (idle != 0u && pool_open) {
            const unsigned c = (unsigned)__popc(idle);
            const int leader = __ffs(idle) - 1;
            uint32_t base = 0;
            if (lane == leader) base = atomicAdd(fetch, c);
            base = __shfl_sync(FULL, base, leader);
            if (base + c >= n) pool_open = false;
            if (!busy) {
                const uint32_t mine = base + (uint32_t)__popc(idle & ((1u << lane) - 1u));
                if (mine < n) {
                    e = q_in[checked_index(P.sc.oob, mine, P.npath)];
                    uint32_t pix;
                    wf_decode(P, wn, e, pix, path);
                    const float4 ot = P.path[path].ot, dh = P.path[path].dh;
                    r = ray_pre(mk(ot.x, ot.y, ot.z), mk(dh.x, dh.y, dh.z), P.sc.neg_zero);
                    rfast = scene_fast && r.fast;
                    bvh_begin(P.bvh, r, rfast, T, cnt);
                    busy = true;
                    ++segs;
                }
            }
        }
        if (__ballot_sync(FULL, busy) == 0u && !pool_open) break;
        // traversal steps until min_idle lanes are done (at least one step)
        for (bool first = true;; first = false) {
            const bool wl = busy && T.lmask != 0u;
            const bool wn = busy && T.lmask == 0u && T.cur >= 0;
            const unsigned lm = __ballot_sync(FULL, wl), nm = __ballot_sync(FULL, wn);
            const unsigned act = lm | nm;
            if (act == 0u || (!first && 32u - (unsigned)__popc(act) >= P.min_idle)) break;
            // leaf lanes count twice, as in the megakernel (+0.6% here)
            if (2 * __popc(lm) >= __popc(nm)) {
                if (wl) bvh_leaf_step(P.bvh, r, rfast, T, cnt);
            } else if (wn) {
                bvh_step(P.bvh, r, rfast, T, stack, cnt);
                if (T.lmask == 0u && T.cur >= 0) bvh_step(P.bvh, r, rfast, T, stack, cnt);
            }
        }
    }
    unsigned long long s2 = segs;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) s2 += __shfl_down_sync(FULL, s2, off);
    if (lane == 0 && s2 != 0ull) atomicAdd(P.segments, s2);
    unsigned long long v = cnt.visits, t = cnt.tests;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        v += __shfl_down_sync(FULL, v, off);
        t += __shfl_down_sync(FULL, t, off);
    }
    if (lane == 0 && P.bvh_counters) {
        if (v) atomicAdd(P.bvh_counters, v);
        if (t) atomicAdd(P.bvh_counters + 1, t);
    }
}

__global__ void __launch_bounds__(256) wf_shade(const WfParams P, uint32_t bounce, uint32_t* __restrict__ q_out,
                                                 uint32_t* __restrict__ n_out) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const uint32_t c0 = P.counts[2], c1 = P.counts[3], c2 = P.counts[4], c3 = P.counts[5];
    const uint32_t e0 = c0, e1 = e0 + c1, e2 = e1 + c2, total = e2 + c3;
    const uint32_t sample0 = *P.sample;
    const uint32_t wn = *P.wave_n;
    const bool more = bounce + 1u < P.max_bounces;
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t base0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31u);
    for (uint32_t wbase = base0; wbase < total; wbase += stride) {
        const uint32_t k = wbase + lane;
        bool requeue = false;
        uint32_t e = 0;
        if (k < total) {
            const int c = k < e0 ? 0 : (k < e1 ? 1 : (k < e2 ? 2 : 3));
            const uint32_t pos = k - (c == 0 ? 0u : (c == 1 ? e0 : (c == 2 ? e1 : e2)));
            e = P.cls[(size_t)c * P.npath + checked_index(P.sc.oob, pos, P.npath)];
            uint32_t pix, path;
            wf_decode(P, wn, e, pix, path);
            const uint32_t sample = sample0 + wf_sub(e);
            WfPath& w = P.path[path];
            const float4 ot = w.ot, dh = w.dh, at4 = w.atten, li4 = w.light;
            const V3 d = mk(dh.x, dh.y, dh.z);
            V3 atten = mk(at4.x, at4.y, at4.z);
            V3 light = mk(li4.x, li4.y, li4.z);
            if (c == 3) {
                // miss: the sky weighted by the throughput ends the path (cpu.rs:330-341)
                const V3 sky = world_sample(P.sc, d);
                light = vadd(light, mk(sky.x * atten.x, sky.y * atten.y, sky.z * atten.z));
            } else {
                const V3 o = mk(ot.x, ot.y, ot.z);
                const int idx = (int)checked_index(P.sc.oob, __float_as_int(dh.w), P.sc.nobj);
                const MatDev m = load_mat(P.sc.mat, idx);
                const HitRec h = closest_hit(o, d, ot.w, __ldg(&P.sc.hit[idx]), __float_as_int(m.d.y));
                V3 no, nd;
                scatter_drawn(d, h, m, pix, sample, bounce * 4u, P.stream_id, P.key0, P.key1, no, nd);
                w.ot = make_float4(no.x, no.y, no.z, 0.0f);
                w.dh = make_float4(nd.x, nd.y, nd.z, __int_as_float(-1));
                atten = mk(atten.x * m.a.x, atten.y * m.a.y, atten.z * m.a.z);
                light = vadd(light, mk(m.b.x, m.b.y, m.b.z));
                w.atten = make_float4(atten.x, atten.y, atten.z, 0.0f);
                requeue = more;
            }
            w.light = make_float4(light.x, light.y, light.z, 0.0f);
        }
        const unsigned m = __ballot_sync(FULL, requeue);
        if (m != 0u) {
            const int leader = __ffs(m) - 1;
            uint32_t b = 0;
            if (lane == leader) b = atomicAdd(n_out, (uint32_t)__popc(m));
            b = __shfl_sync(FULL, b, leader);
            if (requeue) q_out[checked_index(P.sc.oob, b + __popc(m & ((1u << lane) - 1u)), P.npath)] = e;
        }
    }
}

// Each pixel adds its wave's radiances in sample order.
__global__ void wf_accumulate(const WfParams P) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t wn = *P.wave_n;
    if (i < P.npix) {
        float4 a = P.accum[i];
        for (uint32_t sub = 0; sub < wn; ++sub) {
            const size_t k = (size_t)checked_index(P.sc.oob, (long long)i * wn + sub, P.npath);
            const float4 li = P.path[k].light;
            a.x = a.x + li.x;
            a.y = a.y + li.y;
            a.z = a.z + li.z;
            a.w = a.w + 1.0f;
        }
        P.accum[i] = a;
    }
    if (i == 0) *P.sample += wn;  // nothing in this launch reads it
}

__global__ void wf_set_word(uint32_t* word, uint32_t v) { *word = v; }

}  // namespace

size_t wavefront_state_bytes(uint32_t npath) {
    // a 64-byte record + 2 ray queues and 4 class queues of 4-byte entries per path
    return (size_t)npath * (sizeof(WfPath) + 4u * 6u);
}

uint32_t wavefront_wave_spp(uint32_t npix, uint32_t spp) {
    uint32_t w = (npix == 0u || npix >= kWfWavePaths) ? 1u : kWfWavePaths / npix;
    if (w > kWfMaxWaveSpp) w = kWfMaxWaveSpp;
    if (w > spp) w = spp;
    return w < 1u ? 1u : w;
}

size_t wavefront_bvh_smem_bytes() { return (size_t)kWfBvhBlock * kShortStack * sizeof(uint2); }

cudaError_t wavefront_occupancy(bool bvh, int block, size_t smem, int* intersect_per_sm, int* shade_per_sm) {
    cudaError_t e = cudaSuccess;
    if (bvh) {
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(intersect_per_sm, wf_intersect_bvh, kWfBvhBlock,
                                                          wavefront_bvh_smem_bytes());
    } else {
        e = cudaFuncSetAttribute(wf_intersect, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)(smem < 48 * 1024 ? 48 * 1024 : smem));
        if (e == cudaSuccess)
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(intersect_per_sm, wf_intersect, block, smem);
    }
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(shade_per_sm, wf_shade, block, 0);
    return e;
}

cudaError_t wavefront_set_word(uint32_t* word, uint32_t v, cudaStream_t s) {
    wf_set_word<<<1, 1, 0, s>>>(word, v);
    return cudaGetLastError();
}

// Enqueue one wave (up to p.npath / p.npix samples of every pixel; *p.wave_n
// of them) on s; captured into a graph by the caller.  grid_i / grid_s:
// persistent grids of the two queue kernels (the intersect kernel is
// wf_intersect_bvh when p.use_bvh).
cudaError_t enqueue_wave(const WfParams& p, int grid_i, int grid_s, size_t smem, cudaStream_t s) {
    const uint32_t b = 256, g = (p.npix + b - 1) / b, gg = (p.npath + b - 1) / b;
    wf_generate<<<gg, b, 0, s>>>(p);
    cudaError_t e = cudaGetLastError();
    for (uint32_t bounce = 0; bounce < p.max_bounces && e == cudaSuccess; ++bounce) {
        uint32_t* q_in = (bounce & 1u) ? p.queue1 : p.queue0;
        uint32_t* q_out = (bounce & 1u) ? p.queue0 : p.queue1;
        uint32_t* n_in = p.counts + (bounce & 1u);
        uint32_t* n_out = p.counts + ((bounce + 1u) & 1u);
        e = cudaMemsetAsync(n_out, 0, sizeof(uint32_t), s);
        if (e == cudaSuccess) e = cudaMemsetAsync(p.counts + 2, 0, 4 * sizeof(uint32_t), s);
        if (e == cudaSuccess && p.use_bvh) e = cudaMemsetAsync(p.counts + 7, 0, sizeof(uint32_t), s);
        if (e != cudaSuccess) break;
        if (p.use_bvh)
            wf_intersect_bvh<<<grid_i, kWfBvhBlock, wavefront_bvh_smem_bytes(), s>>>(p, q_in, n_in, p.counts + 7);
        else
            wf_intersect<<<grid_i, 256, smem, s>>>(p, q_in, n_in);
        e = cudaGetLastError();
        if (e != cudaSuccess) break;
        wf_shade<<<grid_s, 256, 0, s>>>(p, bounce, q_out, n_out);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        wf_accumulate<<<g, b, 0, s>>>(p);
        e = cudaGetLastError();
    }
    return e;
}

}  // namespace rdc
