// rdc_kernels.cu -- CUDA kernels of the GB300 path tracer (sm_103a).
//
// render_kernel is a persistent kernel: one grid of (SMs x resident blocks),
// every block stages the scene geometry in shared memory once, and every
// lane owns one pixel at a time.  A lane traces that pixel's samples
// back to back: when a path ends it immediately starts the next sample
// (path regeneration), and when the pixel's samples are done it takes a new
// pixel from a global counter (one warp-aggregated atomic per refill).  The
// warp therefore always runs one segment -- one trace_ray of
// src/renderer/cpu.rs:257 -- per active lane per iteration, and the brute-force
// primitive loop, which dominates, stays converged.  A pixel never leaves its
// lane, so its samples are summed in sample order exactly as
// render_next_sample does (src/renderer/cpu.rs:198-210): the result does not
// depend on scheduling.
#include <cstdint>

#include "rdc_device.cuh"

namespace rdc {

__global__ void __launch_bounds__(kRenderBlock, 4) render_kernel(const RenderParams P) {
    extern __shared__ float4 smem[];
    float4* s_rec = smem;
    int4* s_runs = reinterpret_cast<int4*>(smem + P.sc.nrec);
    for (uint32_t i = threadIdx.x; i < P.sc.nrec; i += blockDim.x) s_rec[i] = P.sc.rec[i];
    for (uint32_t i = threadIdx.x; i < P.sc.nruns; i += blockDim.x) s_runs[i] = P.sc.runs[i];
    __syncthreads();

    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int nruns = (int)P.sc.nruns;

    int pix = -1;
    uint32_t sample = 0, send = 0, bounce = 0;
    V3 o = mk(0.f, 0.f, 0.f), d = o, atten = o, light = o;
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    uint32_t segs = 0;
    bool pool_open = true;

    for (;;) {
        // Refill idle lanes with new pixels (warp-aggregated atomic).
        const unsigned need = __ballot_sync(FULL, pix < 0);
        if (need != 0u && pool_open) {
            const unsigned cnt = __popc(need);
            const int leader = __ffs(need) - 1;
            unsigned base = 0;
            if (lane == leader) base = atomicAdd(P.work_counter, cnt);
            base = __shfl_sync(FULL, base, leader);
            if (base + cnt >= P.npix) pool_open = false;
            if (pix < 0) {
                const unsigned mine = base + __popc(need & ((1u << lane) - 1u));
                if (mine < P.npix) {
                    pix = (int)mine;
                    acc = P.accum[pix];
                    primary_ray(P.sc, mine % P.sc.width, mine / P.sc.width, o, d);
                    sample = P.s0;
                    send = P.s0 + P.nspp;
                    bounce = 0;
                    atten = mk(1.f, 1.f, 1.f);
                    light = mk(0.f, 0.f, 0.f);
                }
            }
        }
        if (__ballot_sync(FULL, pix >= 0) == 0u) break;
        if (pix < 0) continue;  // idle lane: rejoins the warp at the refill ballot

        bool done;
        if (bounce < P.max_bounces) {
            ++segs;
            const RayPre r = ray_pre(o, d, P.sc.neg_zero);
            float t;
            int idx;
            intersect_all(s_rec, s_runs, nruns, P.sc.fast_div != 0u, r, t, idx);
            if (idx >= 0) {
                const float4 hi = __ldg(&P.sc.hit[idx]);
                const MatDev m = P.sc.mat[idx];
                const HitRec h = closest_hit(o, d, t, hi, __float_as_int(m.d.y));
                uint32_t w[12];
                const uint32_t c2 = bounce * 4u;
                const U4 w0 = philox(pix, sample, c2, P.stream_id, P.key0, P.key1);
                const U4 w1 = philox(pix, sample, c2 + 1u, P.stream_id, P.key0, P.key1);
                w[0] = w0.x; w[1] = w0.y; w[2] = w0.z; w[3] = w0.w;
                w[4] = w1.x; w[5] = w1.y; w[6] = w1.z; w[7] = w1.w;
                const U4 w2 = philox(pix, sample, c2 + 2u, P.stream_id, P.key0, P.key1);
                w[8] = w2.x; w[9] = w2.y; w[10] = w2.z; w[11] = w2.w;
                V3 no, nd;
                scatter(d, h, m, w, no, nd);
                o = no;
                d = nd;
                atten = mk(atten.x * m.a.x, atten.y * m.a.y, atten.z * m.a.z);
                light = vadd(light, mk(m.b.x, m.b.y, m.b.z));
                ++bounce;
                done = bounce >= P.max_bounces;
            } else {
                const V3 sky = world_sample(P.sc, d);
                light = vadd(light, mk(sky.x * atten.x, sky.y * atten.y, sky.z * atten.z));
                done = true;
            }
        } else {
            done = true;  // max_bounces == 0: the path adds (0, 0, 0, 1)
        }
        if (done) {
            acc.x = acc.x + light.x;
            acc.y = acc.y + light.y;
            acc.z = acc.z + light.z;
            acc.w = acc.w + 1.0f;
            ++sample;
            if (sample == send) {
                P.accum[pix] = acc;
                pix = -1;
            } else {
                // Next sample of the same pixel: the primary ray is recomputed
                // (identical every sample) rather than kept in registers.
                primary_ray(P.sc, (uint32_t)pix % P.sc.width, (uint32_t)pix / P.sc.width, o, d);
                atten = mk(1.f, 1.f, 1.f);
                light = mk(0.f, 0.f, 0.f);
                bounce = 0;
            }
        }
    }

    // Segment counter: warp sum, one 64-bit atomic per warp.
    unsigned long long s = segs;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(FULL, s, off);
    if (lane == 0 && s != 0ull) atomicAdd(P.segments, s);
}

// print_frame_buffer, src/renderer/cpu.rs:221-230.
__global__ void tonemap_kernel(const float4* __restrict__ acc, uint32_t npix, float n,
                               uchar4* __restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npix) return;
    const float4 a = acc[i];
    auto ch = [n](float s) -> unsigned char {
        const float v = fminf(fmaxf(s / n, 0.0f), 1.0f);  // NaN -> 0, as Rust `as u8`
        return (unsigned char)__float2uint_rz(v * 255.0f);
    };
    out[i] = make_uchar4(ch(a.x), ch(a.y), ch(a.z), ch(a.w));
}

__global__ void intersect_rays_kernel(const SceneView sc, const float* __restrict__ o,
                                      const float* __restrict__ d, uint32_t n, float* t_out,
                                      int32_t* idx_out, float* n_out, uint8_t* f_out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const V3 ro = mk(o[3 * i], o[3 * i + 1], o[3 * i + 2]);
    const V3 rd = mk(d[3 * i], d[3 * i + 1], d[3 * i + 2]);
    const RayPre r = ray_pre(ro, rd, sc.neg_zero);
    float t;
    int idx;
    intersect_all(sc.rec, sc.runs, (int)sc.nruns, sc.fast_div != 0u, r, t, idx);
    idx_out[i] = idx;
    if (idx >= 0) {
        const MatDev m = sc.mat[idx];
        const HitRec h = closest_hit(ro, rd, t, sc.hit[idx], __float_as_int(m.d.y));
        t_out[i] = t;
        n_out[3 * i] = h.n.x;
        n_out[3 * i + 1] = h.n.y;
        n_out[3 * i + 2] = h.n.z;
        f_out[i] = h.front ? 1 : 0;
    } else {
        t_out[i] = 0.0f;
        n_out[3 * i] = 0.0f;
        n_out[3 * i + 1] = 0.0f;
        n_out[3 * i + 2] = 0.0f;
        f_out[i] = 0;
    }
}

__global__ void scatter_fixed_kernel(const SceneView sc, const float* __restrict__ o,
                                     const float* __restrict__ d, const float* __restrict__ t,
                                     const int32_t* __restrict__ idx,
                                     const uint32_t* __restrict__ words, uint32_t n,
                                     float* o_out, float* d_out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int k = idx[i];
    if (k < 0 || (uint32_t)k >= sc.nobj) return;  // rejected on the host; never reached
    const V3 ro = mk(o[3 * i], o[3 * i + 1], o[3 * i + 2]);
    const V3 rd = mk(d[3 * i], d[3 * i + 1], d[3 * i + 2]);
    const MatDev m = sc.mat[k];
    const HitRec h = closest_hit(ro, rd, t[i], sc.hit[k], __float_as_int(m.d.y));
    uint32_t w[12];
#pragma unroll
    for (int j = 0; j < 12; ++j) w[j] = words[12 * i + j];
    V3 no, nd;
    scatter(rd, h, m, w, no, nd);
    o_out[3 * i] = no.x;
    o_out[3 * i + 1] = no.y;
    o_out[3 * i + 2] = no.z;
    d_out[3 * i] = nd.x;
    d_out[3 * i + 1] = nd.y;
    d_out[3 * i + 2] = nd.z;
}

// FP32 issue-rate probe: kProbeChains independent FFMA chains per thread,
// so every scheduler can issue one FFMA per clock.  The sink write is
// conditional on a value that never occurs, which keeps the chains live.
__global__ void fp32_probe_kernel(float* sink, int iters) {
    float a[kProbeChains];
#pragma unroll
    for (int j = 0; j < kProbeChains; ++j) a[j] = __int2float_rn(threadIdx.x + j);
    const float m = 0.999999f, c = 1e-7f;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 16; ++k) {
#pragma unroll
            for (int j = 0; j < kProbeChains; ++j) a[j] = __fmaf_rn(a[j], m, c);
        }
    }
    float s = 0.f;
#pragma unroll
    for (int j = 0; j < kProbeChains; ++j) s += a[j];
    if (s == -1.2345f) sink[blockIdx.x] = s;
}

cudaError_t launch_fp32_probe(float* sink, int grid, int block, int iters, cudaStream_t s) {
    fp32_probe_kernel<<<grid, block, 0, s>>>(sink, iters);
    return cudaGetLastError();
}

cudaError_t launch_render(const RenderParams& p, int grid, int block, size_t smem, cudaStream_t s) {
    render_kernel<<<grid, block, smem, s>>>(p);
    return cudaGetLastError();
}

cudaError_t render_occupancy(int block, size_t smem, int* blocks_per_sm) {
    cudaError_t e = cudaFuncSetAttribute(render_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)(smem < 48 * 1024 ? 48 * 1024 : smem));
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, render_kernel, block, smem);
}

cudaError_t launch_tonemap(const float4* accum, uint32_t npix, uint32_t sample_count, uchar4* out,
                           cudaStream_t s) {
    const uint32_t b = 256, g = (npix + b - 1) / b;
    tonemap_kernel<<<g, b, 0, s>>>(accum, npix, (float)sample_count, out);
    return cudaGetLastError();
}

cudaError_t launch_intersect_rays(const SceneView& sc, const float* o, const float* d, uint32_t n,
                                  float* t, int32_t* idx, float* nrm, uint8_t* front,
                                  cudaStream_t s) {
    const uint32_t b = 128, g = (n + b - 1) / b;
    intersect_rays_kernel<<<g, b, 0, s>>>(sc, o, d, n, t, idx, nrm, front);
    return cudaGetLastError();
}

cudaError_t launch_scatter_fixed(const SceneView& sc, const float* o, const float* d,
                                 const float* t, const int32_t* idx, const uint32_t* words,
                                 uint32_t n, float* o_out, float* d_out, cudaStream_t s) {
    const uint32_t b = 128, g = (n + b - 1) / b;
    scatter_fixed_kernel<<<g, b, 0, s>>>(sc, o, d, t, idx, words, n, o_out, d_out);
    return cudaGetLastError();
}

}  // namespace rdc
