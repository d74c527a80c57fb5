// rdc_internal.hpp -- device data layout and launch parameters shared by the
// C-ABI layer (rdc_api.cpp) and the kernels (rdc_kernels.cu).
//
// Device layout of an uploaded scene (all in HBM; rec and runs are staged in
// shared memory per block):
//   rec[]    intersection records (rdc_flatten.hpp): spheres in packed pairs
//            (48 B per pair), cubes as (min, max) pairs per axis (32 B)
//   hit[i]   (cx, cy, cz, side/2): what closest_hit needs (16 B)
//   mat[i]   MatDev, 64 B: everything the scatter step reads for one object
//   runs[r]  (geometry, begin, end, first record): maximal runs of one
//            geometry kind in scene order, so the intersection loop visits
//            objects in scene order (the first-minimum tie rule) with a
//            warp-uniform branch per run instead of one per object.
// The per-object constants (c.c, r*r, min/max, roughness^2, 1/ior, Schlick
// r0, emission colour * strength) are the exact float values the reference
// computes inline, so hoisting them does not change a single bit.
#pragma once

#include <cmath>
#include <cstdint>
#include <string>

#include <cuda_runtime.h>

namespace rdc {

struct alignas(16) MatDev {
    float4 a;  // albedo.rgb, roughness^2
    float4 b;  // emission_color * emission_strength (rgb), metallic
    float4 c;  // transmission, ratio on a front-face hit (1/ior), ratio on a back-face hit (ior), r0 front
    float4 d;  // r0 back, geometry kind (int bits), 0, 0
};

struct SceneView {
    const float4* rec;  // intersection records (rdc_flatten.hpp), staged in shared memory
    uint32_t nrec;      // float4 records
    const float4* hit;
    const MatDev* mat;
    const int4* runs;
    uint32_t nobj;
    uint32_t nruns;
    uint32_t fast_div;  // every object passes cube_fast_div_ok / sphere_fast_ok (guarded fast path allowed)
    float2 neg_zero;    // (-0, -0): the addend of packed products (rdc_device.cuh, mul2)
    uint32_t width;
    uint32_t height;
    float cam_pos[3];
    uint32_t world_kind;
    float inv_view[16];
    float inv_proj[16];
    float top[3];
    float bottom[3];
    float solid[3];
    unsigned long long* oob;  // bounds-checked build: count of out-of-range indices caught
};

struct Bvh4Node;  // rdc_bvh.cuh

// Device LBVH of a scene (rdc_bvh.cu), collapsed to 4-wide nodes (root 0),
// and 2 records per object in scene order.
struct BvhView {
    const Bvh4Node* nodes;
    const float4* prims;
    uint32_t nobj;
    float scene_r;  // bound on |centre| + size over the objects
    float o_max;    // sphere leaf boxes are grown for ray origins with |o| <= o_max
    uint32_t nnodes;
    unsigned long long* oob;  // bounds-checked build: count of out-of-range indices caught
};

struct BvhDevice {
    Bvh4Node* nodes = nullptr;
    uint32_t nnodes = 0;  // 4-wide nodes
    float4* prims = nullptr;
    void* scratch = nullptr;
    size_t scratch_bytes = 0;
    uint32_t nobj = 0;
    float scene_r = 0.0f;
    float o_max = 0.0f;
    void release();
    BvhView view(unsigned long long* oob) const { return BvhView{nodes, prims, nobj, scene_r, o_max, nnodes, oob}; }
};

// Device sort and prefix sum (rdc_sort.cu).  radix_sort_pairs sorts the n
// pairs (keys, vals) by the low key_bits bits of the keys, stably, using
// (keys_alt, vals_alt) as the second buffer; the sorted arrays are whichever
// pair *keys_sorted / *vals_sorted name.  exclusive_scan: out[i] = in[0] +
// ... + in[i-1], n <= 2^24, out == in allowed.  Scratch of the stated sizes.
size_t radix_sort_scratch_bytes(uint32_t n);
cudaError_t radix_sort_pairs(uint32_t* keys, uint32_t* vals, uint32_t* keys_alt, uint32_t* vals_alt, uint32_t n,
                             int key_bits, void* scratch, cudaStream_t s, uint32_t** keys_sorted,
                             uint32_t** vals_sorted);
size_t exclusive_scan_scratch_bytes(uint32_t n);
cudaError_t exclusive_scan(const uint32_t* in, uint32_t* out, uint32_t n, void* scratch, cudaStream_t s);

// Build the LBVH of `sc` on stream `s` (synchronises it).  depth_out: the
// deepest leaf of the binary tree (at most 63; the 4-wide tree is at most
// 32 deep and its traversal stack holds 3 entries per level).
cudaError_t build_lbvh(const struct rdc_scene_desc* sc, BvhDevice& out, cudaStream_t s, uint32_t* depth_out);

struct RenderParams {
    SceneView sc;
    BvhView bvh;                      // used by render_bvh_kernel
    unsigned long long* bvh_counters; // [0] node visits, [1] primitive tests
    float4* accum;
    uint32_t s0;
    uint32_t nspp;
    uint32_t max_bounces;
    uint32_t stream_id;
    uint32_t key0;
    uint32_t key1;
    uint32_t npix;
    uint32_t* work_counter;
    unsigned long long* segments;
    uint32_t min_idle;                // render_bvh_kernel: lanes done before a warp shades
    unsigned long long* errors;       // device errors (shared-memory staging that did not complete)
};

// Path-replay adjoint (rdc_adjoint.cu).  grad holds 8 floats per object:
// dL/dalbedo (3), dL/demission (3), dL/d(roughness^2), unused.
constexpr uint32_t kAdjMaxBounces = 16;
struct AdjParams {
    SceneView sc;
    BvhView bvh;        // used when the scene has an LBVH
    const float* dl;    // dL/dimage, npix * 3 (RGB of the mean-radiance image)
    float* grad;        // nobj * 8, zeroed by the caller
    uint32_t s0, nspp, max_bounces, stream_id, key0, key1;
    uint64_t npaths;    // npix * nspp
    unsigned long long* segments;
    uint32_t smem_grad; // 1: per-block shared accumulators (8 * nobj floats)
    uint32_t shared_vert_stride;  // words between threads' vertex records in shared memory (shared records only)
    unsigned long long* errors;  // device errors (shared-memory staging that did not complete)
};
// Dynamic shared memory of the adjoint kernel: staged records (brute force),
// the gradient table (smem_grad) and, for shared_vert_bounces > 0, that many
// vertex records per thread of a block of `block` threads, each thread's
// adjoint_shared_vert_stride(bounces) words apart.
uint32_t adjoint_shared_vert_stride(uint32_t bounces);
size_t adjoint_smem_bytes(const SceneView& sc, bool bvh, bool smem_grad, uint32_t shared_vert_bounces, int block);
cudaError_t adjoint_occupancy(bool bvh, bool shared_vert, int block, size_t smem, int* blocks_per_sm);
cudaError_t launch_adjoint(const AdjParams& p, bool bvh, bool shared_vert, int grid, int block, size_t smem,
                           cudaStream_t s);

// The message rdc_last_error(NULL) returns on this thread (calls without a
// context: rdc_create, the .rscn reader/writer).
void set_thread_error(const std::string& msg);

// Every device allocation of the library (rdc_render_static makes none) goes
// through dev_malloc.  Fault injection for tests, on the host: when
// RDC_FAIL_ALLOC_AFTER=n is set in the environment at rdc_create, the
// allocations after the next n fail with cudaErrorMemoryAllocation without
// calling cudaMalloc (until the next rdc_create reads the variable again), so
// every caller's out-of-memory path runs on a healthy GPU.
cudaError_t dev_malloc(void** ptr, size_t bytes);
void reset_alloc_injection();

// Wavefront render (rdc_wavefront.cu): the path records and queues of one
// wave in one buffer of wavefront_state_bytes(npath).
// One path's state in the wavefront form, 64 B: the queue kernels take paths
// in queue order, not path order, so a record per path makes each access one
// or two whole sectors (as planes, each 4-byte field would pull a sector of
// its own).
struct alignas(16) WfPath {
    float4 ot;  // the next ray's origin; w: its closest-hit distance
    float4 dh;  // its direction; w: the hit object's index (int bits, -1 for none)
    float4 atten;  // throughput (w unused)
    float4 light;  // radiance gathered so far (w unused)
};
static_assert(sizeof(WfPath) == 64, "wavefront path record");

struct WfParams {
    SceneView sc;
    float4* accum;
    uint32_t npix, max_bounces, stream_id, key0, key1;
    uint32_t npath;     // paths a wave holds: npix x the wave's sample capacity W
    uint32_t* sample;   // the wave's first sample index (device), advanced per wave
    uint32_t* wave_n;   // samples in the current wave (device), W or the remainder in the last
    WfPath* path;               // npath records, one per path of the wave
    uint32_t *queue0, *queue1;  // ray queues of path entries, alternating per bounce
    uint32_t* cls;              // 4 class queues of npath entries: mix, metal, glass, miss
    uint32_t* counts;           // [0], [1] ray queue lengths, [2..5] class queue lengths, [6] the
                                // wave's first sample index, [7] the LBVH intersect kernel's fetch
                                // counter, [8] the wave's sample count
    unsigned long long* segments;
    unsigned long long* errors;  // device errors (shared-memory staging that did not complete)
    uint32_t use_bvh;            // 1: the LBVH intersect kernel over bvh, 0: brute force
    BvhView bvh;
    unsigned long long* bvh_counters;  // node visits, object tests (LBVH)
    uint32_t min_idle;           // LBVH intersect: idle lanes of a warp before it refills
};
constexpr int kWfBvhBlock = 128;      // wf_intersect_bvh: threads per block
constexpr int kWfBvhMinBlocks = 6;    // and the resident blocks its registers are sized for (80; 8 blocks at
                                      // 64 registers measured 5% slower)
constexpr uint32_t kWfPixBits = 28;          // a queue entry: the path's place in its wave << 28 | its pixel
constexpr uint32_t kWfMaxWaveSpp = 16;        // so a wave holds at most 16 samples of a pixel
// and at most this many paths (88 B of state and queue entries each: 2.9 GB).
// Measured at 1080p with 2, 4, 8 and 16 samples per wave: brute force 34.1 /
// 30.7 / 29.4 / 29.0 ms per 64-spp frame (fewer launches over thin
// deep-bounce queues), the LBVH 58.6 / 55.3 / 54.9 / 54.8 ms per 16-spp frame
// (1 sample: 68.3 ms).
constexpr uint32_t kWfWavePaths = 1u << 25;
size_t wavefront_state_bytes(uint32_t npath);
uint32_t wavefront_wave_spp(uint32_t npix, uint32_t spp);  // the wave's sample capacity W
size_t wavefront_bvh_smem_bytes();
cudaError_t wavefront_occupancy(bool bvh, int block, size_t smem, int* intersect_per_sm, int* shade_per_sm);
cudaError_t wavefront_set_word(uint32_t* word, uint32_t v, cudaStream_t s);
cudaError_t enqueue_wave(const WfParams& p, int grid_i, int grid_s, size_t smem, cudaStream_t s);

// One scene of a batch (rdc_batch_upload): its view, accumulator, sample
// count, bounce limit, RNG key and share of the batch's estimated work.
struct BatchScene {
    SceneView sc;
    float4* accum;
    uint32_t npix;
    uint32_t spp;
    uint32_t max_bounces;
    uint32_t key0;
    uint32_t key1;
    float work_begin;  // cumulative estimated work before this scene, in [0, 1)
    float pixel_work;  // estimated work of one pixel (relative)
};

struct BatchParams {
    const BatchScene* scenes;
    uint32_t nscenes;
    uint32_t refill_min;      // idle lanes of a warp that trigger a refill (regroup period)
    uint32_t* pixel_counters; // per scene: next pixel to hand out
    unsigned long long* segments;
    unsigned long long* errors;  // device errors (shared-memory staging that did not complete)
};

// Kernel launchers (rdc_kernels.cu).  Each returns the cudaError_t of its
// launch.
cudaError_t launch_render(const RenderParams& p, int grid, int block, size_t smem, cudaStream_t s);
cudaError_t launch_render_bvh(const RenderParams& p, int grid, int block, cudaStream_t s);
cudaError_t render_bvh_occupancy(int block, int* blocks_per_sm);
cudaError_t render_occupancy(int block, size_t smem, int* blocks_per_sm);
cudaError_t launch_batch(const BatchParams& p, int grid, int block, size_t smem, cudaStream_t s);
cudaError_t batch_occupancy(int block, size_t smem, int* blocks_per_sm);
cudaError_t launch_tonemap(const float4* accum, uint32_t npix, uint32_t sample_count, uchar4* out,
                           cudaStream_t s);
// bvh.nodes == nullptr: brute force over sc.rec; otherwise through the BVH.
cudaError_t launch_intersect_rays(const SceneView& sc, const BvhView& bvh, const float* o, const float* d,
                                  uint32_t n, float* t, int32_t* idx, float* nrm, uint8_t* front,
                                  cudaStream_t s);
cudaError_t launch_scatter_fixed(const SceneView& sc, const float* o, const float* d,
                                 const float* t, const int32_t* idx, const uint32_t* words,
                                 uint32_t n, float* o_out, float* d_out, cudaStream_t s);

cudaError_t launch_fp32_probe(float* sink, int grid, int block, int iters, bool packed, cudaStream_t s);
cudaError_t launch_staging_timeout(unsigned long long* errors, cudaStream_t s);

// A cube whose slab bounds keep the kernels' exact reciprocal division in
// range (rdc_device.cuh): positive finite side, every bound 0 or with
// magnitude in [2^-60, 2^60].
inline bool slab_bound_ok(float b) {
    const float m = std::fabs(b);
    return b == 0.0f || (m >= 0x1p-60f && m <= 0x1p60f);
}
inline bool cube_fast_div_ok(float side, const float4& g0, const float4& g1) {
    return side > 0.0f && std::isfinite(side) && slab_bound_ok(g0.x) && slab_bound_ok(g0.y) &&
           slab_bound_ok(g0.z) && slab_bound_ok(g0.w) && slab_bound_ok(g1.x) && slab_bound_ok(g1.y);
}

// A sphere whose centre and radius keep the candidate pass finite
// (rdc_device.cuh): finite, magnitudes at most 2^50.
inline bool sphere_fast_ok(const float c[3], float radius) {
    return std::fabs(c[0]) <= 0x1p50f && std::fabs(c[1]) <= 0x1p50f && std::fabs(c[2]) <= 0x1p50f &&
           std::fabs(radius) <= 0x1p50f;
}

constexpr int kRenderBlock = 256;
constexpr int kRenderBlocksPerSm = 3;  // render_kernel's launch bound (80 registers)
constexpr int kRenderBvhBlock = 128;  // largest block of render_bvh_kernel
constexpr int kProbeChains = 8;  // independent FFMA chains per thread in the FP32 probe

inline size_t render_smem_bytes(uint32_t nrec, uint32_t nruns) {
    return (size_t)nrec * 16u + (size_t)nruns * 16u;
}

}  // namespace rdc
