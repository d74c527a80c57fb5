// rdc_static.cu -- rdc_render_static: the path-tracing render for callers
// that cannot allocate GPU memory.
//
// Some callers cannot call cudaMalloc: a host application whose device memory
// is owned by another allocator (a game engine or a Vulkan/OpenGL interop
// layer that hands out only its own buffers), a real-time loop that forbids
// allocation after start-up, or a plugin whose memory budget is fixed by its
// host.  They still own the output (the accumulator) and pass the scene; the
// renderer's own scratch -- the flattened scene copy and the counters the
// persistent kernel works from -- lives here, in one file-scope device array
// of fixed size, instead of in memory a context allocates.
//
// Set-up: the first call on a device (with that device current) resolves the
// array's device address with cudaGetSymbolAddress and caches it with the SM
// count; that first call should therefore come before any stream capture.
// The array is shared by every call on a device and keeps the last call's
// contents: each call rewrites the scene copy and clears the counters before
// launching, so calls that overlap on the GPU (two streams, or two threads)
// race on it and must be serialised by the caller.
#include <cstdio>
#include <cstring>
#include <mutex>

#include "raydar_cuda.h"
#include "rdc_flatten.hpp"
#include "rdc_internal.hpp"

namespace {

constexpr size_t kCounterBytes = 256;
// Intersection records per object, worst case: a run of L objects takes
// 3 * ceil(L / 2) float4 (spheres) or 1 + 3 * ceil(L / 2) (cubes, with the
// run header), at most 4 per object, reached by a one-cube run.  A scene of
// alternating spheres and cubes takes 3.5 per object.
constexpr size_t kRecPerObject = 4;
constexpr size_t kMaxRec = (size_t)RDC_STATIC_MAX_OBJECTS * kRecPerObject;
constexpr size_t kRecBytes = kMaxRec * 16;
constexpr bool run_records_fit(uint32_t max_len) {
    for (uint32_t len = 1; len <= max_len; ++len)
        if (1u + 3u * ((len + 1u) / 2u) > kRecPerObject * len) return false;
    return true;
}
static_assert(run_records_fit(RDC_STATIC_MAX_OBJECTS), "a run can take more records than the scratch allows");
constexpr size_t kHitBytes = (size_t)RDC_STATIC_MAX_OBJECTS * 16;
constexpr size_t kMatBytes = (size_t)RDC_STATIC_MAX_OBJECTS * sizeof(rdc::MatDev);
constexpr size_t kRunBytes = (size_t)RDC_STATIC_MAX_OBJECTS * 16;
constexpr size_t kRecOff = kCounterBytes;
constexpr size_t kHitOff = kRecOff + kRecBytes;
constexpr size_t kMatOff = kHitOff + kHitBytes;
constexpr size_t kRunOff = kMatOff + kMatBytes;
constexpr size_t kScratchBytes = kRunOff + kRunBytes;
static_assert(kScratchBytes == RDC_STATIC_SCRATCH_BYTES, "scratch layout and header disagree");
static_assert(kRecOff % 256 == 0 && kHitOff % 256 == 0 && kMatOff % 256 == 0 && kRunOff % 256 == 0,
              "scratch regions must stay 256-byte aligned");

// The scratch.  Its name in host code is only a stand-in for the symbol, not
// a device address: the address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_rdc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
unsigned char* g_scratch_ptr[kMaxDevices] = {};
int g_num_sms[kMaxDevices] = {};

void set_error(char* buf, size_t cap, const char* msg) {
    if (buf && cap > 0) std::snprintf(buf, cap, "%s", msg);
}

rdc_status cuda_error(char* buf, size_t cap, cudaError_t e, const char* what) {
    char m[256];
    std::snprintf(m, sizeof(m), "%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
    set_error(buf, cap, m);
    return RDC_ERR_CUDA;
}

// Per-device set-up on the calling thread's current device.
rdc_status setup(int device, unsigned char** scratch, int* sms, char* err, size_t cap) {
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_ptr[device]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_rdc_scratch);
        if (e != cudaSuccess) return cuda_error(err, cap, e, "cudaGetSymbolAddress(scratch)");
        int n = 0;
        e = cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, device);
        if (e != cudaSuccess) return cuda_error(err, cap, e, "cudaDeviceGetAttribute(SM count)");
        g_num_sms[device] = n;
        g_scratch_ptr[device] = static_cast<unsigned char*>(p);
    }
    *scratch = g_scratch_ptr[device];
    *sms = g_num_sms[device];
    return RDC_OK;
}

// Host staging for the flattened scene: static storage (no allocation),
// guarded by a mutex while a call flattens and copies it.
std::mutex g_stage_mutex;
float4 g_stage_rec[kMaxRec];
float4 g_stage_hit[RDC_STATIC_MAX_OBJECTS];
rdc::MatDev g_stage_mat[RDC_STATIC_MAX_OBJECTS];
int4 g_stage_runs[RDC_STATIC_MAX_OBJECTS];

}  // namespace

extern "C" rdc_status rdc_render_static(const rdc_scene_desc* sc, float* accum_device, uint32_t spp_begin,
                                        uint32_t spp_count, uint32_t max_bounces, uint64_t seed,
                                        void* stream, uint64_t* segments_out, char* error_out,
                                        size_t error_capacity) {
    set_error(error_out, error_capacity, "");
    if (!sc || !accum_device) {
        set_error(error_out, error_capacity, "rdc_render_static: scene or accumulator is NULL");
        return RDC_ERR_INVALID_ARGUMENT;
    }
    const rdc_camera& cam = sc->camera;
    if (cam.resolution_x == 0 || cam.resolution_y == 0) {
        set_error(error_out, error_capacity, "rdc_render_static: zero resolution");
        return RDC_ERR_INVALID_ARGUMENT;
    }
    if (cam.resolution_x > RDC_MAX_RESOLUTION || cam.resolution_y > RDC_MAX_RESOLUTION) {
        set_error(error_out, error_capacity, "rdc_render_static: resolution above RDC_MAX_RESOLUTION");
        return RDC_ERR_LIMIT;
    }
    if (sc->object_count > RDC_STATIC_MAX_OBJECTS) {
        char m[160];
        std::snprintf(m, sizeof(m),
                      "rdc_render_static: %u objects exceed RDC_STATIC_MAX_OBJECTS (%u) of the fixed scratch",
                      sc->object_count, RDC_STATIC_MAX_OBJECTS);
        set_error(error_out, error_capacity, m);
        return RDC_ERR_LIMIT;
    }
    if (sc->object_count > 0 && !sc->objects) {
        set_error(error_out, error_capacity, "rdc_render_static: objects is NULL");
        return RDC_ERR_INVALID_ARGUMENT;
    }
    if (sc->world.kind == RDC_WORLD_TRANSPARENT) {
        set_error(error_out, error_capacity,
                  "rdc_render_static: World::Transparent is not supported (todo!() in the reference)");
        return RDC_ERR_UNSUPPORTED;
    }
    if (sc->world.kind > RDC_WORLD_TRANSPARENT) {
        set_error(error_out, error_capacity, "rdc_render_static: unknown world kind");
        return RDC_ERR_INVALID_ARGUMENT;
    }
    if (max_bounces > RDC_MAX_BOUNCES) {
        set_error(error_out, error_capacity, "rdc_render_static: max_bounces above RDC_MAX_BOUNCES");
        return RDC_ERR_LIMIT;
    }
    if ((uint64_t)spp_begin + spp_count > 0xFFFFFFFFull) {
        set_error(error_out, error_capacity, "rdc_render_static: sample range overflows 32 bits");
        return RDC_ERR_INVALID_ARGUMENT;
    }
    for (uint32_t i = 0; i < sc->object_count; ++i) {
        if (sc->objects[i].geometry != RDC_GEOMETRY_SPHERE && sc->objects[i].geometry != RDC_GEOMETRY_CUBE) {
            set_error(error_out, error_capacity, "rdc_render_static: object with unknown geometry");
            return RDC_ERR_INVALID_ARGUMENT;
        }
    }

    int device = 0;
    cudaError_t e = cudaGetDevice(&device);
    if (e != cudaSuccess) return cuda_error(error_out, error_capacity, e, "cudaGetDevice");
    if (device < 0 || device >= kMaxDevices) {
        set_error(error_out, error_capacity, "rdc_render_static: device ordinal above 63");
        return RDC_ERR_LIMIT;
    }
    unsigned char* scratch = nullptr;
    int sms = 0;
    if (rdc_status st = setup(device, &scratch, &sms, error_out, error_capacity)) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);

    float4* d_rec = reinterpret_cast<float4*>(scratch + kRecOff);
    float4* d_hit = reinterpret_cast<float4*>(scratch + kHitOff);
    rdc::MatDev* d_mat = reinterpret_cast<rdc::MatDev*>(scratch + kMatOff);
    int4* d_runs = reinterpret_cast<int4*>(scratch + kRunOff);
    unsigned long long* d_counters = reinterpret_cast<unsigned long long*>(scratch);

    // Flatten into the static host staging area and copy it into the scratch
    // (pageable copies are staged before cudaMemcpyAsync returns).
    const uint32_t n = sc->object_count;
    const rdc::FlatCounts fc = rdc::flat_counts(sc);
    // Never above the regions by the worst case above; checked all the same,
    // before anything is written to the staging arrays or the scratch.
    if (fc.nrec > kMaxRec || fc.nruns > RDC_STATIC_MAX_OBJECTS) {
        set_error(error_out, error_capacity, "rdc_render_static: flattened scene exceeds the fixed scratch");
        return RDC_ERR_LIMIT;
    }
    bool fast_div = true;
    {
        std::lock_guard<std::mutex> lock(g_stage_mutex);
        fast_div = rdc::flatten(sc, g_stage_rec, g_stage_hit, g_stage_mat, g_stage_runs);
        if (fc.nrec) e = cudaMemcpyAsync(d_rec, g_stage_rec, fc.nrec * sizeof(float4), cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess && n) e = cudaMemcpyAsync(d_hit, g_stage_hit, n * sizeof(float4), cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess && n) e = cudaMemcpyAsync(d_mat, g_stage_mat, n * sizeof(rdc::MatDev), cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess && fc.nruns)
            e = cudaMemcpyAsync(d_runs, g_stage_runs, fc.nruns * sizeof(int4), cudaMemcpyHostToDevice, s);
    }
    if (e != cudaSuccess) return cuda_error(error_out, error_capacity, e, "cudaMemcpyAsync(scene)");
    // The work counter, the segment counter and the device-error count start at zero.
    e = cudaMemsetAsync(d_counters, 0, 5 * sizeof(unsigned long long), s);
    if (e != cudaSuccess) return cuda_error(error_out, error_capacity, e, "cudaMemsetAsync(counters)");

    if (spp_count > 0) {
        rdc::RenderParams p{};  // fields the brute-force kernel does not read stay zero
        rdc::SceneView& v = p.sc;
        v.rec = d_rec;
        v.nrec = fc.nrec;
        v.hit = d_hit;
        v.mat = d_mat;
        v.runs = d_runs;
        v.nobj = n;
        v.nruns = fc.nruns;
        v.fast_div = fast_div ? 1u : 0u;
        v.neg_zero = make_float2(-0.0f, -0.0f);
        v.oob = d_counters + 4;  // reported with the device-error count
        v.width = cam.resolution_x;
        v.height = cam.resolution_y;
        for (int i = 0; i < 3; ++i) v.cam_pos[i] = cam.position[i];
        for (int i = 0; i < 16; ++i) {
            v.inv_view[i] = cam.inverse_view_matrix[i];
            v.inv_proj[i] = cam.inverse_proj_matrix[i];
        }
        v.world_kind = sc->world.kind;
        for (int i = 0; i < 3; ++i) {
            v.top[i] = sc->world.top_color[i];
            v.bottom[i] = sc->world.bottom_color[i];
            v.solid[i] = sc->world.solid_color[i];
        }
        p.accum = reinterpret_cast<float4*>(accum_device);
        p.s0 = spp_begin;
        p.nspp = spp_count;
        p.max_bounces = max_bounces;
        p.stream_id = 0;
        p.key0 = (uint32_t)seed;
        p.key1 = (uint32_t)(seed >> 32);
        p.npix = cam.resolution_x * cam.resolution_y;
        p.work_counter = reinterpret_cast<uint32_t*>(d_counters);
        p.segments = d_counters + 1;
        p.errors = d_counters + 4;
        p.min_idle = 1;

        const size_t smem = rdc::render_smem_bytes(fc.nrec, fc.nruns);
        int per_sm = 0;
        e = rdc::render_occupancy(rdc::kRenderBlock, smem, &per_sm);
        if (e != cudaSuccess) return cuda_error(error_out, error_capacity, e, "render occupancy");
        if (per_sm < 1) {
            set_error(error_out, error_capacity, "rdc_render_static: scene does not fit in shared memory");
            return RDC_ERR_LIMIT;
        }
        const uint64_t warps = ((uint64_t)p.npix + 31) / 32;
        uint64_t grid = (uint64_t)sms * per_sm;
        const uint64_t grid_needed = (warps * 32 + rdc::kRenderBlock - 1) / rdc::kRenderBlock;
        if (grid > grid_needed) grid = grid_needed;
        e = rdc::launch_render(p, (int)grid, rdc::kRenderBlock, smem, s);
        if (e != cudaSuccess) return cuda_error(error_out, error_capacity, e, "render launch");
    }
    if (segments_out) {
        unsigned long long c[5] = {0, 0, 0, 0, 0};
        e = cudaMemcpyAsync(c, d_counters, sizeof(c), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return cuda_error(error_out, error_capacity, e, "segment read-back");
        *segments_out = c[1];
        if (c[4] != 0) {
            set_error(error_out, error_capacity,
                      "rdc_render_static: a block could not stage the scene into shared memory");
            return RDC_ERR_DEVICE;
        }
    }
    return RDC_OK;
}
