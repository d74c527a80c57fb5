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
#include "rdc_internal.hpp"

namespace {

constexpr size_t kCounterBytes = 256;
constexpr size_t kGeomBytes = (size_t)RDC_STATIC_MAX_OBJECTS * 32;
constexpr size_t kHitBytes = (size_t)RDC_STATIC_MAX_OBJECTS * 16;
constexpr size_t kMatBytes = (size_t)RDC_STATIC_MAX_OBJECTS * sizeof(rdc::MatDev);
constexpr size_t kRunBytes = (size_t)RDC_STATIC_MAX_OBJECTS * 16;
constexpr size_t kGeomOff = kCounterBytes;
constexpr size_t kHitOff = kGeomOff + kGeomBytes;
constexpr size_t kMatOff = kHitOff + kHitBytes;
constexpr size_t kRunOff = kMatOff + kMatBytes;
constexpr size_t kScratchBytes = kRunOff + kRunBytes;
static_assert(kScratchBytes == RDC_STATIC_SCRATCH_BYTES, "scratch layout and header disagree");
static_assert(kGeomOff % 256 == 0 && kHitOff % 256 == 0 && kMatOff % 256 == 0 && kRunOff % 256 == 0,
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

// Per-object constants, the same floats rdc_scene_upload computes.
void flatten_object(const rdc_object& o, float4* geom2, float4* hit, rdc::MatDev* mat) {
    const float cx = o.center[0], cy = o.center[1], cz = o.center[2];
    if (o.geometry == RDC_GEOMETRY_SPHERE) {
        geom2[0] = make_float4(cx, cy, cz, (cx * cx + cy * cy) + cz * cz);
        geom2[1] = make_float4(o.radius * o.radius, 0, 0, 0);
        *hit = make_float4(cx, cy, cz, 0.0f);
    } else {
        const float h = o.side_length * 0.5f;
        geom2[0] = make_float4(cx - h, cy - h, cz - h, cx + h);
        geom2[1] = make_float4(cy + h, cz + h, 0, 0);
        *hit = make_float4(cx, cy, cz, o.side_length / 2.0f);
    }
    const rdc_material& m = o.material;
    mat->a = make_float4(m.albedo[0], m.albedo[1], m.albedo[2], m.roughness * m.roughness);
    mat->b = make_float4(m.emission_color[0] * m.emission_strength, m.emission_color[1] * m.emission_strength,
                         m.emission_color[2] * m.emission_strength, m.metallic);
    const float ratio_front = 1.0f / m.ior;
    const float qf = (ratio_front - 1.0f) / (ratio_front + 1.0f);
    const float qb = (m.ior - 1.0f) / (m.ior + 1.0f);
    mat->c = make_float4(m.transmission, ratio_front, m.ior, qf * qf);
    int kind = (int)o.geometry;
    float kind_bits;
    std::memcpy(&kind_bits, &kind, 4);
    mat->d = make_float4(qb * qb, kind_bits, 0, 0);
}

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

    float4* d_geom = reinterpret_cast<float4*>(scratch + kGeomOff);
    float4* d_hit = reinterpret_cast<float4*>(scratch + kHitOff);
    rdc::MatDev* d_mat = reinterpret_cast<rdc::MatDev*>(scratch + kMatOff);
    int4* d_runs = reinterpret_cast<int4*>(scratch + kRunOff);
    unsigned long long* d_counters = reinterpret_cast<unsigned long long*>(scratch);

    // Flatten the scene in fixed chunks on the stack and copy each chunk into
    // the scratch (pageable copies are staged before cudaMemcpyAsync returns).
    constexpr uint32_t kChunk = 32;
    float4 cg[2 * kChunk];
    float4 ch[kChunk];
    rdc::MatDev cm[kChunk];
    int4 cr[kChunk];
    uint32_t nruns = 0, runs_flushed = 0, run_fill = 0;
    int4 cur = make_int4(-1, 0, 0, 0);
    const uint32_t n = sc->object_count;
    for (uint32_t base = 0; base < n; base += kChunk) {
        const uint32_t cnt = n - base < kChunk ? n - base : kChunk;
        for (uint32_t j = 0; j < cnt; ++j) {
            const rdc_object& o = sc->objects[base + j];
            flatten_object(o, &cg[2 * j], &ch[j], &cm[j]);
            const int kind = (int)o.geometry;
            if (cur.x == kind) {
                cur.z = (int)(base + j) + 1;
            } else {
                if (cur.x >= 0) {
                    cr[run_fill++] = cur;
                    ++nruns;
                    if (run_fill == kChunk) {
                        e = cudaMemcpyAsync(d_runs + runs_flushed, cr, kChunk * sizeof(int4), cudaMemcpyHostToDevice, s);
                        if (e != cudaSuccess) return cuda_error(error_out, error_capacity, e, "cudaMemcpyAsync(runs)");
                        runs_flushed += kChunk;
                        run_fill = 0;
                    }
                }
                cur = make_int4(kind, (int)(base + j), (int)(base + j) + 1, 0);
            }
        }
        e = cudaMemcpyAsync(d_geom + 2 * base, cg, 2 * cnt * sizeof(float4), cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(d_hit + base, ch, cnt * sizeof(float4), cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(d_mat + base, cm, cnt * sizeof(rdc::MatDev), cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) return cuda_error(error_out, error_capacity, e, "cudaMemcpyAsync(scene)");
    }
    if (cur.x >= 0) {
        cr[run_fill++] = cur;
        ++nruns;
    }
    if (run_fill > 0) {
        e = cudaMemcpyAsync(d_runs + runs_flushed, cr, run_fill * sizeof(int4), cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) return cuda_error(error_out, error_capacity, e, "cudaMemcpyAsync(runs)");
    }
    // The work counter and the segment counter must start at zero.
    e = cudaMemsetAsync(d_counters, 0, 2 * sizeof(unsigned long long), s);
    if (e != cudaSuccess) return cuda_error(error_out, error_capacity, e, "cudaMemsetAsync(counters)");

    if (spp_count > 0) {
        rdc::RenderParams p;
        rdc::SceneView& v = p.sc;
        v.geom = d_geom;
        v.hit = d_hit;
        v.mat = d_mat;
        v.runs = d_runs;
        v.nobj = n;
        v.nruns = nruns;
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

        const size_t smem = rdc::render_smem_bytes(n, nruns);
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
        unsigned long long segs = 0;
        e = cudaMemcpyAsync(&segs, d_counters + 1, sizeof(segs), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return cuda_error(error_out, error_capacity, e, "segment read-back");
        *segments_out = segs;
    }
    return RDC_OK;
}
