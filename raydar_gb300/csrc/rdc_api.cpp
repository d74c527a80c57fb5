// rdc_api.cpp -- the C ABI of include/raydar_cuda.h: context lifetime, scene
// validation and flattening, launches, read-back and statistics.
//
// Host code only, compiled with -ffp-contract=off: the per-object constants
// computed here (c.c, r*r, slab bounds, roughness^2, 1/ior, Schlick r0,
// emission colour * strength) must be the same floats the reference
// computes inline in src/renderer/cpu.rs.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "raydar_cuda.h"
#include "rdc_flatten.hpp"
#include "rdc_internal.hpp"

using rdc::MatDev;

// Shared memory a block may use for the staged scene (records + runs).
constexpr size_t kMaxSceneSmem = 200 * 1024;
// Dynamic shared memory a block may use at all (227 KB on sm_103a).
constexpr size_t kMaxDynSmem = 227 * 1024;
#ifndef RDC_ADJ_SHARED_VERT_MIN_BLOCKS
#define RDC_ADJ_SHARED_VERT_MIN_BLOCKS 3
#endif
// The adjoint keeps its vertex records in shared memory only while this many
// 256-thread blocks still fit on an SM.
constexpr int kAdjSharedVertMinBlocks = RDC_ADJ_SHARED_VERT_MIN_BLOCKS;
constexpr size_t kCounters = 8;       // device counters per context
constexpr size_t kErrorCounter = 4;   // index of the device-error count
constexpr size_t kBoundsCounter = 5;  // out-of-range indices caught (bounds-checked build)

struct rdc_ctx {
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::string err;

    // scene
    bool has_scene = false;
    rdc::SceneView view{};
    float4* d_rec = nullptr;
    float4* d_hit = nullptr;
    MatDev* d_mat = nullptr;
    int4* d_runs = nullptr;
    size_t cap_obj = 0, cap_runs = 0, cap_rec = 0;

    // frame
    float4* d_accum = nullptr;
    uint32_t width = 0, height = 0;
    uint32_t sample_count = 0;
    uchar4* d_rgba = nullptr;
    size_t cap_rgba = 0;

    // counters: [0] work counter (u32 in the low word), [1] segments, [2] node
    // visits, [3] object tests (cleared per launch), [4] device errors (sticky
    // until reported)
    unsigned long long* d_counters = nullptr;

    // last render
    uint64_t last_paths = 0;
    bool last_timed = false;
    uint32_t last_launches = 0;
    rdc_launch_config render_cfg{(uint32_t)rdc::kRenderBlock, 0, 16};
    uint32_t render_form = RDC_FORM_AUTO;
    uint64_t h2d_bytes = 0, d2h_bytes = 0;

    // closest-hit acceleration
    uint32_t accel_mode = RDC_ACCEL_AUTO;
    bool bvh_active = false;
    uint32_t bvh_depth = 0;
    rdc::BvhDevice bvh;
    bool brute_fits = false;  // records + runs fit the shared-memory budget
    std::vector<rdc_object> host_objects;  // copy of the uploaded scene (LBVH rebuilds)
    rdc_scene_desc host_desc{};

    // wavefront render (rdc_render_wavefront)
    char* d_wf = nullptr;
    size_t cap_wf = 0;
    uint32_t* d_wf_counts = nullptr;  // queue lengths, the wave's first sample and sample count
    cudaGraphExec_t wf_exec = nullptr;

    // differentiation (rdc_forward / rdc_backward)
    bool adj_valid = false;
    uint32_t adj_s0 = 0, adj_n = 0, adj_bounces = 0;
    uint64_t adj_seed = 0;
    float* d_grad = nullptr;
    float* d_dl = nullptr;
    size_t cap_grad = 0, cap_dl = 0;

    // batch (rdc_batch_upload)
    struct Batch {
        uint32_t n = 0;
        rdc::BatchScene* d_scenes = nullptr;
        float4* d_rec = nullptr;
        float4* d_hit = nullptr;
        MatDev* d_mat = nullptr;
        int4* d_runs = nullptr;
        float4* d_accum = nullptr;
        uint32_t* d_pixel_counters = nullptr;
        std::vector<size_t> accum_off;  // in float4
        std::vector<uint32_t> width, height;
        size_t accum_total = 0;         // float4
        size_t smem = 0;                // dynamic shared memory: the largest scene's records + runs
        uint64_t paths = 0;
        rdc_launch_config cfg{256, 0, 1};
        cudaGraph_t graph = nullptr;
        cudaGraphExec_t exec = nullptr;
    } batch;
};

namespace {

thread_local std::string g_create_error;  // failures without a context: rdc_last_error(NULL)

rdc_status fail(rdc_ctx* ctx, rdc_status st, const std::string& msg) {
    if (ctx) ctx->err = msg;
    return st;
}

rdc_status cuda_fail(rdc_ctx* ctx, cudaError_t e, const char* what) {
    std::string m = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
    if (e == cudaErrorMemoryAllocation) return fail(ctx, RDC_ERR_OUT_OF_MEMORY, m);
    return fail(ctx, RDC_ERR_CUDA, m);
}

#define RDC_CUDA(ctx, call)                                   \
    do {                                                      \
        cudaError_t e_ = (call);                              \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call); \
    } while (0)

template <typename T>
rdc_status ensure(rdc_ctx* ctx, T** ptr, size_t* cap, size_t n, const char* what) {
    if (n == 0) n = 1;
    if (*ptr && *cap >= n) return RDC_OK;
    if (*ptr) cudaFree(*ptr);
    *ptr = nullptr;
    *cap = 0;
    cudaError_t e = rdc::dev_malloc((void**)ptr, n * sizeof(T));
    if (e != cudaSuccess) return cuda_fail(ctx, e, what);
    *cap = n;
    return RDC_OK;
}

rdc_status set_device(rdc_ctx* ctx) {
    RDC_CUDA(ctx, cudaSetDevice(ctx->device));
    return RDC_OK;
}

// Kernels count blocks that could not stage the scene into shared memory
// (a bulk copy whose completion they stopped waiting for, rdc_device.cuh);
// after a synchronisation the count is reported once as RDC_ERR_DEVICE.
rdc_status check_device_errors(rdc_ctx* ctx) {
    static_assert(kBoundsCounter == kErrorCounter + 1, "the two device-error counters are adjacent");
    unsigned long long n[2] = {0, 0};
    RDC_CUDA(ctx, cudaMemcpy(n, ctx->d_counters + kErrorCounter, sizeof(n), cudaMemcpyDeviceToHost));
    if (n[0] == 0 && n[1] == 0) return RDC_OK;
    RDC_CUDA(ctx, cudaMemset(ctx->d_counters + kErrorCounter, 0, sizeof(n)));
    if (n[1] != 0)
        return fail(ctx, RDC_ERR_DEVICE,
                    std::to_string(n[1]) + " out-of-range device index(es) caught by the bounds-checked build");
    return fail(ctx, RDC_ERR_DEVICE,
                std::to_string(n[0]) + " block(s) could not stage the scene into shared memory (bulk copy did not "
                                       "complete); their pixels were not rendered");
}

// Checks shared by every scene entry point.  The reference accepts any
// numbers (a NaN sphere is simply never hit); what it cannot render -- the
// Transparent world, a todo!() panic -- is reported instead of panicking.
rdc_status check_scene(rdc_ctx* ctx, const rdc_scene_desc* sc, const std::string& who) {
    if (!sc) return fail(ctx, RDC_ERR_INVALID_ARGUMENT, who + ": scene is NULL");
    const rdc_camera& cam = sc->camera;
    if (cam.resolution_x == 0 || cam.resolution_y == 0)
        return fail(ctx, RDC_ERR_INVALID_ARGUMENT, who + ": zero resolution");
    if (cam.resolution_x > RDC_MAX_RESOLUTION || cam.resolution_y > RDC_MAX_RESOLUTION)
        return fail(ctx, RDC_ERR_LIMIT, who + ": resolution above RDC_MAX_RESOLUTION");
    if (sc->object_count > RDC_MAX_OBJECTS)
        return fail(ctx, RDC_ERR_LIMIT,
                    who + ": object_count " + std::to_string(sc->object_count) + " above RDC_MAX_OBJECTS");
    if (sc->object_count > 0 && !sc->objects) return fail(ctx, RDC_ERR_INVALID_ARGUMENT, who + ": objects is NULL");
    if (sc->world.kind == RDC_WORLD_TRANSPARENT)
        return fail(ctx, RDC_ERR_UNSUPPORTED,
                    who + ": World::Transparent is not supported (todo!() in the reference)");
    if (sc->world.kind > RDC_WORLD_TRANSPARENT) return fail(ctx, RDC_ERR_INVALID_ARGUMENT, who + ": unknown world kind");
    for (uint32_t i = 0; i < sc->object_count; ++i)
        if (sc->objects[i].geometry != RDC_GEOMETRY_SPHERE && sc->objects[i].geometry != RDC_GEOMETRY_CUBE)
            return fail(ctx, RDC_ERR_INVALID_ARGUMENT, who + ": object " + std::to_string(i) + " has unknown geometry");
    return RDC_OK;
}

void fill_view(rdc::SceneView& v, const rdc_scene_desc* sc, const float4* rec, uint32_t nrec, const float4* hit,
               const MatDev* mat, const int4* runs, uint32_t nruns, bool fast_div, unsigned long long* oob) {
    const rdc_camera& cam = sc->camera;
    v.oob = oob;
    v.rec = rec;
    v.nrec = nrec;
    v.hit = hit;
    v.mat = mat;
    v.runs = runs;
    v.nobj = sc->object_count;
    v.nruns = nruns;
    v.fast_div = fast_div ? 1u : 0u;
    v.neg_zero = make_float2(-0.0f, -0.0f);
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
}

void free_batch(rdc_ctx* ctx);
rdc_status capture_batch_graph(rdc_ctx* ctx);

// Pick brute force or the LBVH for the stored scene and build / drop the LBVH.
rdc_status apply_accel(rdc_ctx* ctx, bool scene_changed) {
    const uint32_t n = ctx->host_desc.object_count;
    bool want_bvh;
    if (ctx->accel_mode == RDC_ACCEL_BRUTE_FORCE) {
        want_bvh = false;  // rdc_render refuses it if the records do not fit shared memory
    } else if (ctx->accel_mode == RDC_ACCEL_LBVH) {
        want_bvh = true;
    } else {
        want_bvh = n > RDC_ACCEL_AUTO_LBVH_ABOVE || !ctx->brute_fits;
    }
    if (!want_bvh) {
        ctx->bvh.release();
        ctx->bvh_active = false;
        ctx->bvh_depth = 0;
        return RDC_OK;
    }
    if (ctx->bvh_active && !scene_changed) return RDC_OK;  // already built for this scene
    uint32_t depth = 0;
    const cudaError_t e = rdc::build_lbvh(&ctx->host_desc, ctx->bvh, ctx->stream, &depth);
    if (e != cudaSuccess) {
        ctx->bvh.release();
        ctx->bvh_active = false;
        return cuda_fail(ctx, e, "LBVH build");
    }
    if (depth > 64) {
        ctx->bvh.release();
        ctx->bvh_active = false;
        return fail(ctx, RDC_ERR_LIMIT, "LBVH deeper than the traversal stack allows (3 entries per 4-wide level)");
    }
    ctx->bvh_active = n > 0;
    ctx->bvh_depth = depth;
    ctx->h2d_bytes += (uint64_t)n * 64;
    return RDC_OK;
}

}  // namespace

namespace rdc {
void set_thread_error(const std::string& msg) { g_create_error = msg; }

namespace {
std::mutex g_alloc_mutex;
bool g_alloc_inject = false;      // RDC_FAIL_ALLOC_AFTER was set at the last rdc_create
unsigned long long g_alloc_left = 0;  // allocations that still succeed
}  // namespace

void reset_alloc_injection() {
    std::lock_guard<std::mutex> lock(g_alloc_mutex);
    const char* v = std::getenv("RDC_FAIL_ALLOC_AFTER");
    g_alloc_inject = v != nullptr && *v != '\0';
    g_alloc_left = g_alloc_inject ? std::strtoull(v, nullptr, 10) : 0;
}

cudaError_t dev_malloc(void** ptr, size_t bytes) {
    {
        std::lock_guard<std::mutex> lock(g_alloc_mutex);
        if (g_alloc_inject) {
            if (g_alloc_left == 0) {
                *ptr = nullptr;
                return cudaErrorMemoryAllocation;
            }
            --g_alloc_left;
        }
    }
    return cudaMalloc(ptr, bytes);
}
}  // namespace rdc

extern "C" {

const char* rdc_version(void) { return "raydar_cuda 0.1.0 (sm_103a)"; }

rdc_status rdc_create(rdc_ctx** out, int device) {
    g_create_error.clear();
    if (!out) {
        g_create_error = "rdc_create: out is NULL";
        return RDC_ERR_INVALID_ARGUMENT;
    }
    *out = nullptr;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || device < 0 || device >= n) {
        g_create_error = std::string("rdc_create: no CUDA device ") + std::to_string(device) +
                         (e != cudaSuccess ? std::string(" (") + cudaGetErrorString(e) + ")" : "");
        return e != cudaSuccess ? RDC_ERR_CUDA : RDC_ERR_INVALID_ARGUMENT;
    }
    cudaDeviceProp prop;
    e = cudaGetDeviceProperties(&prop, device);
    if (e != cudaSuccess) {
        g_create_error = std::string("cudaGetDeviceProperties: ") + cudaGetErrorString(e);
        return RDC_ERR_CUDA;
    }
    if (prop.major * 10 + prop.minor < 100) {
        g_create_error = std::string("rdc_create: device ") + prop.name +
                         " is not a Blackwell (sm_10x) GPU; this library is built for sm_103a only";
        return RDC_ERR_UNSUPPORTED;
    }
    rdc::reset_alloc_injection();
    rdc_ctx* ctx = new rdc_ctx();
    ctx->device = device;
    ctx->num_sms = prop.multiProcessorCount;
    auto bail = [&](cudaError_t err, const char* what) {
        g_create_error = std::string(what) + ": " + cudaGetErrorString(err);
        rdc_destroy(ctx);
        return err == cudaErrorMemoryAllocation ? RDC_ERR_OUT_OF_MEMORY : RDC_ERR_CUDA;
    };
    if ((e = cudaSetDevice(device)) != cudaSuccess) return bail(e, "cudaSetDevice");
    if ((e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking)) != cudaSuccess)
        return bail(e, "cudaStreamCreate");
    if ((e = cudaEventCreate(&ctx->ev0)) != cudaSuccess) return bail(e, "cudaEventCreate");
    if ((e = cudaEventCreate(&ctx->ev1)) != cudaSuccess) return bail(e, "cudaEventCreate");
    if ((e = rdc::dev_malloc((void**)&ctx->d_counters, kCounters * sizeof(unsigned long long))) != cudaSuccess)
        return bail(e, "cudaMalloc(counters)");
    if ((e = cudaMemset(ctx->d_counters, 0, kCounters * sizeof(unsigned long long))) != cudaSuccess)
        return bail(e, "cudaMemset(counters)");
    *out = ctx;
    return RDC_OK;
}

void rdc_destroy(rdc_ctx* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    free_batch(ctx);
    ctx->bvh.release();
    cudaFree(ctx->d_rec);
    cudaFree(ctx->d_hit);
    cudaFree(ctx->d_mat);
    cudaFree(ctx->d_runs);
    cudaFree(ctx->d_accum);
    cudaFree(ctx->d_rgba);
    cudaFree(ctx->d_counters);
    cudaFree(ctx->d_grad);
    cudaFree(ctx->d_dl);
    if (ctx->wf_exec) cudaGraphExecDestroy(ctx->wf_exec);
    cudaFree(ctx->d_wf);
    cudaFree(ctx->d_wf_counts);
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

const char* rdc_last_error(const rdc_ctx* ctx) {
    if (!ctx) return g_create_error.c_str();
    return ctx->err.c_str();
}

rdc_status rdc_get_stream(rdc_ctx* ctx, void** stream_out) {
    if (!ctx || !stream_out) return fail(ctx, RDC_ERR_INVALID_ARGUMENT, "rdc_get_stream: NULL argument");
    *stream_out = (void*)ctx->stream;
    return RDC_OK;
}

rdc_status rdc_synchronize(rdc_ctx* ctx) {
    if (!ctx) return RDC_ERR_INVALID_ARGUMENT;
    if (rdc_status st = set_device(ctx)) return st;
    RDC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return check_device_errors(ctx);
}

rdc_status rdc_scene_upload(rdc_ctx* ctx, const rdc_scene_desc* sc) {
    if (!ctx) return RDC_ERR_INVALID_ARGUMENT;
    if (!sc) return fail(ctx, RDC_ERR_INVALID_ARGUMENT, "rdc_scene_upload: scene is NULL");
    if (rdc_status st = check_scene(ctx, sc, "rdc_scene_upload")) return st;
    const rdc_camera& cam = sc->camera;
    const uint32_t n = sc->object_count;
    const rdc::FlatCounts fc = rdc::flat_counts(sc);
    const bool brute_fits = n <= RDC_MAX_BRUTE_OBJECTS && rdc::render_smem_bytes(fc.nrec, fc.nruns) <= kMaxSceneSmem;
    std::vector<float4> rec(fc.nrec ? fc.nrec : 1, make_float4(0, 0, 0, 0));
    std::vector<float4> hit(n ? n : 1, make_float4(0, 0, 0, 0));
    std::vector<MatDev> mat(n ? n : 1);
    std::vector<int4> runs(fc.nruns ? fc.nruns : 1, make_int4(0, 0, 0, 0));
    const bool fast_div = rdc::flatten(sc, rec.data(), hit.data(), mat.data(), runs.data());

    if (rdc_status st = set_device(ctx)) return st;
    // From here on the old scene's buffers may be freed or replaced: a failure
    // below must leave the context with no scene, never with stale pointers.
    ctx->has_scene = false;
    ctx->adj_valid = false;
    if (rdc_status st = ensure(ctx, &ctx->d_rec, &ctx->cap_rec, rec.size(), "cudaMalloc(records)")) return st;
    size_t cap = ctx->cap_obj;
    if (rdc_status st = ensure(ctx, &ctx->d_hit, &cap, hit.size(), "cudaMalloc(hit)")) return st;
    cap = ctx->cap_obj;
    if (rdc_status st = ensure(ctx, &ctx->d_mat, &cap, mat.size(), "cudaMalloc(materials)")) return st;
    ctx->cap_obj = cap;
    if (rdc_status st = ensure(ctx, &ctx->d_runs, &ctx->cap_runs, runs.size(), "cudaMalloc(runs)")) return st;
    // The previous frame may still read the old scene: order the copies.
    RDC_CUDA(ctx, cudaMemcpyAsync(ctx->d_rec, rec.data(), rec.size() * sizeof(float4),
                                  cudaMemcpyHostToDevice, ctx->stream));
    RDC_CUDA(ctx, cudaMemcpyAsync(ctx->d_hit, hit.data(), hit.size() * sizeof(float4),
                                  cudaMemcpyHostToDevice, ctx->stream));
    RDC_CUDA(ctx, cudaMemcpyAsync(ctx->d_mat, mat.data(), mat.size() * sizeof(MatDev),
                                  cudaMemcpyHostToDevice, ctx->stream));
    RDC_CUDA(ctx, cudaMemcpyAsync(ctx->d_runs, runs.data(), runs.size() * sizeof(int4),
                                  cudaMemcpyHostToDevice, ctx->stream));
    ctx->h2d_bytes += rec.size() * sizeof(float4) + hit.size() * sizeof(float4) + mat.size() * sizeof(MatDev) +
                      runs.size() * sizeof(int4);
    // Host staging vectors die at return: wait for the copies.
    RDC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));

    fill_view(ctx->view, sc, ctx->d_rec, fc.nrec, ctx->d_hit, ctx->d_mat, ctx->d_runs, fc.nruns, fast_div,
              ctx->d_counters + kBoundsCounter);
    ctx->brute_fits = brute_fits;
    ctx->has_scene = false;
    ctx->host_objects.assign(sc->objects, sc->objects + n);
    ctx->host_desc = *sc;
    ctx->host_desc.objects = ctx->host_objects.data();
    if (rdc_status bst = apply_accel(ctx, true)) return bst;

    // Frame buffer follows the resolution (CpuRenderer::frame_buffer, cpu.rs:400-417).
    if (!ctx->d_accum || ctx->width != cam.resolution_x || ctx->height != cam.resolution_y) {
        if (ctx->d_accum) cudaFree(ctx->d_accum);
        ctx->d_accum = nullptr;
        const size_t npix = (size_t)cam.resolution_x * cam.resolution_y;
        cudaError_t e = rdc::dev_malloc((void**)&ctx->d_accum, npix * sizeof(float4));
        if (e != cudaSuccess) {
            ctx->has_scene = false;
            return cuda_fail(ctx, e, "cudaMalloc(accumulator)");
        }
        RDC_CUDA(ctx, cudaMemsetAsync(ctx->d_accum, 0, npix * sizeof(float4), ctx->stream));
        ctx->width = cam.resolution_x;
        ctx->height = cam.resolution_y;
        ctx->sample_count = 0;
    }
    ctx->has_scene = true;
    ctx->adj_valid = false;
    return RDC_OK;
}

rdc_status rdc_update_materials(rdc_ctx* ctx, const rdc_material* materials, uint32_t count) {
    if (!ctx) return RDC_ERR_INVALID_ARGUMENT;
    if (!ctx->has_scene) return fail(ctx, RDC_ERR_NO_SCENE, "rdc_update_materials: no scene uploaded");
    const uint32_t n = ctx->host_desc.object_count;
    if (count != n)
        return fail(ctx, RDC_ERR_INVALID_ARGUMENT, "rdc_update_materials: count differs from the scene's object count");
    if (n == 0) return RDC_OK;
    if (!materials) return fail(ctx, RDC_ERR_INVALID_ARGUMENT, "rdc_update_materials: materials is NULL");
    if (rdc_status st = set_device(ctx)) return st;
    std::vector<MatDev> mat(n);
    for (uint32_t i = 0; i < n; ++i) {
        ctx->host_objects[i].material = materials[i];
        mat[i] = rdc::flat_material(ctx->host_objects[i]);
    }
    RDC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));  // no kernel may read mat[] while it changes
    RDC_CUDA(ctx, cudaMemcpyAsync(ctx->d_mat, mat.data(), mat.size() * sizeof(MatDev), cudaMemcpyHostToDevice,
                                  ctx->stream));
    RDC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    ctx->h2d_bytes += mat.size() * sizeof(MatDev);
    ctx->adj_valid = false;
    return RDC_OK;
}

rdc_status rdc_set_accel(rdc_ctx* ctx, uint32_t mode) {
    if (!ctx) return RDC_ERR_INVALID_ARGUMENT;
    if (mode > RDC_ACCEL_LBVH) return fail(ctx, RDC_ERR_INVALID_ARGUMENT, "rdc_set_accel: unknown mode");
    const uint32_t old_mode = ctx->accel_mode;
    ctx->accel_mode = mode;
    if (!ctx->has_scene) return RDC_OK;
    if (rdc_status st = set_device(ctx)) return st;
    RDC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (rdc_status st = apply_accel(ctx, false)) {
        ctx->accel_mode = old_mode;
        return st;
    }
    return RDC_OK;
}

rdc_status rdc_reset(rdc_ctx* ctx) {
    if (!ctx) return RDC_ERR_INVALID_ARGUMENT;
    if (!ctx->has_scene) return fail(ctx, RDC_ERR_NO_SCENE, "rdc_reset: no scene uploaded");
    if (rdc_status st = set_device(ctx)) return st;
    RDC_CUDA(ctx, cudaMemsetAsync(ctx->d_accum, 0, (size_t)ctx->width * ctx->height * sizeof(float4),
                                  ctx->stream));
    ctx->sample_count = 0;
    return RDC_OK;
}

rdc_status rdc_set_render_form(rdc_ctx* ctx, uint32_t form) {
    if (!ctx) return RDC_ERR_INVALID_ARGUMENT;
    if (form > RDC_FORM_WAVEFRONT) return fail(ctx, RDC_ERR_INVALID_ARGUMENT, "rdc_set_render_form: unknown form");
    ctx->render_form = form;
    return RDC_OK;
}

rdc_status rdc_render(rdc_ctx* ctx, uint32_t spp_begin, uint32_t spp_count, uint32_t max_bounces,
                      uint64_t seed) {
    if (!ctx) return RDC_ERR_INVALID_ARGUMENT;
    if (!ctx->has_scene) return fail(ctx, RDC_ERR_NO_SCENE, "rdc_render: no scene uploaded");
    // AUTO: the wavefront once a wave holds RDC_FORM_AUTO_WAVE_SAMPLES samples of every pixel, for LBVH
    // scenes at any size and for brute-force images of at most 1.5 pixels per resident megakernel lane (with
    // fewer pixels than that the megakernel's lanes, each owning whole pixels, run out of work early)
    const uint64_t npix = (uint64_t)ctx->width * ctx->height;
    const uint64_t lanes = (uint64_t)ctx->num_sms * rdc::kRenderBlock * rdc::kRenderBlocksPerSm;
    const bool wavefront =
        ctx->render_form == RDC_FORM_WAVEFRONT ||
        (ctx->render_form == RDC_FORM_AUTO && spp_count > 0 && (ctx->bvh_active || 2 * npix <= 3 * lanes) &&
         rdc::wavefront_wave_spp((uint32_t)npix, spp_count) >= RDC_FORM_AUTO_WAVE_SAMPLES);
    if (wavefront) return rdc_render_wavefront(ctx, spp_begin, spp_count, max_bounces, seed);
    if (max_bounces > RDC_MAX_BOUNCES) return fail(ctx, RDC_ERR_LIMIT, "rdc_render: max_bounces above RDC_MAX_BOUNCES");
    if ((uint64_t)spp_begin + spp_count > 0xFFFFFFFFull)
        return fail(ctx, RDC_ERR_INVALID_ARGUMENT, "rdc_render: sample range overflows 32 bits");
    if (rdc_status st = set_device(ctx)) return st;
    ctx->last_paths = (uint64_t)ctx->width * ctx->height * spp_count;
    ctx->last_launches = 0;
    ctx->last_timed = false;
    RDC_CUDA(ctx, cudaMemsetAsync(ctx->d_counters, 0, 4 * sizeof(unsigned long long), ctx->stream));
    if (spp_count == 0) return RDC_OK;

    rdc::RenderParams p;
    p.sc = ctx->view;
    p.accum = ctx->d_accum;
    p.s0 = spp_begin;
    p.nspp = spp_count;
    p.max_bounces = max_bounces;
    p.stream_id = 0;
    p.key0 = (uint32_t)seed;
    p.key1 = (uint32_t)(seed >> 32);
    p.npix = ctx->width * ctx->height;
    p.work_counter = reinterpret_cast<uint32_t*>(ctx->d_counters);
    p.segments = ctx->d_counters + 1;
    p.errors = ctx->d_counters + kErrorCounter;

    if (!ctx->bvh_active && !ctx->brute_fits)
        return fail(ctx, RDC_ERR_LIMIT,
                    "rdc_render: brute force needs the scene's records in shared memory (at most "
                    "RDC_MAX_BRUTE_OBJECTS objects); use RDC_ACCEL_LBVH or RDC_ACCEL_AUTO");
    p.bvh = ctx->bvh_active ? ctx->bvh.view(ctx->d_counters + kBoundsCounter) : rdc::BvhView{nullptr, nullptr, 0, 0.0f, 0.0f, 0, nullptr};
    p.bvh_counters = ctx->d_counters + 2;
    p.min_idle = ctx->render_cfg.refill_min_idle;
    const int block = ctx->bvh_active ? std::min<int>((int)ctx->render_cfg.block_size, rdc::kRenderBvhBlock)
                                      : (int)ctx->render_cfg.block_size;
    const size_t smem = ctx->bvh_active ? 0 : rdc::render_smem_bytes(ctx->view.nrec, ctx->view.nruns);
    int per_sm = 0;
    if (ctx->bvh_active)
        RDC_CUDA(ctx, rdc::render_bvh_occupancy(block, &per_sm));
    else
        RDC_CUDA(ctx, rdc::render_occupancy(block, smem, &per_sm));
    if (per_sm < 1) return fail(ctx, RDC_ERR_LIMIT, "rdc_render: scene does not fit in shared memory");
    if (ctx->render_cfg.blocks_per_sm != 0) per_sm = std::min<int>(per_sm, (int)ctx->render_cfg.blocks_per_sm);
    const uint64_t warps_needed = ((uint64_t)p.npix + 31) / 32;
    uint64_t grid = (uint64_t)ctx->num_sms * per_sm;
    const uint64_t grid_needed = (warps_needed * 32 + block - 1) / block;
    if (grid > grid_needed) grid = grid_needed;

    RDC_CUDA(ctx, cudaEventRecord(ctx->ev0, ctx->stream));
    if (ctx->bvh_active)
        RDC_CUDA(ctx, rdc::launch_render_bvh(p, (int)grid, block, ctx->stream));
    else
        RDC_CUDA(ctx, rdc::launch_render(p, (int)grid, block, smem, ctx->stream));
    RDC_CUDA(ctx, cudaEventRecord(ctx->ev1, ctx->stream));
    ctx->last_timed = true;
    ctx->last_launches = 1;
    ctx->sample_count = spp_begin + spp_count > ctx->sample_count ? spp_begin + spp_count : ctx->sample_count;
    return RDC_OK;
}

rdc_status rdc_read_accum(rdc_ctx* ctx, float* rgba_out, size_t count) {
    if (!ctx) return RDC_ERR_INVALID_ARGUMENT;
    if (!ctx->has_scene) return fail(ctx, RDC_ERR_NO_SCENE, "rdc_read_accum: no scene uploaded");
    const size_t need = (size_t)ctx->width * ctx->height * 4;
    if (!rgba_out || count < need)
        return fail(ctx, RDC_ERR_INVALID_ARGUMENT, "rdc_read_accum: output buffer smaller than width*height*4");
    if (rdc_status st = set_device(ctx)) return st;
    RDC_CUDA(ctx, cudaMemcpyAsync(rgba_out, ctx->d_accum, need * sizeof(float), cudaMemcpyDeviceToHost,
                                  ctx->stream));
    RDC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    ctx->d2h_bytes += need * sizeof(float);
    return check_device_errors(ctx);
}

rdc_status rdc_write_accum(rdc_ctx* ctx, const float* rgba_in, size_t count, uint32_t sample_count) {
    if (!ctx) return RDC_ERR_INVALID_ARGUMENT;
    if (!ctx->has_scene) return fail(ctx, RDC_ERR_NO_SCENE, "rdc_write_accum: no scene uploaded");
    const size_t need = (size_t)ctx->width * ctx->height * 4;
    if (!rgba_in || count != need)
        return fail(ctx, RDC_ERR_INVALID_ARGUMENT, "rdc_write_accum: input must hold width*height*4 floats");
    if (rdc_status st = set_device(ctx)) return st;
    RDC_CUDA(ctx, cudaMemcpyAsync(ctx->d_accum, rgba_in, need * sizeof(float), cudaMemcpyHostToDevice,
                                  ctx->stream));
    RDC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    ctx->h2d_bytes += need * sizeof(float);
    ctx->sample_count = sample_count;
    return RDC_OK;
}

rdc_status rdc_read_rgba8(rdc_ctx* ctx, uint32_t sample_count, uint8_t* rgba_out, size_t count) {
    if (!ctx) return RDC_ERR_INVALID_ARGUMENT;
    if (!ctx->has_scene) return fail(ctx, RDC_ERR_NO_SCENE, "rdc_read_rgba8: no scene uploaded");
    const size_t npix = (size_t)ctx->width * ctx->height;
    if (!rgba_out || count < npix * 4)
        return fail(ctx, RDC_ERR_INVALID_ARGUMENT, "rdc_read_rgba8: output buffer smaller than width*height*4");
    if (rdc_status st = set_device(ctx)) return st;
    if (rdc_status st = ensure(ctx, &ctx->d_rgba, &ctx->cap_rgba, npix, "cudaMalloc(rgba8)")) return st;
    RDC_CUDA(ctx, rdc::launch_tonemap(ctx->d_accum, (uint32_t)npix, sample_count, ctx->d_rgba, ctx->stream));
    RDC_CUDA(ctx, cudaMemcpyAsync(rgba_out, ctx->d_rgba, npix * 4, cudaMemcpyDeviceToHost, ctx->stream));
    RDC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    ctx->d2h_bytes += npix * 4;
    return check_device_errors(ctx);
}

rdc_status rdc_stats_get(rdc_ctx* ctx, rdc_stats* out) {
    if (!ctx || !out) return fail(ctx, RDC_ERR_INVALID_ARGUMENT, "rdc_stats_get: NULL argument");
    if (rdc_status st = set_device(ctx)) return st;
    RDC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (rdc_status st = check_device_errors(ctx)) return st;
    unsigned long long c[4] = {0, 0, 0, 0};
    RDC_CUDA(ctx, cudaMemcpy(c, ctx->d_counters, sizeof(c), cudaMemcpyDeviceToHost));
    out->segments = c[1];
    out->node_visits = c[2];
    out->prim_tests = c[3];
    out->accel = ctx->bvh_active ? RDC_ACCEL_LBVH : RDC_ACCEL_BRUTE_FORCE;
    out->bvh_depth = ctx->bvh_depth;
    out->paths = ctx->last_paths;
    out->device_ms = 0.0f;
    if (ctx->last_timed) RDC_CUDA(ctx, cudaEventElapsedTime(&out->device_ms, ctx->ev0, ctx->ev1));
    out->sample_count = ctx->sample_count;
    out->kernel_launches = ctx->last_launches;
    out->h2d_bytes = ctx->h2d_bytes;
    out->d2h_bytes = ctx->d2h_bytes;
    return RDC_OK;
}

rdc_status rdc_render_wavefront(rdc_ctx* ctx, uint32_t spp_begin, uint32_t spp_count, uint32_t max_bounces,
                                uint64_t seed) {
    if (!ctx) return RDC_ERR_INVALID_ARGUMENT;
    if (!ctx->has_scene) return fail(ctx, RDC_ERR_NO_SCENE, "rdc_render_wavefront: no scene uploaded");
    if (max_bounces > RDC_MAX_BOUNCES)
        return fail(ctx, RDC_ERR_LIMIT, "rdc_render_wavefront: max_bounces above RDC_MAX_BOUNCES");
    if ((uint64_t)spp_begin + spp_count > 0xFFFFFFFFull)
        return fail(ctx, RDC_ERR_INVALID_ARGUMENT, "rdc_render_wavefront: sample range overflows 32 bits");
    if (!ctx->bvh_active && !ctx->brute_fits)
        return fail(ctx, RDC_ERR_LIMIT,
                    "rdc_render_wavefront: brute force needs the scene's records in shared memory; use the LBVH");
    if (rdc_status st = set_device(ctx)) return st;
    const uint32_t npix = ctx->width * ctx->height;
    ctx->last_paths = (uint64_t)npix * spp_count;
    ctx->last_launches = 0;
    ctx->last_timed = false;
    RDC_CUDA(ctx, cudaMemsetAsync(ctx->d_counters, 0, 4 * sizeof(unsigned long long), ctx->stream));
    if (spp_count == 0) return RDC_OK;
    RDC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));  // the previous graph may still run
    if (ctx->wf_exec) {
        cudaGraphExecDestroy(ctx->wf_exec);
        ctx->wf_exec = nullptr;
    }
    static_assert((uint64_t)RDC_MAX_RESOLUTION * RDC_MAX_RESOLUTION <= (1ull << rdc::kWfPixBits),
                  "a queue entry holds any pixel index");
    static_assert(rdc::kWfMaxWaveSpp <= (1u << (32 - rdc::kWfPixBits)), "and any place in a wave");
    const uint32_t wave = rdc::wavefront_wave_spp(npix, spp_count);
    const uint32_t npath = npix * wave;
    if (rdc_status st = ensure(ctx, &ctx->d_wf, &ctx->cap_wf, rdc::wavefront_state_bytes(npath), "wavefront state"))
        return st;
    if (!ctx->d_wf_counts) RDC_CUDA(ctx, rdc::dev_malloc((void**)&ctx->d_wf_counts, 16 * sizeof(uint32_t)));
    rdc::WfParams p;
    p.sc = ctx->view;
    p.accum = ctx->d_accum;
    p.npix = npix;
    p.npath = npath;
    p.max_bounces = max_bounces;
    p.stream_id = 0;
    p.key0 = (uint32_t)seed;
    p.key1 = (uint32_t)(seed >> 32);
    p.counts = ctx->d_wf_counts;
    p.sample = ctx->d_wf_counts + 6;
    p.wave_n = ctx->d_wf_counts + 8;
    p.segments = ctx->d_counters + 1;
    p.errors = ctx->d_counters + kErrorCounter;
    p.use_bvh = ctx->bvh_active ? 1u : 0u;
    p.bvh = ctx->bvh_active ? ctx->bvh.view(ctx->d_counters + kBoundsCounter)
                            : rdc::BvhView{nullptr, nullptr, 0, 0.0f, 0.0f, 0, nullptr};
    p.bvh_counters = ctx->d_counters + 2;
    p.min_idle = ctx->render_cfg.refill_min_idle;
    p.path = reinterpret_cast<rdc::WfPath*>(ctx->d_wf);  // device allocations are 256-byte aligned
    uint32_t* u = reinterpret_cast<uint32_t*>(p.path + npath);
    p.queue0 = u;
    p.queue1 = u + npath;
    p.cls = u + 2 * (size_t)npath;
    const size_t smem = ctx->bvh_active ? 0 : rdc::render_smem_bytes(ctx->view.nrec, ctx->view.nruns);
    int per_i = 0, per_s = 0;
    RDC_CUDA(ctx, rdc::wavefront_occupancy(ctx->bvh_active, 256, smem, &per_i, &per_s));
    if (per_i < 1 || per_s < 1) return fail(ctx, RDC_ERR_LIMIT, "rdc_render_wavefront: kernels do not fit on an SM");
    const int grid_i = ctx->num_sms * per_i, grid_s = ctx->num_sms * per_s;
    RDC_CUDA(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = rdc::enqueue_wave(p, grid_i, grid_s, smem, ctx->stream);
    cudaGraph_t g = nullptr;
    const cudaError_t e2 = cudaStreamEndCapture(ctx->stream, &g);
    if (e != cudaSuccess || e2 != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return cuda_fail(ctx, e != cudaSuccess ? e : e2, "rdc_render_wavefront: capture");
    }
    e = cudaGraphInstantiate(&ctx->wf_exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaGraphInstantiate");
    RDC_CUDA(ctx, rdc::wavefront_set_word(p.sample, spp_begin, ctx->stream));
    RDC_CUDA(ctx, rdc::wavefront_set_word(p.wave_n, wave, ctx->stream));
    const uint32_t nwaves = (spp_count + wave - 1) / wave, last = spp_count - (nwaves - 1) * wave;
    RDC_CUDA(ctx, cudaEventRecord(ctx->ev0, ctx->stream));
    for (uint32_t k = 0; k < nwaves; ++k) {
        if (k + 1 == nwaves && last != wave) RDC_CUDA(ctx, rdc::wavefront_set_word(p.wave_n, last, ctx->stream));
        RDC_CUDA(ctx, cudaGraphLaunch(ctx->wf_exec, ctx->stream));
    }
    RDC_CUDA(ctx, cudaEventRecord(ctx->ev1, ctx->stream));
    ctx->last_timed = true;
    ctx->last_launches = nwaves * (2u + 2u * max_bounces) + (last != wave ? 1u : 0u);
    ctx->sample_count = spp_begin + spp_count > ctx->sample_count ? spp_begin + spp_count : ctx->sample_count;
    return RDC_OK;
}

rdc_status rdc_forward(rdc_ctx* ctx, uint32_t spp_begin, uint32_t spp_count, uint32_t max_bounces, uint64_t seed,
                       float* image_out) {
    if (!ctx) return RDC_ERR_INVALID_ARGUMENT;
    if (!ctx->has_scene) return fail(ctx, RDC_ERR_NO_SCENE, "rdc_forward: no scene uploaded");
    if (spp_count == 0) return fail(ctx, RDC_ERR_INVALID_ARGUMENT, "rdc_forward: spp_count is 0");
    if (max_bounces > rdc::kAdjMaxBounces)
        return fail(ctx, RDC_ERR_LIMIT, "rdc_forward: max_bounces above RDC_MAX_ADJOINT_BOUNCES");
    if (rdc_status st = rdc_reset(ctx)) return st;
    if (rdc_status st = rdc_render(ctx, spp_begin, spp_count, max_bounces, seed)) return st;
    ctx->adj_valid = true;
    ctx->adj_s0 = spp_begin;
    ctx->adj_n = spp_count;
    ctx->adj_bounces = max_bounces;
    ctx->adj_seed = seed;
    if (!image_out) return RDC_OK;
    const size_t npix = (size_t)ctx->width * ctx->height;
    std::vector<float> acc(npix * 4);
    if (rdc_status st = rdc_read_accum(ctx, acc.data(), acc.size())) return st;
    const float inv = 1.0f / (float)spp_count;
    for (size_t i = 0; i < npix; ++i)
        for (int c = 0; c < 3; ++c) image_out[3 * i + c] = acc[4 * i + c] * inv;
    return RDC_OK;
}

rdc_status rdc_backward(rdc_ctx* ctx, const float* dl_dimage, float* grad_albedo, float* grad_roughness,
                        float* grad_emission) {
    if (!ctx) return RDC_ERR_INVALID_ARGUMENT;
    if (!ctx->has_scene) return fail(ctx, RDC_ERR_NO_SCENE, "rdc_backward: no scene uploaded");
    if (!ctx->adj_valid)
        return fail(ctx, RDC_ERR_INVALID_ARGUMENT, "rdc_backward: no rdc_forward since the scene was uploaded");
    if (!dl_dimage) return fail(ctx, RDC_ERR_INVALID_ARGUMENT, "rdc_backward: dl_dimage is NULL");
    if (rdc_status st = set_device(ctx)) return st;
    const uint32_t nobj = ctx->host_desc.object_count;
    const size_t npix = (size_t)ctx->width * ctx->height;
    if (rdc_status st = ensure(ctx, &ctx->d_dl, &ctx->cap_dl, npix * 3, "rdc_backward: dL/dimage")) return st;
    if (rdc_status st = ensure(ctx, &ctx->d_grad, &ctx->cap_grad, (size_t)nobj * 8, "rdc_backward: gradients"))
        return st;
    RDC_CUDA(ctx, cudaMemcpyAsync(ctx->d_dl, dl_dimage, npix * 3 * sizeof(float), cudaMemcpyHostToDevice,
                                  ctx->stream));
    ctx->h2d_bytes += npix * 3 * sizeof(float);
    RDC_CUDA(ctx, cudaMemsetAsync(ctx->d_grad, 0, (size_t)(nobj ? nobj : 1) * 8 * sizeof(float), ctx->stream));
    RDC_CUDA(ctx, cudaMemsetAsync(ctx->d_counters, 0, 4 * sizeof(unsigned long long), ctx->stream));
    ctx->last_launches = 0;
    ctx->last_timed = false;
    ctx->last_paths = npix * ctx->adj_n;
    if (nobj > 0 && npix > 0) {
        rdc::AdjParams p;
        p.sc = ctx->view;
        p.bvh = ctx->bvh_active ? ctx->bvh.view(ctx->d_counters + kBoundsCounter) : rdc::BvhView{nullptr, nullptr, 0, 0.0f, 0.0f, 0, nullptr};
        p.dl = ctx->d_dl;
        p.grad = ctx->d_grad;
        p.s0 = ctx->adj_s0;
        p.nspp = ctx->adj_n;
        p.max_bounces = ctx->adj_bounces;
        p.stream_id = 0;
        p.key0 = (uint32_t)ctx->adj_seed;
        p.key1 = (uint32_t)(ctx->adj_seed >> 32);
        p.npaths = (uint64_t)npix * ctx->adj_n;
        p.shared_vert_stride = 0;
        p.segments = ctx->d_counters + 1;
        p.errors = ctx->d_counters + kErrorCounter;
        const bool bvh = ctx->bvh_active;
        if (!bvh && !ctx->brute_fits)
            return fail(ctx, RDC_ERR_LIMIT, "rdc_backward: brute force needs the records in shared memory");
        const int block = rdc::kRenderBlock;
        size_t smem = rdc::adjoint_smem_bytes(ctx->view, bvh, true, 0, block);
        p.smem_grad = smem <= kMaxSceneSmem ? 1u : 0u;
        if (!p.smem_grad) smem = rdc::adjoint_smem_bytes(ctx->view, bvh, false, 0, block);
        int per_sm = 0;
        RDC_CUDA(ctx, rdc::adjoint_occupancy(bvh, false, block, smem, &per_sm));
        if (per_sm < 1) return fail(ctx, RDC_ERR_LIMIT, "rdc_backward: scene does not fit in shared memory");
        // Vertex records in shared memory when that still leaves
        // kAdjSharedVertMinBlocks blocks per SM (short paths: 6 bounces at 256
        // threads is 66 KB per block), else in local memory.
        bool shared_vert = false;
        {
            const size_t smem_sh = rdc::adjoint_smem_bytes(ctx->view, bvh, p.smem_grad != 0u, p.max_bounces, block);
            int per_sm_sh = 0;
            if (smem_sh <= kMaxDynSmem && rdc::adjoint_occupancy(bvh, true, block, smem_sh, &per_sm_sh) == cudaSuccess &&
                per_sm_sh >= kAdjSharedVertMinBlocks) {
                shared_vert = true;
                smem = smem_sh;
                per_sm = per_sm_sh;
                p.shared_vert_stride = rdc::adjoint_shared_vert_stride(p.max_bounces);
            }
            (void)cudaGetLastError();
        }
        uint64_t grid = (uint64_t)ctx->num_sms * per_sm;
        const uint64_t need = (p.npaths + block - 1) / block;
        if (grid > need) grid = need;
        RDC_CUDA(ctx, cudaEventRecord(ctx->ev0, ctx->stream));
        RDC_CUDA(ctx, rdc::launch_adjoint(p, bvh, shared_vert, (int)grid, block, smem, ctx->stream));
        RDC_CUDA(ctx, cudaEventRecord(ctx->ev1, ctx->stream));
        ctx->last_timed = true;
        ctx->last_launches = 1;
    }
    std::vector<float> g((size_t)nobj * 8);
    if (nobj > 0) {
        RDC_CUDA(ctx, cudaMemcpyAsync(g.data(), ctx->d_grad, g.size() * sizeof(float), cudaMemcpyDeviceToHost,
                                      ctx->stream));
        ctx->d2h_bytes += g.size() * sizeof(float);
    }
    RDC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    for (uint32_t j = 0; j < nobj; ++j) {
        for (int c = 0; c < 3; ++c) {
            if (grad_albedo) grad_albedo[3 * (size_t)j + c] = g[8 * (size_t)j + c];
            if (grad_emission) grad_emission[3 * (size_t)j + c] = g[8 * (size_t)j + 3 + c];
        }
        // the kernels see roughness^2 (MatDev); d(r^2)/dr = 2r
        if (grad_roughness)
            grad_roughness[j] = g[8 * (size_t)j + 6] * 2.0f * ctx->host_objects[j].material.roughness;
    }
    return RDC_OK;
}

namespace {
// Best lane-operation rate of the FFMA (packed: FP32x2 FMA, two lane
// operations per instruction) probe over a few launches of growing length.
rdc_status fp32_probe(rdc_ctx* ctx, bool packed, double* best_out) {
    const int block = 256, blocks_per_sm = 8;  // 64 warps per SM
    const int grid = ctx->num_sms * blocks_per_sm;
    float* sink = nullptr;
    RDC_CUDA(ctx, rdc::dev_malloc((void**)&sink, grid * sizeof(float)));
    int iters = 256;
    double best = 0.0;
    cudaError_t e = cudaSuccess;
    for (int rep = 0; rep < 6 && e == cudaSuccess; ++rep) {
        e = cudaEventRecord(ctx->ev0, ctx->stream);
        if (e == cudaSuccess) e = rdc::launch_fp32_probe(sink, grid, block, iters, packed, ctx->stream);
        if (e == cudaSuccess) e = cudaEventRecord(ctx->ev1, ctx->stream);
        if (e == cudaSuccess) e = cudaEventSynchronize(ctx->ev1);
        float ms = 0.f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
        if (e != cudaSuccess) break;
        const double ops = (double)grid * block * iters * 16.0 * rdc::kProbeChains * (packed ? 2.0 : 1.0);
        if (ms > 0.f) best = ops / (ms * 1e-3) > best ? ops / (ms * 1e-3) : best;
        if (ms < 20.f) iters *= 2;  // grow to a few tens of milliseconds
    }
    cudaFree(sink);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "FP32 probe");
    *best_out = best;
    ctx->last_timed = false;
    return RDC_OK;
}
}  // namespace

rdc_status rdc_selftest_staging_timeout(rdc_ctx* ctx) {
    if (!ctx) return RDC_ERR_INVALID_ARGUMENT;
    if (rdc_status st = set_device(ctx)) return st;
    RDC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (rdc_status st = check_device_errors(ctx)) return st;  // report anything earlier first
    RDC_CUDA(ctx, rdc::launch_staging_timeout(ctx->d_counters + kErrorCounter, ctx->stream));
    RDC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return check_device_errors(ctx);
}

namespace {
// Device buffers of a self-test, freed on every exit.
struct SelftestBuffers {
    std::vector<void*> p;
    ~SelftestBuffers() {
        for (void* q : p) cudaFree(q);
    }
    cudaError_t alloc(void** out, size_t bytes) {
        *out = nullptr;
        const cudaError_t e = rdc::dev_malloc(out, bytes > 0 ? bytes : 4);
        if (e == cudaSuccess) p.push_back(*out);
        return e;
    }
};
}  // namespace

rdc_status rdc_selftest_radix_sort(rdc_ctx* ctx, const uint32_t* keys, const uint32_t* vals, uint32_t n,
                                   uint32_t key_bits, uint32_t* keys_out, uint32_t* vals_out) {
    if (!ctx) return RDC_ERR_INVALID_ARGUMENT;
    if (n > 0 && (!keys || !vals || !keys_out || !vals_out))
        return fail(ctx, RDC_ERR_INVALID_ARGUMENT, "rdc_selftest_radix_sort: NULL argument");
    if (key_bits < 1 || key_bits > 32)
        return fail(ctx, RDC_ERR_INVALID_ARGUMENT, "rdc_selftest_radix_sort: key_bits must be in 1..32");
    if (n > RDC_MAX_OBJECTS) return fail(ctx, RDC_ERR_LIMIT, "rdc_selftest_radix_sort: n above RDC_MAX_OBJECTS");
    if (rdc_status st = set_device(ctx)) return st;
    if (n == 0) return RDC_OK;
    SelftestBuffers b;
    uint32_t *k0, *v0, *k1, *v1;
    void* scratch;
    const size_t bytes = (size_t)n * 4;
    RDC_CUDA(ctx, b.alloc((void**)&k0, bytes));
    RDC_CUDA(ctx, b.alloc((void**)&v0, bytes));
    RDC_CUDA(ctx, b.alloc((void**)&k1, bytes));
    RDC_CUDA(ctx, b.alloc((void**)&v1, bytes));
    RDC_CUDA(ctx, b.alloc(&scratch, rdc::radix_sort_scratch_bytes(n)));
    RDC_CUDA(ctx, cudaMemcpyAsync(k0, keys, bytes, cudaMemcpyHostToDevice, ctx->stream));
    RDC_CUDA(ctx, cudaMemcpyAsync(v0, vals, bytes, cudaMemcpyHostToDevice, ctx->stream));
    uint32_t *ks = nullptr, *vs = nullptr;
    RDC_CUDA(ctx, rdc::radix_sort_pairs(k0, v0, k1, v1, n, (int)key_bits, scratch, ctx->stream, &ks, &vs));
    RDC_CUDA(ctx, cudaMemcpyAsync(keys_out, ks, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    RDC_CUDA(ctx, cudaMemcpyAsync(vals_out, vs, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    RDC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return RDC_OK;
}

rdc_status rdc_selftest_exclusive_scan(rdc_ctx* ctx, const uint32_t* in, uint32_t n, uint32_t* out) {
    if (!ctx) return RDC_ERR_INVALID_ARGUMENT;
    if (n > 0 && (!in || !out)) return fail(ctx, RDC_ERR_INVALID_ARGUMENT, "rdc_selftest_exclusive_scan: NULL argument");
    if (n > RDC_MAX_OBJECTS) return fail(ctx, RDC_ERR_LIMIT, "rdc_selftest_exclusive_scan: n above RDC_MAX_OBJECTS");
    if (rdc_status st = set_device(ctx)) return st;
    if (n == 0) return RDC_OK;
    SelftestBuffers b;
    uint32_t *d_in, *d_out;
    void* scratch;
    const size_t bytes = (size_t)n * 4;
    RDC_CUDA(ctx, b.alloc((void**)&d_in, bytes));
    RDC_CUDA(ctx, b.alloc((void**)&d_out, bytes));
    RDC_CUDA(ctx, b.alloc(&scratch, rdc::exclusive_scan_scratch_bytes(n)));
    RDC_CUDA(ctx, cudaMemcpyAsync(d_in, in, bytes, cudaMemcpyHostToDevice, ctx->stream));
    RDC_CUDA(ctx, rdc::exclusive_scan(d_in, d_out, n, scratch, ctx->stream));
    RDC_CUDA(ctx, cudaMemcpyAsync(out, d_out, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    RDC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return RDC_OK;
}

rdc_status rdc_measure_fp32x2_issue(rdc_ctx* ctx, double* lane_ops_per_second) {
    if (!ctx || !lane_ops_per_second)
        return fail(ctx, RDC_ERR_INVALID_ARGUMENT, "rdc_measure_fp32x2_issue: NULL argument");
    if (rdc_status st = set_device(ctx)) return st;
    return fp32_probe(ctx, true, lane_ops_per_second);
}

rdc_status rdc_measure_fp32_issue(rdc_ctx* ctx, double* lane_ops_per_second, double* sm_mhz) {
    if (!ctx || !lane_ops_per_second) return fail(ctx, RDC_ERR_INVALID_ARGUMENT, "rdc_measure_fp32_issue: NULL argument");
    if (rdc_status st = set_device(ctx)) return st;
    double best = 0.0;
    if (rdc_status st = fp32_probe(ctx, false, &best)) return st;
    *lane_ops_per_second = best;
    if (sm_mhz) *sm_mhz = best / (ctx->num_sms * 128.0) / 1e6;
    return RDC_OK;
}

rdc_status rdc_intersect_rays(rdc_ctx* ctx, const float* origins, const float* directions, uint32_t n,
                              float* t_out, int32_t* index_out, float* normal_out, uint8_t* front_out) {
    if (!ctx) return RDC_ERR_INVALID_ARGUMENT;
    if (!ctx->has_scene) return fail(ctx, RDC_ERR_NO_SCENE, "rdc_intersect_rays: no scene uploaded");
    if (n == 0) return RDC_OK;
    if (!origins || !directions || !t_out || !index_out || !normal_out || !front_out)
        return fail(ctx, RDC_ERR_INVALID_ARGUMENT, "rdc_intersect_rays: NULL buffer");
    if (rdc_status st = set_device(ctx)) return st;
    const size_t f3 = (size_t)n * 3 * sizeof(float);
    char* buf = nullptr;
    const size_t total = 3 * f3 + n * sizeof(float) + n * sizeof(int32_t) + n;
    RDC_CUDA(ctx, rdc::dev_malloc((void**)&buf, total));
    float* d_o = (float*)buf;
    float* d_d = (float*)(buf + f3);
    float* d_n = (float*)(buf + 2 * f3);
    float* d_t = (float*)(buf + 3 * f3);
    int32_t* d_i = (int32_t*)(buf + 3 * f3 + n * sizeof(float));
    uint8_t* d_f = (uint8_t*)(buf + 3 * f3 + n * sizeof(float) + n * sizeof(int32_t));
    cudaError_t e = cudaMemcpyAsync(d_o, origins, f3, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_d, directions, f3, cudaMemcpyHostToDevice, ctx->stream);
    const rdc::BvhView bv = ctx->bvh_active ? ctx->bvh.view(ctx->d_counters + kBoundsCounter) : rdc::BvhView{nullptr, nullptr, 0, 0.0f, 0.0f, 0, nullptr};
    if (e == cudaSuccess)
        e = rdc::launch_intersect_rays(ctx->view, bv, d_o, d_d, n, d_t, d_i, d_n, d_f, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(t_out, d_t, n * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(index_out, d_i, n * sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(normal_out, d_n, f3, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(front_out, d_f, n, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    cudaFree(buf);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "rdc_intersect_rays");
    return RDC_OK;
}

rdc_status rdc_scatter_fixed(rdc_ctx* ctx, const float* origins, const float* directions, const float* t,
                             const int32_t* index, const uint32_t* words, uint32_t n, float* origin_out,
                             float* direction_out) {
    if (!ctx) return RDC_ERR_INVALID_ARGUMENT;
    if (!ctx->has_scene) return fail(ctx, RDC_ERR_NO_SCENE, "rdc_scatter_fixed: no scene uploaded");
    if (n == 0) return RDC_OK;
    if (!origins || !directions || !t || !index || !words || !origin_out || !direction_out)
        return fail(ctx, RDC_ERR_INVALID_ARGUMENT, "rdc_scatter_fixed: NULL buffer");
    for (uint32_t i = 0; i < n; ++i)
        if (index[i] < 0 || (uint32_t)index[i] >= ctx->view.nobj)
            return fail(ctx, RDC_ERR_INVALID_ARGUMENT,
                        "rdc_scatter_fixed: object index out of range at item " + std::to_string(i));
    if (rdc_status st = set_device(ctx)) return st;
    const size_t f3 = (size_t)n * 3 * sizeof(float);
    const size_t total = 4 * f3 + n * sizeof(float) + n * sizeof(int32_t) + (size_t)n * 12 * sizeof(uint32_t);
    char* buf = nullptr;
    RDC_CUDA(ctx, rdc::dev_malloc((void**)&buf, total));
    float* d_o = (float*)buf;
    float* d_d = (float*)(buf + f3);
    float* d_oo = (float*)(buf + 2 * f3);
    float* d_do = (float*)(buf + 3 * f3);
    float* d_t = (float*)(buf + 4 * f3);
    int32_t* d_i = (int32_t*)(buf + 4 * f3 + n * sizeof(float));
    uint32_t* d_w = (uint32_t*)(buf + 4 * f3 + n * sizeof(float) + n * sizeof(int32_t));
    cudaError_t e = cudaMemcpyAsync(d_o, origins, f3, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_d, directions, f3, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_t, t, n * sizeof(float), cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_i, index, n * sizeof(int32_t), cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_w, words, (size_t)n * 12 * sizeof(uint32_t), cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = rdc::launch_scatter_fixed(ctx->view, d_o, d_d, d_t, d_i, d_w, n, d_oo, d_do, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(origin_out, d_oo, f3, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(direction_out, d_do, f3, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    cudaFree(buf);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "rdc_scatter_fixed");
    return RDC_OK;
}

}  // extern "C"

// ------------------------------------------------------------------ batch --
namespace {

void free_batch(rdc_ctx* ctx) {
    auto& b = ctx->batch;
    if (b.exec) cudaGraphExecDestroy(b.exec);
    if (b.graph) cudaGraphDestroy(b.graph);
    cudaFree(b.d_scenes);
    cudaFree(b.d_rec);
    cudaFree(b.d_hit);
    cudaFree(b.d_mat);
    cudaFree(b.d_runs);
    cudaFree(b.d_accum);
    cudaFree(b.d_pixel_counters);
    b = rdc_ctx::Batch();
}

// Capture clear + persistent batch kernel into the batch graph.
rdc_status capture_batch_graph(rdc_ctx* ctx) {
    auto& b = ctx->batch;
    if (b.exec) cudaGraphExecDestroy(b.exec);
    if (b.graph) cudaGraphDestroy(b.graph);
    b.exec = nullptr;
    b.graph = nullptr;
    int per_sm = 0;
    RDC_CUDA(ctx, rdc::batch_occupancy((int)b.cfg.block_size, b.smem, &per_sm));
    if (per_sm < 1) return fail(ctx, RDC_ERR_LIMIT, "rdc_batch: block size does not fit on an SM");
    const int blocks = b.cfg.blocks_per_sm == 0 ? per_sm : std::min<int>(per_sm, (int)b.cfg.blocks_per_sm);
    const int grid = ctx->num_sms * blocks;
    rdc::BatchParams p;
    p.scenes = b.d_scenes;
    p.nscenes = b.n;
    p.refill_min = b.cfg.refill_min_idle;
    p.pixel_counters = b.d_pixel_counters;
    p.segments = ctx->d_counters + 1;
    p.errors = ctx->d_counters + kErrorCounter;
    RDC_CUDA(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = cudaMemsetAsync(b.d_accum, 0, b.accum_total * sizeof(float4), ctx->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(b.d_pixel_counters, 0, b.n * sizeof(uint32_t), ctx->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(ctx->d_counters, 0, 2 * sizeof(unsigned long long), ctx->stream);
    if (e == cudaSuccess) e = rdc::launch_batch(p, grid, (int)b.cfg.block_size, b.smem, ctx->stream);
    cudaGraph_t g = nullptr;
    const cudaError_t e2 = cudaStreamEndCapture(ctx->stream, &g);
    if (e != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return cuda_fail(ctx, e, "rdc_batch: capture");
    }
    if (e2 != cudaSuccess) return cuda_fail(ctx, e2, "cudaStreamEndCapture");
    b.graph = g;
    RDC_CUDA(ctx, cudaGraphInstantiate(&b.exec, b.graph, 0));
    return RDC_OK;
}

}  // namespace

extern "C" {

rdc_status rdc_batch_upload(rdc_ctx* ctx, const rdc_batch_item* items, uint32_t count) {
    if (!ctx) return RDC_ERR_INVALID_ARGUMENT;
    if (!items || count == 0) return fail(ctx, RDC_ERR_INVALID_ARGUMENT, "rdc_batch_upload: no items");
    for (uint32_t i = 0; i < count; ++i) {
        if (rdc_status st = check_scene(ctx, items[i].scene, "rdc_batch_upload: item " + std::to_string(i)))
            return st;
        if (items[i].max_bounces > RDC_MAX_BOUNCES)
            return fail(ctx, RDC_ERR_LIMIT, "rdc_batch_upload: item " + std::to_string(i) + " max_bounces above limit");
    }
    if (rdc_status st = set_device(ctx)) return st;
    RDC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    const rdc_launch_config cfg = ctx->batch.cfg;
    free_batch(ctx);
    auto& b = ctx->batch;
    b.cfg = cfg;

    // Sizes and offsets of every scene's arrays in the concatenated buffers.
    std::vector<rdc::FlatCounts> fc(count);
    std::vector<size_t> rec_off(count), obj_off(count), run_off(count);
    size_t nrec = 0, nobj = 0, nruns = 0, accum = 0;
    std::vector<double> work(count);
    double total_work = 0.0;
    b.accum_off.resize(count);
    b.width.resize(count);
    b.height.resize(count);
    for (uint32_t i = 0; i < count; ++i) {
        const rdc_scene_desc* sc = items[i].scene;
        fc[i] = rdc::flat_counts(sc);
        rec_off[i] = nrec;
        obj_off[i] = nobj;
        run_off[i] = nruns;
        nrec += fc[i].nrec;
        nobj += fc[i].nobj;
        nruns += fc[i].nruns;
        b.smem = std::max(b.smem, rdc::render_smem_bytes(fc[i].nrec, fc[i].nruns));
        if (b.smem > kMaxSceneSmem) {
            free_batch(ctx);
            return fail(ctx, RDC_ERR_LIMIT,
                        "rdc_batch_upload: item " + std::to_string(i) + " exceeds the shared-memory budget");
        }
        b.width[i] = sc->camera.resolution_x;
        b.height[i] = sc->camera.resolution_y;
        b.accum_off[i] = accum;
        const size_t npix = (size_t)b.width[i] * b.height[i];
        accum += npix;
        b.paths += (uint64_t)npix * items[i].spp;
        // estimated work: paths x (1 + a few segments) x objects tested
        work[i] = (double)npix * items[i].spp * (1.0 + std::min<uint32_t>(items[i].max_bounces, 3u)) *
                  (8.0 + sc->object_count);
        total_work += work[i];
    }
    b.n = count;
    b.accum_total = accum;

    std::vector<float4> rec(std::max<size_t>(nrec, 1), make_float4(0, 0, 0, 0));
    std::vector<float4> hit(std::max<size_t>(nobj, 1), make_float4(0, 0, 0, 0));
    std::vector<MatDev> mat(std::max<size_t>(nobj, 1));
    std::vector<int4> runs(std::max<size_t>(nruns, 1), make_int4(0, 0, 0, 0));
    std::vector<char> fast(count);
    for (uint32_t i = 0; i < count; ++i)
        fast[i] = rdc::flatten(items[i].scene, rec.data() + rec_off[i], hit.data() + obj_off[i],
                               mat.data() + obj_off[i], runs.data() + run_off[i]);

    cudaError_t e = rdc::dev_malloc((void**)&b.d_rec, rec.size() * sizeof(float4));
    if (e == cudaSuccess) e = rdc::dev_malloc((void**)&b.d_hit, hit.size() * sizeof(float4));
    if (e == cudaSuccess) e = rdc::dev_malloc((void**)&b.d_mat, mat.size() * sizeof(MatDev));
    if (e == cudaSuccess) e = rdc::dev_malloc((void**)&b.d_runs, runs.size() * sizeof(int4));
    if (e == cudaSuccess) e = rdc::dev_malloc((void**)&b.d_accum, b.accum_total * sizeof(float4));
    if (e == cudaSuccess) e = rdc::dev_malloc((void**)&b.d_pixel_counters, count * sizeof(uint32_t));
    if (e == cudaSuccess) e = rdc::dev_malloc((void**)&b.d_scenes, count * sizeof(rdc::BatchScene));
    if (e != cudaSuccess) {
        free_batch(ctx);
        return cuda_fail(ctx, e, "rdc_batch_upload: cudaMalloc");
    }
    std::vector<rdc::BatchScene> scenes(count);
    double acc_work = 0.0;
    for (uint32_t i = 0; i < count; ++i) {
        rdc::BatchScene& bs = scenes[i];
        fill_view(bs.sc, items[i].scene, b.d_rec + rec_off[i], fc[i].nrec, b.d_hit + obj_off[i],
                  b.d_mat + obj_off[i], b.d_runs + run_off[i], fc[i].nruns, fast[i] != 0, ctx->d_counters + kBoundsCounter);
        bs.accum = b.d_accum + b.accum_off[i];
        bs.npix = b.width[i] * b.height[i];
        bs.spp = items[i].spp;
        bs.max_bounces = items[i].max_bounces;
        bs.key0 = (uint32_t)items[i].seed;
        bs.key1 = (uint32_t)(items[i].seed >> 32);
        bs.work_begin = (float)(acc_work / total_work);
        bs.pixel_work = bs.npix ? (float)(work[i] / total_work / (double)bs.npix * 1e6) : 0.0f;
        acc_work += work[i];
        if (bs.spp == 0) bs.npix = 0;  // nothing to render: the pool starts empty
    }
    e = cudaMemcpyAsync(b.d_rec, rec.data(), rec.size() * sizeof(float4), cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(b.d_hit, hit.data(), hit.size() * sizeof(float4), cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(b.d_mat, mat.data(), mat.size() * sizeof(MatDev), cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(b.d_runs, runs.data(), runs.size() * sizeof(int4), cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(b.d_scenes, scenes.data(), count * sizeof(rdc::BatchScene), cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) {
        free_batch(ctx);
        return cuda_fail(ctx, e, "rdc_batch_upload: copy");
    }
    ctx->h2d_bytes += rec.size() * sizeof(float4) + hit.size() * sizeof(float4) + mat.size() * sizeof(MatDev) +
                      runs.size() * sizeof(int4) + count * sizeof(rdc::BatchScene);
    if (rdc_status st = capture_batch_graph(ctx)) {
        free_batch(ctx);
        return st;
    }
    return RDC_OK;
}

rdc_status rdc_batch_render(rdc_ctx* ctx) {
    if (!ctx) return RDC_ERR_INVALID_ARGUMENT;
    if (!ctx->batch.exec) return fail(ctx, RDC_ERR_NO_SCENE, "rdc_batch_render: no batch uploaded");
    if (rdc_status st = set_device(ctx)) return st;
    RDC_CUDA(ctx, cudaEventRecord(ctx->ev0, ctx->stream));
    RDC_CUDA(ctx, cudaGraphLaunch(ctx->batch.exec, ctx->stream));
    RDC_CUDA(ctx, cudaEventRecord(ctx->ev1, ctx->stream));
    ctx->last_timed = true;
    ctx->last_launches = 1;
    ctx->last_paths = ctx->batch.paths;
    return RDC_OK;
}

rdc_status rdc_batch_read_accum(rdc_ctx* ctx, uint32_t index, float* rgba_out, size_t count) {
    if (!ctx) return RDC_ERR_INVALID_ARGUMENT;
    auto& b = ctx->batch;
    if (!b.exec) return fail(ctx, RDC_ERR_NO_SCENE, "rdc_batch_read_accum: no batch uploaded");
    if (index >= b.n) return fail(ctx, RDC_ERR_INVALID_ARGUMENT, "rdc_batch_read_accum: index out of range");
    const size_t need = (size_t)b.width[index] * b.height[index] * 4;
    if (!rgba_out || count < need)
        return fail(ctx, RDC_ERR_INVALID_ARGUMENT, "rdc_batch_read_accum: output smaller than width*height*4");
    if (rdc_status st = set_device(ctx)) return st;
    RDC_CUDA(ctx, cudaMemcpyAsync(rgba_out, b.d_accum + b.accum_off[index], need * sizeof(float),
                                  cudaMemcpyDeviceToHost, ctx->stream));
    RDC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    ctx->d2h_bytes += need * sizeof(float);
    return RDC_OK;
}

rdc_status rdc_batch_set_config(rdc_ctx* ctx, const rdc_launch_config* config) {
    if (!ctx) return RDC_ERR_INVALID_ARGUMENT;
    if (!config) return fail(ctx, RDC_ERR_INVALID_ARGUMENT, "rdc_batch_set_config: NULL config");
    if (config->block_size != 64 && config->block_size != 128 && config->block_size != 256)
        return fail(ctx, RDC_ERR_INVALID_ARGUMENT, "rdc_batch_set_config: block_size must be 64, 128 or 256");
    if (config->refill_min_idle < 1 || config->refill_min_idle > 32)
        return fail(ctx, RDC_ERR_INVALID_ARGUMENT, "rdc_batch_set_config: refill_min_idle must be in 1..32");
    if (rdc_status st = set_device(ctx)) return st;
    ctx->batch.cfg = *config;
    if (ctx->batch.n == 0) return RDC_OK;
    RDC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return capture_batch_graph(ctx);
}

rdc_status rdc_set_render_config(rdc_ctx* ctx, const rdc_launch_config* config) {
    if (!ctx) return RDC_ERR_INVALID_ARGUMENT;
    if (!config) return fail(ctx, RDC_ERR_INVALID_ARGUMENT, "rdc_set_render_config: NULL config");
    if (config->block_size != 64 && config->block_size != 128 && config->block_size != 256)
        return fail(ctx, RDC_ERR_INVALID_ARGUMENT, "rdc_set_render_config: block_size must be 64, 128 or 256");
    if (config->refill_min_idle < 1 || config->refill_min_idle > 32)
        return fail(ctx, RDC_ERR_INVALID_ARGUMENT, "rdc_set_render_config: refill_min_idle must be in 1..32");
    ctx->render_cfg = *config;
    return RDC_OK;
}

rdc_status rdc_get_render_config(rdc_ctx* ctx, rdc_launch_config* config) {
    if (!ctx || !config) return fail(ctx, RDC_ERR_INVALID_ARGUMENT, "rdc_get_render_config: NULL argument");
    *config = ctx->render_cfg;
    return RDC_OK;
}

rdc_status rdc_batch_get_config(rdc_ctx* ctx, rdc_launch_config* config) {
    if (!ctx || !config) return fail(ctx, RDC_ERR_INVALID_ARGUMENT, "rdc_batch_get_config: NULL argument");
    *config = ctx->batch.cfg;
    return RDC_OK;
}

rdc_status rdc_batch_autotune(rdc_ctx* ctx, rdc_launch_config* best_out, float* best_ms_out) {
    if (!ctx) return RDC_ERR_INVALID_ARGUMENT;
    if (!ctx->batch.exec) return fail(ctx, RDC_ERR_NO_SCENE, "rdc_batch_autotune: no batch uploaded");
    if (rdc_status st = set_device(ctx)) return st;
    const uint32_t blocks[] = {128, 256};
    const uint32_t refills[] = {1, 4, 16};
    rdc_launch_config best = ctx->batch.cfg;
    float best_ms = 0.0f;
    bool have = false;
    for (uint32_t bsz : blocks) {
        int per_sm = 0;
        RDC_CUDA(ctx, rdc::batch_occupancy((int)bsz, ctx->batch.smem, &per_sm));
        for (int bps = std::max(1, per_sm - 1); bps <= per_sm; ++bps) {
            for (uint32_t rf : refills) {
                const rdc_launch_config c{bsz, (uint32_t)bps, rf};
                if (rdc_status st = rdc_batch_set_config(ctx, &c)) return st;
                float ms = 0.0f;
                for (int rep = 0; rep < 2; ++rep) {  // first run warms up
                    if (rdc_status st = rdc_batch_render(ctx)) return st;
                    RDC_CUDA(ctx, cudaEventSynchronize(ctx->ev1));
                    RDC_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
                }
                if (!have || ms < best_ms) {
                    best = c;
                    best_ms = ms;
                    have = true;
                }
            }
        }
    }
    if (rdc_status st = rdc_batch_set_config(ctx, &best)) return st;
    if (best_out) *best_out = best;
    if (best_ms_out) *best_ms_out = best_ms;
    return RDC_OK;
}

}  // extern "C"
