// oracle_capi.cpp -- extern "C" entry points of the CPU oracle (test
// infrastructure only: loaded by tests/, the smoke check and the benchmark's
// CPU-baseline leg through ctypes; never by the shipped library).
#include <atomic>
#include <thread>

#include "raydar_oracle.hpp"
#include "raydar_oracle_grad.hpp"

using namespace oracle;

extern "C" {

int oracle_abi_version(void) { return RDC_ABI_VERSION; }

// Philox4x32-10 block for known-answer tests.
void oracle_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    Philox4 r = philox4x32_10(ctr[0], ctr[1], ctr[2], ctr[3], key[0], key[1]);
    for (int i = 0; i < 4; ++i) out[i] = r.v[i];
}

void oracle_bounce_words(uint64_t seed, uint32_t stream, uint32_t pixel, uint32_t sample,
                         uint32_t bounce, uint32_t out[12]) {
    bounce_words(seed, stream, pixel, sample, bounce, out);
}

void oracle_uniforms(const uint32_t* words, uint32_t n, float* u01, float* upm1) {
    for (uint32_t i = 0; i < n; ++i) {
        u01[i] = uniform01(words[i]);
        upm1[i] = uniform_pm1(words[i]);
    }
}

// Render samples [s0, s0+n) of every pixel into accum (W*H*4 floats, in/out),
// threads = number of host threads (>= 1).  Returns 0 on success.
int oracle_render(const rdc_scene_desc* desc, uint32_t s0, uint32_t n, uint32_t max_bounces,
                  uint64_t seed, uint32_t stream, float* accum, uint64_t* segments_out,
                  int threads) {
    if (!desc || !accum) return 1;
    const Scene<float> s = scene_from_desc<float>(desc);
    const uint32_t npix = s.width * s.height;
    std::atomic<uint32_t> next{0};
    std::atomic<uint64_t> total{0};
    auto worker = [&]() {
        uint64_t seg = 0;
        for (;;) {
            const uint32_t base = next.fetch_add(64);
            if (base >= npix) break;
            const uint32_t end = base + 64 < npix ? base + 64 : npix;
            for (uint32_t p = base; p < end; ++p)
                render_pixel(s, p, s0, n, max_bounces, seed, stream, accum + 4 * (size_t)p, &seg);
        }
        total += seg;
    };
    if (threads <= 1) {
        worker();
    } else {
        std::vector<std::thread> pool;
        for (int i = 0; i < threads; ++i) pool.emplace_back(worker);
        for (auto& t : pool) t.join();
    }
    if (segments_out) *segments_out = total.load();
    return 0;
}

}  // extern "C"

namespace {

// The gradient of oracle_gradient / oracle_gradient_f32 with dual numbers D.
template <typename D>
int gradient_impl(const rdc_scene_desc* desc, uint32_t s0, uint32_t n, uint32_t max_bounces, uint64_t seed,
                  uint32_t stream, const float* dl_dimage, double* g_albedo, double* g_rough, double* g_emission,
                  double* image, int threads, uint64_t* lost_out, double* g_rough_path) {
    if (!desc || !dl_dimage || !g_albedo || !g_rough || !g_emission || n == 0) return 1;
    if (max_bounces > (uint32_t)kGradSlots) return 2;
    const Scene<float> sf = scene_from_desc<float>(desc);
    const Scene<D> s = scene_from_desc<D>(desc);
    std::atomic<uint64_t> lost{0};
    const uint32_t npix = s.width * s.height;
    const size_t nobj = s.objects.size();
    if (threads < 1) threads = 1;
    std::vector<std::vector<double>> part(threads, std::vector<double>(8 * nobj, 0.0));
    std::atomic<uint32_t> next{0};
    auto worker = [&](int tid) {
        double* ga = part[tid].data();
        double* gr = ga + 3 * nobj;
        double* ge = gr + nobj;
        double* gp = ge + 3 * nobj;
        for (;;) {
            const uint32_t base = next.fetch_add(16);
            if (base >= npix) break;
            const uint32_t end = base + 16 < npix ? base + 16 : npix;
            lost += gradient_pixels(sf, s, base, end, s0, n, max_bounces, seed, stream, dl_dimage, ga, gr, ge,
                                    image, gp);
        }
    };
    if (threads == 1) {
        worker(0);
    } else {
        std::vector<std::thread> pool;
        for (int i = 0; i < threads; ++i) pool.emplace_back(worker, i);
        for (auto& t : pool) t.join();
    }
    for (size_t j = 0; j < nobj; ++j) {
        for (int c = 0; c < 3; ++c) {
            g_albedo[3 * j + c] = 0.0;
            g_emission[3 * j + c] = 0.0;
        }
        g_rough[j] = 0.0;
        if (g_rough_path) g_rough_path[j] = 0.0;
        for (int t = 0; t < threads; ++t) {
            for (int c = 0; c < 3; ++c) {
                g_albedo[3 * j + c] += part[t][3 * j + c];
                g_emission[3 * j + c] += part[t][4 * nobj + 3 * j + c];
            }
            g_rough[j] += part[t][3 * nobj + j];
            if (g_rough_path) g_rough_path[j] += part[t][7 * nobj + j];
        }
    }
    if (lost_out) *lost_out = lost.load();
    return 0;
}

}  // namespace

extern "C" {

// FP64 reference gradient (raydar_oracle_grad.hpp) of sum dL_dimage * image,
// image = mean radiance (RGB) of samples [s0, s0+n).  Writes g_albedo (N*3),
// g_rough (N), g_emission (N*3) and, if not null, image (npix*3).  Returns 1
// on a bad argument, 2 when max_bounces exceeds the tangent slots.  lost_out
// (may be null): paths whose double evaluation lost a recorded hit.
int oracle_gradient(const rdc_scene_desc* desc, uint32_t s0, uint32_t n, uint32_t max_bounces, uint64_t seed,
                    uint32_t stream, const float* dl_dimage, double* g_albedo, double* g_rough,
                    double* g_emission, double* image, int threads, uint64_t* lost_out, double* g_rough_path) {
    return gradient_impl<Dual>(desc, s0, n, max_bounces, seed, stream, dl_dimage, g_albedo, g_rough, g_emission,
                               image, threads, lost_out, g_rough_path);
}

// The same derivative with every per-path intermediate in float (DualF), the
// precision of the CUDA adjoint; the sums over paths stay in double.
int oracle_gradient_f32(const rdc_scene_desc* desc, uint32_t s0, uint32_t n, uint32_t max_bounces, uint64_t seed,
                        uint32_t stream, const float* dl_dimage, double* g_albedo, double* g_rough,
                        double* g_emission, double* image, int threads, uint64_t* lost_out, double* g_rough_path) {
    return gradient_impl<DualF>(desc, s0, n, max_bounces, seed, stream, dl_dimage, g_albedo, g_rough, g_emission,
                                image, threads, lost_out, g_rough_path);
}

// Same, for a list of pixel indices; accum holds npix*4 floats (in/out).
int oracle_render_pixels(const rdc_scene_desc* desc, const uint32_t* pixels, uint32_t npix,
                         uint32_t s0, uint32_t n, uint32_t max_bounces, uint64_t seed,
                         uint32_t stream, float* accum, uint64_t* segments_out) {
    if (!desc || !pixels || !accum) return 1;
    const Scene<float> s = scene_from_desc<float>(desc);
    uint64_t seg = 0;
    for (uint32_t i = 0; i < npix; ++i) {
        if (pixels[i] >= s.width * s.height) return 2;
        render_pixel(s, pixels[i], s0, n, max_bounces, seed, stream, accum + 4 * (size_t)i, &seg);
    }
    if (segments_out) *segments_out = seg;
    return 0;
}

// Closest hit of n rays (origins/directions n*3).
int oracle_intersect(const rdc_scene_desc* desc, const float* o, const float* d, uint32_t n,
                     float* t_out, int32_t* idx_out, float* normal_out, uint8_t* front_out) {
    const Scene<float> s = scene_from_desc<float>(desc);
    for (uint32_t i = 0; i < n; ++i) {
        Ray<float> r{v3(o[3 * i], o[3 * i + 1], o[3 * i + 2]), v3(d[3 * i], d[3 * i + 1], d[3 * i + 2])};
        const Hit<float> h = trace_ray(r, s);
        idx_out[i] = h.index;
        t_out[i] = h.index >= 0 ? h.t : 0.0f;
        normal_out[3 * i] = h.index >= 0 ? h.normal.x : 0.0f;
        normal_out[3 * i + 1] = h.index >= 0 ? h.normal.y : 0.0f;
        normal_out[3 * i + 2] = h.index >= 0 ? h.normal.z : 0.0f;
        front_out[i] = h.index >= 0 ? (uint8_t)h.front : 0;
    }
    return 0;
}

// One scatter step per item, given origin, direction, t, object index and
// 12 random words.
int oracle_scatter(const rdc_scene_desc* desc, const float* o, const float* d, const float* t,
                   const int32_t* idx, const uint32_t* words, uint32_t n, float* o_out,
                   float* d_out) {
    const Scene<float> s = scene_from_desc<float>(desc);
    for (uint32_t i = 0; i < n; ++i) {
        if (idx[i] < 0 || (uint32_t)idx[i] >= s.objects.size()) return 2;
        Ray<float> r{v3(o[3 * i], o[3 * i + 1], o[3 * i + 2]), v3(d[3 * i], d[3 * i + 1], d[3 * i + 2])};
        Hit<float> h;
        h.index = idx[i];
        closest_hit(r, t[i], s.objects[idx[i]], &h);
        Ray<float> out;
        scatter(r, h, s.objects[idx[i]], words + 12 * (size_t)i, &out);
        o_out[3 * i] = out.origin.x;
        o_out[3 * i + 1] = out.origin.y;
        o_out[3 * i + 2] = out.origin.z;
        d_out[3 * i] = out.direction.x;
        d_out[3 * i + 1] = out.direction.y;
        d_out[3 * i + 2] = out.direction.z;
    }
    return 0;
}

void oracle_tonemap(const float* accum, uint32_t npix, uint32_t sample_count, uint8_t* out) {
    for (size_t i = 0; i < (size_t)npix * 4; ++i) out[i] = tonemap_channel(accum[i], sample_count);
}

// Camera::update_matrices in float, including cgmath's float inverse.
int oracle_camera_matrices(const rdc_camera* c, float view[16], float proj[16], float inv_view[16],
                           float inv_proj[16]) {
    const V3<float> eye = v3(c->position[0], c->position[1], c->position[2]);
    const V3<float> tgt = v3(c->target[0], c->target[1], c->target[2]);
    const V3<float> up = v3(c->up[0], c->up[1], c->up[2]);
    look_at_lh(eye, tgt, up, view);
    const float aspect = (float)c->resolution_x / (float)c->resolution_y;
    if (c->projection == RDC_PROJECTION_PERSPECTIVE) {
        perspective(c->fov_degrees, aspect, c->near_clip, c->far_clip, proj);
    } else {
        const float sz = c->ortho_size;
        ortho(-sz * aspect, sz * aspect, -sz, sz, c->near_clip, c->far_clip, proj);
    }
    if (!invert4_cgmath(view, inv_view)) return 1;
    if (!invert4_cgmath(proj, inv_proj)) return 1;
    return 0;
}

}  // extern "C"
