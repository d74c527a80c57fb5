// host_checks.cpp -- a standalone driver for the host-only C++ of the
// library (the .rscn reader and writer, the camera matrices) and the CPU
// oracle, compiled by tests/test_sanitizers.py with AddressSanitizer and
// UndefinedBehaviorSanitizer (-fno-sanitize-recover: the first report ends
// the run with a non-zero status).  No GPU, no CUDA runtime calls.
//
//   host_checks <default.rscn> <benchmark.rscn>
//
// Work: parse both reference scenes (size query, then full), write them back
// and parse the result again; parse every truncation of a scene file at a
// stride of offsets and a few thousand single-byte corruptions (each must
// return a status, not crash); recompute random cameras' matrices; run the
// oracle's render, pixel render, gradient, intersect and scatter entry points
// on a parsed scene with random inputs.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <random>
#include <sstream>
#include <string>
#include <vector>

#include "raydar_cuda.h"

namespace rdc {
// The library's per-thread error message (rdc_api.cpp); the driver keeps the last one.
std::string g_last;
void set_thread_error(const std::string& msg) { g_last = msg; }
}  // namespace rdc

extern "C" {
int oracle_render(const rdc_scene_desc* desc, uint32_t s0, uint32_t n, uint32_t max_bounces, uint64_t seed,
                  uint32_t stream, float* accum, uint64_t* segments_out, int threads);
int oracle_render_pixels(const rdc_scene_desc* desc, const uint32_t* pixels, uint32_t npix, uint32_t s0, uint32_t n,
                         uint32_t max_bounces, uint64_t seed, uint32_t stream, float* accum, uint64_t* segments_out);
int oracle_gradient(const rdc_scene_desc* desc, uint32_t s0, uint32_t n, uint32_t max_bounces, uint64_t seed,
                    uint32_t stream, const float* dl_dimage, double* g_albedo, double* g_rough, double* g_emission,
                    double* image, int threads, uint64_t* lost_out, double* g_rough_path);
int oracle_intersect(const rdc_scene_desc* desc, const float* o, const float* d, uint32_t n, float* t_out,
                     int32_t* idx_out, float* normal_out, uint8_t* front_out);
int oracle_scatter(const rdc_scene_desc* desc, const float* o, const float* d, const float* t, const int32_t* idx,
                   const uint32_t* words, uint32_t n, float* o_out, float* d_out);
}

namespace {

int g_fail = 0;
#define CHECK(c)                                                        \
    do {                                                                \
        if (!(c)) {                                                     \
            std::fprintf(stderr, "check failed at line %d: %s\n", __LINE__, #c); \
            ++g_fail;                                                   \
        }                                                               \
    } while (0)

std::string slurp(const char* path) {
    std::ifstream f(path, std::ios::binary);
    std::stringstream ss;
    ss << f.rdbuf();
    return ss.str();
}

// Parse text; on success fill objs and scene and return RDC_OK.
rdc_status parse(const std::string& text, rdc_scene_desc& scene, std::vector<rdc_object>& objs) {
    uint32_t n = 0;
    rdc_status st = rdc_scene_parse_rscn(text.data(), text.size(), &scene, nullptr, 0, &n);
    if (st != RDC_OK) return st;
    objs.assign(n, rdc_object{});
    st = rdc_scene_parse_rscn(text.data(), text.size(), &scene, objs.data(), n, &n);
    return st;
}

void scene_round_trip(const std::string& text) {
    rdc_scene_desc sc;
    std::vector<rdc_object> objs;
    CHECK(parse(text, sc, objs) == RDC_OK);
    size_t len = 0;
    CHECK(rdc_scene_write_rscn(&sc, nullptr, 0, &len) == RDC_OK || len > 0);
    std::vector<char> buf(len + 1);
    CHECK(rdc_scene_write_rscn(&sc, buf.data(), buf.size(), &len) == RDC_OK);
    rdc_scene_desc sc2;
    std::vector<rdc_object> objs2;
    CHECK(parse(std::string(buf.data(), len), sc2, objs2) == RDC_OK);
    CHECK(objs2.size() == objs.size());
    CHECK(std::memcmp(&sc2.camera, &sc.camera, sizeof(rdc_camera)) == 0);
    if (!objs.empty()) CHECK(std::memcmp(objs2.data(), objs.data(), objs.size() * sizeof(rdc_object)) == 0);
}

void malformed(const std::string& text, std::mt19937& rng) {
    const size_t stride = text.size() > 4000 ? text.size() / 2000 : 1;
    for (size_t cut = 0; cut < text.size(); cut += stride) {
        rdc_scene_desc sc;
        std::vector<rdc_object> objs;
        (void)parse(text.substr(0, cut), sc, objs);  // any status, no crash
    }
    std::uniform_int_distribution<size_t> pos(0, text.size() - 1);
    std::uniform_int_distribution<int> byte(0, 255);
    for (int k = 0; k < 3000; ++k) {
        std::string t = text;
        t[pos(rng)] = (char)byte(rng);
        rdc_scene_desc sc;
        std::vector<rdc_object> objs;
        (void)parse(t, sc, objs);
    }
}

void cameras(std::mt19937& rng) {
    std::normal_distribution<float> g(0.0f, 5.0f);
    std::uniform_real_distribution<float> u(0.0f, 1.0f);
    for (int k = 0; k < 2000; ++k) {
        rdc_camera c;
        std::memset(&c, 0, sizeof(c));
        for (int i = 0; i < 3; ++i) {
            c.position[i] = g(rng);
            c.target[i] = g(rng);
        }
        c.up[1] = 1.0f;
        c.resolution_x = 1 + (uint32_t)(u(rng) * 4000);
        c.resolution_y = 1 + (uint32_t)(u(rng) * 4000);
        c.projection = u(rng) < 0.5f ? RDC_PROJECTION_PERSPECTIVE : RDC_PROJECTION_ORTHOGRAPHIC;
        c.fov_degrees = 1.0f + 170.0f * u(rng);
        c.ortho_size = 0.1f + 20.0f * u(rng);
        c.near_clip = 0.01f;
        c.far_clip = 1000.0f;
        (void)rdc_camera_update_matrices(&c);
    }
}

void oracle_work(const std::string& text, std::mt19937& rng) {
    rdc_scene_desc sc;
    std::vector<rdc_object> objs;
    CHECK(parse(text, sc, objs) == RDC_OK);
    sc.camera.resolution_x = 12;
    sc.camera.resolution_y = 8;
    CHECK(rdc_camera_update_matrices(&sc.camera) == RDC_OK);
    const uint32_t npix = 12 * 8;
    std::vector<float> acc(npix * 4, 0.0f);
    uint64_t segs = 0;
    CHECK(oracle_render(&sc, 0, 2, 12, 7, 0, acc.data(), &segs, 2) == 0);
    CHECK(segs > 0);
    std::vector<uint32_t> px = {0, 5, npix - 1};
    std::vector<float> acc2(px.size() * 4, 0.0f);
    CHECK(oracle_render_pixels(&sc, px.data(), (uint32_t)px.size(), 0, 2, 12, 7, 0, acc2.data(), &segs) == 0);
    const size_t n = objs.size();
    std::vector<float> dl(npix * 3, 0.5f);
    std::vector<double> ga(n * 3), gr(n), ge(n * 3), img(npix * 3), grp(n);
    uint64_t lost = 0;
    CHECK(oracle_gradient(&sc, 0, 2, 6, 9, 0, dl.data(), ga.data(), gr.data(), ge.data(), img.data(), 2, &lost,
                          grp.data()) == 0);
    std::normal_distribution<float> g(0.0f, 1.0f);
    const uint32_t m = 256;
    std::vector<float> o(m * 3), d(m * 3), t(m), nrm(m * 3), oo(m * 3), dd(m * 3);
    std::vector<int32_t> idx(m);
    std::vector<uint8_t> fr(m);
    std::vector<uint32_t> w(m * 12);
    for (uint32_t i = 0; i < m; ++i)
        for (int a = 0; a < 3; ++a) {
            o[3 * i + a] = sc.camera.position[a];
            d[3 * i + a] = g(rng);
        }
    CHECK(oracle_intersect(&sc, o.data(), d.data(), m, t.data(), idx.data(), nrm.data(), fr.data()) == 0);
    for (auto& x : w) x = (uint32_t)rng();
    uint32_t k = 0;
    for (uint32_t i = 0; i < m; ++i)
        if (idx[i] >= 0) {
            for (int a = 0; a < 3; ++a) {
                o[3 * k + a] = o[3 * i + a];
                d[3 * k + a] = d[3 * i + a];
            }
            t[k] = t[i];
            idx[k] = idx[i];
            ++k;
        }
    if (k) CHECK(oracle_scatter(&sc, o.data(), d.data(), t.data(), idx.data(), w.data(), k, oo.data(), dd.data()) == 0);
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 3) {
        std::fprintf(stderr, "usage: host_checks <default.rscn> <benchmark.rscn>\n");
        return 2;
    }
    std::mt19937 rng(12345);
    for (int a = 1; a < 3; ++a) {
        const std::string text = slurp(argv[a]);
        CHECK(!text.empty());
        scene_round_trip(text);
        malformed(text, rng);
        oracle_work(text, rng);
    }
    cameras(rng);
    std::printf("host checks: %s\n", g_fail ? "FAILED" : "ok");
    return g_fail ? 1 : 0;
}
