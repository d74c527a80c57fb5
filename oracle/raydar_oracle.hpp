// raydar_oracle.hpp -- CPU restatement of Raydar's path-tracing hot path.
//
// TEST INFRASTRUCTURE ONLY.  This is the checker the CUDA backend is compared
// against; only tests/, the smoke check and the benchmark's CPU-baseline leg
// may load it.  Nothing in the shipped library includes or links it.
//
// It restates, operation for operation and in the same evaluation order, the
// Rust CPU renderer of bvpav/raydar:
//   src/renderer/cpu.rs:34-62    hit_sphere (expanded quadratic)
//   src/renderer/cpu.rs:64-98    hit_cube (slab test, true division)
//   src/renderer/cpu.rs:344-352  trace_ray (first minimum wins)
//   src/renderer/cpu.rs:354-394  closest_hit (normals, front face)
//   src/renderer/cpu.rs:233-342  per_pixel (camera ray, bounce loop, scatter)
//   src/renderer/cpu.rs:193-219  render_next_sample (accumulation)
//   src/renderer/cpu.rs:221-230  print_frame_buffer (tone map)
//   src/utils/mod.rs:6-55        reflect, refract, can_refract, random_in_unit_sphere
//   src/scene/world.rs:17-31     World::sample
//   src/scene/camera.rs:210-231  update_matrices (look_at_lh, perspective, ortho, invert)
// Third-party arithmetic it restates from the crates' published behaviour
// (pinned in the reference Cargo.lock): cgmath 0.18.0 (dot = (x*x'+y*y')+z*z',
// normalize = v * (1/|v|), lerp = a + (b-a)*t, Matrix4*Vector4 as a left-to-right
// column combination), rand 0.8.5 (Standard f32 = (u>>8)*2^-24;
// gen_range(-1.0..=1.0) = UniformFloat::new_inclusive: ((u>>9 | 1.0 bits) - 1)
// * scale + low with scale = RN(2/(1-2^-23))), ordered-float 4.6.0 (NaN is the
// largest key), f32::min/max (a NaN operand yields the other one).
//
// The reference draws from an unseeded thread_rng (src/utils/mod.rs:48); here
// every draw comes from a counter-based Philox4x32-10 stream (Salmon et al.,
// "Parallel random numbers: as easy as 1, 2, 3", SC'11) keyed by
// (seed, pixel, sample, bounce, slot), the same contract the CUDA backend
// uses, so single paths can be replayed.  The draw ORDER per bounce follows
// cpu.rs:268-309: s1 (3 words, slots 0-2), s2 (slots 3-5), U_transmission
// (slot 6), then U_fresnel or U_metallic (slot 7), then s3 (slots 8-10) or
// U_roughness (slot 8).
//
// PARITY STATUS: camera matrices (view, projection and both inverses, bit
// for bit) are pinned against the matrices the reference serialised into
// scenes/default.rscn and scenes/benchmark.rscn.
// The rest of the path is pinned only by hand-derived known answers: the
// reference has no tests, no fixtures and cannot be built here (no Rust
// toolchain), so per-path arithmetic is "parity unpinned" against the
// reference's own outputs.
//
// Build with -ffp-contract=off (Rust never contracts a*b+c into an FMA; GCC
// does on aarch64 by default) and without -ffast-math.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../include/raydar_cuda.h"

namespace oracle {

// Square root, absolute value and sign bit through argument-dependent lookup:
// the same path code runs on float, double and the forward-mode dual numbers
// of raydar_oracle_grad.hpp.
template <typename T> static inline T r_sqrt(T a) { using std::sqrt; return sqrt(a); }
template <typename T> static inline T r_fabs(T a) { using std::fabs; return fabs(a); }
template <typename T> static inline bool r_signbit(T a) { using std::signbit; return signbit(a); }

// ---------------------------------------------------------------- vectors --
template <typename T>
struct V3 {
    T x, y, z;
};

template <typename T> static inline V3<T> v3(T x, T y, T z) { return V3<T>{x, y, z}; }
template <typename T> static inline V3<T> add(V3<T> a, V3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <typename T> static inline V3<T> sub(V3<T> a, V3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <typename T> static inline V3<T> mul(V3<T> a, T s) { return {a.x * s, a.y * s, a.z * s}; }
template <typename T> static inline V3<T> mulv(V3<T> a, V3<T> b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <typename T> static inline V3<T> divv(V3<T> a, V3<T> b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
template <typename T> static inline V3<T> neg(V3<T> a) { return {-a.x, -a.y, -a.z}; }
// cgmath InnerSpace::dot: sum of the element-wise product, summed x, y, z in order.
template <typename T> static inline T dot(V3<T> a, V3<T> b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
template <typename T> static inline T magnitude2(V3<T> a) { return dot(a, a); }
template <typename T> static inline T magnitude(V3<T> a) { return r_sqrt(magnitude2(a)); }
// cgmath normalize = normalize_to(1) = self * (1 / magnitude).
template <typename T> static inline V3<T> normalize(V3<T> a) { return mul(a, T(1) / magnitude(a)); }
template <typename T> static inline V3<T> cross(V3<T> a, V3<T> b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}

// Rust f32::min / f32::max: a NaN operand yields the other operand.  Equal
// zeros of opposite sign resolve to -0 for min and +0 for max (the CUDA
// fminf/fmaxf behaviour; the reference leaves that case unspecified).
template <typename T> static inline T rmin(T a, T b) {
    if (a != a) return b;
    if (b != b) return a;
    if (a == b) return r_signbit(a) ? a : b;
    return a < b ? a : b;
}
template <typename T> static inline T rmax(T a, T b) {
    if (a != a) return b;
    if (b != b) return a;
    if (a == b) return r_signbit(a) ? b : a;
    return a > b ? a : b;
}
// Rust f32::signum: +-1 by the sign bit (so +-0 map to +-1), NaN stays NaN.
template <typename T> static inline T rsignum(T a) {
    if (a != a) return a;
    return r_signbit(a) ? T(-1) : T(1);
}

// ------------------------------------------------------------- Philox RNG --
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11): 10 rounds of two
// 32x32->64 multiplies with a Weyl-sequence key schedule.
struct Philox4 {
    uint32_t v[4];
};

static inline Philox4 philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                    uint32_t k0, uint32_t k1) {
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
    const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
    for (int r = 0; r < 10; ++r) {
        if (r > 0) {
            k0 += W0;
            k1 += W1;
        }
        const uint64_t p0 = (uint64_t)M0 * c0;
        const uint64_t p1 = (uint64_t)M1 * c2;
        const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        const uint32_t n0 = hi1 ^ c1 ^ k0;
        const uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0;
        c1 = lo1;
        c2 = n2;
        c3 = lo0;
    }
    return Philox4{{c0, c1, c2, c3}};
}

// The 12 random words of one bounce: counter (pixel, sample, bounce*4+call,
// stream) for call = 0,1,2; key = the 64-bit seed.
static inline void bounce_words(uint64_t seed, uint32_t stream, uint32_t pixel, uint32_t sample,
                                uint32_t bounce, uint32_t words[12]) {
    const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
    for (uint32_t call = 0; call < 3; ++call) {
        Philox4 r = philox4x32_10(pixel, sample, bounce * 4u + call, stream, k0, k1);
        for (int i = 0; i < 4; ++i) words[call * 4 + i] = r.v[i];
    }
}

// rand 0.8.5 Standard for f32: 24 high bits scaled by 2^-24, in [0, 1).
static inline float uniform01(uint32_t u) {
    return (float)(u >> 8) * (1.0f / 16777216.0f);
}

// rand 0.8.5 gen_range(-1.0..=1.0) for f32 (UniformFloat::new_inclusive +
// sample): a [1,2) float from 23 random bits, minus 1, times scale, plus low.
static inline float uniform_pm1(uint32_t u) {
    uint32_t bits = (u >> 9) | 0x3F800000u;
    float v12;
    std::memcpy(&v12, &bits, 4);
    const float v01 = v12 - 1.0f;
    // scale = RN(2 / (1 - 2^-23)) = 2 + 2^-22; the rand loop that lowers it
    // until scale*max_rand + low <= high leaves it unchanged for [-1, 1].
    uint32_t sbits = 0x40000001u;
    float scale;
    std::memcpy(&scale, &sbits, 4);
    const float prod = v01 * scale;
    return prod + -1.0f;
}

// ---------------------------------------------------------------- scene ---
template <typename T>
struct Object {
    uint32_t geometry;
    V3<T> center;
    T radius, side_length;
    V3<T> albedo;
    T roughness, metallic;
    V3<T> emission_color;
    T emission_strength, transmission, ior;
};

template <typename T>
struct Scene {
    V3<T> cam_pos;
    T inv_view[16], inv_proj[16];
    uint32_t width, height;
    uint32_t world_kind;
    V3<T> top, bottom, solid;
    std::vector<Object<T>> objects;
};

template <typename T>
static inline Scene<T> scene_from_desc(const rdc_scene_desc* d) {
    Scene<T> s;
    s.cam_pos = v3<T>(d->camera.position[0], d->camera.position[1], d->camera.position[2]);
    for (int i = 0; i < 16; ++i) {
        s.inv_view[i] = (T)d->camera.inverse_view_matrix[i];
        s.inv_proj[i] = (T)d->camera.inverse_proj_matrix[i];
    }
    s.width = d->camera.resolution_x;
    s.height = d->camera.resolution_y;
    s.world_kind = d->world.kind;
    s.top = v3<T>(d->world.top_color[0], d->world.top_color[1], d->world.top_color[2]);
    s.bottom = v3<T>(d->world.bottom_color[0], d->world.bottom_color[1], d->world.bottom_color[2]);
    s.solid = v3<T>(d->world.solid_color[0], d->world.solid_color[1], d->world.solid_color[2]);
    s.objects.resize(d->object_count);
    for (uint32_t i = 0; i < d->object_count; ++i) {
        const rdc_object& o = d->objects[i];
        Object<T>& q = s.objects[i];
        q.geometry = o.geometry;
        q.center = v3<T>(o.center[0], o.center[1], o.center[2]);
        q.radius = o.radius;
        q.side_length = o.side_length;
        q.albedo = v3<T>(o.material.albedo[0], o.material.albedo[1], o.material.albedo[2]);
        q.roughness = o.material.roughness;
        q.metallic = o.material.metallic;
        q.emission_color = v3<T>(o.material.emission_color[0], o.material.emission_color[1],
                                 o.material.emission_color[2]);
        q.emission_strength = o.material.emission_strength;
        q.transmission = o.material.transmission;
        q.ior = o.material.ior;
    }
    return s;
}

// ----------------------------------------------------------- intersection --
template <typename T>
struct Ray {
    V3<T> origin, direction;
};

// src/renderer/cpu.rs:34-62
template <typename T>
static inline bool hit_sphere(const Ray<T>& ray, V3<T> center, T radius, T* t_out) {
    const V3<T> o = ray.origin, d = ray.direction;
    const T a = dot(d, d);
    const T k = dot(o, d) - dot(d, center);
    const T c = ((dot(o, o) - T(2) * dot(o, center)) + dot(center, center)) - radius * radius;
    const T disc = k * k - a * c;
    if (disc < T(0)) return false;
    const T sq = r_sqrt(disc);
    const T t1 = (-k - sq) / a;
    const T t2 = (-k + sq) / a;
    if (t1 >= T(0)) {
        *t_out = t1;
        return true;
    }
    if (t2 >= T(0)) {
        *t_out = t2;
        return true;
    }
    return false;
}

// src/renderer/cpu.rs:64-98
template <typename T>
static inline bool hit_cube(const Ray<T>& ray, V3<T> center, T side, T* t_out) {
    const T h = side * T(0.5);
    const V3<T> half = v3(h, h, h);
    const V3<T> mn = sub(center, half);
    const V3<T> mx = add(center, half);
    const V3<T> t1 = divv(sub(mn, ray.origin), ray.direction);
    const V3<T> t2 = divv(sub(mx, ray.origin), ray.direction);
    const T tmin = rmax(rmax(rmin(t1.x, t2.x), rmin(t1.y, t2.y)), rmin(t1.z, t2.z));
    const T tmax = rmin(rmin(rmax(t1.x, t2.x), rmax(t1.y, t2.y)), rmax(t1.z, t2.z));
    if (tmax < T(0)) return false;
    if (tmin > tmax) return false;
    *t_out = (tmin < T(0)) ? tmax : tmin;
    return true;
}

template <typename T>
static inline bool hit_object(const Ray<T>& ray, const Object<T>& ob, T* t) {
    if (ob.geometry == RDC_GEOMETRY_SPHERE) return hit_sphere(ray, ob.center, ob.radius, t);
    return hit_cube(ray, ob.center, ob.side_length, t);
}

// ordered_float::OrderedFloat ordering: NaN compares greater than everything.
template <typename T>
static inline bool ordered_less(T a, T b) {
    const bool an = a != a, bn = b != b;
    if (an) return false;
    if (bn) return true;
    return a < b;
}

template <typename T>
struct Hit {
    int32_t index;  // -1: miss
    T t;
    bool front;
    V3<T> position, normal;
};

// src/renderer/cpu.rs:354-394
template <typename T>
static inline void closest_hit(const Ray<T>& ray, T t, const Object<T>& ob, Hit<T>* h) {
    const V3<T> p = add(ray.origin, mul(ray.direction, t));  // Ray::at, cpu.rs:30-32
    V3<T> n;
    if (ob.geometry == RDC_GEOMETRY_SPHERE) {
        n = normalize(sub(p, ob.center));
    } else {
        const V3<T> lp = sub(p, ob.center);
        const T hs = ob.side_length / T(2);
        const T xd = r_fabs(r_fabs(lp.x) - hs);
        const T yd = r_fabs(r_fabs(lp.y) - hs);
        const T zd = r_fabs(r_fabs(lp.z) - hs);
        if (xd < yd && xd < zd)
            n = v3(rsignum(lp.x), T(0), T(0));
        else if (yd < zd)
            n = v3(T(0), rsignum(lp.y), T(0));
        else
            n = v3(T(0), T(0), rsignum(lp.z));
    }
    const bool front = dot(n, ray.direction) <= T(0);
    if (!front) n = neg(n);
    h->t = t;
    h->front = front;
    h->position = p;
    h->normal = n;
}

// src/renderer/cpu.rs:344-352: brute force over the objects in scene order,
// min_by_key keeps the FIRST minimum.
template <typename T>
static inline Hit<T> trace_ray(const Ray<T>& ray, const Scene<T>& s) {
    Hit<T> h;
    h.index = -1;
    T best = T(0);
    for (size_t i = 0; i < s.objects.size(); ++i) {
        T t;
        if (!hit_object(ray, s.objects[i], &t)) continue;
        if (h.index < 0 || ordered_less(t, best)) {
            best = t;
            h.index = (int32_t)i;
        }
    }
    if (h.index >= 0) closest_hit(ray, best, s.objects[h.index], &h);
    return h;
}

// ------------------------------------------------------------- shading ----
// src/utils/mod.rs:14-16
template <typename T>
static inline V3<T> reflect(V3<T> v, V3<T> n) {
    return sub(v, mul(mul(n, dot(v, n)), T(2)));
}

// src/utils/mod.rs:25-35 (the unit-length asserts are not evaluated)
template <typename T>
static inline V3<T> refract(V3<T> v, V3<T> n, T ratio) {
    const T cos_theta = rmin(dot(v, neg(n)), T(1));
    const V3<T> perp = mul(add(v, mul(n, cos_theta)), ratio);
    const T s = -r_sqrt(r_fabs(T(1) - magnitude2(perp)));
    const V3<T> par = mul(n, s);
    return add(perp, par);
}

// src/utils/mod.rs:37-44
template <typename T>
static inline bool can_refract(V3<T> v, V3<T> n, T ratio) {
    const T cos_theta = rmin(dot(v, neg(n)), T(1));
    const T sin_theta = r_sqrt(T(1) - cos_theta * cos_theta);
    return ratio * sin_theta <= T(1);
}

// src/utils/mod.rs:47-55: normalised U[-1,1]^3 (drawn x, y, z).
template <typename T>
static inline V3<T> random_in_unit_sphere(const uint32_t* w) {
    const V3<T> r = v3<T>(uniform_pm1(w[0]), uniform_pm1(w[1]), uniform_pm1(w[2]));
    return normalize(r);
}

// src/scene/world.rs:17-31
template <typename T>
static inline V3<T> world_sample(const Scene<T>& s, V3<T> d) {
    if (s.world_kind == RDC_WORLD_SOLID_COLOR) return s.solid;
    // cos = d.(0,1,0) / (|d| * |up|); the dot is exactly d.y and |up| = 1.
    const V3<T> up = v3(T(0), T(1), T(0));
    const T cosine = dot(d, up) / (magnitude(d) * magnitude(up));
    const T amt = (cosine + T(1)) * T(0.5);
    return add(s.bottom, mul(sub(s.top, s.bottom), amt));  // cgmath lerp
}

// The discrete choices of one scatter: which lobe, the diffuse flip, the
// transmission branch and the |dir|^2 < 1e-10 fallback, and which coin with
// a parameter-dependent probability decided the lobe: the roughness coin
// (U_rough < roughness^2, cpu.rs:309) or the Fresnel coin (Schlick's R <
// U_fresnel where refraction is possible, cpu.rs:296-297).  The gradient
// oracle records them on the float path and replays that path in double with
// them held fixed (the same estimator, evaluated at higher precision).
enum { kLobeDiffuse = 0, kLobeSpecular = 1, kLobeRefract = 2 };
struct Choice {
    int lobe;
    bool flip, trans, to_normal;
    bool rough_coin, fresnel_coin;
};

// The hit branch of per_pixel, src/renderer/cpu.rs:262-333, given the
// bounce's random words.  Updates the ray.  ch: if force, the choices to
// take; else, when not null, receives the choices taken.  coin_p, when not
// null, receives the probability of the outcome the deciding coin gave
// (T(1) when no such coin decided).
template <typename T>
static inline void scatter(const Ray<T>& ray, const Hit<T>& h, const Object<T>& ob,
                           const uint32_t* w, Ray<T>* out, Choice* ch = nullptr, bool force = false,
                           T* coin_p = nullptr) {
    const T roughness = ob.roughness * ob.roughness;
    const T metallic = ob.metallic;
    const T transmission = ob.transmission;

    V3<T> diffuse = add(h.normal, random_in_unit_sphere<T>(w + 0));
    const bool flip = force ? ch->flip : dot(diffuse, h.normal) < T(0);
    if (flip) diffuse = neg(diffuse);

    const V3<T> perfect = reflect(ray.direction, h.normal);
    const V3<T> offset2 = mul(random_in_unit_sphere<T>(w + 3), roughness);
    const V3<T> specular = normalize(add(perfect, offset2));

    const bool transmission_ray = force ? ch->trans : (T)uniform01(w[6]) < transmission;
    V3<T> direction;
    int lobe = kLobeSpecular;
    bool rough_coin = false, fresnel_coin = false;
    T p_coin = T(1);
    if (transmission_ray) {
        T ior = ob.ior;
        if (h.front) ior = T(1) / ior;
        const V3<T> rd = normalize(ray.direction);
        const T cos_theta = rmin(dot(rd, neg(h.normal)), T(1));
        const T q = (ior - T(1)) / (ior + T(1));
        const T r0 = q * q;                          // powi(2)
        const T m = T(1) - cos_theta;
        const T m2 = m * m;
        const T m5 = m * (m2 * m2);                  // powi(5), square-and-multiply
        const T refl = r0 + (T(1) - r0) * m5;
        bool refr;
        if (force) {
            refr = ch->lobe == kLobeRefract;
            fresnel_coin = ch->fresnel_coin;
        } else {
            const bool can = can_refract(rd, h.normal, ior);
            refr = refl < (T)uniform01(w[7]) && can;
            fresnel_coin = can;  // under total internal reflection the coin decides nothing
        }
        if (fresnel_coin) p_coin = refr ? T(1) - refl : refl;
        if (refr) {
            const V3<T> refracted = refract(rd, h.normal, ior);
            const V3<T> offset3 = mul(random_in_unit_sphere<T>(w + 8), roughness);
            direction = normalize(add(refracted, offset3));
            lobe = kLobeRefract;
        } else {
            direction = specular;
        }
    } else if (force ? ch->lobe == kLobeSpecular && (T)uniform01(w[7]) < metallic
                     : (T)uniform01(w[7]) < metallic) {
        direction = specular;
    } else {
        rough_coin = true;
        if (force ? ch->lobe == kLobeDiffuse : (T)uniform01(w[8]) < roughness) {
            direction = diffuse;
            lobe = kLobeDiffuse;
            p_coin = roughness;
        } else {
            direction = specular;
            p_coin = T(1) - roughness;
        }
    }
    const V3<T> off = transmission_ray ? direction : h.normal;
    out->origin = add(h.position, mul(off, T(0.0001f)));
    out->direction = direction;
    const bool to_normal = force ? ch->to_normal : magnitude2(out->direction) < T(1e-10f);
    if (to_normal) out->direction = h.normal;
    if (ch && !force) *ch = Choice{lobe, flip, transmission_ray, to_normal, rough_coin, fresnel_coin};
    if (coin_p) *coin_p = p_coin;
}

// Primary ray of pixel (x, y): src/renderer/cpu.rs:199-202, 234-251.
template <typename T>
static inline Ray<T> primary_ray(const Scene<T>& s, uint32_t x, uint32_t y) {
    const T u = (T)(float)x / (T)(float)s.width;
    const T v = T(1) - (T)(float)y / (T)(float)s.height;
    const T clip[4] = {u * T(2) - T(1), v * T(2) - T(1), T(-1), T(-1)};
    T cam[4];
    for (int i = 0; i < 4; ++i)  // Matrix4 * Vector4, columns combined left to right
        cam[i] = ((s.inv_proj[0 * 4 + i] * clip[0] + s.inv_proj[1 * 4 + i] * clip[1]) +
                  s.inv_proj[2 * 4 + i] * clip[2]) +
                 s.inv_proj[3 * 4 + i] * clip[3];
    const T w = cam[3];
    for (int i = 0; i < 4; ++i) cam[i] = cam[i] / w;
    T wd[4];
    for (int i = 0; i < 4; ++i)
        wd[i] = ((s.inv_view[0 * 4 + i] * cam[0] + s.inv_view[1 * 4 + i] * cam[1]) +
                 s.inv_view[2 * 4 + i] * cam[2]) +
                s.inv_view[3 * 4 + i] * cam[3];
    Ray<T> r;
    r.origin = s.cam_pos;
    r.direction = neg(normalize(v3(wd[0], wd[1], wd[2])));
    return r;
}

// One path: src/renderer/cpu.rs:253-341.  Returns RGB light; counts segments.
template <typename T>
static inline V3<T> trace_path(const Scene<T>& s, Ray<T> ray, uint32_t max_bounces, uint64_t seed,
                               uint32_t stream, uint32_t pixel, uint32_t sample,
                               uint64_t* segments) {
    V3<T> light = v3(T(0), T(0), T(0));
    V3<T> atten = v3(T(1), T(1), T(1));
    for (uint32_t b = 0; b < max_bounces; ++b) {
        ++*segments;
        const Hit<T> h = trace_ray(ray, s);
        if (h.index >= 0) {
            const Object<T>& ob = s.objects[h.index];
            uint32_t w[12];
            bounce_words(seed, stream, pixel, sample, b, w);
            Ray<T> next;
            scatter(ray, h, ob, w, &next);
            ray = next;
            atten = mulv(atten, ob.albedo);
            light = add(light, mul(ob.emission_color, ob.emission_strength));
        } else {
            light = add(light, mulv(world_sample(s, ray.direction), atten));
            break;
        }
    }
    return light;
}

// Accumulate samples [s0, s0+n) of one pixel into acc[4] in sample order:
// src/renderer/cpu.rs:198-210.
template <typename T>
static inline void render_pixel(const Scene<T>& s, uint32_t pix, uint32_t s0, uint32_t n,
                                uint32_t max_bounces, uint64_t seed, uint32_t stream, T* acc,
                                uint64_t* segments) {
    const uint32_t x = pix % s.width, y = pix / s.width;
    const Ray<T> prim = primary_ray(s, x, y);
    for (uint32_t k = 0; k < n; ++k) {
        const V3<T> c = trace_path(s, prim, max_bounces, seed, stream, pix, s0 + k, segments);
        acc[0] = acc[0] + c.x;
        acc[1] = acc[1] + c.y;
        acc[2] = acc[2] + c.z;
        acc[3] = acc[3] + T(1);
    }
}

// src/renderer/cpu.rs:221-230: ((sum / N).clamp(0, 1) * 255) as u8.
static inline uint8_t tonemap_channel(float sum, uint32_t n) {
    float v = sum / (float)n;
    if (v != v) return 0;  // Rust `as u8` maps NaN to 0
    v = v < 0.0f ? 0.0f : (v > 1.0f ? 1.0f : v);
    return (uint8_t)(v * 255.0f);
}

// ------------------------------------------------------------- camera -----
// Camera::update_matrices, src/scene/camera.rs:210-231, restated from the
// published definitions of cgmath 0.18 look_at_lh / perspective / ortho.
// Matrices are column-major m[col*4+row].
template <typename T>
static inline void look_at_lh(V3<T> eye, V3<T> center, V3<T> up, T m[16]) {
    const V3<T> f = normalize(sub(center, eye));
    const V3<T> s = normalize(cross(up, f));
    const V3<T> u = cross(f, s);
    const T cols[16] = {s.x, u.x, f.x, T(0), s.y, u.y, f.y, T(0),
                        s.z, u.z, f.z, T(0), -dot(eye, s), -dot(eye, u), -dot(eye, f), T(1)};
    for (int i = 0; i < 16; ++i) m[i] = cols[i];
}

template <typename T>
static inline void perspective(T fovy_deg, T aspect, T near, T far, T m[16]) {
    const T half = (fovy_deg * (T)(3.14159265358979323846 / 180.0)) / T(2);
    const T f = T(1) / std::tan(half);
    for (int i = 0; i < 16; ++i) m[i] = T(0);
    m[0] = f / aspect;
    m[5] = f;
    m[10] = (far + near) / (near - far);
    m[11] = T(-1);
    m[14] = (T(2) * far * near) / (near - far);
}

template <typename T>
static inline void ortho(T l, T r, T b, T t, T n, T f, T m[16]) {
    for (int i = 0; i < 16; ++i) m[i] = T(0);
    m[0] = T(2) / (r - l);
    m[5] = T(2) / (t - b);
    m[10] = T(-2) / (f - n);
    m[12] = -(r + l) / (r - l);
    m[13] = -(t + b) / (t - b);
    m[14] = -(f + n) / (f - n);
    m[15] = T(1);
}

// cgmath 0.18.0 Matrix3::determinant for a matrix given as m[col][row]:
// m00 (m11 m22 - m21 m12) - m10 (m01 m22 - m21 m02) + m20 (m01 m12 - m11 m02),
// evaluated left to right in float.
static inline float det3(const float m[3][3]) {
    return m[0][0] * (m[1][1] * m[2][2] - m[2][1] * m[1][2]) - m[1][0] * (m[0][1] * m[2][2] - m[2][1] * m[0][2]) +
           m[2][0] * (m[0][1] * m[1][2] - m[1][1] * m[0][2]);
}

// cgmath 0.18.0 Matrix4::invert in float (the reference's call at
// src/scene/camera.rs:229-230).  a is column-major, a[c*4+r].
//   determinant: Laplace expansion along row 0, a00 d0 - a10 d1 + a20 d2 - a30 d3,
//     where d_k is the Matrix3::new(...) of rows 1..3 without column k, built
//     column by column from the ORIGINAL ROWS (so it is the transposed minor).
//   singular when |det| <= f32::EPSILON (approx's ulps_eq! against zero; the
//     reference then unwraps None and panics).
//   entry (column i, row j) = det3(minor) * sign * (1 / det), the minor being
//     Matrix3::from_cols of the transpose's rows != i, each truncated at j,
//     sign = -1 when i + j is odd.
static inline bool invert4_cgmath(const float a[16], float out[16]) {
    auto at = [&](int c, int r) { return a[c * 4 + r]; };
    float d[4];
    for (int k = 0; k < 4; ++k) {
        float m[3][3];
        int mc = 0;
        for (int c = 0; c < 4; ++c) {
            if (c == k) continue;
            // Matrix3::new(c0r0, c0r1, c0r2, ...) with c0 = (a[1][c], ...) over the kept columns
            m[0][mc] = at(c, 1);
            m[1][mc] = at(c, 2);
            m[2][mc] = at(c, 3);
            ++mc;
        }
        d[k] = det3(m);
    }
    const float det = at(0, 0) * d[0] - at(1, 0) * d[1] + at(2, 0) * d[2] - at(3, 0) * d[3];
    if (!(std::fabs(det) > 1.1920929e-7f)) return false;  // also NaN
    const float inv_det = 1.0f / det;
    for (int i = 0; i < 4; ++i) {
        for (int j = 0; j < 4; ++j) {
            float m[3][3];
            int mc = 0;
            for (int rr = 0; rr < 4; ++rr) {  // transpose's vector rr = row rr of a
                if (rr == i) continue;
                int mr = 0;
                for (int cc = 0; cc < 4; ++cc) {
                    if (cc == j) continue;
                    m[mc][mr++] = at(cc, rr);
                }
                ++mc;
            }
            const float sign = ((i + j) & 1) ? -1.0f : 1.0f;
            out[i * 4 + j] = det3(m) * sign * inv_det;
        }
    }
    return true;
}

}  // namespace oracle
