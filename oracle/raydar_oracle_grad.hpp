// raydar_oracle_grad.hpp -- FP64 reference gradient of an image loss (TEST
// INFRASTRUCTURE ONLY: the checker of the CUDA adjoint).
//
// The estimator is the forward path of raydar_oracle.hpp (src/renderer/cpu.rs:
// 253-341) evaluated in double, with the same Philox words per bounce.  A
// path's radiance is
//     L = sum_k E(obj_k) + [miss after K hits] sky(d_K) * prod_k albedo(obj_k)
// (emission is added without attenuation, cpu.rs:330-341).  Its derivatives:
//   - emission E (the emitted radiance emission_color * emission_strength):
//     dL/dE(j) = number of hits on j;
//   - albedo: dL_c/dalbedo_c(j) = sky_c * sum over hits k on j of the product
//     of the other hits' albedos;
//   - roughness, two parts:
//     * pathwise: through the miss direction d_K, which every scatter after
//       the first roughness use moves.  Computed here by forward-mode
//       automatic differentiation: the roughness of the object hit at bounce
//       k is seeded as tangent slot k of a dual number, and the unchanged
//       path code (intersection, normal, reflect, refract, normalize, sky)
//       carries the tangents;
//     * lobe choice (score function): where a coin with a parameter-
//       dependent probability picked the lobe -- U_rough < roughness^2
//       (cpu.rs:309) or Schlick's R < U_fresnel (cpu.rs:296-297) -- the
//       probability P of the outcome taken is evaluated in dual numbers too,
//       and the path adds (radiance gathered after that vertex's scatter) *
//       dP/P for every slot.  R depends on the incoming direction, so its
//       tangents reach the roughness of every earlier bounce.
//     This is a different derivation from the CUDA backward kernel's
//     hand-written reverse sweep, so the two check each other.
// Discrete choices (which object is hit, which lobe, the diffuse flip, the
// front face) are those of the float path, recorded first and then held
// fixed: the gradient of the same path-replay estimator the CUDA kernels
// evaluate, computed in double.  (Re-deciding them in double would follow a
// different path wherever float and double rounding part ways, which after a
// few bounces off curved mirrors is common.)
#pragma once

#include <cmath>

#include "raydar_oracle.hpp"

namespace oracle {

constexpr int kGradSlots = 16;  // bounces with a roughness tangent slot each

// Forward-mode dual number: a value and kGradSlots partial derivatives, in R.
// DualT<double> is the reference gradient.  DualT<float> evaluates the same
// derivative with every intermediate in float, as the CUDA adjoint does: on a
// path whose derivative is ill-conditioned (hits a few ulp apart inside one
// object, where 1/t and grazing normals amplify rounding) the float and
// double evaluations part ways, and the float one says what FP32 can give.
// The operators are hidden friends, so the path code's implicit conversions
// (T(2), x * 0.0001f) resolve as for a plain class.
template <typename R>
struct DualT {
    R v;
    R d[kGradSlots];
    DualT() : v(R(0)) {
        for (int i = 0; i < kGradSlots; ++i) d[i] = R(0);
    }
    DualT(R x) : v(x) {  // NOLINT: implicit, as the path code writes T(2), T(0.0001f)
        for (int i = 0; i < kGradSlots; ++i) d[i] = R(0);
    }

    friend DualT operator+(const DualT& a, const DualT& b) {
        DualT r(a.v + b.v);
        for (int i = 0; i < kGradSlots; ++i) r.d[i] = a.d[i] + b.d[i];
        return r;
    }
    friend DualT operator-(const DualT& a, const DualT& b) {
        DualT r(a.v - b.v);
        for (int i = 0; i < kGradSlots; ++i) r.d[i] = a.d[i] - b.d[i];
        return r;
    }
    friend DualT operator-(const DualT& a) {
        DualT r(-a.v);
        for (int i = 0; i < kGradSlots; ++i) r.d[i] = -a.d[i];
        return r;
    }
    friend DualT operator*(const DualT& a, const DualT& b) {
        DualT r(a.v * b.v);
        for (int i = 0; i < kGradSlots; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
        return r;
    }
    friend DualT operator/(const DualT& a, const DualT& b) {
        DualT r(a.v / b.v);
        const R inv = R(1) / b.v;
        for (int i = 0; i < kGradSlots; ++i) r.d[i] = (a.d[i] - r.v * b.d[i]) * inv;
        return r;
    }
    friend bool operator<(const DualT& a, const DualT& b) { return a.v < b.v; }
    friend bool operator<=(const DualT& a, const DualT& b) { return a.v <= b.v; }
    friend bool operator>(const DualT& a, const DualT& b) { return a.v > b.v; }
    friend bool operator>=(const DualT& a, const DualT& b) { return a.v >= b.v; }
    friend bool operator==(const DualT& a, const DualT& b) { return a.v == b.v; }
    friend bool operator!=(const DualT& a, const DualT& b) { return a.v != b.v; }

    // Found by argument-dependent lookup from r_sqrt / r_fabs / r_signbit.
    friend DualT sqrt(const DualT& a) {
        DualT r(std::sqrt(a.v));
        const R g = r.v > R(0) ? R(0.5) / r.v : R(0);
        for (int i = 0; i < kGradSlots; ++i) r.d[i] = a.d[i] * g;
        return r;
    }
    friend DualT fabs(const DualT& a) { return std::signbit(a.v) ? -a : a; }
    friend bool signbit(const DualT& a) { return std::signbit(a.v); }
};
using Dual = DualT<double>;
using DualF = DualT<float>;

// One path's discrete history on the float path: the object hit, its front
// flag and the scatter choices per bounce, and whether it ended in a miss.
struct PathRecord {
    int nv = 0;
    bool missed = false;
    int obj[kGradSlots];
    bool front[kGradSlots];
    Choice ch[kGradSlots];
    V3<float> o[kGradSlots], d[kGradSlots];  // the ray reaching each vertex
    float t[kGradSlots];
    V3<float> d_end;  // the direction after the last vertex
};

// The float path of trace_path (src/renderer/cpu.rs:253-341), recorded.
inline void record_path(const Scene<float>& s, Ray<float> ray, uint32_t max_bounces, uint64_t seed,
                        uint32_t stream, uint32_t pixel, uint32_t sample, PathRecord* rec) {
    rec->nv = 0;
    rec->missed = false;
    for (uint32_t b = 0; b < max_bounces; ++b) {
        rec->d_end = ray.direction;
        const Hit<float> h = trace_ray(ray, s);
        if (h.index < 0) {
            rec->missed = true;
            return;
        }
        rec->o[rec->nv] = ray.origin;
        rec->d[rec->nv] = ray.direction;
        rec->t[rec->nv] = h.t;
        uint32_t w[12];
        bounce_words(seed, stream, pixel, sample, b, w);
        Ray<float> next;
        scatter(ray, h, s.objects[h.index], w, &next, &rec->ch[rec->nv]);
        rec->obj[rec->nv] = h.index;
        rec->front[rec->nv] = h.front;
        ++rec->nv;
        ray = next;
    }
    rec->d_end = ray.direction;
}

// A dual number with its value replaced and its tangents kept.
template <typename R>
inline DualT<R> at_value(const DualT<R>& a, double v) {
    DualT<R> r = a;
    r.v = (R)v;
    return r;
}
template <typename R>
inline V3<DualT<R>> at_value(const V3<DualT<R>>& a, V3<float> v) {
    return v3(at_value(a.x, v.x), at_value(a.y, v.y), at_value(a.z, v.z));
}

// Gradient of sum_p,c dL_dimage[p,c] * image[p,c] with image = the mean
// radiance of samples [s0, s0+n) of pixel p, for the pixels in [p0, p1).
// Each path is traced in float to fix its discrete history and its points;
// the tangents are then carried in double along that history, each vertex
// evaluated at the float path's ray and hit distance (re-tracing the values
// in double would drift from the float path by rounding that a few bounces
// off curved surfaces amplify, and the derivative would be taken elsewhere).  Adds into
// g_albedo (N*3), g_rough (N), g_emission (N*3); writes the mean image (RGB,
// double) of those pixels into image (npix*3) when it is not null.  Returns
// the number of paths whose double evaluation lost a recorded hit (grazing
// rays; they add no albedo or roughness term).
// g_rough receives both roughness parts; g_rough_path (when not null) the
// pathwise part alone.
// D: Dual (the reference) or DualF (the same derivative in float).
template <typename D>
inline uint64_t gradient_pixels(const Scene<float>& sf, const Scene<D>& s, uint32_t p0, uint32_t p1,
                                uint32_t s0, uint32_t n, uint32_t max_bounces, uint64_t seed, uint32_t stream,
                                const float* dl_dimage, double* g_albedo, double* g_rough, double* g_emission,
                                double* image, double* g_rough_path = nullptr) {
    uint64_t lost = 0;
    for (uint32_t pix = p0; pix < p1; ++pix) {
        const Ray<float> prim_f = primary_ray(sf, pix % s.width, pix / s.width);
        const Ray<D> prim = primary_ray(s, pix % s.width, pix / s.width);
        double w[3], img[3] = {0.0, 0.0, 0.0};
        for (int c = 0; c < 3; ++c) w[c] = (double)dl_dimage[3 * (size_t)pix + c] / (double)n;
        for (uint32_t k = 0; k < n; ++k) {
            PathRecord rec;
            record_path(sf, prim_f, max_bounces, seed, stream, pix, s0 + k, &rec);
            Ray<D> ray = prim;
            bool ok = true;
            // d log P / d(slot j) of the coin that decided vertex v's lobe (0 without one)
            double dlogp[kGradSlots][kGradSlots];
            for (int v = 0; v < rec.nv && ok; ++v) {
                Object<D> ob = s.objects[rec.obj[v]];
                // evaluate at the float path's ray and hit distance, with the
                // tangents carried in double
                ray.origin = at_value(ray.origin, rec.o[v]);
                ray.direction = at_value(ray.direction, rec.d[v]);
                D t;
                if (!hit_object(ray, ob, &t)) {
                    ok = false;
                    break;
                }
                t = at_value(t, rec.t[v]);
                Hit<D> h;
                h.index = rec.obj[v];
                closest_hit(ray, t, ob, &h);
                if (h.front != rec.front[v]) {  // grazing: keep the float path's side
                    h.front = rec.front[v];
                    h.normal = neg(h.normal);
                }
                ob.roughness.d[v] = 1.0;  // tangent slot v: this bounce's roughness
                uint32_t words[12];
                bounce_words(seed, stream, pix, s0 + k, (uint32_t)v, words);
                Ray<D> next;
                D pc;
                scatter(ray, h, ob, words, &next, &rec.ch[v], true, &pc);
                for (int j = 0; j < kGradSlots; ++j) dlogp[v][j] = (double)(pc.d[j] / pc.v);
                ray = next;
            }
            double light[3] = {0.0, 0.0, 0.0};
            for (int v = 0; v < rec.nv; ++v) {
                const Object<D>& ob = s.objects[rec.obj[v]];
                const double e[3] = {ob.emission_color.x.v * ob.emission_strength.v,
                                     ob.emission_color.y.v * ob.emission_strength.v,
                                     ob.emission_color.z.v * ob.emission_strength.v};
                for (int c = 0; c < 3; ++c) {
                    light[c] += e[c];
                    g_emission[3 * (size_t)rec.obj[v] + c] += w[c];
                }
            }
            if (!ok) ++lost;
            // radiance gathered after each vertex's scatter: later emission + the sky term
            double after[kGradSlots][3];
            if (ok) {
                double S[3] = {0.0, 0.0, 0.0};
                if (rec.missed) {
                    const V3<D> sky = world_sample(s, at_value(ray.direction, rec.d_end));
                    const double sk[3] = {sky.x.v, sky.y.v, sky.z.v};
                    for (int c = 0; c < 3; ++c) {
                        double prod = 1.0;
                        for (int v = 0; v < rec.nv; ++v) {
                            const V3<D>& a = s.objects[rec.obj[v]].albedo;
                            prod *= c == 0 ? a.x.v : (c == 1 ? a.y.v : a.z.v);
                        }
                        S[c] = sk[c] * prod;
                    }
                }
                for (int v = rec.nv - 1; v >= 0; --v) {
                    for (int c = 0; c < 3; ++c) after[v][c] = S[c];
                    const Object<D>& ob = s.objects[rec.obj[v]];
                    S[0] += ob.emission_color.x.v * ob.emission_strength.v;
                    S[1] += ob.emission_color.y.v * ob.emission_strength.v;
                    S[2] += ob.emission_color.z.v * ob.emission_strength.v;
                }
                for (int v = 0; v < rec.nv; ++v) {
                    const double wv = w[0] * after[v][0] + w[1] * after[v][1] + w[2] * after[v][2];
                    if (wv == 0.0) continue;
                    for (int j = 0; j <= v; ++j) g_rough[rec.obj[j]] += wv * dlogp[v][j];
                }
            }
            if (rec.missed && ok) {
                const V3<D> sky = world_sample(s, at_value(ray.direction, rec.d_end));
                const D skyc[3] = {sky.x, sky.y, sky.z};
                for (int c = 0; c < 3; ++c) {
                    double alb[kGradSlots];
                    double prod = 1.0;
                    for (int v = 0; v < rec.nv; ++v) {
                        const V3<D>& a = s.objects[rec.obj[v]].albedo;
                        alb[v] = c == 0 ? a.x.v : (c == 1 ? a.y.v : a.z.v);
                        prod *= alb[v];
                    }
                    light[c] += skyc[c].v * prod;
                    for (int v = 0; v < rec.nv; ++v) {
                        double others = 1.0;
                        for (int m = 0; m < rec.nv; ++m)
                            if (m != v) others *= alb[m];
                        g_albedo[3 * (size_t)rec.obj[v] + c] += w[c] * skyc[c].v * others;
                        g_rough[rec.obj[v]] += w[c] * prod * skyc[c].d[v];
                        if (g_rough_path) g_rough_path[rec.obj[v]] += w[c] * prod * skyc[c].d[v];
                    }
                }
            }
            for (int c = 0; c < 3; ++c) img[c] += light[c];
        }
        if (image)
            for (int c = 0; c < 3; ++c) image[3 * (size_t)pix + c] = img[c] / (double)n;
    }
    return lost;
}

}  // namespace oracle
