// rdc_flatten.hpp -- host-side flattening of an rdc_scene_desc into the device
// layout (shared by rdc_scene_upload and rdc_render_static).
//
// Output arrays, all indexed in scene order where per object:
//   rec[]   float4 records the intersection loop stages in shared memory:
//           per sphere run, pairs of consecutive spheres (packed for the
//           kernels' two-wide float instructions), 3 float4 per pair
//             (c1.x, c2.x, c1.y, c2.y) (c1.z, c2.z, s1, s2) (c1.c1, c2.c2, r1*r1, r2*r2)
//           s = c.c - q rounded down, q the sphere filter's margin-widened
//           r^2 (sphere_filter_s)
//           (an odd run's last pair repeats its sphere in the second half;
//           the kernel masks that half out);
//           per cube run, a header (R, 0, 0, 0) with R >= |centre| + half
//           side * sqrt(3) over the run (cube_run_bound), then pairs of
//           consecutive cubes, 3 float4 per pair
//             (min1.x, min2.x, max1.x, max2.x) and likewise y, z
//           (an odd run's last pair repeats its cube, as for spheres)
//   hit[i]  (cx, cy, cz, side/2): what closest_hit needs
//   mat[i]  MatDev
//   runs[r] (geometry, first object, end object, first record) per maximal
//           run of one geometry kind
// The constants are the exact floats the reference computes inline
// (src/renderer/cpu.rs:39-43, 65-71, 262-263, 282-293, 332-333); compiled
// with -ffp-contract=off.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>

#include "raydar_cuda.h"
#include "rdc_internal.hpp"

namespace rdc {

struct FlatCounts {
    uint32_t nobj = 0;
    uint32_t nruns = 0;
    uint32_t nrec = 0;  // float4 records
};

// Sizes of the flattened arrays (geometry kinds must be valid).
inline FlatCounts flat_counts(const rdc_scene_desc* sc) {
    FlatCounts f;
    f.nobj = sc->object_count;
    uint32_t i = 0;
    while (i < f.nobj) {
        const uint32_t kind = sc->objects[i].geometry;
        uint32_t j = i;
        while (j < f.nobj && sc->objects[j].geometry == kind) ++j;
        const uint32_t len = j - i;
        f.nrec += (kind == RDC_GEOMETRY_SPHERE) ? 3u * ((len + 1u) / 2u) : 1u + 3u * ((len + 1u) / 2u);
        ++f.nruns;
        i = j;
    }
    return f;
}

inline MatDev flat_material(const rdc_object& o) {
    const rdc_material& m = o.material;
    MatDev md;
    md.a = make_float4(m.albedo[0], m.albedo[1], m.albedo[2], m.roughness * m.roughness);
    md.b = make_float4(m.emission_color[0] * m.emission_strength, m.emission_color[1] * m.emission_strength,
                       m.emission_color[2] * m.emission_strength, m.metallic);
    const float ratio_front = 1.0f / m.ior;
    const float qf = (ratio_front - 1.0f) / (ratio_front + 1.0f);
    const float qb = (m.ior - 1.0f) / (m.ior + 1.0f);
    md.c = make_float4(m.transmission, ratio_front, m.ior, qf * qf);
    int kind = (int)o.geometry;
    float kind_bits;
    std::memcpy(&kind_bits, &kind, 4);
    md.d = make_float4(qb * qb, kind_bits, 0, 0);
    return md;
}

// The sphere filter's per-sphere constant (sphere_candidates,
// rdc_device.cuh): s <= c.c - q with q >= r^2 + 2^-16 (2 c.c + r^2) + 2^-70,
// computed in double (c.c and q within 2^-51 relative of exact, far inside
// the 2^-50 (c.c + q) subtracted) and rounded down to float.
inline float sphere_filter_s(const float c[3], float rr) {
    const double cc = (double)c[0] * c[0] + (double)c[1] * c[1] + (double)c[2] * c[2];
    const double q = ((double)rr + std::ldexp(2.0 * cc + (double)rr, -16) + 0x1p-70) * (1.0 + 0x1p-40);
    const double v = cc - q;
    const double s = v - std::fabs(v) * 0x1p-45 - std::ldexp(cc + q, -50);
    float f = (float)s;
    if ((double)f > s) f = std::nextafter(f, -INFINITY);
    return f;
}

// R of a cube run's header: at least |centre| + half side * sqrt(3) for each
// cube of objects [i, j), with 1e-4 relative slack, rounded up to float.
inline float cube_run_bound(const rdc_scene_desc* sc, uint32_t i, uint32_t j) {
    double R = 0.0;
    for (uint32_t p = i; p < j; ++p) {
        const rdc_object& q = sc->objects[p];
        const double cl = (double)q.center[0] * q.center[0] + (double)q.center[1] * q.center[1] +
                          (double)q.center[2] * q.center[2];
        const double h = std::fabs((double)(q.side_length * 0.5f));
        R = std::max(R, std::sqrt(cl) + h * 1.7320508075688772);
    }
    R *= 1.0001;
    float f = (float)R;
    if ((double)f < R) f = std::nextafter(f, INFINITY);
    return f;
}

// Fill the arrays sized by flat_counts; returns whether every object allows
// the kernels' guarded fast path (cube_fast_div_ok, sphere_fast_ok).
inline bool flatten(const rdc_scene_desc* sc, float4* rec, float4* hit, MatDev* mat, int4* runs) {
    const uint32_t n = sc->object_count;
    bool fast_div = true;
    uint32_t r = 0, off = 0, i = 0;
    while (i < n) {
        const uint32_t kind = sc->objects[i].geometry;
        uint32_t j = i;
        while (j < n && sc->objects[j].geometry == kind) ++j;
        runs[r++] = make_int4((int)kind, (int)i, (int)j, (int)off);
        if (kind == RDC_GEOMETRY_SPHERE) {
            for (uint32_t p = i; p < j; p += 2) {
                const rdc_object& s1 = sc->objects[p];
                const rdc_object& s2 = sc->objects[p + 1 < j ? p + 1 : p];
                const float* c1 = s1.center;
                const float* c2 = s2.center;
                const float cc1 = (c1[0] * c1[0] + c1[1] * c1[1]) + c1[2] * c1[2];
                const float cc2 = (c2[0] * c2[0] + c2[1] * c2[1]) + c2[2] * c2[2];
                const float rr1 = s1.radius * s1.radius, rr2 = s2.radius * s2.radius;
                rec[off++] = make_float4(c1[0], c2[0], c1[1], c2[1]);
                rec[off++] = make_float4(c1[2], c2[2], sphere_filter_s(c1, rr1), sphere_filter_s(c2, rr2));
                rec[off++] = make_float4(cc1, cc2, rr1, rr2);
                fast_div = fast_div && sphere_fast_ok(s1.center, s1.radius) && sphere_fast_ok(s2.center, s2.radius);
            }
        } else {
            rec[off++] = make_float4(cube_run_bound(sc, i, j), 0.0f, 0.0f, 0.0f);
            for (uint32_t p = i; p < j; p += 2) {
                const rdc_object& q1 = sc->objects[p];
                const rdc_object& q2 = sc->objects[p + 1 < j ? p + 1 : p];
                const float h1 = q1.side_length * 0.5f, h2 = q2.side_length * 0.5f;
                const float* c1 = q1.center;
                const float* c2 = q2.center;
                for (int k = 0; k < 3; ++k)
                    rec[off++] = make_float4(c1[k] - h1, c2[k] - h2, c1[k] + h1, c2[k] + h2);
                for (const rdc_object* q : {&q1, &q2}) {
                    const float h = q->side_length * 0.5f;
                    const float* c = q->center;
                    const float4 g0 = make_float4(c[0] - h, c[0] + h, c[1] - h, c[1] + h);
                    const float4 g1 = make_float4(c[2] - h, c[2] + h, 0.0f, 0.0f);
                    fast_div = fast_div && cube_fast_div_ok(q->side_length, g0, g1);
                }
            }
        }
        i = j;
    }
    for (uint32_t k = 0; k < n; ++k) {
        const rdc_object& o = sc->objects[k];
        if (o.geometry == RDC_GEOMETRY_SPHERE)
            hit[k] = make_float4(o.center[0], o.center[1], o.center[2], 0.0f);
        else
            hit[k] = make_float4(o.center[0], o.center[1], o.center[2], o.side_length / 2.0f);
        mat[k] = flat_material(o);
    }
    return fast_div;
}

}  // namespace rdc
