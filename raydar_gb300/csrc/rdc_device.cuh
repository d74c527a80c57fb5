// rdc_device.cuh -- device-side arithmetic of the path-tracing hot path.
//
// Every function evaluates the reference's float expressions in the
// reference's order (src/renderer/cpu.rs, src/utils/mod.rs,
// src/scene/world.rs); this file is compiled with -fmad=false so no a*b+c is
// contracted into an FMA (Rust never contracts), and with IEEE division and
// square root.  Per-ray and per-object subexpressions that the reference
// recomputes for every test are hoisted only where the hoisted value is the
// same float (d.d, o.d, o.o per ray; c.c, r*r, slab bounds per object).
#pragma once

#include <cstdint>

#include "rdc_internal.hpp"

namespace rdc {

// ------------------------------------------------------------- Philox RNG --
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
// easy as 1, 2, 3", SC'11): counter (pixel, sample, bounce*4+call, stream),
// key = 64-bit seed.  Each bounce draws up to 11 words from 3 blocks.
struct U4 {
    uint32_t x, y, z, w;
};

__device__ __forceinline__ U4 philox(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                     uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r > 0) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        const uint32_t lo0 = 0xD2511F53u * c0;
        const uint32_t hi0 = __umulhi(0xD2511F53u, c0);
        const uint32_t lo1 = 0xCD9E8D57u * c2;
        const uint32_t hi1 = __umulhi(0xCD9E8D57u, c2);
        const uint32_t n0 = hi1 ^ c1 ^ k0;
        const uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0;
        c1 = lo1;
        c2 = n2;
        c3 = lo0;
    }
    return U4{c0, c1, c2, c3};
}

// rand 0.8.5 Standard f32: top 24 bits * 2^-24 in [0, 1).
__device__ __forceinline__ float u01(uint32_t u) {
    return __fmul_rn(__uint2float_rn(u >> 8), 5.9604644775390625e-8f);
}

// rand 0.8.5 gen_range(-1.0..=1.0): ([1,2) from 23 bits - 1) * (2 + 2^-22) - 1.
__device__ __forceinline__ float upm1(uint32_t u) {
    const float v01 = __fsub_rn(__uint_as_float((u >> 9) | 0x3F800000u), 1.0f);
    return __fadd_rn(__fmul_rn(v01, __uint_as_float(0x40000001u)), -1.0f);
}

// ------------------------------------------------------------- vectors ----
struct V3 {
    float x, y, z;
};

__device__ __forceinline__ V3 mk(float x, float y, float z) { return V3{x, y, z}; }
__device__ __forceinline__ V3 vadd(V3 a, V3 b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ V3 vsub(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ V3 vmul(V3 a, float s) { return V3{a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ V3 vneg(V3 a) { return V3{-a.x, -a.y, -a.z}; }
__device__ __forceinline__ float vdot(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
__device__ __forceinline__ V3 vnormalize(V3 a) {
    const float inv = 1.0f / sqrtf(vdot(a, a));
    return vmul(a, inv);
}
__device__ __forceinline__ float rsignum(float a) { return a != a ? a : copysignf(1.0f, a); }

// --------------------------------------------------------- intersection ---
// Per-ray values every primitive test reuses (the same floats the reference
// recomputes inside each test).
struct RayPre {
    V3 o, d;
    float a;   // d.d
    float od;  // o.d
    float oo;  // o.o
};

__device__ __forceinline__ RayPre ray_pre(V3 o, V3 d) {
    RayPre r;
    r.o = o;
    r.d = d;
    r.a = vdot(d, d);
    r.od = vdot(o, d);
    r.oo = vdot(o, o);
    return r;
}

// hit_sphere, src/renderer/cpu.rs:34-62, then the first-minimum update of
// trace_ray (cpu.rs:345-349): replace only on a strictly smaller t.
__device__ __forceinline__ void sphere_test(const RayPre& r, float4 g0, float rr, int i,
                                            float& best, int& bidx) {
    const float dc = (r.d.x * g0.x + r.d.y * g0.y) + r.d.z * g0.z;
    const float k = r.od - dc;
    const float oc = (r.o.x * g0.x + r.o.y * g0.y) + r.o.z * g0.z;
    const float c = ((r.oo - 2.0f * oc) + g0.w) - rr;
    const float disc = k * k - r.a * c;
    if (disc >= 0.0f) {
        const float sq = sqrtf(disc);
        const float t1 = (-k - sq) / r.a;
        float t = t1;
        bool ok = t1 >= 0.0f;
        if (!ok) {
            const float t2 = (-k + sq) / r.a;
            t = t2;
            ok = t2 >= 0.0f;
        }
        if (ok && (bidx < 0 || t < best)) {
            best = t;
            bidx = i;
        }
    }
}

// hit_cube, src/renderer/cpu.rs:64-98 (true division per axis).
__device__ __forceinline__ void cube_test(const RayPre& r, float4 g0, float4 g1, int i,
                                          float& best, int& bidx) {
    const float tx1 = (g0.x - r.o.x) / r.d.x;
    const float tx2 = (g0.w - r.o.x) / r.d.x;
    const float ty1 = (g0.y - r.o.y) / r.d.y;
    const float ty2 = (g1.x - r.o.y) / r.d.y;
    const float tz1 = (g0.z - r.o.z) / r.d.z;
    const float tz2 = (g1.y - r.o.z) / r.d.z;
    const float tmin = fmaxf(fmaxf(fminf(tx1, tx2), fminf(ty1, ty2)), fminf(tz1, tz2));
    const float tmax = fminf(fminf(fmaxf(tx1, tx2), fmaxf(ty1, ty2)), fmaxf(tz1, tz2));
    if (!(tmax < 0.0f) && !(tmin > tmax)) {
        const float t = tmin < 0.0f ? tmax : tmin;
        if (bidx < 0 || t < best) {
            best = t;
            bidx = i;
        }
    }
}

// Brute-force closest hit over all objects in scene order.
__device__ __forceinline__ void intersect_all(const float4* __restrict__ geom,
                                              const int4* __restrict__ runs, int nruns,
                                              const RayPre& r, float& best, int& bidx) {
    best = __int_as_float(0x7f800000);
    bidx = -1;
    for (int q = 0; q < nruns; ++q) {
        const int4 run = runs[q];
        if (run.x == 0) {
#pragma unroll 4
            for (int i = run.y; i < run.z; ++i) {
                const float4 g0 = geom[2 * i];
                const float rr = geom[2 * i + 1].x;
                sphere_test(r, g0, rr, i, best, bidx);
            }
        } else {
#pragma unroll 2
            for (int i = run.y; i < run.z; ++i) {
                const float4 g0 = geom[2 * i];
                const float4 g1 = geom[2 * i + 1];
                cube_test(r, g0, g1, i, best, bidx);
            }
        }
    }
}

struct HitRec {
    V3 p, n;
    bool front;
};

// closest_hit, src/renderer/cpu.rs:354-394.
__device__ __forceinline__ HitRec closest_hit(V3 o, V3 d, float t, float4 hi, int kind) {
    HitRec h;
    h.p = vadd(o, vmul(d, t));
    const V3 c = mk(hi.x, hi.y, hi.z);
    V3 n;
    if (kind == 0) {
        n = vnormalize(vsub(h.p, c));
    } else {
        const V3 lp = vsub(h.p, c);
        const float hs = hi.w;
        const float xd = fabsf(fabsf(lp.x) - hs);
        const float yd = fabsf(fabsf(lp.y) - hs);
        const float zd = fabsf(fabsf(lp.z) - hs);
        if (xd < yd && xd < zd)
            n = mk(rsignum(lp.x), 0.0f, 0.0f);
        else if (yd < zd)
            n = mk(0.0f, rsignum(lp.y), 0.0f);
        else
            n = mk(0.0f, 0.0f, rsignum(lp.z));
    }
    h.front = vdot(n, d) <= 0.0f;
    h.n = h.front ? n : vneg(n);
    return h;
}

// random_in_unit_sphere, src/utils/mod.rs:47-55.
__device__ __forceinline__ V3 unit_sphere(uint32_t a, uint32_t b, uint32_t c) {
    return vnormalize(mk(upm1(a), upm1(b), upm1(c)));
}

// The hit branch of per_pixel (src/renderer/cpu.rs:262-328): new ray from a
// hit, the object's material and the bounce's random words w[0..10].
__device__ __forceinline__ void scatter(V3 d, const HitRec& h, const MatDev& m,
                                        const uint32_t* w, V3& o_out, V3& d_out) {
    const float rough = m.a.w;
    const float metallic = m.b.w;
    const float transmission = m.c.x;

    V3 diffuse = vadd(h.n, unit_sphere(w[0], w[1], w[2]));
    if (vdot(diffuse, h.n) < 0.0f) diffuse = vneg(diffuse);

    // reflect, src/utils/mod.rs:14-16: v - n * (v.n) * 2
    const float dn = vdot(d, h.n);
    const V3 perfect = vsub(d, vmul(vmul(h.n, dn), 2.0f));
    const V3 specular = vnormalize(vadd(perfect, vmul(unit_sphere(w[3], w[4], w[5]), rough)));

    const bool trans = u01(w[6]) < transmission;
    V3 dir;
    if (trans) {
        const float ratio = h.front ? m.c.y : m.c.z;
        const float r0 = h.front ? m.c.w : m.d.x;
        const V3 rd = vnormalize(d);
        const V3 nn = vneg(h.n);
        const float cos_theta = fminf(vdot(rd, nn), 1.0f);
        const float mm = 1.0f - cos_theta;
        const float m2 = mm * mm;
        const float m5 = mm * (m2 * m2);
        const float refl = r0 + (1.0f - r0) * m5;
        bool refracted = false;
        if (refl < u01(w[7])) {
            // can_refract, src/utils/mod.rs:37-44
            const float sin_theta = sqrtf(1.0f - cos_theta * cos_theta);
            refracted = ratio * sin_theta <= 1.0f;
        }
        if (refracted) {
            // refract, src/utils/mod.rs:25-35
            const V3 perp = vmul(vadd(rd, vmul(h.n, cos_theta)), ratio);
            const float s = -sqrtf(fabsf(1.0f - vdot(perp, perp)));
            const V3 rf = vadd(perp, vmul(h.n, s));
            dir = vnormalize(vadd(rf, vmul(unit_sphere(w[8], w[9], w[10]), rough)));
        } else {
            dir = specular;
        }
    } else if (u01(w[7]) < metallic) {
        dir = specular;
    } else if (u01(w[8]) < rough) {
        dir = diffuse;
    } else {
        dir = specular;
    }
    const V3 off = trans ? dir : h.n;
    o_out = vadd(h.p, vmul(off, 0.0001f));
    d_out = vdot(dir, dir) < 1e-10f ? h.n : dir;
}

// World::sample, src/scene/world.rs:17-31 (the dot with +Y is d.x*0 + d.y*1 + d.z*0).
__device__ __forceinline__ V3 world_sample(const SceneView& sc, V3 d) {
    if (sc.world_kind == 1u) return mk(sc.solid[0], sc.solid[1], sc.solid[2]);
    const float dy = (d.x * 0.0f + d.y * 1.0f) + d.z * 0.0f;
    const float cosine = dy / (sqrtf(vdot(d, d)) * 1.0f);
    const float amt = (cosine + 1.0f) * 0.5f;
    return mk(sc.bottom[0] + (sc.top[0] - sc.bottom[0]) * amt,
              sc.bottom[1] + (sc.top[1] - sc.bottom[1]) * amt,
              sc.bottom[2] + (sc.top[2] - sc.bottom[2]) * amt);
}

// Primary ray of pixel (x, y), src/renderer/cpu.rs:199-202 and 234-251.
__device__ __forceinline__ void primary_ray(const SceneView& sc, uint32_t x, uint32_t y, V3& o,
                                            V3& d) {
    const float u = __uint2float_rn(x) / __uint2float_rn(sc.width);
    const float v = 1.0f - __uint2float_rn(y) / __uint2float_rn(sc.height);
    const float clip[4] = {u * 2.0f - 1.0f, v * 2.0f - 1.0f, -1.0f, -1.0f};
    float cam[4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
        cam[i] = ((sc.inv_proj[i] * clip[0] + sc.inv_proj[4 + i] * clip[1]) +
                  sc.inv_proj[8 + i] * clip[2]) +
                 sc.inv_proj[12 + i] * clip[3];
    const float w = cam[3];
#pragma unroll
    for (int i = 0; i < 4; ++i) cam[i] = cam[i] / w;
    float wd[3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
        wd[i] = ((sc.inv_view[i] * cam[0] + sc.inv_view[4 + i] * cam[1]) +
                 sc.inv_view[8 + i] * cam[2]) +
                sc.inv_view[12 + i] * cam[3];
    o = mk(sc.cam_pos[0], sc.cam_pos[1], sc.cam_pos[2]);
    d = vneg(vnormalize(mk(wd[0], wd[1], wd[2])));
}

}  // namespace rdc
