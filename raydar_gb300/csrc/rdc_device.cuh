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

// Bounds-checked build (-DRDC_BOUNDS_CHECK=1, libraydar_cuda_checked.so): the
// stand-in for a memory checker.  Every data-dependent index into a device
// array goes through checked_index, which counts an index outside [0, n) in
// *oob and substitutes 0 (every such array has at least one element), so a
// stray index is reported (RDC_ERR_DEVICE at the next synchronisation)
// instead of faulting, and never traps.  The normal build compiles it away.
#ifndef RDC_BOUNDS_CHECK
#define RDC_BOUNDS_CHECK 0
#endif

__device__ __forceinline__ long long checked_index(unsigned long long* oob, long long i, long long n) {
#if RDC_BOUNDS_CHECK
    if (i >= 0 && i < n) return i;
    atomicAdd(oob, 1ull);
    return 0;
#else
    (void)oob;
    (void)n;
    return i;
#endif
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
// cgmath normalize: v * RN(1 / RN(sqrt(v.v))); __frcp_rn is the IEEE quotient 1/x.
__device__ __forceinline__ V3 vnormalize(V3 a) {
    const float inv = __frcp_rn(__fsqrt_rn(vdot(a, a)));
    return vmul(a, inv);
}
__device__ __forceinline__ float rsignum(float a) { return a != a ? a : copysignf(1.0f, a); }

// --------------------------------------------------------- intersection ---
// Division.  The reference divides with IEEE round-to-nearest (`/` in Rust).
// Along one ray every slab test divides by the same three direction
// components and every sphere test by the same d.d, so the kernels divide by
// multiplying with a per-ray correctly rounded reciprocal y = RN(1/b) and
// applying Markstein's final correction step (P. Markstein, "Computation of
// elementary functions on the IBM RISC System/6000 processor", IBM J. Res.
// Dev. 34(1), 1990): q0 = RN(a*y) is a faithful quotient, the residual
// a - b*q0 is exact in an FMA, and RN(q0 + residual*y) is exactly RN(a/b) --
// the IEEE quotient, bit for bit -- as long as a, b, the quotient and the
// residual stay clear of overflow and the subnormal range.  The guards below
// (per ray: direction components in [2^-40, 16], origin components 0 or in
// [2^-60, 2^50], d.d in [2^-34, 2^10]; per scene: cube sides > 0 and slab
// bounds 0 or in [2^-60, 2^60], sphere centres and radii finite and at most
// 2^50; per sphere hit: numerator in [2^-60, 2^60])
// keep every operand there; a ray outside them takes IEEE division.  The
// same guards (with origins and sphere centres and radii at most 2^50) keep
// every value of the sphere candidate pass finite.
__device__ __forceinline__ float div_recip(float a, float b, float y) {
    const float q0 = __fmul_rn(a, y);
    const float r = __fmaf_rn(-q0, b, a);
    return __fmaf_rn(r, y, q0);
}

// A 32-byte record (two float4, 32-byte aligned) with one 256-bit read-only
// load: half the load instructions and L1 wavefronts of two 128-bit loads
// when the lanes of a warp read different records (BVH nodes, primitives,
// materials).
__device__ __forceinline__ void ldg_pair(const float4* p, float4& a, float4& b) {
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
        : "l"(p));
}

__device__ __forceinline__ bool in_range(float v, float lo, float hi) {
    const float m = fabsf(v);
    return m >= lo && m <= hi;
}

// Two-wide float arithmetic (Blackwell's packed FP32x2 instructions).  Each
// component is rounded exactly like the scalar instruction, so pairing two
// spheres, or the two slab planes of one axis, changes no bit; it halves the
// issue slots the FP32 work takes in this issue-bound loop.
//
// Contraction: ptxas fuses a packed multiply into a following packed add
// (one rounding instead of the reference's two) even for .rn instructions
// under -fmad=false, and folds fma(a, b, -0) + c the same way.  A packed
// product is therefore computed as fma.rn(a, b, z) with z = (-0, -0) taken
// from a kernel parameter: RN(a*b + -0) is exactly RN(a*b) for every input
// (a zero product keeps its sign), and ptxas cannot prove z is zero, so the
// product is rounded on its own as the reference rounds it.
__device__ __forceinline__ float2 f2(float x, float y) { return make_float2(x, y); }
#define RDC_F32X2_BINARY(name, op)                                                           \
    __device__ __forceinline__ float2 name(float2 a, float2 b) {                               \
        float2 d;                                                                              \
        asm("{\n\t.reg .b64 ra, rb, rd;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t" \
            op " rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;\n\t}"                                  \
            : "=f"(d.x), "=f"(d.y)                                                             \
            : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));                                         \
        return d;                                                                              \
    }
RDC_F32X2_BINARY(add2, "add.rn.f32x2")
RDC_F32X2_BINARY(sub2, "sub.rn.f32x2")  // a - b (IEEE: a + (-b))
#undef RDC_F32X2_BINARY
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) {
    float2 d;
    asm("{\n\t.reg .b64 ra, rb, rc, rd;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
        "mov.b64 rc, {%6, %7};\n\tfma.rn.f32x2 rd, ra, rb, rc;\n\tmov.b64 {%0, %1}, rd;\n\t}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
    return d;
}
// RN(a*b) per component; nz must be the (-0, -0) kernel parameter.
__device__ __forceinline__ float2 mul2(float2 a, float2 b, float2 nz) { return fma2(a, b, nz); }

// Two quotients by one divisor b (reciprocal y = RN(1/b), nb = -b): the
// Markstein step above on both components.
__device__ __forceinline__ float2 div2_recip(float2 a, float2 nb, float2 y, float2 nz) {
    const float2 q0 = mul2(a, y, nz);
    const float2 r = fma2(q0, nb, a);
    return fma2(r, y, q0);
}

// Per-ray values every primitive test reuses (the same floats the reference
// recomputes inside each test) and the reciprocals of the divisors.
struct RayPre {
    V3 o, d;
    float a;   // d.d
    float od;  // o.d
    float oo;  // o.o
    float ra;  // RN(1/a)
    V3 rd;     // RN(1/d) per component
    bool fast; // operands inside the exact-reciprocal-division range
    float2 nz; // (-0, -0), opaque to the compiler (see mul2)
    float P;   // 2^-15 a oo: the per-ray part of the sphere filter's margin
    float ol1; // |o.x| + |o.y| + |o.z| >= |o|: the cube filter's growth
};

__device__ __forceinline__ RayPre ray_pre(V3 o, V3 d, float2 nz) {
    RayPre r;
    r.nz = nz;
    r.o = o;
    r.d = d;
    r.a = vdot(d, d);
    r.od = vdot(o, d);
    r.oo = vdot(o, o);
    r.ra = __frcp_rn(r.a);
    r.P = (r.a * 3.0517578e-05f /* 2^-15 */) * r.oo;
    r.ol1 = (fabsf(o.x) + fabsf(o.y)) + fabsf(o.z);
    r.rd = mk(__frcp_rn(d.x), __frcp_rn(d.y), __frcp_rn(d.z));
    const float D0 = 9.094947e-13f /* 2^-40 */, D1 = 16.0f;
    const float O0 = 8.6736174e-19f /* 2^-60 */, O1 = 1.1258999e15f /* 2^50 */;
    r.fast = in_range(d.x, D0, D1) && in_range(d.y, D0, D1) && in_range(d.z, D0, D1) &&
             (o.x == 0.0f || in_range(o.x, O0, O1)) && (o.y == 0.0f || in_range(o.y, O0, O1)) &&
             (o.z == 0.0f || in_range(o.z, O0, O1)) && in_range(r.a, 5.820766e-11f /* 2^-34 */, 1024.0f);
    return r;
}

template <bool Fast>
__device__ __forceinline__ float sphere_div(float num, const RayPre& r) {
    if (Fast) {
        if (in_range(num, 8.6736174e-19f, 1.1529215e18f)) return div_recip(num, r.a, r.ra);
    }
    return num / r.a;
}

// hit_sphere (src/renderer/cpu.rs:34-62), pass 1: a bit mask of the spheres
// of a run (up to 32, packed pairs, rdc_flatten.hpp) that can return a hit,
// two spheres per instruction.  Pass 2 (sphere_exact) decides each
// candidate with the reference's own arithmetic, so pass 1 only has to be
// conservative: it may keep a sphere the reference misses, never drop one
// it hits.
//
// Exact pass 1 (Fast = false): the reference's discriminant itself; disc < 0
// (sign bit set: disc is never -0 since k*k >= +0) returns None.
//
// Filter (Fast = true, range-guarded operands: no overflow, a >= 2^-34): as
// FMA chains, b = o.d - c.d (from the reference's own o.d) and e = (o.o + s)
// - 2 o.c, where s = c.c - q rounded down and q = r^2 + 2^-16 (2 c.c + r^2)
// + 2^-70 rounded up (flatten), and P = 2^-15 a o.o per ray; the filter's
// discriminant is disc' = RN(b^2 + RN(P - a e)).  Exactly, with w = o - c,
// b = w.d and e = |w|^2 - q, and b^2 - a(|w|^2 - r^2) = A (r^2 - rho^2) = Q
// (Lagrange's identity; A = d.d, rho the distance from c to the ray's line).
// With u = 2^-24 and S = |o| + |c|, first-order rounding bounds: the
// reference's disc is within u A (21 S^2 + 6 r^2) of Q; the filter's b within
// 6u sqrt(A) S of w.d and 10u sqrt(A) S of the reference's k, e within
// 8u S^2 + 5u q of |w|^2 - q; so disc' >= disc_ref + M - u A (45 S^2 +
// 15 r^2), where the margin M = A (q - r^2) + P >= 256u A (S^2 + r^2)
// (2 c.c + 2 o.o >= S^2).  Hence disc' >= disc_ref + 40u A S^2: disc_ref >= 0
// keeps the sphere.  9 lane operations per sphere against the exact pass's
// 21; the filter keeps spheres passing within about sqrt(r^2 + 2^-16 (2|o|^2
// + 2|c|^2 + r^2)) of the line, a band far narrower than the spheres
// themselves at the scales scenes use.  Spheres behind the origin whose line
// passes that close are kept too and rejected by pass 2: a cull of them here
// (2 more operations per sphere) measured 9% slower overall.
template <bool Fast, int Unroll>
__device__ __forceinline__ uint32_t sphere_candidates(const float4* __restrict__ pr, int n,
                                                      const RayPre& r) {
    const float2 dx = f2(r.d.x, r.d.x), dy = f2(r.d.y, r.d.y), dz = f2(r.d.z, r.d.z);
    const float2 ox = f2(r.o.x, r.o.x), oy = f2(r.o.y, r.o.y), oz = f2(r.o.z, r.o.z);
    // Each sphere's decision is the sign bit of a word (clear = candidate),
    // shifted into the mask with one funnel shift: sphere j of the chunk ends
    // at bit n-1-j.  A NaN discriminant (possible only off the fast path) is
    // kept or dropped by its sign bit; either is right, as the reference
    // returns None for it and pass 2 rejects a kept one.
    uint32_t m = 0;
    const int np = (n + 1) >> 1;
    if (Fast) {
        const float2 na = f2(-r.a, -r.a), P = f2(r.P, r.P);
        const float2 od = f2(r.od, r.od), oo = f2(r.oo, r.oo);
        const float2 ndx = f2(-r.d.x, -r.d.x), ndy = f2(-r.d.y, -r.d.y), ndz = f2(-r.d.z, -r.d.z);
        const float2 mx = f2(-2.0f * r.o.x, -2.0f * r.o.x), my = f2(-2.0f * r.o.y, -2.0f * r.o.y),
                     mz = f2(-2.0f * r.o.z, -2.0f * r.o.z);
#pragma unroll Unroll
        for (int p = 0; p < np; ++p) {
            const float4 A = pr[3 * p];
            const float4 B = pr[3 * p + 1];
            const float2 cx = f2(A.x, A.y), cy = f2(A.z, A.w), cz = f2(B.x, B.y);
            const float2 b = fma2(ndz, cz, fma2(ndy, cy, fma2(ndx, cx, od)));
            const float2 e = fma2(mz, cz, fma2(my, cy, fma2(mx, cx, add2(oo, f2(B.z, B.w)))));  // B.zw = s
            const float2 disc = fma2(b, b, fma2(na, e, P));
            const uint32_t w0 = __float_as_uint(disc.x);
            const uint32_t w1 = __float_as_uint(disc.y);
            m = __funnelshift_l(~w0, m, 1);
            m = __funnelshift_l(~w1, m, 1);
        }
    } else {
        const float2 od = f2(r.od, r.od), oo = f2(r.oo, r.oo), a = f2(r.a, r.a);
#pragma unroll Unroll
        for (int p = 0; p < np; ++p) {
            const float4 A = pr[3 * p];
            const float4 B = pr[3 * p + 1];
            const float4 C = pr[3 * p + 2];
            const float2 cx = f2(A.x, A.y), cy = f2(A.z, A.w), cz = f2(B.x, B.y);
            const float2 cc = f2(C.x, C.y), rr = f2(C.z, C.w);
            const float2 dc = add2(add2(mul2(dx, cx, r.nz), mul2(dy, cy, r.nz)), mul2(dz, cz, r.nz));
            const float2 k = sub2(od, dc);
            const float2 oc = add2(add2(mul2(ox, cx, r.nz), mul2(oy, cy, r.nz)), mul2(oz, cz, r.nz));
            const float2 c = sub2(add2(sub2(oo, add2(oc, oc)), cc), rr);
            const float2 disc = sub2(mul2(k, k, r.nz), mul2(a, c, r.nz));
            m = __funnelshift_l(~__float_as_uint(disc.x), m, 1);
            m = __funnelshift_l(~__float_as_uint(disc.y), m, 1);
        }
    }
    if (2 * np > n) m >>= 1;  // drop the padding half of an odd chunk
    return m;
}

// hit_sphere pass 2 for one candidate (run-relative index j of the chunk's
// records), then the first-minimum update of trace_ray (cpu.rs:345-349):
// replace only on a strictly smaller t.  Candidates are visited in scene
// order, so the tie rule is the reference's.
template <bool Fast>
__device__ __forceinline__ void sphere_exact(const float4* __restrict__ pr, int j, int obj,
                                             const RayPre& r, float& best, int& bidx) {
    const float* q = reinterpret_cast<const float*>(pr + 3 * (j >> 1)) + (j & 1);
    const float cx = q[0], cy = q[2], cz = q[4], cc = q[8], rr = q[10];
    const float dc = (r.d.x * cx + r.d.y * cy) + r.d.z * cz;
    const float k = r.od - dc;
    const float oc = (r.o.x * cx + r.o.y * cy) + r.o.z * cz;
    const float c = ((r.oo - 2.0f * oc) + cc) - rr;
    const float disc = k * k - r.a * c;
    const float sq = __fsqrt_rn(disc);
    const float t1 = sphere_div<Fast>(-k - sq, r);
    float t = t1;
    bool ok = t1 >= 0.0f;
    if (!ok) {
        const float t2 = sphere_div<Fast>(-k + sq, r);
        t = t2;
        ok = t2 >= 0.0f;
    }
    if (ok && (bidx < 0 || t < best)) {
        best = t;
        bidx = obj;
    }
}

// hit_cube, src/renderer/cpu.rs:64-98: the two slab planes of each axis
// divided as a pair; X, Y, Z hold (min, max) of each axis.
template <bool Fast>
__device__ __forceinline__ void cube_slab(float2 X, float2 Y, float2 Z, int i, const RayPre& r, float& best,
                                          int& bidx) {
    const float2 ax = sub2(X, f2(r.o.x, r.o.x));
    const float2 ay = sub2(Y, f2(r.o.y, r.o.y));
    const float2 az = sub2(Z, f2(r.o.z, r.o.z));
    float2 tx, ty, tz;
    if (Fast) {
        tx = div2_recip(ax, f2(-r.d.x, -r.d.x), f2(r.rd.x, r.rd.x), r.nz);
        ty = div2_recip(ay, f2(-r.d.y, -r.d.y), f2(r.rd.y, r.rd.y), r.nz);
        tz = div2_recip(az, f2(-r.d.z, -r.d.z), f2(r.rd.z, r.rd.z), r.nz);
    } else {
        tx = f2(ax.x / r.d.x, ax.y / r.d.x);
        ty = f2(ay.x / r.d.y, ay.y / r.d.y);
        tz = f2(az.x / r.d.z, az.y / r.d.z);
    }
    const float tmin = fmaxf(fmaxf(fminf(tx.x, tx.y), fminf(ty.x, ty.y)), fminf(tz.x, tz.y));
    const float tmax = fminf(fminf(fmaxf(tx.x, tx.y), fmaxf(ty.x, ty.y)), fmaxf(tz.x, tz.y));
    if (!(tmax < 0.0f) && !(tmin > tmax)) {
        const float t = tmin < 0.0f ? tmax : tmin;
        if (bidx < 0 || t < best) {
            best = t;
            bidx = i;
        }
    }
}

// The same test on a cube record in the slab pair layout (min.x, max.x,
// min.y, max.y) (min.z, max.z, ...): the LBVH's primitives.
template <bool Fast>
__device__ __forceinline__ void cube_test(const float4* __restrict__ cr, int i, const RayPre& r, float& best,
                                          int& bidx) {
    const float4 A = cr[0];
    const float4 B = cr[1];
    cube_slab<Fast>(f2(A.x, A.y), f2(A.z, A.w), f2(B.x, B.y), i, r, best, bidx);
}

// The same test on cube j of a brute-force chunk (pairs of cubes, rdc_flatten.hpp:
// (min.x, min.x', max.x, max.x') and likewise y, z per pair).
template <bool Fast>
__device__ __forceinline__ void cube_exact(const float4* __restrict__ pr, int j, int obj, const RayPre& r,
                                           float& best, int& bidx) {
    const float* q = reinterpret_cast<const float*>(pr + 3 * (j >> 1)) + (j & 1);
    cube_slab<Fast>(f2(q[0], q[2]), f2(q[4], q[6]), f2(q[8], q[10]), obj, r, best, bidx);
}

__device__ __forceinline__ float fmax3(float a, float b, float c) {
    float d;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}
__device__ __forceinline__ float fmin3(float a, float b, float c) {
    float d;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}

// hit_cube pass 1 on the guarded fast path: a conservative filter, the
// LBVH's box test (rdc_bvh.cuh) on every cube of a chunk (up to 32, two per
// packed instruction), into a bit mask of the cubes the exact pass 2
// (cube_exact) has to decide.  A cube is dropped only when the grown box
// [min - m, max + m] lies wholly behind the origin or is missed (dropping
// boxes entered beyond the best hit too measured slower on cube-heavy
// scenes: the extra candidates cost pass 2 less than the test cost here).  The growth
// m = 2^-20 (|o| + 2R) + 1e-30, R >= |centre| + half side * sqrt(3) over the
// run, covers the reference's slab rounding and this test's own (the bound
// is proven for the LBVH's leaves, which run the same exact test after the
// same box test).  Per ray, the near and far plane of each axis are known
// from the sign of 1/d, so each cube takes two plane distances per axis
// (one FMA each, FMA(plane, 1/d, -(o +- m)/d)) and one three-input max and
// min; far distances subtract a subtrahend lowered by 2^-120, which never
// lets them be -0 and keeps `exit >= 0` an exact sign test.
constexpr int kCubeFilterMinRun = 4;  // shortest cube run the filter is used on

struct CubeFilterRay {
    float2 inv[3];    // RN(1/d) per axis, both halves
    float2 nnear[3];  // -(o + m)/d or -(o - m)/d: the near plane's subtrahend, negated
    float2 nfar[3];   // the far plane's, negated and raised by 2^-120
    int near_off[3];  // float2 index of the near planes within the axis's float4: 0 (min) or 1 (max)
};

__device__ __forceinline__ CubeFilterRay cube_filter_ray(const RayPre& r, float R) {
    CubeFilterRay c;
    const float m = 9.536743e-7f /* 2^-20 */ * (r.ol1 + 2.0f * R) + 1e-30f;
    const float o[3] = {r.o.x, r.o.y, r.o.z};
    const float inv[3] = {r.rd.x, r.rd.y, r.rd.z};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float oa = (o[k] + m) * inv[k];  // subtrahend of the min plane
        const float ob = (o[k] - m) * inv[k];  // of the max plane
        const bool pos = inv[k] >= 0.0f;
        const float nn = -(pos ? oa : ob);
        const float nf = 7.5231638e-37f /* 2^-120 */ - (pos ? ob : oa);
        c.inv[k] = f2(inv[k], inv[k]);
        c.nnear[k] = f2(nn, nn);
        c.nfar[k] = f2(nf, nf);
        c.near_off[k] = pos ? 0 : 1;
    }
    return c;
}

// Plane distances of the two cubes of a pair, one packed FMA.
__device__ __forceinline__ float2 cube_planes(float2 p, float2 inv, float2 ns) { return fma2(p, inv, ns); }

template <int Unroll>
__device__ __forceinline__ uint32_t cube_candidates(const float4* __restrict__ pr, int n, const CubeFilterRay& c) {
    const float2* p2 = reinterpret_cast<const float2*>(pr);
    const float2* nx = p2 + c.near_off[0];
    const float2* fx = p2 + (1 - c.near_off[0]);
    const float2* ny = p2 + 2 + c.near_off[1];
    const float2* fy = p2 + 2 + (1 - c.near_off[1]);
    const float2* nz = p2 + 4 + c.near_off[2];
    const float2* fz = p2 + 4 + (1 - c.near_off[2]);
    uint32_t m = 0;
    const int np = (n + 1) >> 1;
#pragma unroll Unroll
    for (int p = 0; p < np; ++p) {
        const int o = 6 * p;
        const float2 ex = cube_planes(nx[o], c.inv[0], c.nnear[0]), xx = cube_planes(fx[o], c.inv[0], c.nfar[0]);
        const float2 ey = cube_planes(ny[o], c.inv[1], c.nnear[1]), xy = cube_planes(fy[o], c.inv[1], c.nfar[1]);
        const float2 ez = cube_planes(nz[o], c.inv[2], c.nnear[2]), xz = cube_planes(fz[o], c.inv[2], c.nfar[2]);
        const float2 entry = f2(fmax3(ex.x, ey.x, ez.x), fmax3(ex.y, ey.y, ez.y));
        const float2 exit = f2(fmin3(xx.x, xy.x, xz.x), fmin3(xx.y, xy.y, xz.y));
        const float2 span = sub2(exit, entry);  // exit >= entry
        // bit 31 set <=> dropped (exit < 0 or exit < entry)
        const uint32_t w0 = __float_as_uint(span.x) | __float_as_uint(exit.x);
        const uint32_t w1 = __float_as_uint(span.y) | __float_as_uint(exit.y);
        m = __funnelshift_l(~w0, m, 1);
        m = __funnelshift_l(~w1, m, 1);
    }
    if (2 * np > n) m >>= 1;  // drop the padding half of an odd chunk
    return m;
}

// Brute-force closest hit over all objects in scene order.  Unroll: pass 1's
// unroll factor (4 in the render kernels; the adjoint kernel, bound by
// instruction fetch, runs faster with the loops rolled).
template <bool Fast, int Unroll>
__device__ __forceinline__ void intersect_runs(const float4* __restrict__ rec,
                                               const int4* __restrict__ runs, int nruns,
                                               const RayPre& r, float& best, int& bidx) {
    best = __int_as_float(0x7f800000);
    bidx = -1;
    for (int q = 0; q < nruns; ++q) {
        const int4 run = runs[q];
        if (run.x == 0) {
            for (int cb = run.y; cb < run.z; cb += 32) {
                const int n = min(32, run.z - cb);
                const float4* pr = rec + run.w + 3 * ((cb - run.y) >> 1);
                uint32_t m = sphere_candidates<Fast, Unroll>(pr, n, r);
                while (m != 0u) {  // highest bit first = scene order
                    const int pos = 31 - __clz(m);
                    m ^= 1u << pos;
                    const int j = n - 1 - pos;
                    sphere_exact<Fast>(pr, j, cb + j, r, best, bidx);
                }
            }
        } else {
            // a cube run: a header (R, 0, 0, 0), then 3 float4 per pair of cubes
            const float4* pr0 = rec + run.w + 1;
            // the filter's per-ray setup pays off from a few cubes on (a
            // lone ground cube, which most rays hit, goes straight to pass 2)
            if (Fast && run.z - run.y >= kCubeFilterMinRun) {
                const CubeFilterRay c = cube_filter_ray(r, rec[run.w].x);
                for (int cb = run.y; cb < run.z; cb += 32) {
                    const int n = min(32, run.z - cb);
                    const float4* pr = pr0 + 3 * ((cb - run.y) >> 1);
                    uint32_t m = cube_candidates<Unroll>(pr, n, c);
                    while (m != 0u) {  // highest bit first = scene order
                        const int pos = 31 - __clz(m);
                        m ^= 1u << pos;
                        const int j = n - 1 - pos;
                        cube_exact<Fast>(pr, j, cb + j, r, best, bidx);
                    }
                }
            } else {
                for (int i = run.y; i < run.z; ++i) cube_exact<Fast>(pr0, i - run.y, i, r, best, bidx);
            }
        }
    }
}

// `scene_fast`: every slab bound of the scene is inside the exact-division
// range (computed on upload).
template <int Unroll = 4>
__device__ __forceinline__ void intersect_all(const float4* __restrict__ rec,
                                              const int4* __restrict__ runs, int nruns,
                                              bool scene_fast, const RayPre& r, float& best,
                                              int& bidx) {
    if (scene_fast && r.fast)
        intersect_runs<true, Unroll>(rec, runs, nruns, r, best, bidx);
    else
        intersect_runs<false, Unroll>(rec, runs, nruns, r, best, bidx);
}

struct HitRec {
    V3 p, n;
    bool front;
};

// An object's material record (64 bytes, 64-byte aligned): two 256-bit loads.
__device__ __forceinline__ MatDev load_mat(const MatDev* mats, int i) {
    MatDev m;
    const float4* p = reinterpret_cast<const float4*>(mats + i);
    ldg_pair(p, m.a, m.b);
    ldg_pair(p + 2, m.c, m.d);
    return m;
}

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

// What the adjoint needs to replay a scatter backwards: the lobe taken, the
// diffuse flip, the transmission offset, the |dir| < 1e-5 fallback, which
// coin with a parameter-dependent probability decided the lobe, and the
// unit-sphere vector the lobe added (scaled by roughness^2).  The flags fit
// in 8 bits.
enum : uint32_t {
    kLobeDiffuse = 0u,
    kLobeSpecular = 1u,
    kLobeRefract = 2u,
    kScatFlip = 4u,      // diffuse = -(n + s1)
    kScatTrans = 8u,     // transmission ray: origin offset along the new direction
    kScatNormal = 16u,   // |dir|^2 < 1e-10: the new direction is the normal
    kScatFront = 32u,    // the hit's front-face flag
    kScatRoughCoin = 64u,    // U_rough < roughness^2 chose diffuse or specular (cpu.rs:309-313)
    kScatFresnelCoin = 128u, // Schlick's R < U_fresnel chose refraction or reflection (cpu.rs:296-297)
};
struct ScatterRec {
    uint32_t flags;
    V3 s;
};

// The hit branch of per_pixel (src/renderer/cpu.rs:262-328): the new ray
// from a hit, the object's material and the bounce's random words, lobe
// first.  The reference builds both the diffuse and the specular candidate
// direction and keeps one of them (or the refracted one); only the kept
// direction's arithmetic reaches the new ray, so deciding the lobe from the
// coin words first and building that direction alone gives the same bits
// with one unit-sphere vector and one or two normalisations instead of two
// and three (measured +1.4% on the 81-object brute-force frame, +1.7%
// through the LBVH).  a, b and q are the bounce's three Philox blocks (words
// 0-3, 4-7, 8-11).  With Rec, also fills *rec for the adjoint's replay (the
// flip bit is set for the diffuse lobe only, the one lobe that reads it).
// (Drawing q only for the lanes that read it -- the roughness coin inside
// (0, 1) and the refracted lobe -- measured 2.5% slower on the brute-force
// frame: a warp's lanes rarely all skip it, and the branch costs more than
// the block.)
template <bool Rec>
__device__ __forceinline__ void scatter_lobe_first(V3 d, const HitRec& h, const MatDev& m, const U4 a, const U4 b,
                                                   const U4 q, V3& o_out, V3& d_out, ScatterRec* rec) {
    const float rough = m.a.w;
    const float metallic = m.b.w;
    const float transmission = m.c.x;
    const bool trans = u01(b.z) < transmission;  // word 6
    bool refracted = false, diffuse = false;
    uint32_t coin = 0u;
    float ratio = 0.0f, cos_theta = 0.0f;
    V3 rd = h.n;
    if (trans) {
        ratio = h.front ? m.c.y : m.c.z;
        const float r0 = h.front ? m.c.w : m.d.x;
        rd = vnormalize(d);
        const V3 nn = vneg(h.n);
        cos_theta = fminf(vdot(rd, nn), 1.0f);
        const float mm = 1.0f - cos_theta;
        const float m2 = mm * mm;
        const float m5 = mm * (m2 * m2);
        const float refl = r0 + (1.0f - r0) * m5;
        const bool coin_refracts = refl < u01(b.w);  // word 7
        if (coin_refracts || Rec) {  // the record also needs can_refract when the coin says reflect
            // can_refract, src/utils/mod.rs:37-44
            const float sin_theta = sqrtf(1.0f - cos_theta * cos_theta);
            const bool can = ratio * sin_theta <= 1.0f;
            refracted = coin_refracts && can;
            // under total internal reflection the lobe is reflection whatever the coin says
            coin = can ? kScatFresnelCoin : 0u;
        }
    } else if (!(u01(b.w) < metallic)) {  // word 7
        diffuse = u01(q.x) < rough;          // word 8
        coin = kScatRoughCoin;
    }
    // the lobe's unit-sphere vector: words 0-2 (diffuse), 8-10 (refracted), 3-5 (specular)
    const uint32_t ua = diffuse ? a.x : refracted ? q.x : a.w;
    const uint32_t ub = diffuse ? a.y : refracted ? q.y : b.x;
    const uint32_t uc = diffuse ? a.z : refracted ? q.z : b.y;
    const V3 sv = unit_sphere(ua, ub, uc);
    V3 dir;
    bool flip = false;
    if (diffuse) {
        dir = vadd(h.n, sv);
        flip = vdot(dir, h.n) < 0.0f;
        if (flip) dir = vneg(dir);
    } else {
        V3 base;
        if (refracted) {
            // refract, src/utils/mod.rs:25-35
            const V3 perp = vmul(vadd(rd, vmul(h.n, cos_theta)), ratio);
            const float sq = -sqrtf(fabsf(1.0f - vdot(perp, perp)));
            base = vadd(perp, vmul(h.n, sq));
        } else {
            // reflect, src/utils/mod.rs:14-16: v - n * (v.n) * 2
            const float dn = vdot(d, h.n);
            base = vsub(d, vmul(vmul(h.n, dn), 2.0f));
        }
        dir = vnormalize(vadd(base, vmul(sv, rough)));
    }
    const V3 off = trans ? dir : h.n;
    o_out = vadd(h.p, vmul(off, 0.0001f));
    const bool to_normal = vdot(dir, dir) < 1e-10f;
    d_out = to_normal ? h.n : dir;
    if (Rec) {
        const uint32_t lobe = diffuse ? kLobeDiffuse : refracted ? kLobeRefract : kLobeSpecular;
        rec->flags = lobe | (flip ? kScatFlip : 0u) | (trans ? kScatTrans : 0u) | (to_normal ? kScatNormal : 0u) |
                     (h.front ? kScatFront : 0u) | coin;
        rec->s = sv;
    }
}

// The scatter from twelve given words.
__device__ __forceinline__ void scatter(V3 d, const HitRec& h, const MatDev& m, const uint32_t* w, V3& o_out,
                                        V3& d_out) {
    scatter_lobe_first<false>(d, h, m, U4{w[0], w[1], w[2], w[3]}, U4{w[4], w[5], w[6], w[7]},
                              U4{w[8], w[9], w[10], w[11]}, o_out, d_out, nullptr);
}

// One bounce's scatter with its random words drawn from the Philox blocks
// (pix, sample, c2 .. c2 + 2, stream).
__device__ __forceinline__ void scatter_drawn(V3 d, const HitRec& h, const MatDev& m, uint32_t pix, uint32_t sample,
                                              uint32_t c2, uint32_t stream_id, uint32_t k0, uint32_t k1, V3& o_out,
                                              V3& d_out) {
    scatter_lobe_first<false>(d, h, m, philox(pix, sample, c2, stream_id, k0, k1),
                              philox(pix, sample, c2 + 1u, stream_id, k0, k1),
                              philox(pix, sample, c2 + 2u, stream_id, k0, k1), o_out, d_out, nullptr);
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

// --------------------------------------------------------------- a path ---
// Scene staging into shared memory with the Tensor Memory Accelerator's bulk
// copy (cp.async.bulk, global -> shared), completing on an mbarrier.  One
// thread initialises the barrier (bulk_init) and issues the copies
// (bulk_issue); every thread of the block waits for the barrier's phase
// (bulk_wait), polling at most kBulkWaitPolls times so that a copy that never
// lands cannot hang the block: the kernel then records a device error and
// returns.  Sources and destinations are 16-byte aligned and the sizes are
// 16-byte multiples (float4 / int4 records).
constexpr uint32_t kBulkWaitPolls = 1u << 20;

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void bulk_init(uint64_t* bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void bulk_issue(uint64_t* bar, void* s0, const void* g0, uint32_t n0, void* s1,
                                           const void* g1, uint32_t n1) {
    const uint32_t b = smem_addr(bar);
    // order the block's earlier generic reads of this shared memory before the async writes
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(b),
                 "r"(n0 + n1)
                 : "memory");
    if (n0)
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                         smem_addr(s0)),
                     "l"(g0), "r"(n0), "r"(b)
                     : "memory");
    if (n1)
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                         smem_addr(s1)),
                     "l"(g1), "r"(n1), "r"(b)
                     : "memory");
}

// true once the barrier's phase `parity` has completed.  Each poll suspends
// the thread for at most kBulkPollNs (the instruction's suspend-time hint), so
// the whole wait is bounded by about kBulkWaitPolls * kBulkPollNs (~1 s).
constexpr uint32_t kBulkPollNs = 1000;

__device__ __forceinline__ bool bulk_wait(uint64_t* bar, uint32_t parity) {
    const uint32_t b = smem_addr(bar);
    for (uint32_t i = 0; i < kBulkWaitPolls; ++i) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(b), "r"(parity), "r"(kBulkPollNs)
            : "memory");
        if (done) return true;
    }
    return false;
}

// Stage a scene's records and runs (brute-force kernels): thread 0 issues,
// all wait.  Returns false for the whole block if the copy did not land
// (then errors[0] is incremented once and the block must return).
__device__ __forceinline__ bool stage_scene(uint64_t* bar, uint32_t parity, float4* s_rec, const float4* rec,
                                            uint32_t nrec, int4* s_runs, const int4* runs, uint32_t nruns,
                                            unsigned long long* errors) {
    if (threadIdx.x == 0) bulk_issue(bar, s_rec, rec, 16u * nrec, s_runs, runs, 16u * nruns);
    const bool ok = __syncthreads_and(bulk_wait(bar, parity)) != 0;
    if (!ok && threadIdx.x == 0) {
        if (errors) atomicAdd(errors, 1ull);
        bulk_wait(bar, parity);  // give copies still in flight a last bounded chance to land
    }
    return ok;
}

struct PathState {
    V3 o, d, atten, light;
    uint32_t bounce;
};

__device__ __forceinline__ void path_start(const SceneView& sc, uint32_t pix, PathState& s) {
    primary_ray(sc, pix % sc.width, pix / sc.width, s.o, s.d);
    s.atten = mk(1.f, 1.f, 1.f);
    s.light = mk(0.f, 0.f, 0.f);
    s.bounce = 0;
}

// The next sample of the same pixel: the primary ray is a function of the
// pixel alone (the same floats every sample), so the kernels keep its
// direction in a per-thread shared-memory slot (`dir`, written after
// path_start) instead of recomputing it (six IEEE divisions and a
// normalisation per sample).
__device__ __forceinline__ void path_keep(const PathState& s, float4* dir) {
    *dir = make_float4(s.d.x, s.d.y, s.d.z, 0.0f);
}
__device__ __forceinline__ void path_restart(const SceneView& sc, const float4* dir, PathState& s) {
    const float4 d = *dir;
    s.o = mk(sc.cam_pos[0], sc.cam_pos[1], sc.cam_pos[2]);
    s.d = mk(d.x, d.y, d.z);
    s.atten = mk(1.f, 1.f, 1.f);
    s.light = mk(0.f, 0.f, 0.f);
    s.bounce = 0;
}

// Brute-force closest hit over a scene's records (shared or global memory).
struct BruteIsect {
    const float4* rec;
    const int4* runs;
    int nruns;
    bool scene_fast;
    __device__ __forceinline__ void operator()(const RayPre& r, float& t, int& idx) {
        intersect_all(rec, runs, nruns, scene_fast, r, t, idx);
    }
};

// The same with pass 1's loops rolled: smaller code for the kernels whose
// instruction fetch stalls them most (measured: adjoint backward 10.1 -> 9.45
// ms, batch 99.8 -> 102.6 scenes/s; the single-scene render kernel is faster
// unrolled).
struct BruteIsectRolled {
    const float4* rec;
    const int4* runs;
    int nruns;
    bool scene_fast;
    __device__ __forceinline__ void operator()(const RayPre& r, float& t, int& idx) {
        intersect_all<1>(rec, runs, nruns, scene_fast, r, t, idx);
    }
};

// path_segment (below) runs one segment of a path (src/renderer/cpu.rs:256-338):
// trace_ray, then the scatter of a hit or the world sample of a miss.  `isect`
// finds the closest hit (brute force or BVH: the same result).  It returns
// true when the path has ended (a miss, or max_bounces segments traced).
//
// segment_shade is its second half: given the closest hit (t, idx; idx < 0
// for none) of the ray (s.o, s.d), apply the world sample or the scatter.
__device__ __forceinline__ bool segment_shade(const SceneView& sc, PathState& s, float t, int idx, uint32_t pix,
                                              uint32_t sample, uint32_t max_bounces, uint32_t stream_id,
                                              uint32_t k0, uint32_t k1) {
    if (idx < 0) {
        const V3 sky = world_sample(sc, s.d);
        s.light = vadd(s.light, mk(sky.x * s.atten.x, sky.y * s.atten.y, sky.z * s.atten.z));
        return true;
    }
    const int ci = (int)checked_index(sc.oob, idx, sc.nobj);
    const float4 hi = __ldg(&sc.hit[ci]);
    const MatDev m = load_mat(sc.mat, ci);
    const HitRec h = closest_hit(s.o, s.d, t, hi, __float_as_int(m.d.y));
    V3 no, nd;
    scatter_drawn(s.d, h, m, pix, sample, s.bounce * 4u, stream_id, k0, k1, no, nd);
    s.o = no;
    s.d = nd;
    s.atten = mk(s.atten.x * m.a.x, s.atten.y * m.a.y, s.atten.z * m.a.z);
    s.light = vadd(s.light, mk(m.b.x, m.b.y, m.b.z));
    ++s.bounce;
    return s.bounce >= max_bounces;
}

template <class Isect>
__device__ __forceinline__ bool path_segment(const SceneView& sc, Isect& isect, PathState& s, uint32_t pix,
                                             uint32_t sample, uint32_t max_bounces, uint32_t stream_id,
                                             uint32_t k0, uint32_t k1, uint32_t& segs) {
    if (s.bounce >= max_bounces) return true;  // max_bounces == 0: the path adds (0, 0, 0, 1)
    ++segs;
    const RayPre r = ray_pre(s.o, s.d, sc.neg_zero);
    float t;
    int idx;
    isect(r, t, idx);
    return segment_shade(sc, s, t, idx, pix, sample, max_bounces, stream_id, k0, k1);
}

}  // namespace rdc
