// rdc_bvh.cuh -- traversal of the device-built LBVH (rdc_bvh.cu builds it).
//
// The reference tests every object (src/renderer/cpu.rs:344-352).  For large
// scenes the kernels instead walk a linear BVH: Morton-ordered objects, a
// Karras (2012) radix tree of N-1 internal nodes, collapsed into a 4-wide
// tree (every binary node at even depth keeps its grandchildren, or its leaf
// children, as up to four children): half the dependent node loads per ray,
// four independent box tests per load.  The result must be the reference's
// exactly:
//   - leaves run the same exact sphere / cube tests as the brute-force loop;
//   - the first-minimum rule (lowest object index among equal t) becomes a
//     lexicographic minimum over (t, index), independent of visiting order;
//   - a box is skipped only when its entry distance is strictly greater than
//     the best t so far (an equal-t object with a lower index must be seen);
//   - box tests are conservative with respect to the reference's arithmetic.
//     Its sphere test is the expanded quadratic.  With u = 2^-24,
//     S = |o| + |c| and A = d.d, first-order rounding analysis of
//     a = d.d, k = o.d - d.c, c = ((o.o - 2 o.c) + c.c) - r^2 and
//     disc = k^2 - a c gives |disc - A (r^2 - rho^2)| <= u A (21 S^2 + 6 r^2),
//     rho the distance from the centre to the ray's line.  A hit can thus be
//     reported only when rho^2 <= r^2 (1 + 2^-20) + 2^-19 S^2.  Sphere leaf
//     boxes are built with that radius for |o| <= o_max (rdc_bvh.cu); a ray
//     from further away adds 2^-9.5 (|o| - o_max), the slope of that radius
//     in S.  Every ray also adds 2^-20 (|o| + 2R) = 16u (|o| + 2R), R bounding
//     |centre| + size: it covers the computed t lying before the grown ball's
//     entry (at most ~5u S along the ray), the reference slab test's rounding
//     for cubes (2u (|o| + |c| + h) per axis) and the box test's own
//     (4u |o| + 2u |lo|), 11u |o| + 13u R in all.  The per-ray growth is
//     folded into the two per-axis origin terms, so it costs nothing per box.
#pragma once

#include "raydar_cuda.h"
#include "rdc_device.cuh"

namespace rdc {

// Binary node of the build (rdc_bvh.cu).
struct alignas(16) BvhNode {
    float4 a;  // child 0 box min (xyz), child 0 (int bits: >= 0 node, < 0 leaf ~object)
    float4 b;  // child 0 box max (xyz), child 1 (int bits)
    float4 c;  // child 1 box min (xyz), 0
    float4 d;  // child 1 box max (xyz), 0
};

// 4-wide node, 128 bytes: child j's box in v[2j] (min xyz, child in w as
// int bits: >= 0 node, < 0 leaf ~object) and v[2j+1] (max xyz).  An unused
// slot has min = max = +inf, which no ray hits (1/d is never 0).
struct alignas(16) Bvh4Node {
    float4 v[8];
};

// BvhView (rdc_internal.hpp): nodes (root 0), prims (2 per object, scene
// order: sphere (c, c.c) (r*r, 0, 0, kind); cube in the slab pair layout with
// kind in the last word), scene_r and o_max for the per-ray box growth.

// Per-thread counters of the last traversal work (for the ops/segment model).
struct BvhCounters {
    uint32_t visits = 0;
    uint32_t tests = 0;
};

template <bool Fast>
__device__ __forceinline__ void bvh_sphere_leaf(const RayPre& r, float4 p0, float rr, int obj, float& best,
                                                int& bidx) {
    const float dc = (r.d.x * p0.x + r.d.y * p0.y) + r.d.z * p0.z;
    const float k = r.od - dc;
    const float oc = (r.o.x * p0.x + r.o.y * p0.y) + r.o.z * p0.z;
    const float c = ((r.oo - 2.0f * oc) + p0.w) - rr;
    const float kk = k * k;
    const float disc = kk - r.a * c;
    if (!(disc >= 0.0f)) return;  // None (NaN too: the reference ends in None)
    // Both roots behind the origin: k >= 2^-63 keeps k*k normal, and disc <
    // RN(k*k (1 - 2^-20)) gives sqrt(disc) < k (1 - 2^-21 + 2^-24), so
    // RN(sqrt(disc)) < k and -k -+ RN(sqrt(disc)) < 0: the reference returns None.
    if (Fast && k >= 1.0842022e-19f && disc < kk * 0.99999905f) return;
    const float sq = __fsqrt_rn(disc);
    const float t1 = sphere_div<Fast>(-k - sq, r);
    float t = t1;
    bool ok = t1 >= 0.0f;
    if (!ok) {
        const float t2 = sphere_div<Fast>(-k + sq, r);
        t = t2;
        ok = t2 >= 0.0f;
    }
    if (ok && (bidx < 0 || t < best || (t == best && obj < bidx))) {
        best = t;
        bidx = obj;
    }
}

template <bool Fast>
__device__ __forceinline__ void bvh_leaf(const BvhView& bv, const RayPre& r, int obj, float& best, int& bidx) {
    float4 p0, p1;
    ldg_pair(bv.prims + 2 * checked_index(bv.oob, obj, bv.nobj), p0, p1);
    if (__float_as_int(p1.w) == RDC_GEOMETRY_SPHERE) {
        bvh_sphere_leaf<Fast>(r, p0, p1.x, obj, best, bidx);
    } else {
        // cube_test keeps strict <; reproduce the lexicographic rule around it.
        float tb = best;
        int ib = -1;
        const float4 rec[2] = {p0, p1};
        cube_test<Fast>(rec, obj, r, tb, ib);
        if (ib >= 0 && (bidx < 0 || tb < best || (tb == best && obj < bidx))) {
            best = tb;
            bidx = obj;
        }
    }
}

// Conservative slab test of a box [lo - m, hi + m] (m the per-ray growth):
// with oa = (o + m) / d and ob = (o - m) / d per axis, the plane distances
// are lo / d - oa and hi / d - ob, one FMA each.  Their rounding (a few ulp
// of |o| + |lo| along the ray) is far inside the 2^-20 (|o| + 2R) part of m,
// so the box's entry and exit are compared as computed.
__device__ __forceinline__ bool bvh_box(float3 lo, float3 hi, float3 oa, float3 ob, float3 inv, float limit,
                                        float& entry) {
    const float lx = __fmaf_rn(lo.x, inv.x, -oa.x), hx = __fmaf_rn(hi.x, inv.x, -ob.x);
    const float ly = __fmaf_rn(lo.y, inv.y, -oa.y), hy = __fmaf_rn(hi.y, inv.y, -ob.y);
    const float lz = __fmaf_rn(lo.z, inv.z, -oa.z), hz = __fmaf_rn(hi.z, inv.z, -ob.z);
    const float tmin = fmaxf(fmaxf(fminf(lx, hx), fminf(ly, hy)), fminf(lz, hz));
    const float tmax = fminf(fminf(fmaxf(lx, hx), fmaxf(ly, hy)), fmaxf(lz, hz));
    entry = tmin;
    return fmaxf(tmin, 0.0f) <= fminf(tmax, limit);
}

// One ray's traversal, resumable one node visit at a time.  The stack lives
// with the caller: a binary Karras tree over 30-bit codes with 32-bit index
// tie-breaks is at most 63 deep, the 4-wide tree at most 32, and a visit
// leaves at most 3 siblings pending per level.
struct BvhTrav {
    float3 oa, ob, inv;  // (o + m) / d, (o - m) / d per axis (m: see the file comment), 1/d
    float best;          // closest hit so far (+inf: none)
    int bidx;            // its object (-1: none)
    int cur;             // next node to visit; -1 when no node is left
    int sp;              // stack depth
    int lnode;           // node whose leaf children in lmask are still to be tested
    unsigned lmask;      // the traversal is over when cur < 0 and lmask == 0
};

constexpr int kBvhStack = 96;

__device__ __forceinline__ void bvh_leaf_any(const BvhView& bv, const RayPre& r, bool fast, int obj, float& best,
                                             int& bidx) {
    if (fast)
        bvh_leaf<true>(bv, r, obj, best, bidx);
    else
        bvh_leaf<false>(bv, r, obj, best, bidx);
}

// Set up the traversal of ray r; one- and zero-object trees finish here.
// fast: the scene and the ray allow the exact reciprocal division.
__device__ __forceinline__ void bvh_begin(const BvhView& bv, const RayPre& r, bool fast, BvhTrav& T,
                                          BvhCounters& cnt) {
    T.best = __int_as_float(0x7f800000);
    T.bidx = -1;
    T.sp = 0;
    T.cur = -1;
    T.lnode = 0;
    T.lmask = 0u;
    if (bv.nobj == 0) return;
    if (bv.nobj == 1) {
        ++cnt.tests;
        bvh_leaf_any(bv, r, fast, 0, T.best, T.bidx);
        return;
    }
    // Per-ray box growth (see the file comment) and inverse direction.
    const float olen = sqrtf(vdot(r.o, r.o));
    const float far = olen > bv.o_max ? 1.3810679e-3f * 1.001f * (olen - bv.o_max) : 0.0f;  // 2^-9.5
    const float m = far + 9.536743e-7f * (olen + 2.0f * bv.scene_r) + 1e-30f;            // 2^-20
    // 1/d clamped to +-cap (a direction component below 1/cap tests its slab
    // as if it were 1/cap): cap * (|o| + 2R + 1) stays below 1e37, so no
    // plane distance overflows.
    const float cap = fminf(1e30f, 1e37f / (olen + 2.0f * bv.scene_r + 1.0f));
    auto inv1 = [cap](float v) { return fabsf(v) * cap < 1.0f ? copysignf(cap, v) : 1.0f / v; };
    T.inv = make_float3(inv1(r.d.x), inv1(r.d.y), inv1(r.d.z));
    T.oa = make_float3((r.o.x + m) * T.inv.x, (r.o.y + m) * T.inv.y, (r.o.z + m) * T.inv.z);
    T.ob = make_float3((r.o.x - m) * T.inv.x, (r.o.y - m) * T.inv.y, (r.o.z - m) * T.inv.z);
    T.cur = 0;
}

// Traversal stacks of (node, entry distance bits) words.  LocalStack: one
// per-thread local array.  SplitStack: the first kShortStack entries in
// shared memory (entry k of thread t at sh[k * stride], sh already offset by
// t; consecutive threads, consecutive words, no bank conflicts), deeper ones
// in the local array; shared memory needs no tag lookup and leaves the L1 to
// the nodes.
constexpr int kShortStack = 16;

struct LocalStack {
    uint2* a;
    __device__ __forceinline__ void push(int& sp, uint2 e) { a[sp++] = e; }
    __device__ __forceinline__ uint2 pop(int& sp) { return a[--sp]; }
};

struct SplitStack {
    uint2* sh;
    uint32_t stride;
    uint2* loc;
    __device__ __forceinline__ void push(int& sp, uint2 e) {
        if (sp < kShortStack)
            sh[(uint32_t)sp * stride] = e;
        else
            loc[sp - kShortStack] = e;
        ++sp;
    }
    __device__ __forceinline__ uint2 pop(int& sp) {
        --sp;
        return sp < kShortStack ? sh[(uint32_t)sp * stride] : loc[sp - kShortStack];
    }
};

// Compare-exchange of (entry, node) pairs, ascending by entry.
__device__ __forceinline__ void bvh_cswap(float& ka, int& va, float& kb, int& vb) {
    const bool sw = kb < ka;
    const float k = sw ? kb : ka;
    const int v = sw ? vb : va;
    kb = sw ? ka : kb;
    vb = sw ? va : vb;
    ka = k;
    va = v;
}

// One node visit (T.cur >= 0, T.lmask == 0): the four child boxes; leaf
// children hit are left in T.lmask for bvh_leaf_step (a warp tests them
// together instead of one lane at a time inside the visit); the nearest
// internal child hit is visited next and the others pushed, farthest first;
// with none, the next stacked box still in front of the best hit, or none
// (T.cur = -1).
template <class Stack>
__device__ __forceinline__ void bvh_step(const BvhView& bv, const RayPre& r, bool fast, BvhTrav& T, Stack& stack,
                                         BvhCounters& cnt) {
    const float4* np = bv.nodes[checked_index(bv.oob, T.cur, bv.nnodes)].v;
    float4 lo[4], hi[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) ldg_pair(np + 2 * j, lo[j], hi[j]);
    ++cnt.visits;
    // limit: skip a box whose entry exceeds best (relative slack for the box test's rounding)
    const float limit = T.best * 1.0000038f + 1e-30f;
    float e[4];
    int c[4];
    unsigned hits = 0u;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        c[j] = __float_as_int(lo[j].w);
        if (bvh_box(make_float3(lo[j].x, lo[j].y, lo[j].z), make_float3(hi[j].x, hi[j].y, hi[j].z), T.oa, T.ob,
                    T.inv, limit, e[j]))
            hits |= 1u << j;
    }
    T.lmask = hits & ((c[0] < 0 ? 1u : 0u) | (c[1] < 0 ? 2u : 0u) | (c[2] < 0 ? 4u : 0u) | (c[3] < 0 ? 8u : 0u));
    T.lnode = T.cur;
    const float lim = limit;
    const float INF = __int_as_float(0x7f800000);
    float k0 = ((hits & 1u) && c[0] >= 0) ? e[0] : INF;
    float k1 = ((hits & 2u) && c[1] >= 0) ? e[1] : INF;
    float k2 = ((hits & 4u) && c[2] >= 0) ? e[2] : INF;
    float k3 = ((hits & 8u) && c[3] >= 0) ? e[3] : INF;
    int v0 = c[0], v1 = c[1], v2 = c[2], v3 = c[3];
    bvh_cswap(k0, v0, k1, v1);
    bvh_cswap(k2, v2, k3, v3);
    bvh_cswap(k0, v0, k2, v2);
    bvh_cswap(k1, v1, k3, v3);
    bvh_cswap(k1, v1, k2, v2);
    if (k0 != INF) {
        // an entry is (node, entry distance bits): one 8-byte local store or load
        if (k3 != INF) stack.push(T.sp, make_uint2((unsigned)v3, __float_as_uint(k3)));
        if (k2 != INF) stack.push(T.sp, make_uint2((unsigned)v2, __float_as_uint(k2)));
        if (k1 != INF) stack.push(T.sp, make_uint2((unsigned)v1, __float_as_uint(k1)));
        T.cur = v0;
    } else {
        // pop the next box still in front of the best hit
        int next = -1;
        while (T.sp > 0) {
            const uint2 top = stack.pop(T.sp);
            if (__uint_as_float(top.y) <= lim) {
                next = (int)top.x;
                break;
            }
        }
        T.cur = next;
    }
}

// Test the next pending leaf child (T.lmask != 0) of node T.lnode.
__device__ __forceinline__ void bvh_leaf_step(const BvhView& bv, const RayPre& r, bool fast, BvhTrav& T,
                                              BvhCounters& cnt) {
    const int j = __ffs(T.lmask) - 1;
    T.lmask &= T.lmask - 1u;
    const int child = __float_as_int(__ldg(&bv.nodes[checked_index(bv.oob, T.lnode, bv.nnodes)].v[2 * j].w));
    ++cnt.tests;
    bvh_leaf_any(bv, r, fast, ~child, T.best, T.bidx);
}

// Closest hit through the BVH: the same (t, index) the brute-force loop gives.
__device__ __forceinline__ void bvh_intersect(const BvhView& bv, const RayPre& r, bool fast, float& best, int& bidx,
                                              BvhCounters& cnt) {
    uint2 st[kBvhStack];
    LocalStack stack{st};
    BvhTrav T;
    bvh_begin(bv, r, fast, T, cnt);
    while (T.cur >= 0 || T.lmask != 0u) {
        if (T.lmask != 0u)
            bvh_leaf_step(bv, r, fast, T, cnt);
        else
            bvh_step(bv, r, fast, T, stack, cnt);
    }
    best = T.best;
    bidx = T.bidx;
}

}  // namespace rdc
