// rdc_bvh.cuh -- traversal of the device-built LBVH (rdc_bvh.cu builds it).
//
// The reference tests every object (src/renderer/cpu.rs:344-352).  For large
// scenes the kernels instead walk a linear BVH: Morton-ordered objects, a
// Karras (2012) radix tree of N-1 internal nodes, each node holding the boxes
// of its two children.  The result must be the reference's exactly:
//   - leaves run the same exact sphere / cube tests as the brute-force loop;
//   - the first-minimum rule (lowest object index among equal t) becomes a
//     lexicographic minimum over (t, index), independent of visiting order;
//   - a box is skipped only when its entry distance is strictly greater than
//     the best t so far (an equal-t object with a lower index must be seen);
//   - box tests are conservative with respect to the reference's arithmetic.
//     Its sphere test is the expanded quadratic.  With u = 2^-24,
//     S = |o| + |c| and A = d.d, first-order rounding analysis of
//     a = d.d, k = o.d - d.c, c = ((o.o - 2 o.c) + c.c) - r^2 and
//     disc = k^2 - a c gives |disc - A (r^2 - rho^2)| <= u A (21 S^2 + 4 r^2),
//     rho the distance from the centre to the ray's line.  A hit can thus be
//     reported only when rho^2 <= r^2 (1 + 2^-20) + 2^-19 S^2.  Sphere leaf
//     boxes are built with that radius for |o| <= o_max (rdc_bvh.cu); a ray
//     from further away adds 2^-9.5 (|o| - o_max), the slope of that radius
//     in S.  Every ray also adds 2^-20 (|o| + 2R), R bounding |centre| + size:
//     it covers the computed t lying before the grown ball's entry (at most
//     ~5u S along the ray) and the slab test's rounding for cubes
//     (2u (|o| + |c| + h) per axis).  The per-ray growth is folded into two
//     origin offsets, so it costs nothing per box.
#pragma once

#include "raydar_cuda.h"
#include "rdc_device.cuh"

namespace rdc {

struct alignas(16) BvhNode {
    float4 a;  // child 0 box min (xyz), child 0 (int bits: >= 0 node, < 0 leaf ~object)
    float4 b;  // child 0 box max (xyz), child 1 (int bits)
    float4 c;  // child 1 box min (xyz), 0
    float4 d;  // child 1 box max (xyz), 0
};

// BvhView (rdc_internal.hpp): nodes (N-1, root 0), prims (2 per object, scene
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
    if (Fast && k >= 1.0842022e-19f && disc < kk * 0.99999905f) return;  // both roots behind (proof in rdc_device.cuh)
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
    const float4 p0 = __ldg(&bv.prims[2 * obj]);
    const float4 p1 = __ldg(&bv.prims[2 * obj + 1]);
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

// Conservative slab test of a box [lo - m, hi + m]: oa = o + m, ob = o - m.
__device__ __forceinline__ bool bvh_box(float3 lo, float3 hi, float3 oa, float3 ob, float3 inv, float limit,
                                        float& entry) {
    const float lx = (lo.x - oa.x) * inv.x, hx = (hi.x - ob.x) * inv.x;
    const float ly = (lo.y - oa.y) * inv.y, hy = (hi.y - ob.y) * inv.y;
    const float lz = (lo.z - oa.z) * inv.z, hz = (hi.z - ob.z) * inv.z;
    const float tmin = fmaxf(fmaxf(fminf(lx, hx), fminf(ly, hy)), fminf(lz, hz));
    const float tmax = fminf(fminf(fmaxf(lx, hx), fmaxf(ly, hy)), fmaxf(lz, hz));
    entry = tmin;
    return tmax >= -1e-30f - fabsf(tmax) * 3.8146973e-6f && tmin <= tmax + fabsf(tmax) * 3.8146973e-6f &&
           tmin <= limit;
}

// One ray's traversal, resumable one node visit at a time (the stack lives
// with the caller: 64 entries, deeper than any tree Karras' construction
// builds from 30-bit codes + 32-bit indices).
struct BvhTrav {
    float3 oa, ob, inv;  // origin grown by +m / -m (see the file comment), 1/d
    float best;          // closest hit so far (+inf: none)
    int bidx;            // its object (-1: none)
    int cur;             // next node to visit; -1 when the traversal is over
    int sp;              // stack depth
};

constexpr int kBvhStack = 64;

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
    T.oa = make_float3(r.o.x + m, r.o.y + m, r.o.z + m);
    T.ob = make_float3(r.o.x - m, r.o.y - m, r.o.z - m);
    auto inv1 = [](float v) {
        const float a = fabsf(v) < 1e-30f ? copysignf(1e-30f, v) : v;
        return 1.0f / a;
    };
    T.inv = make_float3(inv1(r.d.x), inv1(r.d.y), inv1(r.d.z));
    T.cur = 0;
}

// One node visit of a running traversal (T.cur >= 0): both child boxes,
// leaf children tested at once, the nearer internal child next and the
// other pushed; with none, the next stacked box still in front of the best
// hit, or the end of the traversal (T.cur = -1).
__device__ __forceinline__ void bvh_step(const BvhView& bv, const RayPre& r, bool fast, BvhTrav& T,
                                         int* stack_node, float* stack_entry, BvhCounters& cnt) {
    const BvhNode* np = bv.nodes + T.cur;
    const float4 na = __ldg(&np->a), nb = __ldg(&np->b), nc = __ldg(&np->c), ndd = __ldg(&np->d);
    ++cnt.visits;
    // limit: skip a box whose entry exceeds best (relative slack for the box test's rounding)
    const float limit = T.best * 1.0000038f + 1e-30f;
    float e0, e1;
    bool h0 = bvh_box(make_float3(na.x, na.y, na.z), make_float3(nb.x, nb.y, nb.z), T.oa, T.ob, T.inv, limit, e0);
    bool h1 = bvh_box(make_float3(nc.x, nc.y, nc.z), make_float3(ndd.x, ndd.y, ndd.z), T.oa, T.ob, T.inv, limit, e1);
    const int c0 = __float_as_int(na.w), c1 = __float_as_int(nb.w);
    if (h0 && c0 < 0) {
        ++cnt.tests;
        bvh_leaf_any(bv, r, fast, ~c0, T.best, T.bidx);
        h0 = false;
    }
    if (h1 && c1 < 0) {
        ++cnt.tests;
        bvh_leaf_any(bv, r, fast, ~c1, T.best, T.bidx);
        h1 = false;
    }
    if (h0 && h1) {
        const bool first0 = e0 <= e1;
        stack_node[T.sp] = first0 ? c1 : c0;
        stack_entry[T.sp] = first0 ? e1 : e0;
        ++T.sp;  // depth <= 62 (30 Morton bits + 32 index bits)
        T.cur = first0 ? c0 : c1;
    } else if (h0) {
        T.cur = c0;
    } else if (h1) {
        T.cur = c1;
    } else {
        // pop the next box still in front of the best hit
        const float lim = T.best * 1.0000038f + 1e-30f;
        int next = -1;
        while (T.sp > 0) {
            --T.sp;
            if (stack_entry[T.sp] <= lim) {
                next = stack_node[T.sp];
                break;
            }
        }
        T.cur = next;
    }
}

// Closest hit through the BVH: the same (t, index) the brute-force loop gives.
__device__ __forceinline__ void bvh_intersect(const BvhView& bv, const RayPre& r, bool fast, float& best, int& bidx,
                                              BvhCounters& cnt) {
    int stack_node[kBvhStack];
    float stack_entry[kBvhStack];
    BvhTrav T;
    bvh_begin(bv, r, fast, T, cnt);
    while (T.cur >= 0) bvh_step(bv, r, fast, T, stack_node, stack_entry, cnt);
    best = T.best;
    bidx = T.bidx;
}

}  // namespace rdc
