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
//     Its sphere test is the expanded quadratic, whose c term carries an
//     absolute error up to ~2^-20 (|o| + |c| + r)^2, so a computed hit point can
//     lie outside the sphere by up to sqrt(r^2 + dc) - r.  Each ray therefore
//     grows every box by m = sqrt(rmin^2 + 2^-20 (|o| + 2R)^2) - rmin
//     + 2^-20 (|o| + 2R), where R bounds |centre| + size over the scene and
//     rmin is the smallest sphere radius; the growth is folded into two
//     per-ray origin offsets, so it costs nothing per box.
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
// kind in the last word), scene_r and rmin for the per-ray box growth.

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

// Closest hit through the BVH: the same (t, index) the brute-force loop gives.
template <bool Fast>
__device__ __forceinline__ void bvh_intersect(const BvhView& bv, const RayPre& r, float& best, int& bidx,
                                              BvhCounters& cnt) {
    best = __int_as_float(0x7f800000);
    bidx = -1;
    if (bv.nobj == 0) return;
    if (bv.nobj == 1) {
        ++cnt.tests;
        bvh_leaf<Fast>(bv, r, 0, best, bidx);
        return;
    }
    // Per-ray box growth (see the file comment) and inverse direction.
    const float olen = sqrtf(vdot(r.o, r.o));
    const float span = olen + 2.0f * bv.scene_r;
    const float dc_max = 9.536743e-7f * span * span;  // 2^-20 (|o| + 2R)^2
    const float m = (sqrtf(bv.rmin * bv.rmin + dc_max) - bv.rmin) * 1.001f + 9.536743e-7f * span + 1e-30f;
    const float3 oa = make_float3(r.o.x + m, r.o.y + m, r.o.z + m);
    const float3 ob = make_float3(r.o.x - m, r.o.y - m, r.o.z - m);
    auto inv1 = [](float v) {
        const float a = fabsf(v) < 1e-30f ? copysignf(1e-30f, v) : v;
        return 1.0f / a;
    };
    const float3 inv = make_float3(inv1(r.d.x), inv1(r.d.y), inv1(r.d.z));

    int stack_node[64];
    float stack_entry[64];
    int sp = 0;
    int cur = 0;
    for (;;) {
        const BvhNode nd = bv.nodes[cur];
        ++cnt.visits;
        // limit: skip a box whose entry exceeds best (relative slack for the box test's rounding)
        const float limit = best * 1.0000038f + 1e-30f;
        float e0, e1;
        bool h0 = bvh_box(make_float3(nd.a.x, nd.a.y, nd.a.z), make_float3(nd.b.x, nd.b.y, nd.b.z), oa, ob, inv,
                          limit, e0);
        bool h1 = bvh_box(make_float3(nd.c.x, nd.c.y, nd.c.z), make_float3(nd.d.x, nd.d.y, nd.d.z), oa, ob, inv,
                          limit, e1);
        const int c0 = __float_as_int(nd.a.w), c1 = __float_as_int(nd.b.w);
        if (h0 && c0 < 0) {
            ++cnt.tests;
            bvh_leaf<Fast>(bv, r, ~c0, best, bidx);
            h0 = false;
        }
        if (h1 && c1 < 0) {
            ++cnt.tests;
            bvh_leaf<Fast>(bv, r, ~c1, best, bidx);
            h1 = false;
        }
        if (h0 && h1) {
            const bool first0 = e0 <= e1;
            stack_node[sp] = first0 ? c1 : c0;
            stack_entry[sp] = first0 ? e1 : e0;
            ++sp;  // depth <= 62 (30 Morton bits + 32 index bits), checked at build
            cur = first0 ? c0 : c1;
        } else if (h0) {
            cur = c0;
        } else if (h1) {
            cur = c1;
        } else {
            // pop the next box still in front of the best hit
            bool found = false;
            while (sp > 0) {
                --sp;
                if (stack_entry[sp] <= best * 1.0000038f + 1e-30f) {
                    cur = stack_node[sp];
                    found = true;
                    break;
                }
            }
            if (!found) break;
        }
    }
}

}  // namespace rdc
