// rdc_bvh.cuh -- traversal of the device-built LBVH (rdc_bvh.cu builds it).
//
// The reference tests every object (src/renderer/cpu.rs:344-352).  For large
// scenes the kernels instead walk a linear BVH: Morton-ordered objects, a
// Karras (2012) radix tree of N-1 internal nodes, collapsed into a 4-wide
// tree (each node takes up to four binary descendants as its children):
// about half the dependent node loads per ray, four independent box tests per
// node.  The result must be the reference's exactly:
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

// 4-wide node, 256 bytes.  For each axis a, 64 bytes of its children's box
// planes: pl[4a][j] = min of child j, pl[4a + 1][j] = max, pl[4a + 2][j] =
// max, pl[4a + 3][j] = min.  For a positive direction component a box's near
// plane on that axis is its minimum, for a negative one its maximum, so a ray
// reads the 32 bytes at 64a (positive) or 64a + 32 (negative) and has the
// near planes of all four children in the first half and the far planes in
// the second: one aligned 256-bit load per axis, one L1 access per lane, and
// no per-child min/max to order the planes.  (Planes stored once, near and
// far read with two 16-byte loads per axis, measured 11% slower: seven L1
// accesses per visit instead of four, with the L1 data pipe the bound; 8-wide
// nodes cut node visits per segment from 18.0 to 12.5 but cost 1.56x per
// visit, 7% slower overall.)  child[j]: >= 0 node, < 0 ~object; the internal
// children take the first slots, at consecutive node indices from `first`
// (slot j's node is first + j).  leaves: bit j set when slot j holds an
// object.  An unused slot has min = +inf, max = -inf: every ray's near plane
// there is +inf and its far plane -inf, so it is never entered.
constexpr int kBvhWidth = 4;
struct alignas(32) Bvh4Node {
    float pl[12][4];
    int child[4];
    uint32_t leaves;
    int first;
    uint32_t pad[10];
};
static_assert(sizeof(Bvh4Node) == 256, "4-wide node layout");

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

// Conservative slab tests of a node's children, boxes [lo - m, hi + m] (m
// the per-ray growth).  Per axis, with oa = (o + m) / d and ob = (o - m) / d,
// the plane distances are lo / d - oa and hi / d - ob, one FMA each; the near
// one is lo's for d >= 0 (1/d carries d's sign, zeros included) and hi's
// otherwise, which fixes per ray which plane each load returns and which
// origin term goes with it.  Their rounding (a few ulp of |o| + |lo| along
// the ray) is far inside the 2^-20 (|o| + 2R) part of m, so the box's entry
// and exit are compared as computed; 2m also keeps far - near positive for
// every non-empty box, so ordering the planes by the sign of 1/d gives the
// same entry and exit as ordering them by value.
struct BvhRayBox {
    float inv[3];       // 1/d per axis
    float nn[3], nf[3]; // -(near origin term), -(far origin term) per axis
    uint32_t neg;       // sign bits of 1/d: x in bit 0, y 1, z 2
};

// Entry (max(0, near)) of every child box, and a bit per child whose box is
// entered no later than limit and left no earlier than 0.
__device__ __forceinline__ unsigned bvh_boxes(const char* nb, const BvhRayBox& R, float limit, float (&e)[4]) {
    float4 n[3], f[3];  // per axis: near planes of children 0-3, far planes
#pragma unroll
    for (int a = 0; a < 3; ++a)
        ldg_pair(reinterpret_cast<const float4*>(nb + 64 * a + ((R.neg >> a) & 1u) * 32u), n[a], f[a]);
    const float nx[4] = {n[0].x, n[0].y, n[0].z, n[0].w}, fx[4] = {f[0].x, f[0].y, f[0].z, f[0].w};
    const float ny[4] = {n[1].x, n[1].y, n[1].z, n[1].w}, fy[4] = {f[1].x, f[1].y, f[1].z, f[1].w};
    const float nz[4] = {n[2].x, n[2].y, n[2].z, n[2].w}, fz[4] = {f[2].x, f[2].y, f[2].z, f[2].w};
    unsigned hits = 0u;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const float en = fmax3(__fmaf_rn(nx[j], R.inv[0], R.nn[0]), __fmaf_rn(ny[j], R.inv[1], R.nn[1]),
                               fmaxf(__fmaf_rn(nz[j], R.inv[2], R.nn[2]), 0.0f));
        const float ex = fmin3(__fmaf_rn(fx[j], R.inv[0], R.nf[0]), __fmaf_rn(fy[j], R.inv[1], R.nf[1]),
                               fminf(__fmaf_rn(fz[j], R.inv[2], R.nf[2]), limit));
        e[j] = en;
        hits |= (en <= ex ? 1u : 0u) << j;
    }
    return hits;
}

// One ray's traversal, resumable one node visit at a time.  The stack lives
// with the caller: a visit leaves at most kBvhWidth - 1 siblings pending, and
// the build keeps the wide tree at most kBvhMaxLevels deep (a binary Karras
// tree over 30-bit codes with 32-bit index tie-breaks is at most 63 deep).
struct BvhTrav {
    BvhRayBox box;       // the ray's per-axis box-test terms
    float best;          // closest hit so far (+inf: none)
    int bidx;            // its object (-1: none)
    int cur;             // next node to visit; -1 when no node is left
    int sp;              // stack depth
    int lnode;           // node whose leaf children in lmask are still to be tested
    unsigned lmask;      // the traversal is over when cur < 0 and lmask == 0
};

constexpr int kBvhStack = 96;
constexpr int kBvhMaxLevels = kBvhStack / (kBvhWidth - 1);  // 32

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
    // (r.rd is RN(1/d), the IEEE quotient 1.0f / d)
    auto inv1 = [cap](float v, float rv) { return fabsf(v) * cap < 1.0f ? copysignf(cap, v) : rv; };
    const float iv[3] = {inv1(r.d.x, r.rd.x), inv1(r.d.y, r.rd.y), inv1(r.d.z, r.rd.z)};
    const float ov[3] = {r.o.x, r.o.y, r.o.z};
    uint32_t sg = 0;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float oa = (ov[a] + m) * iv[a], ob = (ov[a] - m) * iv[a];
        const bool neg = __float_as_uint(iv[a]) >> 31;  // near plane: the maximum
        T.box.inv[a] = iv[a];
        T.box.nn[a] = neg ? -ob : -oa;
        T.box.nf[a] = neg ? -oa : -ob;
        sg |= (neg ? 1u : 0u) << a;
    }
    T.box.neg = sg;
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
    __device__ __forceinline__ void put(int i, uint2 e) { a[i] = e; }
    __device__ __forceinline__ void push(int& sp, uint2 e) { a[sp++] = e; }
    __device__ __forceinline__ uint2 pop(int& sp) { return a[--sp]; }
};

struct SplitStack {
    uint2* sh;
    uint32_t stride;
    uint2* loc;
    __device__ __forceinline__ void put(int i, uint2 e) {
        if (i < kShortStack)
            sh[(uint32_t)i * stride] = e;
        else
            loc[i - kShortStack] = e;
    }
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

// Compare-exchange of two sort keys, ascending.
__device__ __forceinline__ void bvh_cswap(uint32_t& a, uint32_t& b) {
    const uint32_t lo = umin(a, b);
    b = umax(a, b);
    a = lo;
}

// Sort network on the visit's four keys, ascending (5 compare-exchanges).
__device__ __forceinline__ void bvh_sort(uint32_t (&k)[4]) {
    bvh_cswap(k[0], k[1]);
    bvh_cswap(k[2], k[3]);
    bvh_cswap(k[0], k[2]);
    bvh_cswap(k[1], k[3]);
    bvh_cswap(k[1], k[2]);
}

// One node visit (T.cur >= 0, T.lmask == 0): the child boxes; leaf children
// hit are left in T.lmask for bvh_leaf_step (a warp tests them together
// instead of one lane at a time inside the visit); the nearest internal child
// hit is visited next and the others pushed, farthest first; with none, the
// next stacked box still in front of the best hit, or none (T.cur = -1).
// Internal children are ordered by a key per slot: the entry distance's bits
// (non-negative: ordered as unsigned integers) with the low bits replaced by
// the slot, at most 3 ulp off the entry; the stack keeps the entry rounded
// down to a multiple of 4 ulp, so its test against the best hit stays
// conservative.
template <class Stack>
__device__ __forceinline__ void bvh_step(const BvhView& bv, const RayPre& r, bool fast, BvhTrav& T, Stack& stack,
                                         BvhCounters& cnt) {
    const Bvh4Node* node = bv.nodes + checked_index(bv.oob, T.cur, bv.nnodes);
    const char* nb = reinterpret_cast<const char*>(node);
    const uint2 meta = __ldg(reinterpret_cast<const uint2*>(&node->leaves));  // (leaves, first)
    ++cnt.visits;
    // limit: skip a box whose entry exceeds best (relative slack for the box test's rounding)
    const float limit = T.best * 1.0000038f + 1e-30f;
    float e[kBvhWidth];
    const unsigned hits = bvh_boxes(nb, T.box, limit, e);
    T.lmask = hits & meta.x;
    T.lnode = T.cur;
    const unsigned inner = hits & ~meta.x;
    const uint32_t NONE = 0xffffffffu;
    const uint32_t SLOT = kBvhWidth - 1u;
    uint32_t k[kBvhWidth];
#pragma unroll
    for (int j = 0; j < kBvhWidth; ++j)
        k[j] = ((inner >> j) & 1u) ? (__float_as_uint(e[j]) & (0x7fffffffu & ~SLOT)) | (uint32_t)j : NONE;
    bvh_sort(k);
    const int first = (int)meta.y;
    if (k[0] != NONE) {
        // an entry is (node, entry distance bits): one 8-byte store or load
#pragma unroll
        for (int j = kBvhWidth - 1; j >= 1; --j)
            if (k[j] != NONE) stack.push(T.sp, make_uint2((unsigned)(first + (int)(k[j] & SLOT)), k[j] & ~SLOT));
        T.cur = first + (int)(k[0] & SLOT);
    } else {
        // pop the next box still in front of the best hit
        int next = -1;
        while (T.sp > 0) {
            const uint2 top = stack.pop(T.sp);
            if (__uint_as_float(top.y) <= limit) {
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
    const int child = __ldg(&bv.nodes[checked_index(bv.oob, T.lnode, bv.nnodes)].child[j]);
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
