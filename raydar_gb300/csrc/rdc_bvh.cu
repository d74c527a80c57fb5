// rdc_bvh.cu -- device build of the linear BVH used for large scenes.
//
//   1. object boxes and primitive records (host, exact reference constants)
//   2. 30-bit Morton code of each box centre in the cube spanning the scene's
//      centre bounds
//   3. stable radix sort of (code, object) pairs (rdc_sort.cu)
//   4. Karras, "Maximizing parallelism in the construction of BVHs, octrees
//      and k-d trees" (HPG 2012): internal node i of N-1 finds its key range
//      and split from the longest common prefixes of (code, position) keys
//   5. bottom-up refit: each leaf walks towards the root; at every node the
//      first arriving child records its box and stops (one atomic per node),
//      the second computes the union and continues.  No thread ever waits.
//   6. agglomerative treelet restructuring, two bottom-up passes (treelets of
//      9 leaves re-clustered by smallest union area; config 5: 18.2 -> 17.8
//      node visits per segment, +2.6%; a third pass adds nothing measurable)
//   6b. tree depth (Karras trees over 30-bit codes with position tie-breaks
//      are at most 63 deep; a restructured tree deeper than 62 is rebuilt
//      without restructuring)
//   7. collapse to 4-wide nodes, top down one level per pass: a 4-wide node
//      starts from its binary node's two children and opens the internal
//      child of largest surface area until it has four (a greedy surface-area
//      collapse); nodes are numbered level by level through a prefix sum
//      (rdc_sort.cu), so the layout is deterministic and every node's internal
//      children have consecutive indices.  If that tree would be deeper than
//      the traversal stack allows, every internal child is opened once
//      instead (each node takes its binary node's grandchildren), which
//      halves the depth.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "raydar_cuda.h"
#include "rdc_bvh.cuh"
#include "rdc_internal.hpp"

#ifndef RDC_BVH_RESTRUCTURE_PASSES
#define RDC_BVH_RESTRUCTURE_PASSES 2
#endif

namespace rdc {

namespace {

// Spread the low 10 bits of v so there are two zero bits between each.
__device__ __forceinline__ uint32_t spread3(uint32_t v) {
    v = (v | (v << 16)) & 0x030000FFu;
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

__global__ void morton_kernel(const float4* __restrict__ box, uint32_t n, float3 lo, float3 inv_ext,
                              uint32_t* keys, uint32_t* vals) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 a = box[2 * i], b = box[2 * i + 1];
    auto q = [](float v) {
        const float s = fminf(fmaxf(v * 1024.0f, 0.0f), 1023.0f);
        return (uint32_t)s;
    };
    const uint32_t x = q(((a.x + b.x) * 0.5f - lo.x) * inv_ext.x);
    const uint32_t y = q(((a.y + b.y) * 0.5f - lo.y) * inv_ext.y);
    const uint32_t z = q(((a.z + b.z) * 0.5f - lo.z) * inv_ext.z);
    keys[i] = (spread3(x) << 2) | (spread3(y) << 1) | spread3(z);
    vals[i] = i;
}

// Longest common prefix of the keys at sorted positions i and j, with the
// position as a tie-break; -1 outside [0, n).
__device__ __forceinline__ int lcp(const uint32_t* __restrict__ code, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    const uint32_t a = code[i], b = code[j];
    if (a != b) return __clz(a ^ b);
    return 32 + __clz((uint32_t)i ^ (uint32_t)j);
}

// parent_* entries are (parent node << 1) | slot, -1 for the root;
// parent_node is indexed by internal node, parent_leaf by object.
__global__ void karras_kernel(const uint32_t* __restrict__ code, const uint32_t* __restrict__ obj, int n,
                              BvhNode* nodes, int* parent_node, int* parent_leaf) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    const int d = (lcp(code, n, i, i + 1) - lcp(code, n, i, i - 1)) >= 0 ? 1 : -1;
    const int dmin = lcp(code, n, i, i - d);
    int lmax = 2;
    while (lcp(code, n, i, i + lmax * d) > dmin) lmax <<= 1;  // ends: lcp is -1 past the array
    int l = 0;
    for (int t = lmax >> 1; t >= 1; t >>= 1)
        if (lcp(code, n, i, i + (l + t) * d) > dmin) l += t;
    const int j = i + l * d;
    const int dnode = lcp(code, n, i, j);
    int s = 0;
    int t = l;
    do {
        t = (t + 1) >> 1;
        if (lcp(code, n, i, i + (s + t) * d) > dnode) s += t;
    } while (t > 1);
    const int g = i + s * d + min(d, 0);
    const int lo = min(i, j), hi = max(i, j);
    int c0, c1;
    if (lo == g) {
        c0 = ~(int)obj[g];
        parent_leaf[obj[g]] = (i << 1) | 0;
    } else {
        c0 = g;
        parent_node[g] = (i << 1) | 0;
    }
    if (hi == g + 1) {
        c1 = ~(int)obj[g + 1];
        parent_leaf[obj[g + 1]] = (i << 1) | 1;
    } else {
        c1 = g + 1;
        parent_node[g + 1] = (i << 1) | 1;
    }
    nodes[i].a.w = __int_as_float(c0);
    nodes[i].b.w = __int_as_float(c1);
    if (i == 0) parent_node[0] = -1;
}

__device__ __forceinline__ void put_box(BvhNode* nd, int slot, float3 lo, float3 hi) {
    if (slot == 0) {
        nd->a.x = lo.x; nd->a.y = lo.y; nd->a.z = lo.z;
        nd->b.x = hi.x; nd->b.y = hi.y; nd->b.z = hi.z;
    } else {
        nd->c.x = lo.x; nd->c.y = lo.y; nd->c.z = lo.z;
        nd->d.x = hi.x; nd->d.y = hi.y; nd->d.z = hi.z;
    }
}

__global__ void refit_kernel(const float4* __restrict__ box, const uint32_t* __restrict__ obj,
                             const int* __restrict__ parent_node, const int* __restrict__ parent_leaf, int n,
                             BvhNode* nodes, uint32_t* flags) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const float4 a = box[2 * obj[k]], b = box[2 * obj[k] + 1];
    float3 lo = make_float3(a.x, a.y, a.z), hi = make_float3(b.x, b.y, b.z);
    int p = parent_leaf[obj[k]];
    for (int level = 0; level < 128 && p >= 0; ++level) {
        const int node = p >> 1;
        put_box(&nodes[node], p & 1, lo, hi);
        __threadfence();
        if (atomicAdd(&flags[node], 1u) == 0u) return;  // the sibling finishes this node
        __threadfence();
        const float4 na = __ldcg(&nodes[node].a), nb = __ldcg(&nodes[node].b);
        const float4 nc = __ldcg(&nodes[node].c), ndd = __ldcg(&nodes[node].d);
        lo = make_float3(fminf(na.x, nc.x), fminf(na.y, nc.y), fminf(na.z, nc.z));
        hi = make_float3(fmaxf(nb.x, ndd.x), fmaxf(nb.y, ndd.y), fmaxf(nb.z, ndd.z));
        p = parent_node[node];
    }
}

__global__ void depth_kernel(const int* __restrict__ parent_node, const int* __restrict__ parent_leaf, int n,
                             uint32_t* max_depth) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    uint32_t depth = 1;
    int p = parent_leaf[k];
    while (p >= 0 && depth < 200) {
        ++depth;
        p = parent_node[p >> 1];
    }
    atomicMax(max_depth, depth);
}

// Agglomerative treelet restructuring (Domingues and Pedrini, "Bounding
// volume hierarchy optimization through agglomerative treelet restructuring",
// HPG 2015) over the Karras tree, which places every object at a leaf by its
// centre alone.  Bottom-up like the refit: one thread per object walks
// towards the root, the second arrival at a node handles it, so both of its
// subtrees are final and no other thread touches them.  At node X: the
// treelet's leaves start as X's two children and the internal one of largest
// surface area is opened until there are kTreelet; the leaves are then
// re-clustered by repeatedly merging the pair whose union has the smallest
// area, and the treelet's internal nodes (X last, as the new root, so X's
// parent link stands) are rewritten when the new sum of internal node areas
// is smaller.  The leaves' set and X's box do not change.
constexpr int kTreelet = 9;
constexpr int kRestructurePasses = RDC_BVH_RESTRUCTURE_PASSES;

__device__ __forceinline__ float area3(float3 lo, float3 hi) {
    const float dx = hi.x - lo.x, dy = hi.y - lo.y, dz = hi.z - lo.z;
    return dx * dy + dy * dz + dz * dx;
}

__device__ __forceinline__ void child_of(const BvhNode& nd, int slot, int& id, float3& lo, float3& hi) {
    const float4 l = slot ? nd.c : nd.a, h = slot ? nd.d : nd.b;
    id = __float_as_int(slot ? nd.b.w : nd.a.w);
    lo = make_float3(l.x, l.y, l.z);
    hi = make_float3(h.x, h.y, h.z);
}

__device__ __forceinline__ BvhNode load_node_cg(const BvhNode* nodes, int i) {
    BvhNode nd;
    nd.a = __ldcg(&nodes[i].a);
    nd.b = __ldcg(&nodes[i].b);
    nd.c = __ldcg(&nodes[i].c);
    nd.d = __ldcg(&nodes[i].d);
    return nd;
}

__device__ void restructure_treelet(int X, BvhNode* nodes, int* parent_node, int* parent_leaf) {
    int id[kTreelet];
    float3 lo[kTreelet], hi[kTreelet];
    int inner[kTreelet - 1];
    int ni = 0, k = 2;
    inner[ni++] = X;
    {
        const BvhNode nd = load_node_cg(nodes, X);
        child_of(nd, 0, id[0], lo[0], hi[0]);
        child_of(nd, 1, id[1], lo[1], hi[1]);
    }
    float old_cost = 0.0f;  // internal areas below X (X's own is the same before and after)
    while (k < kTreelet) {
        int best = -1;
        float ba = -1.0f;
        for (int j = 0; j < k; ++j) {
            if (id[j] < 0) continue;
            const float a = area3(lo[j], hi[j]);
            if (a > ba) {
                ba = a;
                best = j;
            }
        }
        if (best < 0) break;
        old_cost += ba;
        const int node = id[best];
        inner[ni++] = node;
        const BvhNode nd = load_node_cg(nodes, node);
        child_of(nd, 0, id[best], lo[best], hi[best]);
        child_of(nd, 1, id[k], lo[k], hi[k]);
        ++k;
    }
    if (k < 3) return;
    // agglomerative clustering: merge r creates node ml[r] = (left ma[r], right mb[r])
    int cid[kTreelet];
    float3 clo[kTreelet], chi[kTreelet];
    bool alive[kTreelet];
    for (int j = 0; j < k; ++j) {
        cid[j] = id[j];
        clo[j] = lo[j];
        chi[j] = hi[j];
        alive[j] = true;
    }
    int ma[kTreelet - 1], mb[kTreelet - 1];
    int mid_a[kTreelet - 1], mid_b[kTreelet - 1];
    float3 mlo_a[kTreelet - 1], mhi_a[kTreelet - 1], mlo_b[kTreelet - 1], mhi_b[kTreelet - 1];
    float new_cost = 0.0f;
    for (int r = 0; r < k - 1; ++r) {
        int bi = -1, bj = -1;
        float bd = __int_as_float(0x7f800000);
        for (int i = 0; i < k; ++i) {
            if (!alive[i]) continue;
            for (int j = i + 1; j < k; ++j) {
                if (!alive[j]) continue;
                const float3 ul = make_float3(fminf(clo[i].x, clo[j].x), fminf(clo[i].y, clo[j].y),
                                              fminf(clo[i].z, clo[j].z));
                const float3 uh = make_float3(fmaxf(chi[i].x, chi[j].x), fmaxf(chi[i].y, chi[j].y),
                                              fmaxf(chi[i].z, chi[j].z));
                const float d = area3(ul, uh);
                if (d < bd) {
                    bd = d;
                    bi = i;
                    bj = j;
                }
            }
        }
        ma[r] = bi;
        mb[r] = bj;
        mid_a[r] = cid[bi];
        mid_b[r] = cid[bj];
        mlo_a[r] = clo[bi];
        mhi_a[r] = chi[bi];
        mlo_b[r] = clo[bj];
        mhi_b[r] = chi[bj];
        const int node = (r == k - 2) ? X : inner[r + 1];
        if (r < k - 2) new_cost += bd;
        cid[bi] = node;
        clo[bi] = make_float3(fminf(clo[bi].x, clo[bj].x), fminf(clo[bi].y, clo[bj].y), fminf(clo[bi].z, clo[bj].z));
        chi[bi] = make_float3(fmaxf(chi[bi].x, chi[bj].x), fmaxf(chi[bi].y, chi[bj].y), fmaxf(chi[bi].z, chi[bj].z));
        alive[bj] = false;
    }
    if (!(new_cost < old_cost)) return;
    for (int r = 0; r < k - 1; ++r) {
        const int node = (r == k - 2) ? X : inner[r + 1];
        BvhNode nd;
        nd.a = make_float4(mlo_a[r].x, mlo_a[r].y, mlo_a[r].z, __int_as_float(mid_a[r]));
        nd.b = make_float4(mhi_a[r].x, mhi_a[r].y, mhi_a[r].z, __int_as_float(mid_b[r]));
        nd.c = make_float4(mlo_b[r].x, mlo_b[r].y, mlo_b[r].z, 0.0f);
        nd.d = make_float4(mhi_b[r].x, mhi_b[r].y, mhi_b[r].z, 0.0f);
        nodes[node] = nd;
        const int ch[2] = {mid_a[r], mid_b[r]};
        for (int slot = 0; slot < 2; ++slot) {
            if (ch[slot] >= 0)
                parent_node[ch[slot]] = (node << 1) | slot;
            else
                parent_leaf[~ch[slot]] = (node << 1) | slot;
        }
    }
    (void)ma;
    (void)mb;
}

__global__ void restructure_kernel(const int* __restrict__ parent_leaf_start, int n, BvhNode* nodes,
                                   int* parent_node, int* parent_leaf, uint32_t* flags) {
    const int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= n) return;
    int p = parent_leaf_start[o];
    for (int level = 0; level < 128 && p >= 0; ++level) {
        const int node = p >> 1;
        __threadfence();
        if (atomicAdd(&flags[node], 1u) == 0u) return;  // the sibling's thread finishes this node
        __threadfence();
        restructure_treelet(node, nodes, parent_node, parent_leaf);
        __threadfence();
        p = __ldcg(&parent_node[node]);
    }
}

// The children of the 4-wide node of binary node b, from b's two children:
//   greedy (surface-area collapse): open the internal child whose box has
//     the largest surface area (lowest slot on ties) until there are four or
//     only leaves are left;
//   level (the fallback for trees the greedy rule leaves too deep): open
//     every internal child once, so the node holds b's grandchildren and its
//     leaf children, and the 4-wide tree is half as deep as the binary one.
// Returns the count; ids are binary node indices (>= 0) or ~object.
__device__ __forceinline__ float half_area(float4 lo, float4 hi) {
    const float dx = hi.x - lo.x, dy = hi.y - lo.y, dz = hi.z - lo.z;
    return dx * dy + dy * dz + dz * dx;
}

constexpr int W = kBvhWidth;

__device__ __forceinline__ int wide_children(const BvhNode* __restrict__ bin, int b, bool level, int (&id)[W],
                                             float4 (&lo)[W], float4 (&hi)[W]) {
    const BvhNode nd = bin[b];
    id[0] = __float_as_int(nd.a.w);
    lo[0] = nd.a;
    hi[0] = nd.b;
    id[1] = __float_as_int(nd.b.w);
    lo[1] = nd.c;
    hi[1] = nd.d;
    int k = 2;
    if (level) {
        const int kk = k;
        for (int j = 0; j < kk; ++j) {
            if (id[j] < 0) continue;
            const BvhNode m = bin[id[j]];
            id[j] = __float_as_int(m.a.w);
            lo[j] = m.a;
            hi[j] = m.b;
            id[k] = __float_as_int(m.b.w);
            lo[k] = m.c;
            hi[k] = m.d;
            ++k;
        }
        return k;
    }
    while (k < W) {
        int best = -1;
        float ba = -1.0f;
        for (int j = 0; j < k; ++j) {
            if (id[j] < 0) continue;
            const float a = half_area(lo[j], hi[j]);
            if (a > ba) {
                ba = a;
                best = j;
            }
        }
        if (best < 0) break;
        const BvhNode m = bin[id[best]];
        id[best] = __float_as_int(m.a.w);
        lo[best] = m.a;
        hi[best] = m.b;
        id[k] = __float_as_int(m.b.w);
        lo[k] = m.c;
        hi[k] = m.d;
        ++k;
    }
    return k;
}

// Level pass 1: the number of internal children of each frontier node.
__global__ void collapse_count_kernel(const BvhNode* __restrict__ bin, const int2* __restrict__ front, uint32_t m,
                                      bool level, uint32_t* __restrict__ count) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    int id[W];
    float4 lo[W], hi[W];
    const int k = wide_children(bin, front[i].x, level, id, lo, hi);
    uint32_t c = 0;
    for (int j = 0; j < k; ++j) c += id[j] >= 0 ? 1u : 0u;
    count[i] = c;
}

// Level pass 2: write frontier node i's 4-wide node at front[i].y.  Its
// internal children take the first slots (in the order wide_children gives
// them) and become nodes next_base + off[i] + r, r = 0, 1, ..., and the next
// level's frontier entries off[i] + r; the leaf children follow.
__global__ void collapse_write_kernel(const BvhNode* __restrict__ bin, const int2* __restrict__ front, uint32_t m,
                                      bool level, const uint32_t* __restrict__ off, uint32_t next_base,
                                      Bvh4Node* out, int2* __restrict__ next) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    int id[W];
    float4 lo[W], hi[W];
    const int k = wide_children(bin, front[i].x, level, id, lo, hi);
    const float INF = __int_as_float(0x7f800000);
    Bvh4Node q;
    for (int j = 0; j < W; ++j) {
        for (int a = 0; a < 3; ++a) {
            q.pl[4 * a][j] = q.pl[4 * a + 3][j] = INF;
            q.pl[4 * a + 1][j] = q.pl[4 * a + 2][j] = -INF;
        }
        q.child[j] = 0;
    }
    q.leaves = 0u;
    q.first = (int)(next_base + off[i]);
    for (uint32_t& w : q.pad) w = 0u;
    uint32_t r = 0;
    int slot = 0;
    for (int pass = 0; pass < 2; ++pass) {  // internal children, then leaves
        for (int j = 0; j < k; ++j) {
            if ((id[j] >= 0) != (pass == 0)) continue;
            const float l3[3] = {lo[j].x, lo[j].y, lo[j].z}, h3[3] = {hi[j].x, hi[j].y, hi[j].z};
            for (int a = 0; a < 3; ++a) {
                q.pl[4 * a][slot] = l3[a];
                q.pl[4 * a + 1][slot] = h3[a];
                q.pl[4 * a + 2][slot] = h3[a];
                q.pl[4 * a + 3][slot] = l3[a];
            }
            if (id[j] < 0) {
                q.child[slot] = id[j];
                q.leaves |= 1u << slot;
            } else {
                const int idx = (int)(next_base + off[i] + r);
                q.child[slot] = idx;
                next[off[i] + r] = make_int2(id[j], idx);
                ++r;
            }
            ++slot;
        }
    }
    out[front[i].y] = q;
}

}  // namespace

void BvhDevice::release() {
    cudaFree(nodes);
    cudaFree(prims);
    cudaFree(scratch);
    nodes = nullptr;
    nnodes = 0;
    prims = nullptr;
    scratch = nullptr;
    scratch_bytes = 0;
    nobj = 0;
}

cudaError_t build_lbvh(const rdc_scene_desc* sc, BvhDevice& out, cudaStream_t s, uint32_t* depth_out) {
    const uint32_t n = sc->object_count;
    out.release();
    if (n == 0) return cudaSuccess;
    // Primitive records, object boxes, centre bounds and R on the host.
    std::vector<float4> prims(2 * (size_t)n), box(2 * (size_t)n);
    float clo[3] = {INFINITY, INFINITY, INFINITY}, chi[3] = {-INFINITY, -INFINITY, -INFINITY};
    double scene_r = 0.0;
    for (uint32_t i = 0; i < n; ++i) {
        const rdc_object& o = sc->objects[i];
        const double ext = o.geometry == RDC_GEOMETRY_SPHERE ? std::fabs((double)o.radius)
                                                               : std::fabs((double)o.side_length) * 0.5;
        double cl = 0.0;
        for (int a = 0; a < 3; ++a) cl += (double)o.center[a] * (double)o.center[a];
        scene_r = std::max(scene_r, std::sqrt(cl) + ext * 1.7320508075688772);
    }
    // Sphere leaf boxes are grown for origins up to o_max: the camera (its
    // primary rays) or any point of the scene (the hit points that start
    // every later segment).  Rays from further away add the rest per ray.
    const double cam = std::sqrt((double)sc->camera.position[0] * sc->camera.position[0] +
                                 (double)sc->camera.position[1] * sc->camera.position[1] +
                                 (double)sc->camera.position[2] * sc->camera.position[2]);
    const double o_max = std::max(cam, scene_r * 1.0001);
    // float lower / upper neighbours of a double (outward rounding)
    auto down = [](double x) {
        float f = (float)x;
        if ((double)f > x) f = std::nextafter(f, -INFINITY);
        return f;
    };
    auto upr = [](double x) {
        float f = (float)x;
        if ((double)f < x) f = std::nextafter(f, INFINITY);
        return f;
    };
    for (uint32_t i = 0; i < n; ++i) {
        const rdc_object& o = sc->objects[i];
        const float* c = o.center;
        int kind = (int)o.geometry;
        float kb;
        std::memcpy(&kb, &kind, 4);
        double ext;
        if (o.geometry == RDC_GEOMETRY_SPHERE) {
            prims[2 * i] = make_float4(c[0], c[1], c[2], (c[0] * c[0] + c[1] * c[1]) + c[2] * c[2]);
            prims[2 * i + 1] = make_float4(o.radius * o.radius, 0.0f, 0.0f, kb);
            // The expanded quadratic can report a hit for a ray passing within
            // sqrt(r^2 (1 + 2^-20) + 2^-19 (|o| + |c|)^2) of the centre (the
            // rounding bound in the traversal's comment).
            const double r = std::fabs((double)o.radius);
            const double cn = std::sqrt(((double)c[0] * c[0] + (double)c[1] * c[1]) + (double)c[2] * c[2]);
            const double s = o_max + cn;
            ext = std::sqrt(r * r * (1.0 + 0x1p-20) + 0x1p-19 * s * s) * (1.0 + 0x1p-40);
        } else {
            const float h = o.side_length * 0.5f;
            prims[2 * i] = make_float4(c[0] - h, c[0] + h, c[1] - h, c[1] + h);
            prims[2 * i + 1] = make_float4(c[2] - h, c[2] + h, 0.0f, kb);
            ext = std::fabs((double)h);
        }
        box[2 * i] = make_float4(down(c[0] - ext), down(c[1] - ext), down(c[2] - ext), 0.0f);
        box[2 * i + 1] = make_float4(upr(c[0] + ext), upr(c[1] + ext), upr(c[2] + ext), 0.0f);
        for (int a = 0; a < 3; ++a) {
            clo[a] = std::min(clo[a], c[a]);
            chi[a] = std::max(chi[a], c[a]);
        }
    }
    out.nobj = n;
    out.scene_r = upr(scene_r * 1.0001);
    out.o_max = down(o_max);

    // Device buffers: the 4-wide nodes + prims are kept; the rest (binary
    // nodes included) is build scratch.
    const size_t n_int = n >= 2 ? (size_t)n - 1 : 1;
    cudaError_t e = dev_malloc((void**)&out.prims, prims.size() * sizeof(float4));
    const size_t sort_tmp = radix_sort_scratch_bytes(n), scan_tmp = exclusive_scan_scratch_bytes((uint32_t)n_int);
    // scratch: box (2n float4) | binary nodes (n-1) | keys, keys2, vals, vals2 (4n u32) | parents (2n int) |
    //          flags, counts, map (3n u32) | two collapse frontiers (n-1 int2 each) | depth | sort tmp | scan tmp
    const size_t box_b = 2 * (size_t)n * sizeof(float4);
    const size_t bin_b = n_int * sizeof(BvhNode);
    const size_t u32_b = (size_t)n * 4;
    auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const size_t front_b = n_int * sizeof(int2);
    const size_t total =
        up(box_b) + up(bin_b) + 9 * up(u32_b) + 2 * up(front_b) + up(256) + up(sort_tmp) + up(scan_tmp) + 256;
    if (e == cudaSuccess) e = dev_malloc((void**)&out.scratch, total);
    if (e != cudaSuccess) {
        out.release();
        return e;
    }
    out.scratch_bytes = total;
    char* sp = static_cast<char*>(out.scratch);
    auto take = [&](size_t bytes) {
        char* p = sp;
        sp += (bytes + 255) & ~(size_t)255;
        return p;
    };
    float4* d_box = (float4*)take(box_b);
    BvhNode* bin = (BvhNode*)take(bin_b);
    uint32_t* keys = (uint32_t*)take(u32_b);
    uint32_t* keys2 = (uint32_t*)take(u32_b);
    uint32_t* vals = (uint32_t*)take(u32_b);
    uint32_t* vals2 = (uint32_t*)take(u32_b);
    int* parent_node = (int*)take(u32_b);
    int* parent_leaf = (int*)take(u32_b);
    uint32_t* flags = (uint32_t*)take(u32_b);
    uint32_t* counts = (uint32_t*)take(u32_b);
    uint32_t* map = (uint32_t*)take(u32_b);
    int2* front = (int2*)take(front_b);
    int2* front_next = (int2*)take(front_b);
    uint32_t* d_depth = (uint32_t*)take(256);
    void* d_sort = take(sort_tmp);
    void* d_scan = take(scan_tmp);

    e = cudaMemcpyAsync(out.prims, prims.data(), prims.size() * sizeof(float4), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_box, box.data(), box_b, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(flags, 0, u32_b, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_depth, 0, 4, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(bin, 0, bin_b, s);
    if (e != cudaSuccess) return e;
    const float3 lo = make_float3(clo[0], clo[1], clo[2]);
    auto inv = [](float a, float b) { return b > a ? 1.0f / (b - a) : 0.0f; };
    // One scale for all axes (the largest extent): per-axis scaling would split
    // a flat domain's short axis as often as its long ones, giving flat boxes
    // of large surface area (config 5's 40 x 10 x 40 box: 19.8 -> 18.5 node
    // visits per segment, +6%).
    const float ext = std::max(chi[0] - clo[0], std::max(chi[1] - clo[1], chi[2] - clo[2]));
    const float ie = inv(0.0f, ext);
    const float3 inv_ext = make_float3(ie, ie, ie);
    const uint32_t B = 256, G = (n + B - 1) / B;
    morton_kernel<<<G, B, 0, s>>>(d_box, n, lo, inv_ext, keys, vals);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    {
        uint32_t *ks = nullptr, *vs = nullptr;
        e = radix_sort_pairs(keys, vals, keys2, vals2, n, 30, d_sort, s, &ks, &vs);
        if (e != cudaSuccess) return e;
        if (ks != keys2) {  // the sorted pairs are in (keys2, vals2) from here on
            std::swap(keys, keys2);
            std::swap(vals, vals2);
        }
    }
    uint32_t depth = 1;
    if (n >= 2) {
        const uint32_t GI = (uint32_t)((n_int + B - 1) / B);
        // Karras tree, refit, then treelet restructuring passes (each pass
        // bottom-up; the leaves' starting parents are snapshot into keys, free
        // after the sort).  Restructuring can deepen the tree: should it pass
        // the depth the 4-wide traversal allows, the tree is rebuilt without.
        for (int passes = kRestructurePasses;; passes = 0) {
            karras_kernel<<<GI, B, 0, s>>>(keys2, vals2, (int)n, bin, parent_node, parent_leaf);
            if ((e = cudaGetLastError()) != cudaSuccess) return e;
            e = cudaMemsetAsync(flags, 0, u32_b, s);
            if (e != cudaSuccess) return e;
            refit_kernel<<<G, B, 0, s>>>(d_box, vals2, parent_node, parent_leaf, (int)n, bin, flags);
            if ((e = cudaGetLastError()) != cudaSuccess) return e;
            for (int pass = 0; pass < passes; ++pass) {
                e = cudaMemsetAsync(flags, 0, u32_b, s);
                if (e == cudaSuccess) e = cudaMemcpyAsync(keys, parent_leaf, u32_b, cudaMemcpyDeviceToDevice, s);
                if (e != cudaSuccess) return e;
                restructure_kernel<<<G, B, 0, s>>>((const int*)keys, (int)n, bin, parent_node, parent_leaf, flags);
                if ((e = cudaGetLastError()) != cudaSuccess) return e;
            }
            e = cudaMemsetAsync(d_depth, 0, 4, s);
            if (e != cudaSuccess) return e;
            depth_kernel<<<G, B, 0, s>>>(parent_node, parent_leaf, (int)n, d_depth);
            if ((e = cudaGetLastError()) != cudaSuccess) return e;
            e = cudaMemcpyAsync(&depth, d_depth, 4, cudaMemcpyDeviceToHost, s);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
            if (e != cudaSuccess) return e;
            if (depth <= 62 || passes == 0) break;
        }

        // Collapse to 4-wide nodes, one level per pass (count, scan, write):
        // the greedy surface-area rule, or, should that tree be deeper than
        // the traversal stack allows (32 levels, 3 entries each), the level
        // rule (the binary tree is at most 63 deep, so at most 32 levels).  At
        // most n - 1 4-wide nodes (each holds >= 2 children).
        static_assert(kBvhMaxLevels >= 32, "stack too short for the level rule");
        e = dev_malloc((void**)&out.nodes, n_int * sizeof(Bvh4Node));
        if (e != cudaSuccess) return e;
        uint32_t m = 1, total = 1;
        for (int mode = 0; mode < 2; ++mode) {  // 0: greedy surface area, 1: level rule
            const int2 root = make_int2(0, 0);
            e = cudaMemcpyAsync(front, &root, sizeof(int2), cudaMemcpyHostToDevice, s);
            if (e != cudaSuccess) return e;
            m = 1;
            total = 1;
            uint32_t levels = 0;
            while (m > 0 && levels < (uint32_t)kBvhMaxLevels) {
                ++levels;
                const uint32_t GM = (m + B - 1) / B;
                collapse_count_kernel<<<GM, B, 0, s>>>(bin, front, m, mode != 0, counts);
                if ((e = cudaGetLastError()) != cudaSuccess) return e;
                e = exclusive_scan(counts, map, m, d_scan, s);
                if (e != cudaSuccess) return e;
                collapse_write_kernel<<<GM, B, 0, s>>>(bin, front, m, mode != 0, map, total, out.nodes, front_next);
                if ((e = cudaGetLastError()) != cudaSuccess) return e;
                uint32_t tl[2] = {0, 0};
                e = cudaMemcpyAsync(&tl[0], map + m - 1, 4, cudaMemcpyDeviceToHost, s);
                if (e == cudaSuccess) e = cudaMemcpyAsync(&tl[1], counts + m - 1, 4, cudaMemcpyDeviceToHost, s);
                if (e == cudaSuccess) e = cudaStreamSynchronize(s);
                if (e != cudaSuccess) return e;
                m = tl[0] + tl[1];
                total += m;
                std::swap(front, front_next);
            }
            if (m == 0) break;
        }
        if (m != 0) return cudaErrorUnknown;  // unreachable: the level rule's tree fits the stack
        out.nnodes = total;
    }
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return e;
    if (depth_out) *depth_out = depth;
    cudaFree(out.scratch);
    out.scratch = nullptr;
    out.scratch_bytes = 0;
    return e;
}

}  // namespace rdc
