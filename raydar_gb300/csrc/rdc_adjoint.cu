// rdc_adjoint.cu -- path-replay adjoint of the render (sm_103a).
//
// The loss is any function of the mean-radiance image; the caller passes
// dL/dimage (RGB per pixel).  A path of pixel p contributes
//     L = sum_k E(obj_k) + [miss after K hits] sky(d_K) * prod_k albedo(obj_k)
// (src/renderer/cpu.rs:253-341: emission is added without attenuation, the
// miss adds the sky times the albedo product), weighted by
// dL/dimage(p) / spp.  Gradients per object:
//   - emission E = emission_color * emission_strength: the weight, once per hit;
//   - albedo: weight * sky * the product of the path's other albedos;
//   - roughness^2 (the host applies d(r^2)/dr = 2r), two parts:
//     * pathwise: through the miss direction d_K.  The kernel seeds the
//       adjoint of d_K with the sky's derivative and sweeps the path's
//       vertices in reverse, through the scatter (normalize, reflect,
//       refract), the front-face flip, the sphere normal and the ray
//       parameter t (implicit differentiation of the hit surface);
//     * lobe choice (score function): two coins pick a lobe with a
//       probability that depends on the parameters -- U_rough < r^2 picks
//       diffuse over specular (cpu.rs:309-313; P = r^2 or 1 - r^2) and
//       Schlick's R < U_fresnel picks refraction over reflection
//       (cpu.rs:296-297; P = 1 - R or R, where R depends on the incoming
//       direction and so on the roughness of every earlier vertex).  A
//       vertex whose lobe a coin chose adds w_k * d log P / d(params), with
//       w_k the weighted radiance the path gathers after that choice (the
//       emission of later hits and the sky term); d log P flows into r^2
//       directly or, for R, backwards through the incoming ray like the
//       pathwise part.  In expectation this is the derivative of the lobe
//       probabilities; it is exact for 0 < roughness < 1.  At roughness 1 (a
//       lobe that is always diffuse) the specular alternative is never
//       sampled, so the derivative from below misses its -E[specular] half.
// Not differentiated: which object a ray hits (a roughness step can move a
// ray across another object's silhouette: a boundary term), the diffuse
// flip and the total-internal-reflection edge.
//
// Nothing of the forward pass is stored: each path is replayed from its
// Philox counter (pixel, sample, bounce) with the forward kernels' own
// functions, so it retraces the rendered path bit for bit, into a per-thread
// record of at most kAdjMaxBounces vertices of 44 bytes (incoming ray, hit
// distance, object and scatter flags, the lobe's unit-sphere vector; keeping
// the vector measured 13% faster than recomputing its Philox words in the
// sweep).  Gradients are summed per
// warp over lanes that hit the same object (match + pointer-jumping
// reduction) and added with FP32 atomics, into per-block shared accumulators
// when the scene's gradient table fits, else straight into global memory.
#include <cstdint>

#include "rdc_bvh.cuh"
#include "rdc_device.cuh"

namespace rdc {

namespace {

// One vertex of a replayed path (44 bytes): the ray that reaches it, its
// hit distance, the object index (low 24 bits) with the scatter flags (high
// 8) and the unit-sphere vector the lobe added.  After the reverse sweep o
// holds the vertex's albedo gradient without the albedos before it, and t
// its dL/d(roughness^2).
struct AdjVert {
    V3 o, d;
    float t;
    uint32_t objf;
    V3 s;
};

__device__ __forceinline__ V3 vjp_normalize(V3 v, V3 u, float len, V3 g) {
    // u = v / len: du = (dv - u (u . dv)) / len
    (void)v;
    return vmul(vsub(g, vmul(u, vdot(g, u))), 1.0f / len);
}

// Reverse step through vertex v: (go, gd) are the adjoints of the ray that
// leaves v; on return those of the ray that reaches v.  s is the lobe's
// unit-sphere vector, wk the weighted radiance gathered after the vertex's
// scatter (for the coin terms).  Returns dL/d(roughness^2) of this vertex.
__device__ __forceinline__ float vertex_vjp(const SceneView& sc, const AdjVert& v, const MatDev& m, V3 s,
                                            float wk, V3& go, V3& gd) {
    const int obj = (int)(v.objf & 0xFFFFFFu);
    const uint32_t f = v.objf >> 24;
    const float4 hi = __ldg(&sc.hit[checked_index(sc.oob, obj, sc.nobj)]);
    const int kind = __float_as_int(m.d.y);
    const HitRec h = closest_hit(v.o, v.d, v.t, hi, kind);
    const float r = m.a.w;
    const V3 d = v.d, n = h.n;
    V3 g_dir = mk(0.f, 0.f, 0.f), g_n = mk(0.f, 0.f, 0.f);
    if (f & kScatNormal)
        g_n = gd;
    else
        g_dir = gd;
    if (f & kScatTrans)
        g_dir = vadd(g_dir, vmul(go, 0.0001f));
    else
        g_n = vadd(g_n, vmul(go, 0.0001f));
    V3 g_p = go, g_din = mk(0.f, 0.f, 0.f);
    float gr = 0.0f;
    const uint32_t lobe = f & 3u;

    // U_rough < r^2: P(diffuse) = r^2, P(specular) = 1 - r^2
    if (f & kScatRoughCoin) gr += lobe == kLobeDiffuse ? wk / r : -wk / (1.0f - r);

    // Fresnel quantities of a transmission vertex: rd = d / |d|,
    // cos = min(-rd.n, 1), R = r0 + (1 - r0)(1 - cos)^5
    float dl = 1.0f, cr = 0.0f, cs = 0.0f, g_cs = 0.0f;
    V3 rd = d;
    if (f & kScatTrans) {
        dl = sqrtf(vdot(d, d));
        rd = vmul(d, 1.0f / dl);
        cr = -vdot(rd, n);
        cs = fminf(cr, 1.0f);
        if (f & kScatFresnelCoin) {
            const float r0 = (f & kScatFront) ? m.c.w : m.d.x;
            const float mm = 1.0f - cs;
            const float m2 = mm * mm;
            const float R = r0 + (1.0f - r0) * (mm * (m2 * m2));
            const float gR = lobe == kLobeRefract ? -wk / (1.0f - R) : wk / R;
            g_cs = gR * (-5.0f * (1.0f - r0) * (m2 * m2));
        }
    }

    if (lobe == kLobeDiffuse) {
        g_n = (f & kScatFlip) ? vsub(g_n, g_dir) : vadd(g_n, g_dir);  // dir = +-(n + s1)
    } else if (lobe == kLobeSpecular) {
        // dir = X / |X|, X = d - 2 (d.n) n + s2 r
        const float dn = vdot(d, n);
        const V3 X = vadd(vsub(d, vmul(n, 2.0f * dn)), vmul(s, r));
        const float L = sqrtf(vdot(X, X));
        const V3 gX = vjp_normalize(X, vmul(X, 1.0f / L), L, g_dir);
        gr += vdot(s, gX);
        const float ngX = vdot(n, gX);
        g_din = vadd(g_din, vsub(gX, vmul(n, 2.0f * ngX)));
        g_n = vsub(g_n, vadd(vmul(gX, 2.0f * dn), vmul(d, 2.0f * ngX)));
        if ((f & kScatTrans) && cr < 1.0f && g_cs != 0.0f) {
            // a reflection the Fresnel coin chose: R's cos through rd and n
            g_n = vsub(g_n, vmul(rd, g_cs));
            g_din = vadd(g_din, vjp_normalize(d, rd, dl, vmul(n, -g_cs)));
        }
    } else {
        // dir = Z / |Z|, Z = perp + s n + s3 r, perp = ratio (rd + cos n),
        // s = -sqrt|1 - perp.perp|, cos = min(-rd.n, 1), rd = d / |d|
        const float ratio = (f & kScatFront) ? m.c.y : m.c.z;
        const V3 perp = vmul(vadd(rd, vmul(n, cs)), ratio);
        const float q = 1.0f - vdot(perp, perp);
        const float sq = sqrtf(fabsf(q));
        const V3 Z = vadd(vadd(perp, vmul(n, -sq)), vmul(s, r));
        const float L = sqrtf(vdot(Z, Z));
        const V3 gZ = vjp_normalize(Z, vmul(Z, 1.0f / L), L, g_dir);
        gr += vdot(s, gZ);
        V3 g_perp = gZ;
        const float gs = vdot(n, gZ);
        g_n = vadd(g_n, vmul(gZ, -sq));
        if (sq > 1e-12f) g_perp = vadd(g_perp, vmul(perp, gs * (q < 0.0f ? -1.0f : 1.0f) / sq));
        V3 g_rd = vmul(g_perp, ratio);
        const float gcos = ratio * vdot(n, g_perp) + g_cs;
        g_n = vadd(g_n, vmul(g_perp, ratio * cs));
        if (cr < 1.0f) {
            g_rd = vsub(g_rd, vmul(n, gcos));
            g_n = vsub(g_n, vmul(rd, gcos));
        }
        g_din = vadd(g_din, vjp_normalize(d, rd, dl, g_rd));
    }
    // n = +-n0 (front-face flip); sphere n0 = (p - c) / |p - c|, cube n0 constant
    const V3 g_n0 = h.front ? g_n : vneg(g_n);
    const V3 c = mk(hi.x, hi.y, hi.z);
    const V3 pc = vsub(h.p, c);
    if (kind == 0) {
        const float pl = sqrtf(vdot(pc, pc));
        const V3 n0 = vmul(pc, 1.0f / pl);
        g_p = vadd(g_p, vjp_normalize(pc, n0, pl, g_n0));
    }
    // p = o + t d with t(o, d) on the hit surface
    const float g_t = vdot(g_p, d);
    V3 go_new = g_p;
    V3 gd_new = vadd(g_din, vmul(g_p, v.t));
    if (kind == 0) {
        // |o + t d - c|^2 = r^2:  dt = -(p - c).(do + t dd) / ((p - c).d)
        const float den = vdot(pc, d);
        if (fabsf(den) > 1e-20f) {
            const float k = g_t / den;
            go_new = vsub(go_new, vmul(pc, k));
            gd_new = vsub(gd_new, vmul(pc, k * v.t));
        }
    } else {
        // the hit face's plane x_i = const:  dt = -(do_i + t dd_i) / d_i
        const int ax = n.x != 0.0f ? 0 : (n.y != 0.0f ? 1 : 2);
        const float di = ax == 0 ? d.x : (ax == 1 ? d.y : d.z);
        if (fabsf(di) > 1e-20f) {
            const float k = g_t / di;
            if (ax == 0) {
                go_new.x -= k;
                gd_new.x -= k * v.t;
            } else if (ax == 1) {
                go_new.y -= k;
                gd_new.y -= k * v.t;
            } else {
                go_new.z -= k;
                gd_new.z -= k * v.t;
            }
        }
    }
    go = go_new;
    gd = gd_new;
    return gr;
}

// Sum c[0..6] over the lanes of the warp with the same obj (>= 0) and add
// the sums at g + 8 * obj with one atomic per object and component: the
// lanes sharing an object form a list in lane order, and pointer jumping
// (as many rounds as the largest list needs, at most 5) leaves the list's
// total with its first lane.
__device__ __forceinline__ void warp_add_grad(float* g, int obj, float c[7], unsigned long long* oob, uint32_t nobj) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const unsigned peers = __match_any_sync(FULL, obj);
    const unsigned above = lane == 31 ? 0u : (peers & (0xffffffffu << (lane + 1)));
    int next = above ? __ffs(above) - 1 : lane;
    bool has = above != 0u;
    // ceil(log2) of the largest group: after r rounds a lane holds the sum of
    // 2^r consecutive members of its list, so that many rounds give every
    // head its group's total (groups are mostly small after the first vertex;
    // measured 8.29 -> 8.06 ms on config 4 against a fixed 5 rounds)
    const unsigned big = __reduce_max_sync(FULL, obj >= 0 ? (unsigned)__popc(peers) : 1u);  // no vertex: no sum
    const int nrounds = big > 1u ? 32 - __clz((int)(big - 1u)) : 0;
#pragma unroll 1
    for (int round = 0; round < nrounds; ++round) {  // rolled: less code for the fetch-bound kernel
        float o[7];
#pragma unroll
        for (int j = 0; j < 7; ++j) o[j] = __shfl_sync(FULL, c[j], next);
        const int nn = __shfl_sync(FULL, next, next);
        const bool nh = __shfl_sync(FULL, has ? 1 : 0, next) != 0;
        if (has) {
#pragma unroll
            for (int j = 0; j < 7; ++j) c[j] += o[j];
            next = nn;
            has = nh;
        }
    }
    if (obj >= 0 && lane == __ffs(peers) - 1) {
        float* dst = g + 8 * (size_t)checked_index(oob, obj, nobj);
#pragma unroll
        for (int j = 0; j < 7; ++j)
            if (c[j] != 0.0f) atomicAdd(dst + j, c[j]);
    }
}

// Resident blocks per SM the register budget is sized for: with the vertex
// records in local memory 4 (64 registers; 3, 4 and 5 measured within 2% of
// each other on config 4, 4 the fastest); with them in shared memory, which
// holds 3 blocks of 6-bounce records, 3 (80 registers, fewer spills).
#ifndef RDC_ADJ_MIN_BLOCKS
#define RDC_ADJ_MIN_BLOCKS 4
#endif
#ifndef RDC_ADJ_SH_MIN_BLOCKS
#define RDC_ADJ_SH_MIN_BLOCKS 3
#endif

// kShRec: the vertex records in the block's shared memory, after the
// gradient table: thread t's at word t * shared_vert_stride (an odd number
// of words, so a warp reading one field of one vertex hits 32 banks), which
// keeps them out of the L1 and L2 the replay's loads use; otherwise a
// per-thread local array.
template <bool kBvh, bool kShRec>
__global__ void __launch_bounds__(kRenderBlock, kShRec ? RDC_ADJ_SH_MIN_BLOCKS : RDC_ADJ_MIN_BLOCKS)
    adjoint_kernel(const AdjParams P) {
    extern __shared__ float4 smem[];
    const unsigned FULL = 0xffffffffu;
    float4* s_rec = smem;
    int4* s_runs = reinterpret_cast<int4*>(smem + (kBvh ? 0u : P.sc.nrec));
    float* s_grad = reinterpret_cast<float*>(s_runs + (kBvh ? 0u : P.sc.nruns));
    float* s_vert = s_grad + (P.smem_grad ? 8u * P.sc.nobj : 0u);
    __shared__ __align__(8) uint64_t s_bar;
    if (P.smem_grad)
        for (uint32_t i = threadIdx.x; i < 8u * P.sc.nobj; i += blockDim.x) s_grad[i] = 0.0f;
    if (!kBvh && threadIdx.x == 0) bulk_init(&s_bar);
    __syncthreads();
    if (!kBvh &&
        !stage_scene(&s_bar, 0u, s_rec, P.sc.rec, P.sc.nrec, s_runs, P.sc.runs, P.sc.nruns, P.errors))
        return;
    float* gbase = P.smem_grad ? s_grad : P.grad;
    const bool scene_fast = P.sc.fast_div != 0u;
    BruteIsectRolled brute{s_rec, s_runs, (int)P.sc.nruns, scene_fast};
    BvhCounters cnt;
    uint32_t segs = 0;

    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t rounds = (P.npaths + stride - 1) / stride;  // the same for every thread
    for (uint64_t it = 0; it < rounds; ++it) {
        const uint64_t path = it * stride + (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
        AdjVert v_local[kShRec ? 1 : kAdjMaxBounces];
        AdjVert* const v =
            kShRec ? reinterpret_cast<AdjVert*>(s_vert + threadIdx.x * P.shared_vert_stride) : v_local;
        int nv = 0;
        V3 gw = mk(0.f, 0.f, 0.f);
        V3 d = mk(0.f, 0.f, 0.f), atten = mk(1.f, 1.f, 1.f);
        bool active = false, missed = false;
        bool emit_after_first = false;  // an emissive hit after vertex 0
        if (path < P.npaths) {
            const uint32_t pix = (uint32_t)(path / P.nspp);
            const uint32_t sample = P.s0 + (uint32_t)(path % P.nspp);
            const float inv_n = 1.0f / (float)P.nspp;
            const size_t px3 = 3 * (size_t)checked_index(P.sc.oob, pix, (long long)P.sc.width * P.sc.height);
            gw = mk(P.dl[px3] * inv_n, P.dl[px3 + 1] * inv_n, P.dl[px3 + 2] * inv_n);
            if (gw.x != 0.0f || gw.y != 0.0f || gw.z != 0.0f) {
                // replay (the forward kernels' arithmetic, bit for bit)
                active = true;
                V3 o;
                primary_ray(P.sc, pix % P.sc.width, pix / P.sc.width, o, d);
                for (uint32_t b = 0; b < P.max_bounces; ++b) {
                    ++segs;
                    const RayPre r = ray_pre(o, d, P.sc.neg_zero);
                    float t;
                    int idx;
                    if (kBvh)
                        bvh_intersect(P.bvh, r, scene_fast && r.fast, t, idx, cnt);
                    else
                        brute(r, t, idx);
                    if (idx < 0) {
                        missed = true;
                        break;
                    }
                    idx = (int)checked_index(P.sc.oob, idx, P.sc.nobj);
                    const MatDev m = load_mat(P.sc.mat, idx);
                    const HitRec h = closest_hit(o, d, t, __ldg(&P.sc.hit[idx]), __float_as_int(m.d.y));
                    const uint32_t c2 = b * 4u;
                    ScatterRec rec;
                    V3 no, nd;
                    scatter_lobe_first<true>(d, h, m, philox(pix, sample, c2, P.stream_id, P.key0, P.key1),
                                             philox(pix, sample, c2 + 1u, P.stream_id, P.key0, P.key1),
                                             philox(pix, sample, c2 + 2u, P.stream_id, P.key0, P.key1), no, nd,
                                             &rec);
                    AdjVert& vk = v[nv++];
                    vk.o = o;
                    vk.d = d;
                    vk.t = t;
                    vk.objf = (uint32_t)idx | (rec.flags << 24);
                    vk.s = rec.s;
                    atten = mk(atten.x * m.a.x, atten.y * m.a.y, atten.z * m.a.z);
                    emit_after_first = emit_after_first || (b > 0u && (m.b.x != 0.0f || m.b.y != 0.0f || m.b.z != 0.0f));
                    o = no;
                    d = nd;
                }
            }
        }
        // The block's warps go from replay to sweep to accumulation together:
        // the three phases' code does not fit the instruction cache at once,
        // and warps spread over all three stalled on instruction fetch
        // (config 4 backward 10.2 -> 8.3 ms with the barriers).
        __syncthreads();
        if (active) {
            // A path that ends without a miss gathers only emission: with no
            // emissive hit after its first vertex every coin weight is zero
            // and nothing depends on a direction, so its sweep adds nothing.
            const bool sweep = missed || emit_after_first;
            // reverse sweep: S = the radiance gathered after the current
            // vertex's scatter, suf = the albedos after it
            V3 go = mk(0.f, 0.f, 0.f), gd = mk(0.f, 0.f, 0.f);
            V3 sky = mk(0.f, 0.f, 0.f), S = mk(0.f, 0.f, 0.f);
            if (missed) {
                sky = world_sample(P.sc, d);
                S = mk(sky.x * atten.x, sky.y * atten.y, sky.z * atten.z);
                if (P.sc.world_kind == 0u) {
                    // sky = bottom + (top - bottom) (d.y / |d| + 1) / 2
                    const float coef = 0.5f * (gw.x * atten.x * (P.sc.top[0] - P.sc.bottom[0]) +
                                               gw.y * atten.y * (P.sc.top[1] - P.sc.bottom[1]) +
                                               gw.z * atten.z * (P.sc.top[2] - P.sc.bottom[2]));
                    const float len = sqrtf(vdot(d, d));
                    const float cosv = d.y / len;
                    gd = vmul(vsub(mk(0.f, 1.f, 0.f), vmul(d, cosv / len)), coef / len);
                }
            }
            V3 suf = mk(1.f, 1.f, 1.f);
            if (!sweep) {
                for (int k = 0; k < nv; ++k) {
                    v[k].o = mk(0.f, 0.f, 0.f);
                    v[k].t = 0.0f;
                }
            }
            for (int k = sweep ? nv - 1 : -1; k >= 0; --k) {
                AdjVert& vk = v[k];
                const int obj = (int)(vk.objf & 0xFFFFFFu);
                const MatDev m = load_mat(P.sc.mat, (int)checked_index(P.sc.oob, obj, P.sc.nobj));
                const V3 s = vk.s;
                const float wk = gw.x * S.x + gw.y * S.y + gw.z * S.z;
                const float gr = vertex_vjp(P.sc, vk, m, s, wk, go, gd);
                vk.o = mk(gw.x * sky.x * suf.x, gw.y * sky.y * suf.y, gw.z * sky.z * suf.z);
                vk.t = gr;
                suf = mk(suf.x * m.a.x, suf.y * m.a.y, suf.z * m.a.z);
                S = mk(S.x + m.b.x, S.y + m.b.y, S.z + m.b.z);
            }
        }
        __syncthreads();
        // warp-converged accumulation over vertex slots; pre = the albedos
        // before vertex k, which completes its albedo gradient
        const int maxnv = (int)__reduce_max_sync(FULL, (unsigned)nv);
        V3 pre = mk(1.f, 1.f, 1.f);
        for (int k = 0; k < maxnv; ++k) {
            const bool has = k < nv;
            const int obj = has ? (int)(v[k].objf & 0xFFFFFFu) : -1;
            float c[7];
            c[0] = has ? v[k].o.x * pre.x : 0.0f;
            c[1] = has ? v[k].o.y * pre.y : 0.0f;
            c[2] = has ? v[k].o.z * pre.z : 0.0f;
            c[3] = has ? gw.x : 0.0f;
            c[4] = has ? gw.y : 0.0f;
            c[5] = has ? gw.z : 0.0f;
            c[6] = has ? v[k].t : 0.0f;
            if (has) {
                const float4 alb = __ldg(&P.sc.mat[checked_index(P.sc.oob, obj, P.sc.nobj)].a);
                pre = mk(pre.x * alb.x, pre.y * alb.y, pre.z * alb.z);
            }
            warp_add_grad(gbase, obj, c, P.sc.oob, P.sc.nobj);
        }
    }
    // flush the block's shared accumulators; counters
    if (P.smem_grad) {
        __syncthreads();
        for (uint32_t i = threadIdx.x; i < 8u * P.sc.nobj; i += blockDim.x)
            if (s_grad[i] != 0.0f) atomicAdd(P.grad + i, s_grad[i]);
    }
    unsigned long long s = segs;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(FULL, s, off);
    if ((threadIdx.x & 31) == 0 && s != 0ull) atomicAdd(P.segments, s);
}

}  // namespace

uint32_t adjoint_shared_vert_stride(uint32_t bounces) {
    const uint32_t w = bounces * (uint32_t)(sizeof(AdjVert) / 4);
    return w | 1u;
}

size_t adjoint_smem_bytes(const SceneView& sc, bool bvh, bool smem_grad, uint32_t shared_vert_bounces, int block) {
    size_t b = bvh ? 0 : 16u * ((size_t)sc.nrec + sc.nruns);
    if (smem_grad) b += 32u * (size_t)sc.nobj;
    if (shared_vert_bounces) b += 4u * (size_t)adjoint_shared_vert_stride(shared_vert_bounces) * (size_t)block;
    return b;
}

static const void* adjoint_fn(bool bvh, bool sh) {
    if (bvh) return sh ? (const void*)adjoint_kernel<true, true> : (const void*)adjoint_kernel<true, false>;
    return sh ? (const void*)adjoint_kernel<false, true> : (const void*)adjoint_kernel<false, false>;
}

cudaError_t adjoint_occupancy(bool bvh, bool shared_vert, int block, size_t smem, int* blocks_per_sm) {
    const void* fn = adjoint_fn(bvh, shared_vert);
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)(smem < 48 * 1024 ? 48 * 1024 : smem));
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, fn, block, smem);
}

cudaError_t launch_adjoint(const AdjParams& p, bool bvh, bool shared_vert, int grid, int block, size_t smem,
                           cudaStream_t s) {
    if (bvh) {
        if (shared_vert)
            adjoint_kernel<true, true><<<grid, block, smem, s>>>(p);
        else
            adjoint_kernel<true, false><<<grid, block, smem, s>>>(p);
    } else {
        if (shared_vert)
            adjoint_kernel<false, true><<<grid, block, smem, s>>>(p);
        else
            adjoint_kernel<false, false><<<grid, block, smem, s>>>(p);
    }
    return cudaGetLastError();
}

}  // namespace rdc
