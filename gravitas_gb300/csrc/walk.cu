// walk.cu — the FP32 tree walks (compiled with FMA contraction and fast FP32 division/sqrt).
//
// walk_plain: one thread per sorted star, the CUDA twin of the Metal kernel
//   internal/sim/bh/gpu_darwin.go:76-118 (all FP32, uncompensated, per-star opening).
// walk_mixed: one warp per group of 64 consecutive Morton-sorted stars (two per lane, packed
//   FP32x2 arithmetic) walking the skip-pointer tree in lockstep. A node is opened when any star of the group would open it under the
//   reference criterion d2 < crit2 (bh.go:116), so every star sees each accepted node exactly
//   where the reference would accept it or deeper. Positions are FP64 split into hi + lo FP32
//   parts; a separation is formed from hi differences, exact for nearby points (Sterbenz) and
//   relatively small for distant ones, plus the lo parts, so separations stay accurate however
//   far a system lies from the origin: (com_hi - O) + com_lo - ((hi - O) + lo), with O the hi part
//   of the lane's first star (of the star itself for a distant star of a target list). Each star
//   accumulates in FP32 blocks (the interactions of 32 node visits) folded into a Kahan sum.
#include <cuda_runtime.h>

#include "gbh_internal.cuh"

namespace gbh {

namespace {

constexpr unsigned kFull = 0xffffffffu;

constexpr int kPlainThreads = 256;
// Mixed-walk block size (a compile-time tuning knob; 64 and 128 measured equal).
#ifndef GBH_MIXED_THREADS
#define GBH_MIXED_THREADS 128
#endif
constexpr int kMixedThreads = GBH_MIXED_THREADS;

inline unsigned blocks_for(int64_t n, int threads) {
    int64_t b = (n + threads - 1) / threads;
    return unsigned(b < 1 ? 1 : b);
}

__device__ __forceinline__ void set_err(DevInfo *info, int where) {
    atomicExch(&info->err, 1);
    info->err_where = where;
}

// gpu_darwin.go:84-117, with the same float4 node and star records.
__global__ __launch_bounds__(kPlainThreads) void k_walk_plain(const DevInfo *info, const PNode *__restrict__ nodes,
                                                              const float4 *__restrict__ stars,
                                                              const int32_t *__restrict__ order, float eps2,
                                                              double *ax, double *ay, double *az,
                                                              const int32_t *__restrict__ targets,
                                                              const int32_t *__restrict__ sid_sorted,
                                                              const SysGeo *__restrict__ geo, DevInfo *err_info) {
    int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    int64_t ns = info->nstars;
    if (t >= (targets ? int64_t(info->ntargets) : ns)) return;
    int64_t k = targets ? int64_t(targets[t]) : t;
    int64_t nn = info->nnodes;
    float4 p = stars[k];
    float fax = 0.f, fay = 0.f, faz = 0.f;
    int64_t steps = 0;
    int i = nn > 0 ? (sid_sorted ? geo[sid_sorted[k]].root : 0) : -1;  // the star's own system
    while (i >= 0) {
        if (++steps > nn || i >= nn) {
            set_err(err_info, 3);
            break;
        }
        const PNode nd = nodes[i];
        float dx = nd.com.x - p.x, dy = nd.com.y - p.y, dz = nd.com.z - p.z;
        float d2 = dx * dx + dy * dy + dz * dz;
        if (d2 >= nd.q2.z) {
            float inv = 1.0f / (d2 + eps2);
            float inv3 = inv * sqrtf(inv);
            float qx = nd.q1.x * dx + nd.q1.w * dy + nd.q2.x * dz;
            float qy = nd.q1.w * dx + nd.q1.y * dy + nd.q2.y * dz;
            float qz = nd.q2.x * dx + nd.q2.y * dy + nd.q1.z * dz;
            float inv5 = inv3 * inv;
            float f = nd.com.w * inv3 + 2.5f * (dx * qx + dy * qy + dz * qz) * inv5 * inv;
            fax += dx * f - qx * inv5;
            fay += dy * f - qy * inv5;
            faz += dz * f - qz * inv5;
            i = nd.links.y;
            continue;
        }
        if (nd.links.x >= 0) {
            i = nd.links.x;
            continue;
        }
        if (nd.links.z < 0 || nd.links.w > ns || nd.links.z > nd.links.w) {
            set_err(err_info, 6);
            break;
        }
        for (int j = nd.links.z; j < nd.links.w; ++j) {
            if (j == int(k)) continue;
            float4 s = stars[j];
            float ddx = s.x - p.x, ddy = s.y - p.y, ddz = s.z - p.z;
            float ir = rsqrtf(ddx * ddx + ddy * ddy + ddz * ddz + eps2);
            float f = s.w * ir * ir * ir;
            fax += ddx * f;
            fay += ddy * f;
            faz += ddz * f;
        }
        i = nd.links.y;
    }
    int32_t o = order[k];
    ax[o] = fax;
    ay[o] = fay;
    az[o] = faz;
}

// Kahan fold of a block partial into the running sum (s, c): true sum = s - c.
__device__ __forceinline__ void kahan_fold(float &s, float &c, float &part) {
    float y = part - c;
    float t = s + y;
    c = (t - s) - y;
    s = t;
    part = 0.f;
}

// The mixed walk: one warp per group of 64 consecutive sorted stars (or 64 consecutive entries
// of a target list), each lane owning two neighbouring stars; every separation, test and
// interaction is computed for both stars at once with packed FP32x2 arithmetic
// (__fadd2_rn / __fmul2_rn / __ffma2_rn), so the node load, vote and branch of a visit are shared
// by 64 stars and the math issues half the instructions of one star per lane (measured 1.3x).
__device__ __forceinline__ float2 f2(float v) { return make_float2(v, v); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

__device__ __forceinline__ void kahan_fold2(float2 &s, float2 &c, float2 &part) {
    kahan_fold(s.x, c.x, part.x);
    kahan_fold(s.y, c.y, part.y);
}

// kPot: the same walk accumulating psi = sum m / r + (d.Q.d) / (2 r^5) (walkPotential,
// potential.go:44-81) per star instead of the acceleration; psi goes to ax[sorted index].
// kShared: no target list, so a lane's two stars share one origin (see the separations below).
// Without a target list 9 blocks of 128 per SM (56 registers, a few spills) measured 1.8 % faster
// than 8 (64 registers, no room for a ninth block); 10 (48 registers) was slower. The target-list
// form needs more registers and keeps 8.
// kSplit: each group's walk is shared by nparts warps, part p owning the source stars
// [p ns / nparts, (p + 1) ns / nparts): a node is owned by the part that holds its first star
// (nodes are visited in pre-order, so first stars never decrease along the walk); every part
// tests the nodes whose ranges reach into its own, with the group's vote, so all parts agree on
// every node and each accepted node and opened leaf is added by exactly its owner.
template <bool kQuad, bool kSoft, bool kPot, bool kShared, bool kSplit = false>
__global__ __launch_bounds__(kMixedThreads, kShared ? 9 : 8) void k_walk_mixed2(const DevInfo *info, const MNode *__restrict__ nodes,
                                                               const int2 *__restrict__ ranges,
                                                               const float4 *__restrict__ st_hi,
                                                               const float4 *__restrict__ st_lo,
                                                               const float4 *__restrict__ st_off,
                                                               const int32_t *__restrict__ order, float eps2,
                                                               double *ax, double *ay, double *az,
                                                               const int32_t *__restrict__ targets,
                                                               const int4 *__restrict__ groups, int pair,
                                                               const int32_t *__restrict__ gperm, int32_t perm_cap,
                                                               uint32_t *gcost, DevInfo *err_info, int nparts,
                                                               double *part_acc, int64_t part_stride) {
    // pair: 64-star groups, lane l walks stars 2l and 2l + 1; else 32-star groups, one star per
    // lane (the second FP32x2 slot then repeats the first and is not written)
    const int lane = threadIdx.x & 31;
    const int32_t ns = int32_t(info->nstars);  // the C-ABI caps n at 2^30
    const uint32_t nn = uint32_t(info->nnodes);
    const int32_t wid = int32_t((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int32_t g = kSplit ? wid / nparts : wid;
    const int part = kSplit ? wid - g * nparts : 0;
    const int32_t s_lo = kSplit ? int32_t(int64_t(ns) * part / nparts) : 0;
    const int32_t s_hi = kSplit ? int32_t(int64_t(ns) * (part + 1) / nparts) : ns;
    // longest first: walk the group the last walk's costs put at this position (gperm holds a
    // permutation of the groups, valid while its recorded group count matches)
    int32_t base, nt, root = 0, gw = g;
    if (groups) {  // a forest: group g = up to 64 (32) stars of one system, walked from its root
        if (uint32_t(g) >= info->ngroups) return;
        if (gperm && gperm[perm_cap] == int32_t(info->ngroups)) gw = gperm[g];
        const int4 e = groups[gw];
        base = e.x;
        nt = e.x + e.y;
        root = e.z;
    } else {
        const int gsize = pair ? 64 : 32;
        nt = targets ? int32_t(info->ntargets) : ns;
        if (g * gsize >= nt) return;  // uniform over the warp
        if (gperm && gperm[perm_cap] == (nt + gsize - 1) / gsize) gw = gperm[g];
        base = gw * gsize;
    }
    const int32_t t0 = base + (pair ? 2 * lane : lane), t1 = t0 + 1;
    const bool v0 = t0 < nt, v1 = pair && t1 < nt;
    const int32_t first_k = targets ? targets[base] : base;
    const int32_t k0 = v0 ? (targets ? targets[t0] : t0) : first_k;
    const int32_t k1 = v1 ? (targets ? targets[t1] : t1) : first_k;
    const float4 h0 = st_hi[k0], l0 = st_lo[k0];
    const float4 h1 = st_hi[k1], l1 = st_lo[k1];
    // Separations (node com - star) = ((com_hi - O) + com_lo) - ((hi - O) + lo), O the star's
    // origin, formed as sums of negated terms. Consecutive sorted stars are Morton neighbours, so a
    // lane's two stars share one origin, the first star's hi part; the first bracket is then the
    // same for both and is formed in scalar FP32 (kShared). A target list can pair distant stars:
    // there the second star is its own origin unless its sorted index follows the first's, and
    // the first bracket is packed (the same values whenever the origins agree, so a full target
    // list walks exactly as no list).
    const bool near1 = kShared || k1 == k0 + 1;
    const float2 nox = make_float2(-h0.x, near1 ? -h0.x : -h1.x);
    const float2 noy = make_float2(-h0.y, near1 ? -h0.y : -h1.y);
    const float2 noz = make_float2(-h0.z, near1 ? -h0.z : -h1.z);
    const float2 nrx = make_float2(-l0.x, -((h1.x + nox.y) + l1.x));
    const float2 nry = make_float2(-l0.y, -((h1.y + noy.y) + l1.y));
    const float2 nrz = make_float2(-l0.z, -((h1.z + noz.y) + l1.z));
    const float2 e2 = f2(eps2);

    float2 sx = f2(0.f), sy = f2(0.f), sz = f2(0.f), cx = f2(0.f), cy = f2(0.f), cz = f2(0.f);
    float2 px = f2(0.f), py = f2(0.f), pz = f2(0.f);
    uint32_t visits = 0, pairs = 0;
    int i = nn > 0 ? root : -1;
    while (i >= 0) {
        if (uint32_t(i) >= nn) {
            if (lane == 0) set_err(err_info, 4);
            break;
        }
        const MNode nd = nodes[i];
        bool own = true;  // this warp adds the node's interactions (always, unless split)
        if constexpr (kSplit) {
            const int2 rg = ranges[i];
            if (rg.x >= s_hi) break;  // this node and every later one start after the part
            if (rg.y <= s_lo) {       // the whole subtree lies before the part
                i = __float_as_int(nd.d.w);
                if (++visits > nn + 32u) {
                    if (lane == 0) set_err(err_info, 4);
                    break;
                }
                continue;
            }
            own = rg.x >= s_lo;
        }
        float2 dx, dy, dz;
        if constexpr (kShared) {  // 6 scalar adds + 3 packed: measured 2-3 % faster than 9 packed
            dx = add2(f2((nd.a.x + nox.x) + nd.b.x), nrx);
            dy = add2(f2((nd.a.y + noy.x) + nd.b.y), nry);
            dz = add2(f2((nd.a.z + noz.x) + nd.b.z), nrz);
        } else {
            dx = add2(add2(add2(f2(nd.a.x), nox), f2(nd.b.x)), nrx);
            dy = add2(add2(add2(f2(nd.a.y), noy), f2(nd.b.y)), nry);
            dz = add2(add2(add2(f2(nd.a.z), noz), f2(nd.b.z)), nrz);
        }
        const float2 d2 = fma2(dz, dz, fma2(dy, dy, mul2(dx, dx)));
        const bool open = __any_sync(kFull, (d2.x < nd.a.w) | (d2.y < nd.a.w));
        const int first = __float_as_int(nd.d.z), next = __float_as_int(nd.d.w);
        if (!open) {
            if (own) {
                const float2 r2 = add2(d2, e2);
                const float2 ir = make_float2(rsqrtf(r2.x), rsqrtf(r2.y));
                const float2 ir2 = mul2(ir, ir);
                const float2 ir3 = mul2(ir, ir2);
                if constexpr (kPot) {
                    float2 t = mul2(f2(nd.b.w), ir);
                    if (kQuad) {
                        const float2 qx = fma2(f2(nd.d.x), dz, fma2(f2(nd.c.w), dy, mul2(f2(nd.c.x), dx)));
                        const float2 qy = fma2(f2(nd.d.y), dz, fma2(f2(nd.c.y), dy, mul2(f2(nd.c.w), dx)));
                        const float2 qz = fma2(f2(nd.c.z), dz, fma2(f2(nd.d.y), dy, mul2(f2(nd.d.x), dx)));
                        const float2 dqd = fma2(dz, qz, fma2(dy, qy, mul2(dx, qx)));
                        t = fma2(mul2(f2(0.5f), dqd), mul2(ir3, ir2), t);
                    }
                    px = add2(px, t);
                } else if (kQuad) {
                    const float2 qx = fma2(f2(nd.d.x), dz, fma2(f2(nd.c.w), dy, mul2(f2(nd.c.x), dx)));
                    const float2 qy = fma2(f2(nd.d.y), dz, fma2(f2(nd.c.y), dy, mul2(f2(nd.c.w), dx)));
                    const float2 qz = fma2(f2(nd.c.z), dz, fma2(f2(nd.d.y), dy, mul2(f2(nd.d.x), dx)));
                    const float2 ir5 = mul2(ir3, ir2);
                    const float2 dqd = fma2(dz, qz, fma2(dy, qy, mul2(dx, qx)));
                    const float2 u = mul2(mul2(f2(2.5f), ir2), dqd);
                    const float2 f = fma2(ir5, u, mul2(f2(nd.b.w), ir3));
                    const float2 nir5 = mul2(f2(-1.f), ir5);
                    px = fma2(nir5, qx, fma2(f, dx, px));
                    py = fma2(nir5, qy, fma2(f, dy, py));
                    pz = fma2(nir5, qz, fma2(f, dz, pz));
                } else {
                    const float2 f = mul2(f2(nd.b.w), ir3);
                    px = fma2(f, dx, px);
                    py = fma2(f, dy, py);
                    pz = fma2(f, dz, pz);
                }
            }
            i = next;
        } else if (first >= 0) {
            i = first;
        } else {
            const int2 r = ranges[i];
            if (r.x < 0 || r.y > ns || r.x > r.y) {
                if (lane == 0) set_err(err_info, 5);
                break;
            }
            if (own) {
                pairs += uint32_t(r.y - r.x);
                // Leaf stars: separation = (leaf com - star) + (leaf star - com), the first the visit's
                // separation, the second the star's FP32 offset stored by the upsweep. In a star's own
                // leaf the first term is replaced by the negative of the star's own stored offset, so
                // that its self pair is exactly zero and its close pairs are differences of two offsets.
                float2 lx = dx, ly = dy, lz = dz;
                if (k0 >= r.x && k0 < r.y) {
                    const float4 o = st_off[k0];
                    lx.x = -o.x;
                    ly.x = -o.y;
                    lz.x = -o.z;
                }
                if (k1 >= r.x && k1 < r.y) {
                    const float4 o = st_off[k1];
                    lx.y = -o.x;
                    ly.y = -o.y;
                    lz.y = -o.z;
                }
    #pragma unroll 4  // measured 2-3 % faster than no unrolling (independent source stars)
                for (int j = r.x; j < r.y; ++j) {
                    const float4 so = st_off[j];
                    const float2 ex = add2(lx, f2(so.x));
                    const float2 ey = add2(ly, f2(so.y));
                    const float2 ez = add2(lz, f2(so.z));
                    const float2 r2 = fma2(ez, ez, fma2(ey, ey, fma2(ex, ex, e2)));
                    // A star paired with itself gives a separation of exactly 0: with eps2 > 0 that adds
                    // 0, as skipping j == self does (bh.go:142-144). Without softening r2 = 0 is masked.
                    float2 ir;
                    if (kSoft) {
                        ir = make_float2(rsqrtf(r2.x), rsqrtf(r2.y));
                    } else {
                        ir = make_float2(r2.x > 0.f ? rsqrtf(r2.x) : 0.f, r2.y > 0.f ? rsqrtf(r2.y) : 0.f);
                    }
                    if constexpr (kPot) {
                        // the self pair has zero separation but m / eps is not zero: skip j == self
                        float2 t = mul2(f2(so.w), ir);
                        t.x = j == k0 ? 0.f : t.x;
                        t.y = j == k1 ? 0.f : t.y;
                        px = add2(px, t);
                    } else {
                        const float2 f = mul2(mul2(f2(so.w), ir), mul2(ir, ir));
                        px = fma2(f, ex, px);
                        py = fma2(f, ey, py);
                        pz = fma2(f, ez, pz);
                    }
                }
            }
            i = next;
        }
        if ((++visits & 31u) == 0) {  // fold the block partials every 32 visits
            kahan_fold2(sx, cx, px);
            kahan_fold2(sy, cy, py);
            kahan_fold2(sz, cz, pz);
            if (visits > nn + 32u) {  // each node is visited at most once
                if (lane == 0) set_err(err_info, 4);
                break;
            }
        }
    }
    kahan_fold2(sx, cx, px);
    kahan_fold2(sy, cy, py);
    kahan_fold2(sz, cz, pz);
    if constexpr (kSplit) {  // the part's sums, by sorted index; k_split_combine adds the parts
        double *q = part_acc + int64_t(part) * 3 * part_stride;
        if (v0) {
            q[k0] = double(sx.x) - double(cx.x);
            q[part_stride + k0] = double(sy.x) - double(cy.x);
            q[2 * part_stride + k0] = double(sz.x) - double(cz.x);
        }
        if (v1) {
            q[k1] = double(sx.y) - double(cx.y);
            q[part_stride + k1] = double(sy.y) - double(cy.y);
            q[2 * part_stride + k1] = double(sz.y) - double(cz.y);
        }
        return;
    }
    if (gcost && lane == 0) gcost[gw] = 2u * visits + pairs;  // the group's cost
    if constexpr (kPot) {
        if (v0) ax[k0] = double(sx.x) - double(cx.x);
        if (v1) ax[k1] = double(sx.y) - double(cx.y);
        return;
    }
    if (v0) {
        int32_t o = order[k0];
        ax[o] = double(sx.x) - double(cx.x);
        ay[o] = double(sy.x) - double(cy.x);
        az[o] = double(sz.x) - double(cz.x);
    }
    if (v1) {
        int32_t o = order[k1];
        ax[o] = double(sx.y) - double(cx.y);
        ay[o] = double(sy.y) - double(cy.y);
        az[o] = double(sz.y) - double(cz.y);
    }
}

// Register-resident FMA chains: 8 independent chains per thread.
__global__ __launch_bounds__(256) void k_fma_probe(int iters, float *out) {
    float a0 = threadIdx.x * 1e-7f, a1 = a0 + 1e-7f, a2 = a0 + 2e-7f, a3 = a0 + 3e-7f;
    float a4 = a0 + 4e-7f, a5 = a0 + 5e-7f, a6 = a0 + 6e-7f, a7 = a0 + 7e-7f;
    const float m = 0.999999f, c = 1e-7f;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int u = 0; u < 16; ++u) {
            a0 = fmaf(a0, m, c);
            a1 = fmaf(a1, m, c);
            a2 = fmaf(a2, m, c);
            a3 = fmaf(a3, m, c);
            a4 = fmaf(a4, m, c);
            a5 = fmaf(a5, m, c);
            a6 = fmaf(a6, m, c);
            a7 = fmaf(a7, m, c);
        }
    }
    float s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
    if (s == 12345.678f) out[blockIdx.x] = s;  // never true; keeps the chains live
}

}  // namespace

cudaError_t walk_plain(const Launch &L, const TreeBufs &b, int64_t nstars_cap, float eps2, double *ax, double *ay,
                       double *az, bool targets) {
    k_walk_plain<<<blocks_for(nstars_cap, kPlainThreads), kPlainThreads, 0, L.stream>>>(
        b.info, b.pnodes, b.st_hi, b.order, eps2, ax, ay, az, targets ? b.targets : nullptr,
        b.nsys > 1 ? b.sid_sorted : nullptr, b.geo, b.info);
    ++*L.count;
    return cudaGetLastError();
}

// Longest-first order for the next walk from this walk's group costs: groups bucketed by
// floor(log2 cost), most expensive bucket first, ascending group index inside a bucket (so that
// neighbouring warps keep walking neighbouring groups). One block of kLptThreads threads, each
// owning a contiguous run of groups.
constexpr int kLptThreads = 512, kLptBuckets = 16;  // 32 KB of shared counts
static_assert(kLptThreads / 32 == kLptBuckets, "the warp totals reuse the bucket array");
__global__ __launch_bounds__(kLptThreads) void k_lpt_order(const DevInfo *info, int gsize, bool forest,
                                                           const uint32_t *gcost, int32_t *gperm, int32_t perm_cap) {
    __shared__ uint32_t cnt[kLptBuckets][kLptThreads];
    __shared__ uint32_t base[kLptBuckets];
    const int t = threadIdx.x;
    const int32_t ng = forest ? int32_t(info->ngroups) : int32_t((info->nstars + gsize - 1) / gsize);
    if (ng > perm_cap) return;  // no order: the walk keeps launch order
    const int32_t per = (ng + kLptThreads - 1) / kLptThreads;
    const int32_t g0 = t * per, g1 = g0 + per < ng ? g0 + per : ng;
    auto bucket = [&](uint32_t c) {
        int l = 31 - __clz(c | 1u);
        return kLptBuckets - 1 - (l < kLptBuckets ? l : kLptBuckets - 1);
    };
    for (int k = 0; k < kLptBuckets; ++k) cnt[k][t] = 0;
    for (int32_t g = g0; g < g1; ++g) ++cnt[bucket(gcost[g])][t];
    __syncthreads();
    // Exclusive scan of the counts in bucket-major order, kItems consecutive entries per thread:
    // entry (k, q) becomes the position of thread q's first group of bucket k in the order.
    constexpr int kItems = kLptBuckets * kLptThreads / kLptThreads;
    uint32_t *flat = &cnt[0][0];
    uint32_t v[kItems], sum = 0;
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
        v[i] = flat[t * kItems + i];
        sum += v[i];
    }
    const int lane = t & 31, warp = t >> 5;
    uint32_t incl = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(kFull, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) base[warp] = incl;  // warp totals (kLptThreads / 32 == kLptBuckets of them)
    __syncthreads();
    if (warp == 0) {
        const uint32_t w = lane < kLptThreads / 32 ? base[lane] : 0;
        uint32_t wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(kFull, wi, o);
            if (lane >= o) wi += y;
        }
        if (lane < kLptThreads / 32) base[lane] = wi - w;
    }
    __syncthreads();
    uint32_t run = base[warp] + incl - sum;
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
        flat[t * kItems + i] = run;
        run += v[i];
    }
    __syncthreads();
    for (int32_t g = g0; g < g1; ++g) {
        int k = bucket(gcost[g]);
        gperm[cnt[k][t]++] = g;
    }
    __syncthreads();
    if (t == 0) gperm[perm_cap] = ng;
}

// Sum of a split walk's parts for every walked star, in part order, to state order.
__global__ __launch_bounds__(256) void k_split_combine(const DevInfo *info, const int32_t *__restrict__ order,
                                                       const int32_t *__restrict__ targets, int nparts,
                                                       const double *__restrict__ part_acc, int64_t stride,
                                                       double *ax, double *ay, double *az) {
    const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    const int64_t nt = targets ? int64_t(info->ntargets) : info->nstars;
    if (t >= nt) return;
    const int32_t k = targets ? targets[t] : int32_t(t);
    double x = 0, y = 0, z = 0;
    for (int p = 0; p < nparts; ++p) {
        const double *q = part_acc + int64_t(p) * 3 * stride;
        x += q[k];
        y += q[stride + k];
        z += q[2 * stride + k];
    }
    const int32_t o = order[k];
    ax[o] = x;
    ay[o] = y;
    az[o] = z;
}

template <bool kQuad, bool kSoft, bool kPot, bool kShared>
static cudaError_t launch_mixed_t(const Launch &L, const TreeBufs &b, int64_t nstars_cap, float eps2, double *ax,
                                double *ay, double *az, bool targets) {
    const bool forest = b.nsys > 1;
    const int gsize = b.group == 32 ? 32 : 64;
    int64_t groups = forest ? b.cap_groups : (nstars_cap + gsize - 1) / gsize;
    if constexpr (!kPot) {  // few groups: split each group's walk over several warps
        // a target list walks about walk_hint stars (the previous event's count): part by that
        const int64_t walked = targets && b.walk_hint > 0 && b.walk_hint < nstars_cap ? b.walk_hint : nstars_cap;
        int parts = (!forest && b.split) ? walk_parts(walked, gsize) : 1;
        const int budget = walk_parts_budget(nstars_cap);  // a function of n alone, never of capacity
        if (parts > budget) parts = budget;
        if (parts > 1 && b.part_acc && int64_t(parts) * 3 * nstars_cap <= b.part_cap) {
            const int64_t warps = groups * parts;
            const int64_t wblocks = (warps + kMixedThreads / 32 - 1) / (kMixedThreads / 32);
            k_walk_mixed2<kQuad, kSoft, false, kShared, true>
                <<<unsigned(wblocks < 1 ? 1 : wblocks), kMixedThreads, 0, L.stream>>>(
                    b.info, b.mnodes, b.mrange, b.st_hi, b.st_lo, b.st_off, b.order, eps2, ax, ay, az,
                    targets ? b.targets : nullptr, nullptr, gsize == 64 ? 1 : 0, nullptr, int32_t(b.cap_groups),
                    nullptr, b.info, parts, b.part_acc, nstars_cap);
            ++*L.count;
            cudaError_t e = cudaGetLastError();
            if (e != cudaSuccess) return e;
            k_split_combine<<<blocks_for(nstars_cap, 256), 256, 0, L.stream>>>(
                b.info, b.order, targets ? b.targets : nullptr, parts, b.part_acc, nstars_cap, ax, ay, az);
            ++*L.count;
            return cudaGetLastError();
        }
    }
    const bool lpt = b.lpt && !targets && !kPot;
    int64_t blocks = (groups + kMixedThreads / 32 - 1) / (kMixedThreads / 32);
    k_walk_mixed2<kQuad, kSoft, kPot, kShared><<<unsigned(blocks < 1 ? 1 : blocks), kMixedThreads, 0, L.stream>>>(
        b.info, b.mnodes, b.mrange, b.st_hi, b.st_lo, b.st_off, b.order, eps2, ax, ay, az,
        targets ? b.targets : nullptr,
        forest ? b.groups : nullptr, gsize == 64 ? 1 : 0, lpt ? b.gperm : nullptr, int32_t(b.cap_groups),
        lpt ? b.gcost : nullptr, b.info, 1, nullptr, 0);
    ++*L.count;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || !lpt) return e;
    k_lpt_order<<<1, kLptThreads, 0, L.stream>>>(b.info, gsize, forest, b.gcost, b.gperm, int32_t(b.cap_groups));
    ++*L.count;
    return cudaGetLastError();
}

template <bool kQuad, bool kSoft, bool kPot = false>
static cudaError_t launch_mixed(const Launch &L, const TreeBufs &b, int64_t nstars_cap, float eps2, double *ax,
                                double *ay, double *az, bool targets) {
    if constexpr (!kPot) {  // potential walks take no target list
        if (targets) return launch_mixed_t<kQuad, kSoft, false, false>(L, b, nstars_cap, eps2, ax, ay, az, true);
    }
    return launch_mixed_t<kQuad, kSoft, kPot, true>(L, b, nstars_cap, eps2, ax, ay, az, false);
}

cudaError_t lpt_order(const Launch &L, const TreeBufs &b, int gsize) {
    k_lpt_order<<<1, kLptThreads, 0, L.stream>>>(b.info, gsize, b.nsys > 1, b.gcost, b.gperm, int32_t(b.cap_groups));
    ++*L.count;
    return cudaGetLastError();
}

// Parts of a split walk of groups of gsize stars (1: no split), for single systems with few groups
// per SM: by the stars the walk takes (a target list: the previous event's count), within the
// budget of nstars_cap bodies and the part accumulators. The same decision as launch_mixed_t's.
int split_parts(const TreeBufs &b, int64_t nstars_cap, bool targets, int gsize) {
    if (b.nsys > 1 || !b.split || !b.part_acc) return 1;
    const int64_t walked = targets && b.walk_hint > 0 && b.walk_hint < nstars_cap ? b.walk_hint : nstars_cap;
    int parts = walk_parts(walked, gsize);
    const int budget = walk_parts_budget(nstars_cap);
    if (parts > budget) parts = budget;
    return parts > 1 && int64_t(parts) * 3 * nstars_cap <= b.part_cap ? parts : 1;
}

cudaError_t split_combine(const Launch &L, const TreeBufs &b, int nparts, int64_t stride, bool targets, double *ax,
                          double *ay, double *az) {
    k_split_combine<<<blocks_for(stride, 256), 256, 0, L.stream>>>(b.info, b.order, targets ? b.targets : nullptr,
                                                                    nparts, b.part_acc, stride, ax, ay, az);
    ++*L.count;
    return cudaGetLastError();
}


cudaError_t walk_mixed(const Launch &L, const TreeBufs &b, int64_t nstars_cap, float eps2, int quad, double *ax,
                       double *ay, double *az, bool targets) {
    // The list walk (walk_lists.cu) in groups of 32 (one star a lane) or 64 (two), split among
    // warps when the groups are few; the paired walk above with b.paired (GBH_CFG_PAIRED). Measured
    // against the paired walk's split mode on 16k-131k bodies: the split list walk takes half the
    // time or less (0.11 / 0.17 ms at 16k, 0.37 / 0.76 at 65k, 0.78 / 1.54 at 131k, 64-star groups).
    if (b.cap_nodes < (int64_t(1) << 29)) {
        if (b.group == 32) return walk_lists(L, b, nstars_cap, eps2, quad, ax, ay, az, b.list_depth, targets, 1);
        if (!b.paired) return walk_lists(L, b, nstars_cap, eps2, quad, ax, ay, az, b.list_depth, targets, 2);
    }
    bool soft = eps2 > 0.f;
    if (quad && soft) return launch_mixed<true, true>(L, b, nstars_cap, eps2, ax, ay, az, targets);
    if (quad) return launch_mixed<true, false>(L, b, nstars_cap, eps2, ax, ay, az, targets);
    if (soft) return launch_mixed<false, true>(L, b, nstars_cap, eps2, ax, ay, az, targets);
    return launch_mixed<false, false>(L, b, nstars_cap, eps2, ax, ay, az, targets);
}

cudaError_t walk_mixed_potential(const Launch &L, const TreeBufs &b, int64_t nstars_cap, float eps2, int quad,
                                 double *psi) {
    bool soft = eps2 > 0.f;
    // the list walk's potential sink (64-star groups); the paired walk's potential mode otherwise
    if (soft && b.group == 64 && !b.paired && b.cap_nodes < (int64_t(1) << 29))
        return walk_lists_potential(L, b, eps2, quad, psi);
    if (quad && soft) return launch_mixed<true, true, true>(L, b, nstars_cap, eps2, psi, nullptr, nullptr, false);
    if (quad) return launch_mixed<true, false, true>(L, b, nstars_cap, eps2, psi, nullptr, nullptr, false);
    if (soft) return launch_mixed<false, true, true>(L, b, nstars_cap, eps2, psi, nullptr, nullptr, false);
    return launch_mixed<false, false, true>(L, b, nstars_cap, eps2, psi, nullptr, nullptr, false);
}

int walk_parts(int64_t n, int gsize) {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1)
        sms = 152;
    // Measured on the galaxy model at 8k-512k bodies (leaf 32): each part re-tests the nodes
    // above its range and skips the subtrees beside it, so splitting pays only while the unsplit
    // walk leaves most of the GPU idle. Best part counts by groups per SM: up to 2.5 -> 32 (1.2x
    // over 16 parts at 16k bodies), up to 5 -> 16 (5x over no split at 16k), up to 7 -> 8 (1.9x
    // at 64k), up to 14 -> 4 (1.09x at 128k), up to 21 -> 2 (1.15x at 192k), more -> no split
    // (2 parts were 1.2x slower at 256k).
    const int64_t groups = (n + gsize - 1) / gsize;
    if (2 * groups <= 5 * int64_t(sms)) return 32;
    if (groups <= 5 * int64_t(sms)) return 16;
    if (groups <= 7 * int64_t(sms)) return 8;
    if (groups <= 14 * int64_t(sms)) return 4;
    if (groups <= 21 * int64_t(sms)) return 2;
    return 1;
}

int walk_parts_budget(int64_t n) {
    // whenever a walk over these n bodies may split: 16 parts (a target list may walk few enough
    // groups for more parts than all n would take), or 32 where n itself takes 32
    const int np = walk_parts(n, 64);
    return np <= 1 ? 1 : (np > 16 ? np : 16);
}

cudaError_t split_reserve(TreeBufs &b, int64_t n) {
    const int parts = walk_parts_budget(n);
    if (parts <= 1) return cudaSuccess;
    const int64_t need = int64_t(parts) * 3 * n;
    if (need <= b.part_cap) return cudaSuccess;
    if (b.part_acc) cudaFree(b.part_acc);
    b.part_acc = nullptr;
    b.part_cap = 0;
    const int64_t cap = need + need / 4;
    cudaError_t e = dev_alloc(&b.part_acc, sizeof(double) * size_t(cap));
    if (e != cudaSuccess) {
        b.part_acc = nullptr;
        return e;
    }
    b.part_cap = cap;
    return cudaSuccess;
}

cudaError_t fp32_fma_probe(const Launch &L, int blocks, int iters, float *out) {
    k_fma_probe<<<blocks, 256, 0, L.stream>>>(iters, out);
    ++*L.count;
    return cudaGetLastError();
}

}  // namespace gbh
