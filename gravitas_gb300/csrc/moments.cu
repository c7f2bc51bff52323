// moments.cu — node moments for the FP32 walks (FMA contraction on, no FP64 arithmetic).
//
// The FP32 walks read each node's centre of mass as hi + lo FP32 parts, and its mass,
// quadrupole and crit2 in FP32. FP64 runs at a small fraction of the FP32 rate on GB300, so
// this upsweep forms the moments of finish (build.go:176-217) in FP32 about a reference point
// inside the node (its first star, or its first child's centre of mass): offsets
// d = (hi_j - hi_ref) + (lo_j - lo_ref) are exact or relatively small, the mass-weighted mean
// offset gives the centre of mass as ref + mean (renormalised to hi + lo), and the traceless
// quadrupole with its parallel-axis shift (quadrupole.add, build.go:329-337) is summed about
// it. crit2 = (2 half / theta + |com - centre|)^2 (Barnes 1994, build.go:208-211), where the
// offset of the geometric centre from the reference point is formed in double-float arithmetic
// from the FP32 hi + lo views of the root corner and side. Values agree with the FP64 moments
// to FP32 rounding; the FP64 walk uses the bit-exact upsweep of tree.cu instead.
#include <cuda_runtime.h>

#include <cuda/atomic>

#include "gbh_internal.cuh"

namespace gbh {

namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ void set_err(DevInfo *info, int where) {
    atomicExch(&info->err, 1);
    info->err_where = where;
}

// Error-free sum a + b = s + e (Knuth's TwoSum).
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = a + b;
    float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// (ref_hi + ref_lo) + off as a renormalised hi + lo pair.
__device__ __forceinline__ void add_offset(float rh, float rl, float off, float &h, float &l) {
    float s, e;
    two_sum(rh, off, s, e);
    e += rl;
    h = s + e;
    l = e - (h - s);
}

__device__ __forceinline__ uint32_t compact3(uint64_t v) {  // inverse of spread (morton.go:7-15)
    v &= 0x1249249249249249ull;
    v = (v | v >> 2) & 0x10c30c30c30c30c3ull;
    v = (v | v >> 4) & 0x100f00f00f00f00full;
    v = (v | v >> 8) & 0x1f0000ff0000ffull;
    v = (v | v >> 16) & 0x1f00000000ffffull;
    v = (v | v >> 32) & 0x1fffffull;
    return uint32_t(v);
}

// ref - centre along one axis: centre = min + (2 i + 1) half_L, half_L = side 2^-(L+1).
__device__ __forceinline__ float ref_minus_centre(float rh, float rl, float mh, float ml, float sh, float sl,
                                                  uint32_t cell, int L) {
    float k = ldexpf(float(2u * cell + 1u), -(L + 1));  // exact
    float a, ea;
    two_sum(rh, -mh, a, ea);
    float p = k * sh;
    float ep = fmaf(k, sh, -p);  // exact error of the product
    return (a - p) + (((ea + (rl - ml)) - ep) - k * sl);
}

struct FMom {
    float hx, hy, hz, lx, ly, lz, m;
    float qxx, qyy, qzz, qxy, qxz, qyz;
};

__device__ __forceinline__ void quad_add(FMom &q, float m, float ex, float ey, float ez) {
    float r2 = ex * ex + ey * ey + ez * ez;
    q.qxx += m * (3.f * ex * ex - r2);
    q.qyy += m * (3.f * ey * ey - r2);
    q.qzz += m * (3.f * ez * ez - r2);
    float m3 = 3.f * m;
    q.qxy += m3 * ex * ey;
    q.qxz += m3 * ex * ez;
    q.qyz += m3 * ey * ez;
}

// The fields of a node that its moments need: loaded one level ahead of the arrival at the node.
struct UpNode {
    int32_t first = 0, next = 0, lo = 0, hi = 0;
    uint32_t info = 0;  // level in bits 0-7, child count in bits 8-15
};

__device__ __forceinline__ UpNode up_node(const gbh_node *nodes, const uint32_t *n_info, int32_t r) {
    UpNode u;
    u.first = nodes[r].first;
    u.next = nodes[r].next;
    u.lo = nodes[r].lo;
    u.hi = nodes[r].hi;
    u.info = n_info[r];
    return u;
}

// Finishes node r: centre of mass from the reference point and mean offset (or the geometric
// centre for zero mass), crit2, and the walk records (stored when `store`). `key` is the key of
// any star of the node: the node's cell is the prefix of its level.
__device__ __forceinline__ void finish_fast(const SysGeo &inf, FMom &q, float rhx, float rhy, float rhz, float rlx,
                                            float rly, float rlz, float ox, float oy, float oz, uint64_t key,
                                            const UpNode &u, int32_t r, PNode *pn, MNode *mn, int2 *mr, LNode *ln,
                                            bool plain_records, bool store) {
    const int L = int(u.info & 0xffu);
    int sh = 3 * (kMaxLevel - L);
    uint64_t pre = L == 0 ? 0 : key >> sh;
    float cx = ref_minus_centre(rhx, rlx, inf.min_hi[0], inf.min_lo[0], inf.side_hi, inf.side_lo, compact3(pre >> 2), L);
    float cy = ref_minus_centre(rhy, rly, inf.min_hi[1], inf.min_lo[1], inf.side_hi, inf.side_lo, compact3(pre >> 1), L);
    float cz = ref_minus_centre(rhz, rlz, inf.min_hi[2], inf.min_lo[2], inf.side_hi, inf.side_lo, compact3(pre), L);
    if (!(q.m > 0.f)) {  // empty mass: the geometric centre (build.go:189-193)
        ox = -cx;
        oy = -cy;
        oz = -cz;
    }
    add_offset(rhx, rlx, ox, q.hx, q.lx);
    add_offset(rhy, rly, oy, q.hy, q.ly);
    add_offset(rhz, rlz, oz, q.hz, q.lz);
    if (!store) return;
    float dx = ox + cx, dy = oy + cy, dz = oz + cz;  // com - centre
    float crit = inf.crit_base[L] + sqrtf(dx * dx + dy * dy + dz * dz);
    float crit2 = crit * crit;
    const int32_t first = u.first, next = u.next, lo = u.lo, hi = u.hi;
    if (plain_records) {
        PNode p;
        p.com = make_float4(q.hx, q.hy, q.hz, q.m);
        p.q1 = make_float4(q.qxx, q.qyy, q.qzz, q.qxy);
        p.q2 = make_float4(q.qxz, q.qyz, crit2, 0.f);
        p.links = make_int4(first, next, lo, hi);
        pn[r] = p;
    }
    MNode m;
    m.a = make_float4(q.hx, q.hy, q.hz, crit2);
    m.b = make_float4(q.lx, q.ly, q.lz, q.m);
    m.c = make_float4(q.qxx, q.qyy, q.qzz, q.qxy);
    m.d = make_float4(q.qxz, q.qyz, __int_as_float(first), __int_as_float(next));
    mn[r] = m;
    mr[r] = make_int2(lo, hi);
    // the list walk's record (the link packs the children's range; the caller keeps nodes < 2^29)
    const uint32_t link = first >= 0 ? uint32_t(first) | ((((u.info >> 8) & 0xffu) - 1u) & 7u) << 29 : uint32_t(lo);
    LNode l;
    l.a = make_float4(q.hx, q.hy, q.hz, first >= 0 ? crit : -crit);  // the sign marks a leaf
    l.b = make_float4(q.lx, q.ly, q.lz, __uint_as_float(link));
    l.c = make_float4(-q.qxx, -q.qyy, -q.qzz, -q.qxy);
    l.d = make_float4(-q.qxz, -q.qyz, q.m, __int_as_float(hi));
    ln[r] = l;
}

constexpr unsigned kFull = 0xffffffffu;
// Lanes per leaf and per inner node. Measured on the merger (whole build, CUDA events): 2, 4 and
// 8 lanes tie at 16k bodies; from 1M to 4M 2 lanes are fastest (more lanes mean more warps for
// the same leaves), and one thread per leaf was 3-20 % slower below 2M and 3 % faster at 4M.
constexpr int kGroup = 2;
constexpr int kMaxChildren = 8;

// Sum over the kGroup lanes of a group: every lane ends with the same bits (each butterfly step
// adds the same two values in both lanes, and IEEE addition is commutative).
__device__ __forceinline__ float grp_sum(float v) {
#pragma unroll
    for (int o = kGroup / 2; o >= 1; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
    return v;
}

__device__ __forceinline__ void grp_sum_quad(FMom &q) {
    q.qxx = grp_sum(q.qxx);
    q.qyy = grp_sum(q.qyy);
    q.qzz = grp_sum(q.qzz);
    q.qxy = grp_sum(q.qxy);
    q.qxz = grp_sum(q.qxz);
    q.qyz = grp_sum(q.qyz);
}

// One group of kGroup lanes per leaf: the lanes sum the leaf's stars (a star a lane in turn) and
// reduce over the group; then the group walks up the tree. At each node the group leader
// counts its arrival; the last child to arrive finishes the node (child k + i kGroup on lane k). Each
// level costs two dependent round trips to L2 (the arrival, then the children's records
// together with the next node's fields and parent, loaded one level ahead).
__global__ __launch_bounds__(kThreads) void k_upsweep_fast(const uint64_t *__restrict__ keys, const DevInfo *info,
                                                           const int32_t *__restrict__ leaves,
                                                           const uint32_t *__restrict__ cnt,
                                                           const uint32_t *__restrict__ base,
                                                           const int32_t *__restrict__ pre_ref,
                                                           const float4 *__restrict__ st_hi,
                                                           const float4 *__restrict__ st_lo,
                                                           float4 *__restrict__ st_off, const gbh_node *nodes,
                                                           const int32_t *__restrict__ n_parent,
                                                           const uint32_t *__restrict__ n_info, int32_t *n_arrive,
                                                           PNode *pn, MNode *mn, int2 *mr, LNode *ln,
                                                           bool plain_records,
                                                           const int32_t *__restrict__ sid_sorted,
                                                           const SysGeo *__restrict__ geo, DevInfo *err_info) {
    const int lane = threadIdx.x & 31, k = lane & (kGroup - 1), src = lane & ~(kGroup - 1);
    const bool leader = k == 0;
    const int64_t ns = info->nstars, nn = info->nnodes, nleaves = info->nleaves;
    const int64_t stride = int64_t(gridDim.x) * (kThreads / kGroup);
    for (int64_t wb = (int64_t(blockIdx.x) * kThreads + (threadIdx.x & ~31)) / kGroup; wb < nleaves; wb += stride) {
        const int64_t t = wb + lane / kGroup;
        bool act = t < nleaves;
        int32_t r = 0, P = -1, GP = -1;
        UpNode u, pu;
        if (act) {
            const int32_t i = leaves[t];
            if (i < 0 || i >= ns || cnt[i] == 0) {
                act = false;
                if (leader) set_err(err_info, 23);
            } else {
                r = pre_ref[base[i] + cnt[i] - 1];  // the last node of a chain is a leaf
                if (r < 0 || r >= nn) {
                    act = false;
                    if (leader) set_err(err_info, 20);
                } else {
                    u = up_node(nodes, n_info, r);
                    P = n_parent[r];
                    if (u.lo < 0 || u.hi > ns || u.lo >= u.hi) {
                        act = false;
                        if (leader) set_err(err_info, 21);
                    }
                }
            }
        }
        // the leaf: star sums, a star a lane in turn
        float4 rh = make_float4(0.f, 0.f, 0.f, 0.f), rl = rh;
        uint64_t key = 0;
        const SysGeo *g = geo;
        float M = 0.f, sx = 0.f, sy = 0.f, sz = 0.f;
        if (act) {
            rh = st_hi[u.lo];
            rl = st_lo[u.lo];
            key = keys[u.lo];
            if (sid_sorted) g = geo + sid_sorted[u.lo];
            if (P >= 0) {
                pu = up_node(nodes, n_info, P);
                GP = n_parent[P];
            }
            for (int32_t j = u.lo + k; j < u.hi; j += kGroup) {
                const float4 h = st_hi[j], l = st_lo[j];
                const float dx = (h.x - rh.x) + (l.x - rl.x), dy = (h.y - rh.y) + (l.y - rl.y),
                            dz = (h.z - rh.z) + (l.z - rl.z);
                M += h.w;
                sx = fmaf(h.w, dx, sx);
                sy = fmaf(h.w, dy, sy);
                sz = fmaf(h.w, dz, sz);
            }
        }
        M = grp_sum(M);
        sx = grp_sum(sx);
        sy = grp_sum(sy);
        sz = grp_sum(sz);
        FMom q = {};
        q.m = M;
        float ox = 0.f, oy = 0.f, oz = 0.f;
        if (M > 0.f) {
            ox = sx / M;
            oy = sy / M;
            oz = sz / M;
            if (act)
                for (int32_t j = u.lo + k; j < u.hi; j += kGroup) {
                    const float4 h = st_hi[j], l = st_lo[j];
                    const float ex = ((h.x - rh.x) + (l.x - rl.x)) - ox;
                    const float ey = ((h.y - rh.y) + (l.y - rl.y)) - oy;
                    const float ez = ((h.z - rh.z) + (l.z - rl.z)) - oz;
                    quad_add(q, h.w, ex, ey, ez);
                }
        }
        grp_sum_quad(q);
        if (act) {
            finish_fast(*g, q, rh.x, rh.y, rh.z, rl.x, rl.y, rl.z, ox, oy, oz, key, u, r, pn, mn, mr, ln,
                        plain_records, leader);
            // Each star's offset from the leaf's centre of mass, formed with the operations of the
            // mixed walk's separation (com_hi - star_hi) + (com_lo - star_lo), negated: a star
            // paired with itself then gets a separation of exactly 0 (IEEE addition is
            // sign-symmetric).
            for (int32_t j = u.lo + k; j < u.hi; j += kGroup) {
                const float4 h = st_hi[j], l = st_lo[j];
                st_off[j] = make_float4((h.x - q.hx) + (l.x - q.lx), (h.y - q.hy) + (l.y - q.ly),
                                        (h.z - q.hz) + (l.z - q.lz), h.w);
            }
        }
        // up the tree: P is the node to arrive at, pu its fields, GP its parent
        for (int guard = 0; guard <= kMaxLevel + 1; ++guard) {
            act = act && P >= 0;
            if (!__any_sync(kFull, act)) break;
            const uint32_t nch = (pu.info >> 8) & 0xffu;
            int last = 0;
            if (act && leader) {
                // arrival counter with acquire-release ordering: this child's records are visible
                // to the last child to arrive, whose group reads every child's records after the
                // leader's increment and the warp barrier below
                cuda::atomic_ref<int, cuda::thread_scope_device> arrive(n_arrive[P]);
                last = arrive.fetch_add(1, cuda::memory_order_acq_rel) == int(nch) - 1;
            }
            last = __shfl_sync(kFull, last, src);
            __syncwarp(kFull);
            act = act && last;
            if (act && (pu.first < 0 || nch == 0 || nch > uint32_t(kMaxChildren) || int64_t(pu.first) + nch > nn)) {
                act = false;
                if (leader) set_err(err_info, 22);
            }
            constexpr int kPer = kMaxChildren / kGroup;  // children a lane
            float4 a[kPer], b[kPer], c[kPer], d[kPer];
            bool child[kPer];
#pragma unroll
            for (int e = 0; e < kPer; ++e) {
                const int ch = k + e * kGroup;
                child[e] = act && uint32_t(ch) < nch;
                a[e] = b[e] = c[e] = d[e] = make_float4(0.f, 0.f, 0.f, 0.f);
                if (child[e]) {
                    a[e] = __ldcg(&mn[pu.first + ch].a);
                    b[e] = __ldcg(&mn[pu.first + ch].b);
                    c[e] = __ldcg(&mn[pu.first + ch].c);
                    d[e] = __ldcg(&mn[pu.first + ch].d);
                }
            }
            UpNode gu;
            int32_t GGP = -1;
            if (act && GP >= 0) {
                gu = up_node(nodes, n_info, GP);
                GGP = n_parent[GP];
            }
            // reference point: the first child's centre of mass
            const float rax = __shfl_sync(kFull, a[0].x, src), ray = __shfl_sync(kFull, a[0].y, src),
                        raz = __shfl_sync(kFull, a[0].z, src), rbx = __shfl_sync(kFull, b[0].x, src),
                        rby = __shfl_sync(kFull, b[0].y, src), rbz = __shfl_sync(kFull, b[0].z, src);
            float dx[kPer], dy[kPer], dz[kPer];
            M = sx = sy = sz = 0.f;
#pragma unroll
            for (int e = 0; e < kPer; ++e) {
                dx[e] = (a[e].x - rax) + (b[e].x - rbx);
                dy[e] = (a[e].y - ray) + (b[e].y - rby);
                dz[e] = (a[e].z - raz) + (b[e].z - rbz);
                if (child[e]) {
                    M += b[e].w;
                    sx = fmaf(b[e].w, dx[e], sx);
                    sy = fmaf(b[e].w, dy[e], sy);
                    sz = fmaf(b[e].w, dz[e], sz);
                }
            }
            M = grp_sum(M);
            sx = grp_sum(sx);
            sy = grp_sum(sy);
            sz = grp_sum(sz);
            q = FMom{};
            q.m = M;
            ox = oy = oz = 0.f;
            if (M > 0.f) {
                ox = sx / M;
                oy = sy / M;
                oz = sz / M;
            }
#pragma unroll
            for (int e = 0; e < kPer; ++e)
                if (child[e]) {
                    q.qxx += c[e].x;
                    q.qyy += c[e].y;
                    q.qzz += c[e].z;
                    q.qxy += c[e].w;
                    q.qxz += d[e].x;
                    q.qyz += d[e].y;
                    quad_add(q, b[e].w, dx[e] - ox, dy[e] - oy, dz[e] - oz);
                }
            grp_sum_quad(q);
            if (act)
                finish_fast(*g, q, rax, ray, raz, rbx, rby, rbz, ox, oy, oz, key, pu, P, pn, mn, mr, ln,
                            plain_records, leader);
            P = GP;
            pu = gu;
            GP = GGP;
        }
    }
}

// FP64 moment fields of the node table from the MNode records.
__global__ __launch_bounds__(kThreads) void k_export_fast(const DevInfo *info, const MNode *__restrict__ mn,
                                                          gbh_node *nodes) {
    int64_t r = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (r >= info->nnodes) return;
    MNode m = mn[r];
    gbh_node &nd = nodes[r];
    nd.x = double(m.a.x) + double(m.b.x);
    nd.y = double(m.a.y) + double(m.b.y);
    nd.z = double(m.a.z) + double(m.b.z);
    nd.m = m.b.w;
    nd.qxx = m.c.x;
    nd.qyy = m.c.y;
    nd.qzz = m.c.z;
    nd.qxy = m.c.w;
    nd.qxz = m.d.x;
    nd.qyz = m.d.y;
    nd.crit2 = m.a.w;
}

}  // namespace

cudaError_t upsweep_fast(const Launch &L, TreeBufs &b, bool plain_records) {
    const uint32_t *cnt = b.chain_cnt, *base = b.chain_cnt + b.cap_n;
    // a group of 8 lanes per leaf (at most one leaf per node), grid-stride beyond 4096 blocks
    int64_t nb = (b.cap_nodes + kThreads / kGroup - 1) / (kThreads / kGroup);
    nb = nb < 1 ? 1 : nb > 4096 ? 4096 : nb;
    k_upsweep_fast<<<unsigned(nb), kThreads, 0, L.stream>>>(
        b.keys, b.info, b.leaves, cnt, base, b.pre_ref, b.st_hi, b.st_lo, b.st_off, b.nodes, b.n_parent, b.n_info,
        b.n_arrive,
        b.pnodes, b.mnodes, b.mrange, b.lnode, plain_records, b.nsys > 1 ? b.sid_sorted : nullptr, b.geo, b.info);
    ++*L.count;
    return cudaGetLastError();
}

cudaError_t export_fast_moments(const Launch &L, TreeBufs &b) {
    int64_t nb = (b.cap_nodes + kThreads - 1) / kThreads;
    k_export_fast<<<unsigned(nb < 1 ? 1 : nb), kThreads, 0, L.stream>>>(b.info, b.mnodes, b.nodes);
    ++*L.count;
    return cudaGetLastError();
}

}  // namespace gbh
