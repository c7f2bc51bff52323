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

// Finishes node r: centre of mass from the reference point and mean offset (or the geometric
// centre for zero mass), crit2, and the walk records.
__device__ __forceinline__ void finish_fast(const SysGeo &inf, FMom &q, float rhx, float rhy, float rhz, float rlx,
                                            float rly, float rlz, float ox, float oy, float oz, uint64_t key,
                                            uint32_t ninfo, const gbh_node *nodes, int32_t r, PNode *pn, MNode *mn,
                                            int2 *mr, LNode *ln, bool plain_records) {
    const int L = int(ninfo & 0xffu);
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
    float dx = ox + cx, dy = oy + cy, dz = oz + cz;  // com - centre
    float crit = inf.crit_base[L] + sqrtf(dx * dx + dy * dy + dz * dz);
    float crit2 = crit * crit;
    int32_t first = nodes[r].first, next = nodes[r].next, lo = nodes[r].lo, hi = nodes[r].hi;
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
    const uint32_t link = first >= 0 ? uint32_t(first) | ((((ninfo >> 8) & 0xffu) - 1u) & 7u) << 29 : uint32_t(lo);
    LNode l;
    l.a = make_float4(q.hx, q.hy, q.hz, first >= 0 ? crit : -crit);  // the sign marks a leaf
    l.b = make_float4(q.lx, q.ly, q.lz, __uint_as_float(link));
    l.c = make_float4(-q.qxx, -q.qyy, -q.qzz, -q.qxy);
    l.d = make_float4(-q.qxz, -q.qyz, q.m, __int_as_float(hi));
    ln[r] = l;
}

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
    int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= int64_t(info->nleaves)) return;
    const DevInfo inf = *info;
    const int64_t ns = inf.nstars, nn = inf.nnodes;
    int32_t i = leaves[t];
    if (i < 0 || i >= ns || cnt[i] == 0) {
        set_err(err_info, 23);
        return;
    }
    int32_t r = pre_ref[base[i] + cnt[i] - 1];  // the last node of a chain is a leaf
    if (r < 0 || r >= nn) {
        set_err(err_info, 20);
        return;
    }
    {
        int32_t lo = nodes[r].lo, hi = nodes[r].hi;
        if (lo < 0 || hi > ns || lo >= hi) {
            set_err(err_info, 21);
            return;
        }
        const float4 rh = st_hi[lo], rl = st_lo[lo];
        float M = 0.f, sx = 0.f, sy = 0.f, sz = 0.f;
        for (int32_t j = lo; j < hi; ++j) {
            float4 h = st_hi[j], l = st_lo[j];
            float dx = (h.x - rh.x) + (l.x - rl.x), dy = (h.y - rh.y) + (l.y - rl.y), dz = (h.z - rh.z) + (l.z - rl.z);
            M += h.w;
            sx = fmaf(h.w, dx, sx);
            sy = fmaf(h.w, dy, sy);
            sz = fmaf(h.w, dz, sz);
        }
        FMom q = {};
        q.m = M;
        float ox = 0.f, oy = 0.f, oz = 0.f;
        if (M > 0.f) {
            ox = sx / M;
            oy = sy / M;
            oz = sz / M;
            for (int32_t j = lo; j < hi; ++j) {
                float4 h = st_hi[j], l = st_lo[j];
                float ex = ((h.x - rh.x) + (l.x - rl.x)) - ox;
                float ey = ((h.y - rh.y) + (l.y - rl.y)) - oy;
                float ez = ((h.z - rh.z) + (l.z - rl.z)) - oz;
                quad_add(q, h.w, ex, ey, ez);
            }
        }
        finish_fast(geo[sid_sorted ? sid_sorted[lo] : 0], q, rh.x, rh.y, rh.z, rl.x, rl.y, rl.z, ox, oy, oz, keys[lo],
                    n_info[r], nodes, r, pn, mn, mr, ln, plain_records);
        // Each star's offset from the leaf's centre of mass, formed with the operations of the
        // mixed walk's separation (com_hi - star_hi) + (com_lo - star_lo), negated: a star paired
        // with itself then gets a separation of exactly 0 (IEEE addition is sign-symmetric).
        for (int32_t j = lo; j < hi; ++j) {
            float4 h = st_hi[j], l = st_lo[j];
            st_off[j] = make_float4((h.x - q.hx) + (l.x - q.lx), (h.y - q.hy) + (l.y - q.ly),
                                    (h.z - q.hz) + (l.z - q.lz), h.w);
        }
    }
    int32_t cur = r;
    for (int guard = 0; guard <= kMaxLevel + 1; ++guard) {
        int32_t par = n_parent[cur];
        if (par < 0) break;
        uint32_t nch = (n_info[par] >> 8) & 0xffu;
        // arrival counter with acquire-release ordering: this child's records are visible to the
        // last child to arrive, which reads every child's records after its own increment
        cuda::atomic_ref<int, cuda::thread_scope_device> arrive(n_arrive[par]);
        const int old = arrive.fetch_add(1, cuda::memory_order_acq_rel);
        if (old != int(nch) - 1) break;
        int32_t first = nodes[par].first;
        if (first < 0 || int64_t(first) + nch > nn) {
            set_err(err_info, 22);
            break;
        }
        // reference point: the first child's centre of mass
        const float4 ra = __ldcg(&mn[first].a), rb = __ldcg(&mn[first].b);
        float M = 0.f, sx = 0.f, sy = 0.f, sz = 0.f;
        for (int32_t ch = first; ch < first + int32_t(nch); ++ch) {
            float4 a = __ldcg(&mn[ch].a), b = __ldcg(&mn[ch].b);
            float dx = (a.x - ra.x) + (b.x - rb.x), dy = (a.y - ra.y) + (b.y - rb.y), dz = (a.z - ra.z) + (b.z - rb.z);
            M += b.w;
            sx = fmaf(b.w, dx, sx);
            sy = fmaf(b.w, dy, sy);
            sz = fmaf(b.w, dz, sz);
        }
        FMom q = {};
        q.m = M;
        float ox = 0.f, oy = 0.f, oz = 0.f;
        if (M > 0.f) {
            ox = sx / M;
            oy = sy / M;
            oz = sz / M;
        }
        for (int32_t ch = first; ch < first + int32_t(nch); ++ch) {
            float4 a = __ldcg(&mn[ch].a), b = __ldcg(&mn[ch].b), cq = __ldcg(&mn[ch].c), dq = __ldcg(&mn[ch].d);
            q.qxx += cq.x;
            q.qyy += cq.y;
            q.qzz += cq.z;
            q.qxy += cq.w;
            q.qxz += dq.x;
            q.qyz += dq.y;
            float ex = ((a.x - ra.x) + (b.x - rb.x)) - ox;
            float ey = ((a.y - ra.y) + (b.y - rb.y)) - oy;
            float ez = ((a.z - ra.z) + (b.z - rb.z)) - oz;
            quad_add(q, b.w, ex, ey, ez);
        }
        const int32_t plo = nodes[par].lo;
        finish_fast(geo[sid_sorted ? sid_sorted[plo] : 0], q, ra.x, ra.y, ra.z, rb.x, rb.y, rb.z, ox, oy, oz, keys[plo],
                    n_info[par], nodes, par, pn, mn, mr, ln, plain_records);
        cur = par;
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
    int64_t nb = (b.cap_n + kThreads - 1) / kThreads;
    k_upsweep_fast<<<unsigned(nb < 1 ? 1 : nb), kThreads, 0, L.stream>>>(
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
