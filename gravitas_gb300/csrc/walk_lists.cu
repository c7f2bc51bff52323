// walk_lists.cu — the list walk: the mixed-precision FP32 walk with decoupled traversal and
// evaluation (compiled like walk.cu: FMA contraction on, fast FP32 division and square root).
//
// One warp owns a group of up to 32 or 64 consecutive Morton-sorted stars, one or two per lane
// (lane l holds stars l and 32 + l), and builds the group's interaction lists cooperatively before
// evaluating them:
//
// * Traversal is node-parallel. The warp keeps a stack of sibling ranges (an opened inner node's
//   children are contiguous in the reference's serial layout, build.go:142-152) in shared memory
//   and tests up to 32 nodes per step, one per lane, with the opening criterion of the reference
//   walk (bh.go:116: open when d2 < crit2) taken over every star of the group: a node is accepted
//   only when no star of the group would open it. The test is the group's bounding box first; a
//   node the box cannot accept is refined against each star. Both tests add a margin that covers
//   their FP32 rounding, so every star sees each accepted node exactly where the reference would
//   accept it, or deeper.
// * Accepted nodes and the stars of opened leaves are appended (ballot + popc offsets) to two
//   lists in shared memory, staged as FP32 records relative to the group's origin. When a list
//   reaches its depth (a knob of gbh_params.list_depth) the warp evaluates it: every lane takes
//   two list entries at once in packed FP32x2 arithmetic (__ffma2_rn and friends) against each of
//   its stars, the records read as broadcasts from shared memory (once for both stars of a lane),
//   with no branch and no dependence between entries.
// * Persistent warps (one launch of num_SMs x resident blocks) take groups from a counter, longest
//   first in the order the previous walk's group costs give (k_lpt_order). A walk restricted to a
//   target list (block steps) takes groups of 32 or 64 consecutive list entries; a full list
//   walks exactly as no list.
// * The adjoint sink (at the end of the file) hands the same lists to the transposed Jacobian of
//   the walk's force instead: the tree adjoint of the adjoint pair.
//
// Precision: positions are FP64 split into hi + lo FP32 parts. The group's origin O is its first
// star's hi part; a star's or node's offset from O is (hi - O) + lo in FP32, exact for nearby
// points and relatively accurate for distant ones, and a separation is the difference of two
// offsets. That is accurate to FP32 rounding of the group's extent; a group whose extent is large
// against its stars' spacing and the softening (one that straddles a jump of the Morton curve)
// forms every separation as (hi_j - hi_i) + (lo_j - lo_i) instead, accurate to FP32 rounding of
// the separation itself. Each star sums each list in FP32 and folds the sum into a Kahan sum.
#include <cuda_runtime.h>

#include "gbh_internal.cuh"

namespace gbh {

namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kLwWarps = 2;              // warps per block (shared memory ~10 KB per warp)
constexpr int kLwThreads = 32 * kLwWarps;
// Sibling ranges of one depth on the stack were all pushed by one step (ranges are popped only
// from the deepest level, and a step pushes the children of the nodes it tests, one level deeper),
// so at most 32 per depth, and depths run from 1 to kMaxLevel.
constexpr int kStackCap = 32 * (kMaxLevel + 1);
constexpr int kLevels = kMaxLevel + 3;
constexpr int kNodeF4 = 224;  // node list buffer, float4 slots (3,584 B)
constexpr int kSrcF4 = 192;   // source list buffer, float4 slots (3,072 B)

// Record layouts. A pair of list entries (A, B) is stored field by field as (A, B) float pairs,
// so that one packed FP32x2 operand is one 8-byte half of a float4 read.
//   node, compact: (x, y | z, m | qxx, qyy | qzz, qxy | qxz, qyz) — 5 float4 per pair
//   node, exact:   the same with x, y, z the hi parts, then (xlo, ylo | zlo, 0) — 7 float4
//   source, compact: (x, y | z, m) — 2 float4;  exact: (xhi, yhi | zhi, m | xlo, ylo | zlo, 0) — 4
// Quadrupole components are stored negated (the term -Q.d / r^5 becomes a fused add).
template <bool kExact>
struct Layout {
    static constexpr int kNodePair = kExact ? 7 : 5;
    static constexpr int kSrcPair = kExact ? 4 : 2;
    static constexpr int kNodeCap = 2 * (kNodeF4 / kNodePair);  // entries: 88 compact, 64 exact
    static constexpr int kSrcCap = 2 * (kSrcF4 / kSrcPair);     // entries: 192 compact, 96 exact
};

// The traversal's own shared memory.
struct __align__(16) TravMem {
    uint32_t stack[kStackCap];   // sibling ranges: first | (count - 1) << 29
    int32_t lvl[kLevels];        // first stack slot of each depth
    float4 rq[32];               // the nodes of a step that the box test keeps, pair-interleaved
    int32_t owner[32];           // source staging: the lane whose leaf run starts at each slot
};

struct __align__(16) WarpMem {
    float4 nbuf[kNodeF4];
    float4 sbuf[kSrcF4];
    TravMem tm;
};

__device__ __forceinline__ void set_err(DevInfo *info, int where) {
    atomicExch(&info->err, 1);
    info->err_where = where;
}

__device__ __forceinline__ float2 f2(float v) { return make_float2(v, v); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 lo2(float4 v) { return make_float2(v.x, v.y); }
__device__ __forceinline__ float2 hi2(float4 v) { return make_float2(v.z, v.w); }

// Kahan fold of a list's FP32 sum into the running sum (s, c): true sum = s - c.
__device__ __forceinline__ void kahan_fold(float &s, float &c, float part) {
    float y = part - c;
    float t = s + y;
    c = (t - s) - y;
    s = t;
}

// The group's star, as its lane holds it.
struct Target {
    float tx, ty, tz;     // offset from the group origin (compact separations)
    float hx, hy, hz;     // hi parts (exact separations)
    float lx, ly, lz;     // lo parts
};

struct Acc {
    float2 px, py, pz;    // the current list's sums (entry A, entry B halves)
    float sx, sy, sz, cx, cy, cz;  // Kahan sums
    __device__ __forceinline__ void fold() {
        kahan_fold(sx, cx, px.x + px.y);
        kahan_fold(sy, cy, py.x + py.y);
        kahan_fold(sz, cz, pz.x + pz.y);
        px = py = pz = f2(0.f);
    }
};

// Separation (entry - star) along one axis for a pair of entries.
template <bool kExact>
__device__ __forceinline__ float2 sep(float2 h, float2 l, float nt, float nh, float nl) {
    if constexpr (kExact) return add2(add2(h, f2(nh)), add2(l, f2(nl)));
    else return add2(h, f2(nt));
}

// Evaluates the node list (count entries, padded to pairs) for the lane's kS stars: each pair of
// records is read once and evaluated for every star of the lane.
template <bool kExact, bool kQuad, bool kSoft, int kS>
__device__ __forceinline__ void eval_nodes(const float4 *nbuf, int count, const Target (&t)[kS], float eps2,
                                           Acc (&a)[kS]) {
    using Lay = Layout<kExact>;
    const float2 e2 = f2(eps2);
    const int np = (count + 1) >> 1;
#pragma unroll 2
    for (int p = 0; p < np; ++p) {
        const float4 *r = &nbuf[p * Lay::kNodePair];
        const float4 r0 = r[0], r1 = r[1];
        float2 lx = f2(0.f), ly = f2(0.f), lz = f2(0.f);
        if constexpr (kExact) {
            const float4 r5 = r[5], r6 = r[6];
            lx = lo2(r5);
            ly = hi2(r5);
            lz = lo2(r6);
        }
        float4 r2a, r3, r4;
        if constexpr (kQuad) {
            r2a = r[2];
            r3 = r[3];
            r4 = r[4];
        }
#pragma unroll
        for (int q = 0; q < kS; ++q) {
            const float2 dx = sep<kExact>(lo2(r0), lx, -t[q].tx, -t[q].hx, -t[q].lx);
            const float2 dy = sep<kExact>(hi2(r0), ly, -t[q].ty, -t[q].hy, -t[q].ly);
            const float2 dz = sep<kExact>(lo2(r1), lz, -t[q].tz, -t[q].hz, -t[q].lz);
            const float2 r2 = fma2(dz, dz, fma2(dy, dy, fma2(dx, dx, e2)));
            float2 ir;
            if constexpr (kSoft) {
                ir = make_float2(rsqrtf(r2.x), rsqrtf(r2.y));
            } else {  // an accepted node never sits on a star (d2 >= crit2 > 0); kept for safety
                ir = make_float2(r2.x > 0.f ? rsqrtf(r2.x) : 0.f, r2.y > 0.f ? rsqrtf(r2.y) : 0.f);
            }
            const float2 ir2 = mul2(ir, ir);
            const float2 ir3 = mul2(ir2, ir);
            const float2 mir3 = mul2(hi2(r1), ir3);
            if constexpr (kQuad) {
                // q = -Q.d (the record holds -Q): qx = -(qxx dx + qxy dy + qxz dz), ...
                const float2 qx = fma2(lo2(r4), dz, fma2(hi2(r3), dy, mul2(lo2(r2a), dx)));
                const float2 qy = fma2(hi2(r4), dz, fma2(hi2(r2a), dy, mul2(hi2(r3), dx)));
                const float2 qz = fma2(lo2(r3), dz, fma2(hi2(r4), dy, mul2(lo2(r4), dx)));
                const float2 dqd = fma2(dz, qz, fma2(dy, qy, mul2(dx, qx)));  // -(d.Q.d)
                const float2 ir5 = mul2(ir3, ir2);
                // f = m / r^3 + 5/2 (d.Q.d) / r^7;  a += f d - Q.d / r^5 (bh.go:117-133)
                const float2 f = fma2(mul2(dqd, mul2(ir5, ir2)), f2(-2.5f), mir3);
                a[q].px = fma2(ir5, qx, fma2(f, dx, a[q].px));
                a[q].py = fma2(ir5, qy, fma2(f, dy, a[q].py));
                a[q].pz = fma2(ir5, qz, fma2(f, dz, a[q].pz));
            } else {
                a[q].px = fma2(mir3, dx, a[q].px);
                a[q].py = fma2(mir3, dy, a[q].py);
                a[q].pz = fma2(mir3, dz, a[q].pz);
            }
        }
    }
#pragma unroll
    for (int q = 0; q < kS; ++q) a[q].fold();
}

// Evaluates the source list (leaf stars, count entries padded to pairs): m / (r^2 + eps^2)^(3/2).
// A star paired with itself has a separation of exactly 0 (its record and its target are formed by
// the same operations), which adds 0 with softening, as skipping j == self does (bh.go:142-144);
// without softening r2 = 0 is masked.
template <bool kExact, bool kSoft, int kS>
__device__ __forceinline__ void eval_sources(const float4 *sbuf, int count, const Target (&t)[kS], float eps2,
                                             Acc (&a)[kS]) {
    using Lay = Layout<kExact>;
    const float2 e2 = f2(eps2);
    const int np = (count + 1) >> 1;
#pragma unroll(kS == 1 ? 4 : 2)
    for (int p = 0; p < np; ++p) {
        const float4 *r = &sbuf[p * Lay::kSrcPair];
        const float4 r0 = r[0], r1 = r[1];
        float2 lx = f2(0.f), ly = f2(0.f), lz = f2(0.f);
        if constexpr (kExact) {
            const float4 r2a = r[2], r3 = r[3];
            lx = lo2(r2a);
            ly = hi2(r2a);
            lz = lo2(r3);
        }
#pragma unroll
        for (int q = 0; q < kS; ++q) {
            const float2 dx = sep<kExact>(lo2(r0), lx, -t[q].tx, -t[q].hx, -t[q].lx);
            const float2 dy = sep<kExact>(hi2(r0), ly, -t[q].ty, -t[q].hy, -t[q].ly);
            const float2 dz = sep<kExact>(lo2(r1), lz, -t[q].tz, -t[q].hz, -t[q].lz);
            const float2 r2 = fma2(dz, dz, fma2(dy, dy, fma2(dx, dx, e2)));
            float2 ir;
            if constexpr (kSoft) {
                ir = make_float2(rsqrtf(r2.x), rsqrtf(r2.y));
            } else {
                ir = make_float2(r2.x > 0.f ? rsqrtf(r2.x) : 0.f, r2.y > 0.f ? rsqrtf(r2.y) : 0.f);
            }
            const float2 f = mul2(mul2(hi2(r1), ir), mul2(ir, ir));
            a[q].px = fma2(f, dx, a[q].px);
            a[q].py = fma2(f, dy, a[q].py);
            a[q].pz = fma2(f, dz, a[q].pz);
        }
    }
#pragma unroll
    for (int q = 0; q < kS; ++q) a[q].fold();
}

// Writes field f of list entry e into a pair-interleaved record buffer.
__device__ __forceinline__ void put(float4 *buf, int pair_f4, int e, int f, float v) {
    reinterpret_cast<float *>(buf + (e >> 1) * pair_f4)[2 * f + (e & 1)] = v;
}

// Odd counts: entry B of the last pair becomes a copy of A with zero mass and quadrupole (its
// separation is A's, so its terms are exactly zero).
template <int kPairF4, int kFields>
__device__ __forceinline__ void pad_pair(float4 *buf, int count, int lane, int mass_field, int q_first, int q_last) {
    if (!(count & 1)) return;
    if (lane < kFields) {
        float *r = reinterpret_cast<float *>(buf + (count >> 1) * kPairF4);
        const bool zero = lane == mass_field || (lane >= q_first && lane <= q_last);
        r[2 * lane + 1] = zero ? 0.f : r[2 * lane];
    }
    __syncwarp();
}

struct GroupOut {
    uint32_t cost;
    bool ok;
};

// The warp's list buffers and what a full list is handed to: InPlace evaluates the forces of
// the lane's stars (the list walk); the adjoint sink below evaluates the transposed Jacobian.
struct InPlace {
    static constexpr bool kIndices = false;  // no node or star index per entry
    float4 *nbuf, *sbuf;
    int32_t *nidx, *sidx;
    template <bool kExact, bool kQuad, bool kSoft, int kS>
    __device__ __forceinline__ void nodes(int count, const Target (&t)[kS], float eps2, Acc (&a)[kS], int) {
        eval_nodes<kExact, kQuad, kSoft, kS>(nbuf, count, t, eps2, a);
    }
    template <bool kExact, bool kSoft, int kS>
    __device__ __forceinline__ void sources(int count, const Target (&t)[kS], float eps2, Acc (&a)[kS], int) {
        eval_sources<kExact, kSoft, kS>(sbuf, count, t, eps2, a);
    }
};

// Walks one group with the given separation form; a is zeroed by the caller. kSplit: this warp is
// one part of the group's walk, owning the source stars [s_lo, s_hi) (ranges: each node's star
// range): it skips nodes with no star in its range, tests every other node as the whole walk
// would (so all parts agree on every node), adds an accepted node only when the node's first star
// is its own, and an opened leaf's stars only within its range.
template <bool kExact, bool kQuad, bool kSoft, int kS, bool kSplit = false, class Sink, class AccT>
__device__ __forceinline__ GroupOut walk_group(TravMem &W, Sink &sink, int lane, int32_t root, const Target (&t)[kS], float Ox,
                                               float Oy, float Oz, float bx0, float by0, float bz0, float bx1,
                                               float by1, float bz1, float ext, float eps2, int node_depth,
                                               int src_depth, const LNode *__restrict__ nodes,
                                               const float4 *__restrict__ st_hi, const float4 *__restrict__ st_lo,
                                               int32_t nn, int32_t ns, DevInfo *err_info, AccT (&a)[kS],
                                               const int2 *__restrict__ ranges = nullptr, int32_t s_lo = 0,
                                               int32_t s_hi = 0) {
    using Lay = Layout<kExact>;
    constexpr int kNodeFields = kExact ? 13 : 10;
    constexpr int kSrcFields = kExact ? 7 : 4;
    const unsigned lt = (1u << lane) - 1u, upto = kFull >> (31 - lane);
    // one step appends at most 32 entries to a list below its depth
    if (node_depth > Lay::kNodeCap - 32) node_depth = Lay::kNodeCap - 32;
    if (src_depth > Lay::kSrcCap - 32) src_depth = Lay::kSrcCap - 32;
    int ncount = 0, scount = 0, sp = 1, dtop = 0;
    uint32_t tested = 0, acc_nodes = 0, pairs = 0;
    if (lane == 0) {
        W.stack[0] = uint32_t(root);  // the root alone (a range of one)
        W.lvl[0] = 0;
    }
    __syncwarp();
    float2 ntx[kS], nty[kS], ntz[kS];
#pragma unroll
    for (int q = 0; q < kS; ++q) {
        ntx[q] = f2(-t[q].tx);
        nty[q] = f2(-t[q].ty);
        ntz[q] = f2(-t[q].tz);
    }
    auto flush_nodes = [&]() {
        pad_pair<Lay::kNodePair, kNodeFields>(sink.nbuf, ncount, lane, 3, 4, 9);
        sink.template nodes<kExact, kQuad, kSoft, kS>(ncount, t, eps2, a, lane);
        __syncwarp();
        ncount = 0;
    };
    auto flush_sources = [&]() {
        pad_pair<Lay::kSrcPair, kSrcFields>(sink.sbuf, scount, lane, 3, 32, 32);
        sink.template sources<kExact, kSoft, kS>(scount, t, eps2, a, lane);
        __syncwarp();
        scount = 0;
    };
    while (sp > 0) {
        // ---- pop the sibling ranges of the deepest level, at most 32 nodes; lane j takes node j
        // of their concatenation (the range holding it is the last one starting at or before j)
        const int avail = sp - W.lvl[dtop];
        const int nr = avail < 32 ? avail : 32;
        const uint32_t e = lane < nr ? W.stack[sp - 1 - lane] : 0u;
        const int c = lane < nr ? int(e >> 29) + 1 : 0;
        int incl = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(kFull, incl, o);
            if (lane >= o) incl += y;
        }
        const bool taken = lane < nr && incl <= 32;
        const int r = __popc(__ballot_sync(kFull, taken));
        const int total = __shfl_sync(kFull, incl, r - 1);
        const unsigned starts = __reduce_or_sync(kFull, taken ? 1u << (incl - c) : 0u);
        const int q = __popc(starts & upto) - 1;
        const int32_t qfirst = __shfl_sync(kFull, int32_t(e & 0x1fffffffu), q);
        const int qexcl = __shfl_sync(kFull, incl - c, q);
        sp -= r;
        const int depth = dtop;
        int32_t node = lane < total ? qfirst + (lane - qexcl) : -1;
        tested += uint32_t(total);
        // ---- test: the group's box, then (all lanes at once) every star for what the box keeps
        bool acc = false, bad = node >= nn, own = true;
        if constexpr (kSplit) {
            if (node >= 0 && !bad) {
                const int2 rg = ranges[node];
                if (rg.x >= s_hi || rg.y <= s_lo) node = -1;  // no star of this part below it
                else own = rg.x >= s_lo;
            }
        }
        float4 na = make_float4(0.f, 0.f, 0.f, 0.f), nb = na, nc = na, nd = na;
        float cx = 0.f, cy = 0.f, cz = 0.f, lim = 0.f;
        if (node >= 0 && !bad) {
            na = nodes[node].a;
            nb = nodes[node].b;
            if constexpr (kS == 2) {  // the whole record at once (measured faster with two stars a lane)
                nc = nodes[node].c;
                nd = nodes[node].d;
            }
            cx = (na.x - Ox) + nb.x;
            cy = (na.y - Oy) + nb.y;
            cz = (na.z - Oz) + nb.z;
            // Margin for FP32 rounding: every offset (node or star, from O) carries an error below
            // 2^-23 of its size, so accept only when the computed distance exceeds crit by sqrt(3)
            // 2^-22 (|c| + extent) and the squared distance its bound by 2^-21; crit itself (from
            // the FP32 moments) gets 2^-20 against the FP64 moments' value.
            const float slack = (fmaxf(fabsf(cx), fmaxf(fabsf(cy), fabsf(cz))) + ext) * 4.2e-7f;
            const float crit = fabsf(na.w);
            const float cr = fmaf(crit, 9.6e-7f, crit) + slack;
            lim = cr * cr * (1.f + 4.8e-7f);
            const float qx = fmaxf(0.f, fmaxf(bx0 - cx, cx - bx1));
            const float qy = fmaxf(0.f, fmaxf(by0 - cy, cy - by1));
            const float qz = fmaxf(0.f, fmaxf(bz0 - cz, cz - bz1));
            acc = qx * qx + qy * qy + qz * qz >= lim;
        }
        const unsigned mref = __ballot_sync(kFull, node >= 0 && !bad && !acc);
        if (mref) {
            // the box keeps these nodes: each lane tests its own stars against two of them at once
            // (packed FP32x2); stars beyond the group repeat the group's first star
            const int slot = __popc(mref & lt), nref = __popc(mref);
            if ((mref >> lane) & 1u) {
                float *rq = reinterpret_cast<float *>(&W.rq[0]) + (slot >> 1) * 8 + (slot & 1);
                rq[0] = cx;
                rq[2] = cy;
                rq[4] = cz;
                rq[6] = lim;
            }
            if ((nref & 1) && lane == 0) {  // pad the last pair with a copy of its first entry
                float *rq = reinterpret_cast<float *>(&W.rq[0]) + (nref >> 1) * 8;
                rq[1] = rq[0];
                rq[3] = rq[2];
                rq[5] = rq[4];
                rq[7] = rq[6];
            }
            __syncwarp();
            unsigned near = 0;
            for (int p = 0; p < nref; p += 2) {
                const float4 r0 = reinterpret_cast<const float4 *>(&W.rq[0])[p >> 1 << 1];
                const float4 r1 = reinterpret_cast<const float4 *>(&W.rq[0])[(p >> 1 << 1) + 1];
                const float2 ql = hi2(r1);
                bool nx = false, ny = false;
#pragma unroll
                for (int q = 0; q < kS; ++q) {
                    const float2 ex = add2(lo2(r0), ntx[q]), ey = add2(hi2(r0), nty[q]), ez = add2(lo2(r1), ntz[q]);
                    const float2 d2 = fma2(ez, ez, fma2(ey, ey, mul2(ex, ex)));
                    nx |= d2.x < ql.x;
                    ny |= d2.y < ql.y;
                }
                near |= (__any_sync(kFull, nx) ? 1u : 0u) << p;
                near |= (__any_sync(kFull, ny) ? 1u : 0u) << (p + 1);
            }
            __syncwarp();
            if ((mref >> lane) & 1u) acc = !((near >> slot) & 1u);
        }
        const uint32_t link = __float_as_uint(nb.w);
        const bool open_in = node >= 0 && !bad && !acc && !(na.w < 0.f);
        const bool open_leaf = node >= 0 && !bad && !acc && na.w < 0.f;
        if (open_in) bad = int64_t(link & 0x1fffffffu) + int64_t(link >> 29) + 1 > nn;
        const unsigned mi = __ballot_sync(kFull, open_in);
        const int npush = __popc(mi);
        if (__any_sync(kFull, bad) || tested > uint32_t(nn) + 32u || sp + npush > kStackCap ||
            (npush && depth + 1 >= kLevels)) {
            if (lane == 0) set_err(err_info, 8);  // a corrupt tree: stop this group
            return GroupOut{0, false};
        }
        // ---- push the children of opened inner nodes (one level deeper); the link is the range
        if (npush) {
            if (open_in) W.stack[sp + __popc(mi & lt)] = uint32_t(link);
            if (lane == 0) W.lvl[depth + 1] = sp;
            sp += npush;
            dtop = depth + 1;
        }
        __syncwarp();
        if (!npush) {
            while (dtop > 0 && W.lvl[dtop] >= sp) --dtop;
        }
        // ---- append accepted nodes to the node list (a part: the nodes whose first star is its own)
        const bool add = kSplit ? acc && own : acc;
        const unsigned ma = __ballot_sync(kFull, add);
        if (ma) {
            if (add) {
                const int en = ncount + __popc(ma & lt);
                const float4 qc = kS == 2 ? nc : nodes[node].c, qd = kS == 2 ? nd : nodes[node].d;
                constexpr int P = Lay::kNodePair;
                if constexpr (kExact) {
                    put(sink.nbuf, P, en, 0, na.x);
                    put(sink.nbuf, P, en, 1, na.y);
                    put(sink.nbuf, P, en, 2, na.z);
                    put(sink.nbuf, P, en, 10, nb.x);
                    put(sink.nbuf, P, en, 11, nb.y);
                    put(sink.nbuf, P, en, 12, nb.z);
                } else {
                    put(sink.nbuf, P, en, 0, cx);
                    put(sink.nbuf, P, en, 1, cy);
                    put(sink.nbuf, P, en, 2, cz);
                }
                if constexpr (Sink::kIndices) sink.nidx[en] = node;
                put(sink.nbuf, P, en, 3, qd.z);  // m
                put(sink.nbuf, P, en, 4, qc.x);  // -qxx
                put(sink.nbuf, P, en, 5, qc.y);  // -qyy
                put(sink.nbuf, P, en, 6, qc.z);  // -qzz
                put(sink.nbuf, P, en, 7, qc.w);  // -qxy
                put(sink.nbuf, P, en, 8, qd.x);  // -qxz
                put(sink.nbuf, P, en, 9, qd.y);  // -qyz
            }
            const int nacc = __popc(ma);
            ncount += nacc;
            acc_nodes += uint32_t(nacc);
            __syncwarp();
            if (ncount >= node_depth) flush_nodes();
        }
        // ---- stage the stars of opened leaves into the source list, 32 at a time
        const unsigned ml = __ballot_sync(kFull, open_leaf);
        if (ml) {
            int lo = open_leaf ? int(link) : 0;
            int hi = open_leaf ? __float_as_int(kS == 2 ? nd.w : nodes[node].d.w) : 0;
            if (__any_sync(kFull, open_leaf && (lo < 0 || hi > ns || lo >= hi))) {
                if (lane == 0) set_err(err_info, 8);
                return GroupOut{0, false};
            }
            if constexpr (kSplit) {  // the part's own stars of the leaf (at least one: it reaches in)
                if (open_leaf) {
                    lo = lo > s_lo ? lo : s_lo;
                    hi = hi < s_hi ? hi : s_hi;
                    if (hi < lo) hi = lo;  // only a record that disagrees with its range: no stars
                }
            }
            const int lc = hi - lo;
            int inc = lc;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(kFull, inc, o);
                if (lane >= o) inc += y;
            }
            const int excl = inc - lc;
            const int T = __shfl_sync(kFull, inc, 31);
            pairs += uint32_t(T);
            for (int cs = 0; cs < T; cs += 32) {
                // slot cs + j belongs to the last leaf whose (clipped) run starts at or before it
                const bool mine = open_leaf && excl < cs + 32 && excl + lc > cs;
                const int p0 = excl > cs ? excl - cs : 0;
                if (mine) W.owner[p0] = lane;
                const unsigned st = __reduce_or_sync(kFull, mine ? 1u << p0 : 0u);
                __syncwarp();
                const int j = cs + lane;
                const int ow = j < T ? W.owner[31 - __clz(st & upto)] : 0;
                const int olo = __shfl_sync(kFull, lo, ow), oex = __shfl_sync(kFull, excl, ow);
                if (j < T) {
                    const int32_t star = olo + (j - oex);
                    const float4 h = st_hi[star], l = st_lo[star];
                    const int en = scount + lane;
                    constexpr int P = Lay::kSrcPair;
                    if constexpr (kExact) {
                        put(sink.sbuf, P, en, 0, h.x);
                        put(sink.sbuf, P, en, 1, h.y);
                        put(sink.sbuf, P, en, 2, h.z);
                        put(sink.sbuf, P, en, 4, l.x);
                        put(sink.sbuf, P, en, 5, l.y);
                        put(sink.sbuf, P, en, 6, l.z);
                    } else {
                        put(sink.sbuf, P, en, 0, (h.x - Ox) + l.x);
                        put(sink.sbuf, P, en, 1, (h.y - Oy) + l.y);
                        put(sink.sbuf, P, en, 2, (h.z - Oz) + l.z);
                    }
                    put(sink.sbuf, P, en, 3, h.w);
                    if constexpr (Sink::kIndices) sink.sidx[en] = star;
                }
                scount += T - cs < 32 ? T - cs : 32;
                __syncwarp();
                if (scount >= src_depth) flush_sources();
            }
        }
    }
    if (ncount) flush_nodes();
    if (scount) flush_sources();
    return GroupOut{(31u * acc_nodes + 12u * pairs) * uint32_t(kS) / 16u + tested, true};
}

// A group's range of list entries or stars (forest: its table entry; else groups of kG).
struct GroupRange {
    int32_t base, cnt, root;
};
template <int kG>
__device__ __forceinline__ GroupRange group_range(int32_t g, const int4 *__restrict__ groups, int32_t nt) {
    GroupRange r;
    if (groups) {
        const int4 ge = groups[g];
        r.base = ge.x;
        r.cnt = ge.y;
        r.root = ge.z;
    } else {
        r.base = g * kG;
        r.cnt = nt - r.base < kG ? nt - r.base : kG;
        r.root = 0;
    }
    if (r.cnt > kG) r.cnt = kG;
    return r;
}

// The lane's stars of a group (star 32 q + lane; one beyond the group repeats the group's first
// star), their offsets from the group origin O (the first star's hi part) and hi/lo parts.
template <int kS>
struct GroupStars {
    bool valid[kS];
    int32_t k[kS];
    Target t[kS];
    float Ox, Oy, Oz;
};
template <int kS>
__device__ __forceinline__ void group_stars(int lane, const GroupRange &R, const int32_t *__restrict__ targets,
                                            const float4 *__restrict__ st_hi, const float4 *__restrict__ st_lo,
                                            GroupStars<kS> &G) {
    float4 h[kS], l[kS];
#pragma unroll
    for (int q = 0; q < kS; ++q) {
        G.valid[q] = 32 * q + lane < R.cnt;
        const int32_t e = R.base + (G.valid[q] ? 32 * q + lane : 0);
        G.k[q] = targets ? targets[e] : e;
        h[q] = st_hi[G.k[q]];
        l[q] = st_lo[G.k[q]];
    }
    G.Ox = __shfl_sync(kFull, h[0].x, 0);
    G.Oy = __shfl_sync(kFull, h[0].y, 0);
    G.Oz = __shfl_sync(kFull, h[0].z, 0);
#pragma unroll
    for (int q = 0; q < kS; ++q) {
        G.t[q].tx = (h[q].x - G.Ox) + l[q].x;
        G.t[q].ty = (h[q].y - G.Oy) + l[q].y;
        G.t[q].tz = (h[q].z - G.Oz) + l[q].z;
        G.t[q].hx = h[q].x;
        G.t[q].hy = h[q].y;
        G.t[q].hz = h[q].z;
        G.t[q].lx = l[q].x;
        G.t[q].ly = l[q].y;
        G.t[q].lz = l[q].z;
    }
}

// The group's box, its extent from the origin, and whether its separations take hi and lo parts
// apart: offsets from O carry rounding errors of 2^-24 of the group's extent, so separations
// formed from them stay accurate while the extent is within 2^12 of the softening or of the
// closest consecutive stars (star 32 q + lane is followed by the next lane's, or lane 0's next
// star); beyond that (a group across a jump of the Morton curve) they take hi and lo apart.
struct GroupBox {
    float bx0, by0, bz0, bx1, by1, bz1, ext;
    bool exact;
};
template <int kS>
__device__ __forceinline__ GroupBox group_box(int lane, int32_t cnt, const Target (&t)[kS], float eps) {
    GroupBox B;
    B.bx0 = B.bx1 = t[0].tx;
    B.by0 = B.by1 = t[0].ty;
    B.bz0 = B.bz1 = t[0].tz;
    float gap = 3.0e38f;
#pragma unroll
    for (int q = 0; q < kS; ++q) {
        B.bx0 = fminf(B.bx0, t[q].tx);
        B.by0 = fminf(B.by0, t[q].ty);
        B.bz0 = fminf(B.bz0, t[q].tz);
        B.bx1 = fmaxf(B.bx1, t[q].tx);
        B.by1 = fmaxf(B.by1, t[q].ty);
        B.bz1 = fmaxf(B.bz1, t[q].tz);
        float nx = __shfl_down_sync(kFull, t[q].tx, 1), ny = __shfl_down_sync(kFull, t[q].ty, 1),
              nz = __shfl_down_sync(kFull, t[q].tz, 1);
        if (q + 1 < kS) {
            const float wx = __shfl_sync(kFull, t[q + 1 < kS ? q + 1 : q].tx, 0);
            const float wy = __shfl_sync(kFull, t[q + 1 < kS ? q + 1 : q].ty, 0);
            const float wz = __shfl_sync(kFull, t[q + 1 < kS ? q + 1 : q].tz, 0);
            if (lane == 31) {
                nx = wx;
                ny = wy;
                nz = wz;
            }
        }
        if (32 * q + lane + 1 < cnt)
            gap = fminf(gap, fmaxf(fabsf(nx - t[q].tx), fmaxf(fabsf(ny - t[q].ty), fabsf(nz - t[q].tz))));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        B.bx0 = fminf(B.bx0, __shfl_xor_sync(kFull, B.bx0, o));
        B.by0 = fminf(B.by0, __shfl_xor_sync(kFull, B.by0, o));
        B.bz0 = fminf(B.bz0, __shfl_xor_sync(kFull, B.bz0, o));
        B.bx1 = fmaxf(B.bx1, __shfl_xor_sync(kFull, B.bx1, o));
        B.by1 = fmaxf(B.by1, __shfl_xor_sync(kFull, B.by1, o));
        B.bz1 = fmaxf(B.bz1, __shfl_xor_sync(kFull, B.bz1, o));
        gap = fminf(gap, __shfl_xor_sync(kFull, gap, o));
    }
    B.ext = fmaxf(fmaxf(fmaxf(-B.bx0, B.bx1), fmaxf(-B.by0, B.by1)), fmaxf(-B.bz0, B.bz1));
    B.exact = B.ext > 4096.f * fmaxf(eps, gap);
    return B;
}

template <int kS>
__device__ __forceinline__ void zero_acc(Acc (&a)[kS]) {
#pragma unroll
    for (int q = 0; q < kS; ++q) {
        a[q].px = a[q].py = a[q].pz = f2(0.f);
        a[q].sx = a[q].sy = a[q].sz = a[q].cx = a[q].cy = a[q].cz = 0.f;
    }
}

template <int kS>
__device__ __forceinline__ void store_acc(const GroupStars<kS> &G, const Acc (&a)[kS], const int32_t *__restrict__ order,
                                          double *ax, double *ay, double *az) {
#pragma unroll
    for (int q = 0; q < kS; ++q) {
        if (G.valid[q]) {
            const int32_t o = order[G.k[q]];
            ax[o] = double(a[q].sx) - double(a[q].cx);
            ay[o] = double(a[q].sy) - double(a[q].cy);
            az[o] = double(a[q].sz) - double(a[q].cz);
        }
    }
}

// kSplit: work item i walks part i % nparts of group i / nparts (walk_group's split mode) and
// writes its sums by sorted index to part_acc[part][axis][star]; k_split_combine adds the parts.
template <bool kQuad, bool kSoft, int kS, bool kSplit = false>
__global__ __launch_bounds__(kLwThreads) void k_walk_lists(const DevInfo *info, const LNode *__restrict__ nodes,
                                                           const float4 *__restrict__ st_hi,
                                                           const float4 *__restrict__ st_lo,
                                                           const int32_t *__restrict__ order, float eps, float eps2,
                                                           double *ax, double *ay, double *az,
                                                           const int4 *__restrict__ groups,
                                                           const int32_t *__restrict__ targets,
                                                           const int32_t *__restrict__ gperm, int32_t perm_cap,
                                                           uint32_t *gcost, uint32_t *work_ctr, DevInfo *err_info,
                                                           int node_depth, int src_depth, int nparts = 1,
                                                           double *part_acc = nullptr, int64_t part_stride = 0,
                                                           const int2 *__restrict__ ranges = nullptr) {
    constexpr int kG = 32 * kS;  // stars per group: lane l holds stars l, 32 + l, ...
    __shared__ WarpMem smem[kLwWarps];
    WarpMem &W = smem[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    const int32_t ns = int32_t(info->nstars);
    const int32_t nn = int32_t(info->nnodes);
    // a target list (block steps): groups of kG consecutive entries; else every star
    const int32_t nt = targets ? int32_t(info->ntargets) : ns;
    const int32_t ng = nn > 0 ? (groups ? int32_t(info->ngroups) : (nt + kG - 1) / kG) : 0;
    const bool lpt = !kSplit && gperm && gperm[perm_cap] == ng;
    const int32_t items = kSplit ? ng * nparts : ng;
    for (;;) {
        int32_t idx = 0;
        if (lane == 0) idx = int32_t(atomicAdd(work_ctr, 1u));
        idx = __shfl_sync(kFull, idx, 0);
        if (idx >= items) break;
        const int part = kSplit ? idx % nparts : 0;
        if constexpr (kSplit) idx /= nparts;
        const int32_t g = lpt ? gperm[idx] : idx;
        const int32_t s_lo = kSplit ? int32_t(int64_t(ns) * part / nparts) : 0;
        const int32_t s_hi = kSplit ? int32_t(int64_t(ns) * (part + 1) / nparts) : ns;
        const GroupRange R = group_range<kG>(g, groups, nt);
        if (R.cnt <= 0) continue;
        GroupStars<kS> G;
        group_stars<kS>(lane, R, targets, st_hi, st_lo, G);
        const GroupBox B = group_box<kS>(lane, R.cnt, G.t, eps);
        __syncwarp();
        Acc a[kS];
        zero_acc<kS>(a);
        GroupOut r;
        InPlace sink{W.nbuf, W.sbuf, nullptr, nullptr};
        if (B.exact)
            r = walk_group<true, kQuad, kSoft, kS, kSplit>(W.tm, sink, lane, R.root, G.t, G.Ox, G.Oy, G.Oz, B.bx0,
                                                            B.by0, B.bz0, B.bx1, B.by1, B.bz1, B.ext, eps2, node_depth,
                                                            src_depth, nodes, st_hi, st_lo, nn, ns, err_info, a,
                                                            ranges, s_lo, s_hi);
        else
            r = walk_group<false, kQuad, kSoft, kS, kSplit>(W.tm, sink, lane, R.root, G.t, G.Ox, G.Oy, G.Oz, B.bx0,
                                                             B.by0, B.bz0, B.bx1, B.by1, B.bz1, B.ext, eps2, node_depth,
                                                             src_depth, nodes, st_hi, st_lo, nn, ns, err_info, a,
                                                             ranges, s_lo, s_hi);
        __syncwarp();
        if (!r.ok) break;  // the error flag is set; the host reports GBH_ERR_LIMIT
        if constexpr (kSplit) {  // the part's sums by sorted index
            double *q = part_acc + int64_t(part) * 3 * part_stride;
#pragma unroll
            for (int u = 0; u < kS; ++u)
                if (G.valid[u]) {
                    q[G.k[u]] = double(a[u].sx) - double(a[u].cx);
                    q[part_stride + G.k[u]] = double(a[u].sy) - double(a[u].cy);
                    q[2 * part_stride + G.k[u]] = double(a[u].sz) - double(a[u].cz);
                }
            continue;
        }
        if (gcost && lane == 0) gcost[g] = r.cost;
        store_acc<kS>(G, a, order, ax, ay, az);
    }
}

template <bool kQuad, bool kSoft, int kS, bool kSplit>
static int lists_blocks_per_sm() {
    static int blocks_per_sm = 0;  // per instantiation; the same on every device of this architecture
    if (!blocks_per_sm) {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, k_walk_lists<kQuad, kSoft, kS, kSplit>,
                                                          kLwThreads, 0) != cudaSuccess)
            return 0;
        if (blocks_per_sm < 1) blocks_per_sm = 1;
    }
    return blocks_per_sm;
}

template <bool kQuad, bool kSoft, int kS>
cudaError_t launch_lists(const Launch &L, const TreeBufs &b, int64_t nstars_cap, float eps2, double *ax, double *ay,
                         double *az, int node_depth, int src_depth, bool lpt, bool targets, bool &split) {
    const bool forest = b.nsys > 1;
    cudaError_t e = cudaMemsetAsync(b.walk_ctr, 0, sizeof(uint32_t), L.stream);
    if (e != cudaSuccess) return e;
    const int sms = L.num_sms > 0 ? L.num_sms : 152;
    if constexpr (kQuad && kSoft) {
        // few groups: each group's walk shared among several warps (the same part count rule as
        // the paired walk's split mode, by the stars the walk takes)
        const int parts = split_parts(b, nstars_cap, targets, 32 * kS);
        split = parts > 1;
        if (split) {
            const int bps = lists_blocks_per_sm<kQuad, kSoft, kS, true>();
            if (!bps) return cudaErrorUnknown;
            k_walk_lists<kQuad, kSoft, kS, true><<<unsigned(sms * bps), kLwThreads, 0, L.stream>>>(
                b.info, b.lnode, b.st_hi, b.st_lo, b.order, sqrtf(eps2), eps2, ax, ay, az, nullptr,
                targets ? b.targets : nullptr, nullptr, int32_t(b.cap_groups), nullptr, b.walk_ctr, b.info,
                node_depth, src_depth, parts, b.part_acc, nstars_cap, b.mrange);
            ++*L.count;
            if ((e = cudaGetLastError()) != cudaSuccess) return e;
            return split_combine(L, b, parts, nstars_cap, targets, ax, ay, az);
        }
    }
    const int bps = lists_blocks_per_sm<kQuad, kSoft, kS, false>();
    if (!bps) return cudaErrorUnknown;
    k_walk_lists<kQuad, kSoft, kS><<<unsigned(sms * bps), kLwThreads, 0, L.stream>>>(
        b.info, b.lnode, b.st_hi, b.st_lo, b.order, sqrtf(eps2), eps2, ax, ay, az,
        forest ? b.groups : nullptr, targets ? b.targets : nullptr, lpt ? b.gperm : nullptr, int32_t(b.cap_groups),
        lpt ? b.gcost : nullptr,
        b.walk_ctr, b.info, node_depth, src_depth);
    ++*L.count;
    return cudaGetLastError();
}

template <int kS>
cudaError_t walk_lists_s(const Launch &L, const TreeBufs &b, int64_t nstars_cap, float eps2, int quad, double *ax,
                         double *ay, double *az, int nd, int sd, bool lpt, bool targets) {
    const bool soft = eps2 > 0.f;
    cudaError_t e;
    bool split = false;
    if (quad && soft) e = launch_lists<true, true, kS>(L, b, nstars_cap, eps2, ax, ay, az, nd, sd, lpt, targets, split);
    else if (quad) e = launch_lists<true, false, kS>(L, b, nstars_cap, eps2, ax, ay, az, nd, sd, lpt, targets, split);
    else if (soft) e = launch_lists<false, true, kS>(L, b, nstars_cap, eps2, ax, ay, az, nd, sd, lpt, targets, split);
    else e = launch_lists<false, false, kS>(L, b, nstars_cap, eps2, ax, ay, az, nd, sd, lpt, targets, split);
    if (e != cudaSuccess || !lpt || split) return e;  // a split walk records no group costs
    return lpt_order(L, b, 32 * kS);
}

// ---------------------------------------------------------------- adjoint of the list walk
//
// The transposed Jacobian of the list walk's force with its interaction lists frozen (the lists
// the forward walk builds at the same positions: the same traversal runs again). Target star i
// with weight w_i (the adjoint of its velocity) and separation d = source - x_i, r^2 = |d|^2 + eps^2:
//   accepted node n (quadrupole, bh.go:117-133): a = f d - Q d / r^5, f = m / r^3 + 5/2 (d.Q.d) / r^7,
//     J = da/dd = f I + d (grad f)^T - Q / r^5 + 5 (Q d) d^T / r^7 (symmetric),
//     grad f = -3 m d / r^5 + 5 Q d / r^7 - 35/2 (d.Q.d) d / r^9;
//     star i gets -J w_i; the node's centre of mass +J w_i, its mass (d.w_i) / r^3, and each stored
//     quadrupole component its derivative of w_i.a;
//   leaf star j (softened pair, bh.go:145-150): K = I / r^3 - 3 d d^T / r^5, star i gets -m_j K w_i,
//     star j gets +m_j K w_i and (d.w_i) / r^3 on its mass; a star paired with itself adds nothing.
// Each warp sums a list entry's source terms over its 32 stars (a reduce-scatter: lane l ends
// with term l) and adds them to the node's or star's FP64 accumulators with atomics.

constexpr int kAdjNodeTerms = 10;  // centre of mass (3), mass, Q xx yy zz xy xz yz
constexpr int kAdjStarTerms = 4;   // position (3), mass

struct AdjAcc {
    float wx, wy, wz;     // the lane's star's weight
    int32_t k;            // its sorted index (a star's pair with itself is skipped)
    double gx, gy, gz;    // its own terms, summed over the flushed lists
};

// Sums v[0..31] over the warp; afterwards lane l holds the sum of term l in v[0].
__device__ __forceinline__ void reduce_scatter32(float (&v)[32], int lane) {
#pragma unroll
    for (int sft = 16; sft >= 1; sft >>= 1) {
        const bool up = (lane & sft) != 0;
#pragma unroll
        for (int i = 0; i < sft; ++i) {
            const float send = up ? v[i] : v[i + sft];
            const float keep = up ? v[i + sft] : v[i];
            v[i] = keep + __shfl_xor_sync(kFull, send, sft);
        }
    }
}
// The same for 8 terms: full sums over the two upper lane bits, then a scatter over the lower
// three (lane l < 8 ends with term l).
__device__ __forceinline__ void reduce_scatter8(float (&v)[8], int lane) {
#pragma unroll
    for (int sft = 16; sft >= 8; sft >>= 1)
#pragma unroll
        for (int i = 0; i < 8; ++i) v[i] += __shfl_xor_sync(kFull, v[i], sft);
#pragma unroll
    for (int sft = 4; sft >= 1; sft >>= 1) {
        const bool up = (lane & sft) != 0;
#pragma unroll
        for (int i = 0; i < sft; ++i) {
            const float send = up ? v[i] : v[i + sft];
            const float keep = up ? v[i + sft] : v[i];
            v[i] = keep + __shfl_xor_sync(kFull, send, sft);
        }
    }
}

struct AdjSink {
    static constexpr bool kIndices = true;
    float4 *nbuf, *sbuf;
    int32_t *nidx, *sidx;
    double *nadj;  // [node][kAdjNodeTerms]
    double *sadj;  // [sorted star][kAdjStarTerms]

    // With kS stars a lane, each lane adds its stars' source terms before the reduce-scatter, so
    // its shuffles serve 32 kS stars (with one star the sums are the terms themselves, bit for bit).
    template <bool kExact, bool kQuad, bool kSoft, int kS>
    __device__ __forceinline__ void nodes(int count, const Target (&tt)[kS], float eps2, AdjAcc (&aa)[kS],
                                          int lane) {
        static_assert(kQuad && kSoft, "the adjoint walk: quadrupoles, softening");
        using Lay = Layout<kExact>;
        const float2 e2 = f2(eps2);
        float2 gx[kS], gy[kS], gz[kS];
#pragma unroll
        for (int q = 0; q < kS; ++q) gx[q] = gy[q] = gz[q] = f2(0.f);
        const int np = (count + 1) >> 1;
        for (int p = 0; p < np; ++p) {
            const float4 *r = &nbuf[p * Lay::kNodePair];
            const float4 r0 = r[0], r1 = r[1], r2a = r[2], r3 = r[3], r4 = r[4];
            float2 lx = f2(0.f), ly = f2(0.f), lz = f2(0.f);
            if constexpr (kExact) {
                const float4 r5 = r[5], r6 = r[6];
                lx = lo2(r5);
                ly = hi2(r5);
                lz = lo2(r6);
            }
            const float2 m = hi2(r1);
            // the record holds -Q: n = -Q
            const float2 nxx = lo2(r2a), nyy = hi2(r2a), nzz = lo2(r3), nxy = hi2(r3), nxz = lo2(r4), nyz = hi2(r4);
            float v[32];
#pragma unroll
            for (int i = 0; i < 32; ++i) v[i] = 0.f;
#pragma unroll
            for (int q = 0; q < kS; ++q) {
                const Target &t = tt[q];
                const float2 wx = f2(aa[q].wx), wy = f2(aa[q].wy), wz = f2(aa[q].wz);
                const float2 dx = sep<kExact>(lo2(r0), lx, -t.tx, -t.hx, -t.lx);
                const float2 dy = sep<kExact>(hi2(r0), ly, -t.ty, -t.hy, -t.ly);
                const float2 dz = sep<kExact>(lo2(r1), lz, -t.tz, -t.hz, -t.lz);
                const float2 rr = fma2(dz, dz, fma2(dy, dy, fma2(dx, dx, e2)));
                const float2 ir = make_float2(rsqrtf(rr.x), rsqrtf(rr.y));
                const float2 ir2 = mul2(ir, ir), ir3 = mul2(ir2, ir), ir5 = mul2(ir3, ir2), ir7 = mul2(ir5, ir2),
                             ir9 = mul2(ir7, ir2);
                const float2 qx = fma2(nxz, dz, fma2(nxy, dy, mul2(nxx, dx)));  // -(Q d)
                const float2 qy = fma2(nyz, dz, fma2(nyy, dy, mul2(nxy, dx)));
                const float2 qz = fma2(nzz, dz, fma2(nyz, dy, mul2(nxz, dx)));
                const float2 dqd = fma2(dz, qz, fma2(dy, qy, mul2(dx, qx)));      // -(d.Q.d)
                const float2 dw = fma2(dz, wz, fma2(dy, wy, mul2(dx, wx)));
                const float2 qw = fma2(qz, wz, fma2(qy, wy, mul2(qx, wx)));       // -(Q d . w)
                const float2 nwx = fma2(nxz, wz, fma2(nxy, wy, mul2(nxx, wx)));   // -(Q w)
                const float2 nwy = fma2(nyz, wz, fma2(nyy, wy, mul2(nxy, wx)));
                const float2 nwz = fma2(nzz, wz, fma2(nyz, wy, mul2(nxz, wx)));
                const float2 f = fma2(mul2(dqd, ir7), f2(-2.5f), mul2(m, ir3));
                // grad f . w = -3 m dw / r^5 - 5 (-(Qd.w)) / r^7 + 17.5 (-(dQd)) dw / r^9
                const float2 gw = fma2(mul2(mul2(dqd, ir9), dw), f2(17.5f),
                                       fma2(mul2(qw, ir7), f2(-5.f), mul2(mul2(m, ir5), mul2(dw, f2(-3.f)))));
                const float2 c5 = mul2(mul2(ir7, dw), f2(-5.f));  // -5 dw / r^7, times -(Q d)
                const float2 jx = fma2(c5, qx, fma2(ir5, nwx, fma2(dx, gw, mul2(f, wx))));
                const float2 jy = fma2(c5, qy, fma2(ir5, nwy, fma2(dy, gw, mul2(f, wy))));
                const float2 jz = fma2(c5, qz, fma2(ir5, nwz, fma2(dz, gw, mul2(f, wz))));
                gx[q] = add2(gx[q], jx);
                gy[q] = add2(gy[q], jy);
                gz[q] = add2(gz[q], jz);
                // d(w.a)/dQ: xx: 5/2 dw dx^2 / r^7 - wx dx / r^5; xy: 5 dw dx dy / r^7 - (wx dy + wy dx) / r^5
                const float2 qa = mul2(mul2(ir7, dw), f2(2.5f));
                const float2 Gxx = fma2(mul2(qa, dx), dx, mul2(mul2(ir5, wx), mul2(dx, f2(-1.f))));
                const float2 Gyy = fma2(mul2(qa, dy), dy, mul2(mul2(ir5, wy), mul2(dy, f2(-1.f))));
                const float2 Gzz = fma2(mul2(qa, dz), dz, mul2(mul2(ir5, wz), mul2(dz, f2(-1.f))));
                const float2 qa2 = add2(qa, qa);
                const float2 Gxy = fma2(mul2(qa2, dx), dy, mul2(ir5, mul2(fma2(wx, dy, mul2(wy, dx)), f2(-1.f))));
                const float2 Gxz = fma2(mul2(qa2, dx), dz, mul2(ir5, mul2(fma2(wx, dz, mul2(wz, dx)), f2(-1.f))));
                const float2 Gyz = fma2(mul2(qa2, dy), dz, mul2(ir5, mul2(fma2(wy, dz, mul2(wz, dy)), f2(-1.f))));
                const float2 am = mul2(dw, ir3);
                const float2 term[10] = {jx, jy, jz, am, Gxx, Gyy, Gzz, Gxy, Gxz, Gyz};
#pragma unroll
                for (int i = 0; i < kAdjNodeTerms; ++i) {
                    v[i] += term[i].x;
                    v[kAdjNodeTerms + i] += term[i].y;
                }
            }
            const bool hasB = 2 * p + 1 < count;  // the padded last entry is no node
            reduce_scatter32(v, lane);
            if (lane < kAdjNodeTerms || (hasB && lane < 2 * kAdjNodeTerms)) {
                const int e = 2 * p + (lane >= kAdjNodeTerms ? 1 : 0);
                const int term = lane >= kAdjNodeTerms ? lane - kAdjNodeTerms : lane;
                atomicAdd(&nadj[int64_t(nidx[e]) * kAdjNodeTerms + term], double(v[0]));
            }
        }
#pragma unroll
        for (int q = 0; q < kS; ++q) {
            aa[q].gx -= double(gx[q].x) + double(gx[q].y);
            aa[q].gy -= double(gy[q].x) + double(gy[q].y);
            aa[q].gz -= double(gz[q].x) + double(gz[q].y);
        }
    }

    template <bool kExact, bool kSoft, int kS>
    __device__ __forceinline__ void sources(int count, const Target (&tt)[kS], float eps2, AdjAcc (&aa)[kS],
                                            int lane) {
        static_assert(kSoft, "the adjoint walk: softening");
        using Lay = Layout<kExact>;
        const float2 e2 = f2(eps2);
        float2 gx[kS], gy[kS], gz[kS];
#pragma unroll
        for (int q = 0; q < kS; ++q) gx[q] = gy[q] = gz[q] = f2(0.f);
        const int np = (count + 1) >> 1;
        for (int p = 0; p < np; ++p) {
            const float4 *r = &sbuf[p * Lay::kSrcPair];
            const float4 r0 = r[0], r1 = r[1];
            float2 lx = f2(0.f), ly = f2(0.f), lz = f2(0.f);
            if constexpr (kExact) {
                const float4 r2a = r[2], r3 = r[3];
                lx = lo2(r2a);
                ly = hi2(r2a);
                lz = lo2(r3);
            }
            const bool hasB = 2 * p + 1 < count;
            const int32_t sA = sidx[2 * p], sB = hasB ? sidx[2 * p + 1] : -1;
            float v[8];
#pragma unroll
            for (int i = 0; i < 8; ++i) v[i] = 0.f;
#pragma unroll
            for (int q = 0; q < kS; ++q) {
                const Target &t = tt[q];
                const float2 wx = f2(aa[q].wx), wy = f2(aa[q].wy), wz = f2(aa[q].wz);
                const float2 dx = sep<kExact>(lo2(r0), lx, -t.tx, -t.hx, -t.lx);
                const float2 dy = sep<kExact>(hi2(r0), ly, -t.ty, -t.hy, -t.ly);
                const float2 dz = sep<kExact>(lo2(r1), lz, -t.tz, -t.hz, -t.lz);
                const float2 rr = fma2(dz, dz, fma2(dy, dy, fma2(dx, dx, e2)));
                const float2 ir = make_float2(rsqrtf(rr.x), rsqrtf(rr.y));
                const float2 ir2 = mul2(ir, ir), ir3 = mul2(ir2, ir), ir5 = mul2(ir3, ir2);
                // a star and its own pair, and the padded last entry, contribute nothing
                const float keepA = sA == aa[q].k ? 0.f : 1.f;
                const float keepB = hasB && sB != aa[q].k ? 1.f : 0.f;
                const float2 m = mul2(hi2(r1), make_float2(keepA, keepB));
                const float2 dw = fma2(dz, wz, fma2(dy, wy, mul2(dx, wx)));
                // m K w = m (w / r^3 - 3 d dw / r^5)
                const float2 c3 = mul2(mul2(ir5, dw), f2(-3.f));
                const float2 kx = mul2(m, fma2(c3, dx, mul2(ir3, wx)));
                const float2 ky = mul2(m, fma2(c3, dy, mul2(ir3, wy)));
                const float2 kz = mul2(m, fma2(c3, dz, mul2(ir3, wz)));
                gx[q] = add2(gx[q], kx);
                gy[q] = add2(gy[q], ky);
                gz[q] = add2(gz[q], kz);
                const float2 am = mul2(mul2(dw, ir3), make_float2(keepA, keepB));
                v[0] += kx.x;
                v[1] += ky.x;
                v[2] += kz.x;
                v[3] += am.x;
                v[4] += kx.y;
                v[5] += ky.y;
                v[6] += kz.y;
                v[7] += am.y;
            }
            reduce_scatter8(v, lane);
            if (lane < kAdjStarTerms || (hasB && lane < 2 * kAdjStarTerms)) {
                const int e = 2 * p + (lane >= kAdjStarTerms ? 1 : 0);
                const int term = lane >= kAdjStarTerms ? lane - kAdjStarTerms : lane;
                atomicAdd(&sadj[int64_t(sidx[e]) * kAdjStarTerms + term], double(v[0]));
            }
        }
#pragma unroll
        for (int q = 0; q < kS; ++q) {
            aa[q].gx -= double(gx[q].x) + double(gx[q].y);
            aa[q].gy -= double(gy[q].x) + double(gy[q].y);
            aa[q].gz -= double(gz[q].x) + double(gz[q].y);
        }
    }
};

struct __align__(16) AdjWarpMem {
    float4 nbuf[kNodeF4];
    float4 sbuf[kSrcF4];
    int32_t nidx[Layout<false>::kNodeCap];
    int32_t sidx[Layout<false>::kSrcCap];
    TravMem tm;
};

// The adjoint walk over groups of 32 kS stars (the forward's groups in adjoint mode): the same
// traversal as k_walk_lists<quad, soft, kS, kSplit>, with the adjoint sink. w: the weights in
// state order (three arrays); tgt: each sorted star's own terms (3 doubles), or with kSplit each
// part's by sorted index in part_tgt (k_adj_part_combine adds the parts).
template <int kS, bool kSplit>
__global__ __launch_bounds__(kLwThreads) void k_walk_lists_adj(const DevInfo *info, const LNode *__restrict__ nodes,
                                                               const float4 *__restrict__ st_hi,
                                                               const float4 *__restrict__ st_lo,
                                                               const int32_t *__restrict__ order, float eps,
                                                               float eps2, const double *__restrict__ wx,
                                                               const double *__restrict__ wy,
                                                               const double *__restrict__ wz, double *tgt,
                                                               double *nadj, double *sadj, uint32_t *work_ctr,
                                                               DevInfo *err_info, int node_depth, int src_depth,
                                                               int nparts, double *part_tgt, int64_t part_stride,
                                                               const int2 *__restrict__ ranges) {
    constexpr int kG = 32 * kS;
    __shared__ AdjWarpMem smem[kLwWarps];
    AdjWarpMem &W = smem[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    const int32_t ns = int32_t(info->nstars);
    const int32_t nn = int32_t(info->nnodes);
    const int32_t ng = nn > 0 ? (ns + kG - 1) / kG : 0;
    const int32_t items = kSplit ? ng * nparts : ng;
    for (;;) {
        int32_t idx = 0;
        if (lane == 0) idx = int32_t(atomicAdd(work_ctr, 1u));
        idx = __shfl_sync(kFull, idx, 0);
        if (idx >= items) break;
        const int part = kSplit ? idx % nparts : 0;
        if constexpr (kSplit) idx /= nparts;
        const int32_t s_lo = kSplit ? int32_t(int64_t(ns) * part / nparts) : 0;
        const int32_t s_hi = kSplit ? int32_t(int64_t(ns) * (part + 1) / nparts) : ns;
        const GroupRange R = group_range<kG>(idx, nullptr, ns);
        if (R.cnt <= 0) continue;
        GroupStars<kS> G;
        group_stars<kS>(lane, R, nullptr, st_hi, st_lo, G);
        const GroupBox B = group_box<kS>(lane, R.cnt, G.t, eps);
        __syncwarp();
        AdjAcc a[kS];
#pragma unroll
        for (int q = 0; q < kS; ++q) {
            const int32_t o = order[G.k[q]];
            // a star beyond the group (a copy of the first star) weighs nothing: no source terms
            a[q].wx = G.valid[q] ? float(wx[o]) : 0.f;
            a[q].wy = G.valid[q] ? float(wy[o]) : 0.f;
            a[q].wz = G.valid[q] ? float(wz[o]) : 0.f;
            a[q].k = G.k[q];
            a[q].gx = a[q].gy = a[q].gz = 0.0;
        }
        AdjSink sink{W.nbuf, W.sbuf, W.nidx, W.sidx, nadj, sadj};
        GroupOut r;
        if (B.exact)
            r = walk_group<true, true, true, kS, kSplit>(W.tm, sink, lane, R.root, G.t, G.Ox, G.Oy, G.Oz, B.bx0, B.by0,
                                                         B.bz0, B.bx1, B.by1, B.bz1, B.ext, eps2, node_depth,
                                                         src_depth, nodes, st_hi, st_lo, nn, ns, err_info, a, ranges,
                                                         s_lo, s_hi);
        else
            r = walk_group<false, true, true, kS, kSplit>(W.tm, sink, lane, R.root, G.t, G.Ox, G.Oy, G.Oz, B.bx0,
                                                          B.by0, B.bz0, B.bx1, B.by1, B.bz1, B.ext, eps2, node_depth,
                                                          src_depth, nodes, st_hi, st_lo, nn, ns, err_info, a, ranges,
                                                          s_lo, s_hi);
        __syncwarp();
        if (!r.ok) break;
#pragma unroll
        for (int u = 0; u < kS; ++u) {
            if (!G.valid[u]) continue;
            if constexpr (kSplit) {  // the part's own terms by sorted index; k_adj_part_combine adds them
                double *q = part_tgt + int64_t(part) * 3 * part_stride;
                q[G.k[u]] = a[u].gx;
                q[part_stride + G.k[u]] = a[u].gy;
                q[2 * part_stride + G.k[u]] = a[u].gz;
            } else {
                tgt[3 * int64_t(G.k[u])] = a[u].gx;
                tgt[3 * int64_t(G.k[u]) + 1] = a[u].gy;
                tgt[3 * int64_t(G.k[u]) + 2] = a[u].gz;
            }
        }
    }
}

// A split adjoint walk's own terms of every star: the parts' sums in part order.
__global__ __launch_bounds__(256) void k_adj_part_combine(const DevInfo *info, int nparts,
                                                          const double *__restrict__ part_tgt, int64_t stride,
                                                          double *tgt) {
    const int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (k >= info->nstars) return;
    double x = 0, y = 0, z = 0;
    for (int p = 0; p < nparts; ++p) {
        const double *q = part_tgt + int64_t(p) * 3 * stride;
        x += q[k];
        y += q[stride + k];
        z += q[2 * stride + k];
    }
    tgt[3 * k] = x;
    tgt[3 * k + 1] = y;
    tgt[3 * k + 2] = z;
}

// ---- the tree potential with the list walk: psi_i = sum m / r + (d.Q.d) / (2 r^5) over the
// accepted nodes and the opened leaves' stars (walkPotential, potential.go:44-81), a star's pair
// with itself skipped by index (a coincident other star still counts, as in the reference)

struct PotAcc {
    float2 p;      // the current list's sums (entry A, entry B halves)
    float s, c;    // Kahan sum
    int32_t k;     // the star's sorted index
    __device__ __forceinline__ void fold() {
        kahan_fold(s, c, p.x + p.y);
        p = f2(0.f);
    }
};

struct PotSink {
    static constexpr bool kIndices = true;
    float4 *nbuf, *sbuf;
    int32_t *nidx, *sidx;

    template <bool kExact, bool kQuad, bool kSoft, int kS>
    __device__ __forceinline__ void nodes(int count, const Target (&t)[kS], float eps2, PotAcc (&a)[kS], int) {
        using Lay = Layout<kExact>;
        const float2 e2 = f2(eps2);
        const int np = (count + 1) >> 1;
        for (int p = 0; p < np; ++p) {
            const float4 *r = &nbuf[p * Lay::kNodePair];
            const float4 r0 = r[0], r1 = r[1];
            float2 lx = f2(0.f), ly = f2(0.f), lz = f2(0.f);
            if constexpr (kExact) {
                const float4 r5 = r[5], r6 = r[6];
                lx = lo2(r5);
                ly = hi2(r5);
                lz = lo2(r6);
            }
            float4 r2a, r3, r4;
            if constexpr (kQuad) {
                r2a = r[2];
                r3 = r[3];
                r4 = r[4];
            }
#pragma unroll
            for (int q = 0; q < kS; ++q) {
                const float2 dx = sep<kExact>(lo2(r0), lx, -t[q].tx, -t[q].hx, -t[q].lx);
                const float2 dy = sep<kExact>(hi2(r0), ly, -t[q].ty, -t[q].hy, -t[q].ly);
                const float2 dz = sep<kExact>(lo2(r1), lz, -t[q].tz, -t[q].hz, -t[q].lz);
                const float2 rr = fma2(dz, dz, fma2(dy, dy, fma2(dx, dx, e2)));
                float2 ir;
                if constexpr (kSoft) {
                    ir = make_float2(rsqrtf(rr.x), rsqrtf(rr.y));
                } else {
                    ir = make_float2(rr.x > 0.f ? rsqrtf(rr.x) : 0.f, rr.y > 0.f ? rsqrtf(rr.y) : 0.f);
                }
                float2 v = mul2(hi2(r1), ir);
                if constexpr (kQuad) {  // the record holds -Q: dqd = -(d.Q.d)
                    const float2 qx = fma2(lo2(r4), dz, fma2(hi2(r3), dy, mul2(lo2(r2a), dx)));
                    const float2 qy = fma2(hi2(r4), dz, fma2(hi2(r2a), dy, mul2(hi2(r3), dx)));
                    const float2 qz = fma2(lo2(r3), dz, fma2(hi2(r4), dy, mul2(lo2(r4), dx)));
                    const float2 dqd = fma2(dz, qz, fma2(dy, qy, mul2(dx, qx)));
                    const float2 ir2 = mul2(ir, ir);
                    v = fma2(mul2(f2(-0.5f), dqd), mul2(mul2(ir2, ir), ir2), v);
                }
                a[q].p = add2(a[q].p, v);
            }
        }
#pragma unroll
        for (int q = 0; q < kS; ++q) a[q].fold();
    }

    template <bool kExact, bool kSoft, int kS>
    __device__ __forceinline__ void sources(int count, const Target (&t)[kS], float eps2, PotAcc (&a)[kS], int) {
        using Lay = Layout<kExact>;
        const float2 e2 = f2(eps2);
        const int np = (count + 1) >> 1;
        for (int p = 0; p < np; ++p) {
            const float4 *r = &sbuf[p * Lay::kSrcPair];
            const float4 r0 = r[0], r1 = r[1];
            float2 lx = f2(0.f), ly = f2(0.f), lz = f2(0.f);
            if constexpr (kExact) {
                const float4 r2a = r[2], r3 = r[3];
                lx = lo2(r2a);
                ly = hi2(r2a);
                lz = lo2(r3);
            }
            const int32_t sA = sidx[2 * p], sB = 2 * p + 1 < count ? sidx[2 * p + 1] : -1;  // B: a zero-mass pad
#pragma unroll
            for (int q = 0; q < kS; ++q) {
                const float2 dx = sep<kExact>(lo2(r0), lx, -t[q].tx, -t[q].hx, -t[q].lx);
                const float2 dy = sep<kExact>(hi2(r0), ly, -t[q].ty, -t[q].hy, -t[q].ly);
                const float2 dz = sep<kExact>(lo2(r1), lz, -t[q].tz, -t[q].hz, -t[q].lz);
                const float2 rr = fma2(dz, dz, fma2(dy, dy, fma2(dx, dx, e2)));
                float2 ir;
                if constexpr (kSoft) {
                    ir = make_float2(rsqrtf(rr.x), rsqrtf(rr.y));
                } else {
                    ir = make_float2(rr.x > 0.f ? rsqrtf(rr.x) : 0.f, rr.y > 0.f ? rsqrtf(rr.y) : 0.f);
                }
                float2 v = mul2(hi2(r1), ir);
                v.x = sA == a[q].k ? 0.f : v.x;
                v.y = sB == a[q].k ? 0.f : v.y;
                a[q].p = add2(a[q].p, v);
            }
        }
#pragma unroll
        for (int q = 0; q < kS; ++q) a[q].fold();
    }
};

// psi of every star of a single system or forest (groups of 32 kS; forest groups from the build),
// by sorted index: the list walk's traversal with the potential sink.
template <bool kQuad, bool kSoft, int kS>
__global__ __launch_bounds__(kLwThreads) void k_walk_lists_pot(const DevInfo *info, const LNode *__restrict__ nodes,
                                                               const float4 *__restrict__ st_hi,
                                                               const float4 *__restrict__ st_lo, float eps, float eps2,
                                                               double *psi, const int4 *__restrict__ groups,
                                                               uint32_t *work_ctr, DevInfo *err_info, int node_depth,
                                                               int src_depth) {
    constexpr int kG = 32 * kS;
    __shared__ AdjWarpMem smem[kLwWarps];
    AdjWarpMem &W = smem[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    const int32_t ns = int32_t(info->nstars);
    const int32_t nn = int32_t(info->nnodes);
    const int32_t ng = nn > 0 ? (groups ? int32_t(info->ngroups) : (ns + kG - 1) / kG) : 0;
    for (;;) {
        int32_t idx = 0;
        if (lane == 0) idx = int32_t(atomicAdd(work_ctr, 1u));
        idx = __shfl_sync(kFull, idx, 0);
        if (idx >= ng) break;
        const GroupRange R = group_range<kG>(idx, groups, ns);
        if (R.cnt <= 0) continue;
        GroupStars<kS> G;
        group_stars<kS>(lane, R, nullptr, st_hi, st_lo, G);
        const GroupBox B = group_box<kS>(lane, R.cnt, G.t, eps);
        __syncwarp();
        PotAcc a[kS];
#pragma unroll
        for (int q = 0; q < kS; ++q) {
            a[q].p = f2(0.f);
            a[q].s = a[q].c = 0.f;
            a[q].k = G.k[q];
        }
        PotSink sink{W.nbuf, W.sbuf, W.nidx, W.sidx};
        GroupOut r;
        if (B.exact)
            r = walk_group<true, kQuad, kSoft, kS>(W.tm, sink, lane, R.root, G.t, G.Ox, G.Oy, G.Oz, B.bx0, B.by0,
                                                    B.bz0, B.bx1, B.by1, B.bz1, B.ext, eps2, node_depth, src_depth,
                                                    nodes, st_hi, st_lo, nn, ns, err_info, a);
        else
            r = walk_group<false, kQuad, kSoft, kS>(W.tm, sink, lane, R.root, G.t, G.Ox, G.Oy, G.Oz, B.bx0, B.by0,
                                                     B.bz0, B.bx1, B.by1, B.bz1, B.ext, eps2, node_depth, src_depth,
                                                     nodes, st_hi, st_lo, nn, ns, err_info, a);
        __syncwarp();
        if (!r.ok) break;
#pragma unroll
        for (int q = 0; q < kS; ++q)
            if (G.valid[q]) psi[G.k[q]] = double(a[q].s) - double(a[q].c);
    }
}

// The leaf of every sorted star (from the leaves' star ranges in their list records).
__global__ void k_star_leaf(const DevInfo *info, const LNode *__restrict__ nodes, int32_t *star_leaf) {
    const int64_t r = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (r >= info->nnodes) return;
    const LNode nd = nodes[r];
    if (!(nd.a.w < 0.f)) return;  // inner node
    const int32_t lo = int32_t(__float_as_uint(nd.b.w)), hi = __float_as_int(nd.d.w);
    const int32_t ns = int32_t(info->nstars);
    for (int32_t j = lo < 0 ? 0 : lo; j < hi && j < ns; ++j) star_leaf[j] = int32_t(r);
}

// Per sorted star k: its own terms and its pair terms as a source, plus the chain rule through
// the moments of every node that holds it (its leaf and the leaf's ancestors):
//   com = sum m x / M:  x_k gets (m_k / M) A_c, m_k gets (x_k - com).A_c / M;  M: m_k gets A_m;
//   Q = sum m (3 e e^T - |e|^2 I), e = x - com (the com's own dependence drops out, sum m e = 0):
//   x_k gets m_k (dQ/de)^T G and m_k gets the Q of e_k contracted with G.
// Written in state order into out (x, y, z, m terms, n apart).
__global__ void k_adj_downsweep(const DevInfo *info, const LNode *__restrict__ nodes, const int32_t *__restrict__ parent,
                                const int32_t *__restrict__ star_leaf, const int32_t *__restrict__ order,
                                const double *__restrict__ px, const double *__restrict__ py,
                                const double *__restrict__ pz, const double *__restrict__ mass,
                                const double *__restrict__ tgt, const double *__restrict__ nadj,
                                const double *__restrict__ sadj, int64_t n, double *out, DevInfo *err_info) {
    const int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    const int64_t ns = info->nstars;
    if (k >= ns) return;
    const int32_t i = order[k];
    const double x = px[i], y = py[i], z = pz[i], mk = mass[i];
    double gx = tgt[3 * k] + sadj[4 * k], gy = tgt[3 * k + 1] + sadj[4 * k + 1], gz = tgt[3 * k + 2] + sadj[4 * k + 2];
    double gm = sadj[4 * k + 3];
    int32_t r = star_leaf[k];
    const int32_t nn = int32_t(info->nnodes);
    for (int guard = 0; r >= 0 && guard <= kMaxLevel + 1; ++guard) {
        if (r >= nn) {
            atomicExch(&err_info->err, 1);
            err_info->err_where = 24;
            break;
        }
        const LNode nd = nodes[r];
        const double M = double(nd.d.z);
        const double *A = nadj + int64_t(r) * kAdjNodeTerms;
        if (M > 0) {
            const double ex = x - (double(nd.a.x) + double(nd.b.x)), ey = y - (double(nd.a.y) + double(nd.b.y)),
                         ez = z - (double(nd.a.z) + double(nd.b.z));
            const double Gxx = A[4], Gyy = A[5], Gzz = A[6], Gxy = A[7], Gxz = A[8], Gyz = A[9];
            const double s = mk / M;
            gx += s * A[0] + mk * ((4 * Gxx - 2 * Gyy - 2 * Gzz) * ex + 3 * Gxy * ey + 3 * Gxz * ez);
            gy += s * A[1] + mk * ((4 * Gyy - 2 * Gxx - 2 * Gzz) * ey + 3 * Gxy * ex + 3 * Gyz * ez);
            gz += s * A[2] + mk * ((4 * Gzz - 2 * Gxx - 2 * Gyy) * ez + 3 * Gxz * ex + 3 * Gyz * ey);
            const double e2 = ex * ex + ey * ey + ez * ez;
            gm += A[3] + (ex * A[0] + ey * A[1] + ez * A[2]) / M + Gxx * (3 * ex * ex - e2) +
                  Gyy * (3 * ey * ey - e2) + Gzz * (3 * ez * ez - e2) + 3 * (Gxy * ex * ey + Gxz * ex * ez + Gyz * ey * ez);
        } else {
            gm += A[3];
        }
        r = parent[r];
    }
    out[i] = gx;
    out[n + i] = gy;
    out[2 * n + i] = gz;
    out[3 * n + i] = gm;
}

}  // namespace

int list_depth_max(bool exact) { return exact ? Layout<true>::kNodeCap - 32 : Layout<false>::kNodeCap - 32; }

cudaError_t walk_lists(const Launch &L, const TreeBufs &b, int64_t nstars_cap, float eps2, int quad, double *ax,
                       double *ay, double *az, int list_depth, bool targets, int stars_per_lane) {
    // The list depth is the node list's flush threshold (entries per lane and evaluation); the
    // source list flushes at twice it. Both are capped so that one step's appends always fit; an
    // exact-separation group uses the smaller of its own cap and the depth.
    int nd = list_depth > 0 ? list_depth : kDefaultListDepth;
    if (nd < 2) nd = 2;
    if (nd > Layout<false>::kNodeCap - 32) nd = Layout<false>::kNodeCap - 32;
    int sd = 2 * nd;
    if (sd > Layout<false>::kSrcCap - 32) sd = Layout<false>::kSrcCap - 32;
    const bool lpt = b.lpt && !targets;  // a target list changes from event to event
    if (stars_per_lane == 2) return walk_lists_s<2>(L, b, nstars_cap, eps2, quad, ax, ay, az, nd, sd, lpt, targets);
    return walk_lists_s<1>(L, b, nstars_cap, eps2, quad, ax, ay, az, nd, sd, lpt, targets);
}

template <bool kQuad>
static cudaError_t launch_pot(const Launch &L, const TreeBufs &b, float eps2, double *psi) {
    static int blocks_per_sm = 0;  // per instantiation
    cudaError_t e;
    if (!blocks_per_sm) {
        if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, k_walk_lists_pot<kQuad, true, 2>,
                                                               kLwThreads, 0)))
            return e;
        if (blocks_per_sm < 1) blocks_per_sm = 1;
    }
    if ((e = cudaMemsetAsync(b.walk_ctr, 0, sizeof(uint32_t), L.stream))) return e;
    const int sms = L.num_sms > 0 ? L.num_sms : 152;
    k_walk_lists_pot<kQuad, true, 2><<<unsigned(sms * blocks_per_sm), kLwThreads, 0, L.stream>>>(
        b.info, b.lnode, b.st_hi, b.st_lo, sqrtf(eps2), eps2, psi, b.nsys > 1 ? b.groups : nullptr, b.walk_ctr,
        b.info, kDefaultListDepth, 2 * kDefaultListDepth);
    ++*L.count;
    return cudaGetLastError();
}

cudaError_t walk_lists_potential(const Launch &L, const TreeBufs &b, float eps2, int quad, double *psi) {
    return quad ? launch_pot<true>(L, b, eps2, psi) : launch_pot<false>(L, b, eps2, psi);
}

template <int kS>
static cudaError_t launch_adj(const Launch &L, const TreeBufs &b, int64_t n, float eps2, const double *wx,
                              const double *wy, const double *wz, AdjTreeBufs &s) {
    const int parts = split_parts(b, n, false, 32 * kS);
    const int sms = L.num_sms > 0 ? L.num_sms : 152;
    const int nd = kDefaultListDepth, sd = 2 * kDefaultListDepth;
    cudaError_t e;
    if (parts > 1) {
        static int bps_split = 0;  // per instantiation
        if (!bps_split) {
            if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps_split, k_walk_lists_adj<kS, true>, kLwThreads,
                                                                   0)))
                return e;
            if (bps_split < 1) bps_split = 1;
        }
        k_walk_lists_adj<kS, true><<<unsigned(sms * bps_split), kLwThreads, 0, L.stream>>>(
            b.info, b.lnode, b.st_hi, b.st_lo, b.order, sqrtf(eps2), eps2, wx, wy, wz, s.tgt, s.nadj, s.sadj,
            b.walk_ctr, b.info, nd, sd, parts, b.part_acc, n, b.mrange);
        ++*L.count;
        if ((e = cudaGetLastError())) return e;
        k_adj_part_combine<<<unsigned((n + 255) / 256), 256, 0, L.stream>>>(b.info, parts, b.part_acc, n, s.tgt);
        ++*L.count;
        return cudaGetLastError();
    }
    static int blocks_per_sm = 0;  // per instantiation
    if (!blocks_per_sm) {
        if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, k_walk_lists_adj<kS, false>, kLwThreads,
                                                               0)))
            return e;
        if (blocks_per_sm < 1) blocks_per_sm = 1;
    }
    k_walk_lists_adj<kS, false><<<unsigned(sms * blocks_per_sm), kLwThreads, 0, L.stream>>>(
        b.info, b.lnode, b.st_hi, b.st_lo, b.order, sqrtf(eps2), eps2, wx, wy, wz, s.tgt, s.nadj, s.sadj, b.walk_ctr,
        b.info, nd, sd, 1, nullptr, 0, nullptr);
    ++*L.count;
    return cudaGetLastError();
}

cudaError_t walk_lists_adjoint(const Launch &L, const TreeBufs &b, float eps2, const double *px, const double *py,
                               const double *pz, const double *mass, const double *wx, const double *wy,
                               const double *wz, int64_t n, AdjTreeBufs &s, double *out) {
    cudaError_t e;
    if ((e = cudaMemsetAsync(s.nadj, 0, sizeof(double) * kAdjNodeTerms * size_t(b.cap_nodes), L.stream))) return e;
    if ((e = cudaMemsetAsync(s.sadj, 0, sizeof(double) * kAdjStarTerms * size_t(b.cap_n), L.stream))) return e;
    if ((e = cudaMemsetAsync(s.star_leaf, 0xff, sizeof(int32_t) * size_t(b.cap_n), L.stream))) return e;
    if ((e = cudaMemsetAsync(b.walk_ctr, 0, sizeof(uint32_t), L.stream))) return e;
    // few groups: each group's walk shared among several warps, as the forward's (walk_lists)
    if ((e = b.group == 64 ? launch_adj<2>(L, b, n, eps2, wx, wy, wz, s) : launch_adj<1>(L, b, n, eps2, wx, wy, wz, s)))
        return e;
    const unsigned nbn = unsigned((b.cap_nodes + 255) / 256), nbs = unsigned((b.cap_n + 255) / 256);
    k_star_leaf<<<nbn < 1 ? 1 : nbn, 256, 0, L.stream>>>(b.info, b.lnode, s.star_leaf);
    ++*L.count;
    if ((e = cudaGetLastError())) return e;
    k_adj_downsweep<<<nbs < 1 ? 1 : nbs, 256, 0, L.stream>>>(b.info, b.lnode, b.n_parent, s.star_leaf, b.order, px, py,
                                                            pz, mass, s.tgt, s.nadj, s.sadj, n, out, b.info);
    ++*L.count;
    return cudaGetLastError();
}

cudaError_t adj_tree_reserve(AdjTreeBufs &s, const TreeBufs &b) {
    if (s.cap_nodes >= b.cap_nodes && s.cap_n >= b.cap_n) return cudaSuccess;
    adj_tree_free(s);
    cudaError_t e = dev_alloc(&s.nadj, sizeof(double) * kAdjNodeTerms * size_t(b.cap_nodes));
    if (e == cudaSuccess) e = dev_alloc(&s.sadj, sizeof(double) * kAdjStarTerms * size_t(b.cap_n));
    if (e == cudaSuccess) e = dev_alloc(&s.tgt, sizeof(double) * 3 * size_t(b.cap_n));
    if (e == cudaSuccess) e = dev_alloc(&s.star_leaf, sizeof(int32_t) * size_t(b.cap_n));
    if (e != cudaSuccess) {
        adj_tree_free(s);
        return e;
    }
    s.cap_nodes = b.cap_nodes;
    s.cap_n = b.cap_n;
    return cudaSuccess;
}

void adj_tree_free(AdjTreeBufs &s) {
    void *ptrs[] = {s.nadj, s.sadj, s.tgt, s.star_leaf};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    s = AdjTreeBufs{};
}

}  // namespace gbh
