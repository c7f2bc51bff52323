// tree.cu — octree construction and the FP64 kernels of the Barnes-Hut step.
//
// Compiled with -fmad=false: every FP64 a*b+c is a rounded multiply and a rounded add, as in
// the reference's arithmetic, so keys, node moments, the FP64 walk, the direct sum and the
// kick/drift are bit identical to it.
//
// Pipeline of tree_build (one stream, no host round trip):
//   k_flags_bbox -> scan -> k_bbox_final -> k_compact_keys          (collect + keys, build.go:11-31, 62-113)
//   8 x (k_rs_hist -> scan -> k_rs_scatter)                         (stable LSD radix sort, morton.go:25-49)
//   k_gather                                                        (sorted copies, build.go:34-41)
//   k_chain_count -> scan -> k_chain_emit -> scan -> k_ref_index -> k_emit_nodes
//                                                                   (node set and links of buildNode, build.go:134-172)
//   k_upsweep                                                       (finish, build.go:176-217)
//
// Node set without recursion. A cell at level L is the set of sorted stars whose keys share
// their top 3L bits. The reference creates a node for the root and for every non-empty octant
// of a node that splits (count > leaf and level < 21). Counts shrink down the tree, so a
// non-root cell is a node exactly when its parent cell holds more than leaf stars. Every node
// starts at some sorted position i; the nodes starting at i form a chain of consecutive levels
// (a node and its first child share their first star). Sorting nodes by (first star, level) is
// the walk's pre-order, so the skip pointer of a node is the shallowest node that starts where
// it ends. The reference's serial build allocates each node's children as one block when the
// node is visited in that pre-order, so a prefix sum of child counts over pre-order gives every
// node its index in the reference's own serial layout.
#include <cuda_runtime.h>

#include <climits>

#include "gbh_internal.cuh"

namespace gbh {

namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

constexpr int kRsThreads = 256;
constexpr int kRsItems = 8;
constexpr int kRsTile = kRsThreads * kRsItems;
constexpr int kRsWarps = kRsThreads / 32;
constexpr int kRsBins = 256;

constexpr int kThreads = 256;

inline unsigned blocks_for(int64_t n, int threads) {
    int64_t b = (n + threads - 1) / threads;
    return unsigned(b < 1 ? 1 : b);
}

// Records a device-side consistency failure (checked by the host after the call).
__device__ __forceinline__ void dev_error(DevInfo *info, int where) {
    atomicExch(&info->err, 1);
    info->err_where = where;
}

// ---------------------------------------------------------------- exclusive scan (uint32)

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v) {
    int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

// Block-wide exclusive scan of one value per thread; returns the exclusive prefix and the total.
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t *s_warp, uint32_t &total) {
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t incl = warp_incl_scan(v);
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < (kScanThreads / 32) ? s_warp[lane] : 0;
        uint32_t wi = warp_incl_scan(w);
        if (lane < (kScanThreads / 32)) s_warp[lane] = wi - w;
        if (lane == (kScanThreads / 32) - 1) s_warp[kScanThreads / 32] = wi;
    }
    __syncthreads();
    uint32_t r = s_warp[warp] + incl - v;
    total = s_warp[kScanThreads / 32];
    __syncthreads();
    return r;
}

__device__ __forceinline__ int64_t dyn_len(int64_t n, const int64_t *ndyn) {
    if (ndyn) {
        int64_t m = *ndyn;
        return m < n ? m : n;
    }
    return n;
}

__global__ __launch_bounds__(kScanThreads) void k_scan_reduce(const uint32_t *__restrict__ in, int64_t n,
                                                              const int64_t *ndyn, uint32_t *__restrict__ sums) {
    __shared__ uint32_t s_warp[kScanThreads / 32 + 1];
    int64_t ne = dyn_len(n, ndyn);
    int64_t base = int64_t(blockIdx.x) * kScanTile + int64_t(threadIdx.x) * kScanItems;
    uint32_t v = 0;
    if (int64_t(blockIdx.x) * kScanTile < ne) {
#pragma unroll
        for (int k = 0; k < kScanItems; ++k)
            if (base + k < ne) v += in[base + k];
    }
    uint32_t total;
    block_excl_scan(v, s_warp, total);
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

__global__ __launch_bounds__(kScanThreads) void k_scan_apply(const uint32_t *in, uint32_t *out, int64_t n,
                                                             const int64_t *ndyn, const uint32_t *__restrict__ sums) {
    __shared__ uint32_t s_warp[kScanThreads / 32 + 1];
    int64_t ne = dyn_len(n, ndyn);
    if (int64_t(blockIdx.x) * kScanTile >= ne) return;
    int64_t base = int64_t(blockIdx.x) * kScanTile + int64_t(threadIdx.x) * kScanItems;
    uint32_t v[kScanItems];
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        v[k] = base + k < ne ? in[base + k] : 0;
        s += v[k];
    }
    uint32_t total;
    uint32_t run = block_excl_scan(s, s_warp, total) + (sums ? sums[blockIdx.x] : 0);
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        if (base + k < ne) out[base + k] = run;
        run += v[k];
    }
}

// One block of kSingleThreads scanning up to kSingleThreads * kSingleItems entries in one launch
// (each thread a run of consecutive entries): the small scans of a small build take one launch
// instead of three.
constexpr int kSingleThreads = 1024, kSingleItems = 8;
__global__ __launch_bounds__(kSingleThreads) void k_scan_single(const uint32_t *in, uint32_t *out, int64_t n,
                                                                const int64_t *ndyn) {
    __shared__ uint32_t s_warp[kSingleThreads / 32];
    const int64_t ne = dyn_len(n, ndyn);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t base = int64_t(threadIdx.x) * kSingleItems;
    uint32_t v[kSingleItems];
    uint32_t sum = 0;
#pragma unroll
    for (int k = 0; k < kSingleItems; ++k) {
        v[k] = base + k < ne ? in[base + k] : 0;
        sum += v[k];
    }
    const uint32_t incl = warp_incl_scan(sum);
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        const uint32_t w = s_warp[lane];  // kSingleThreads / 32 == 32 warp totals
        s_warp[lane] = warp_incl_scan(w) - w;
    }
    __syncthreads();
    uint32_t run = s_warp[warp] + incl - sum;
#pragma unroll
    for (int k = 0; k < kSingleItems; ++k) {
        if (base + k < ne) out[base + k] = run;
        run += v[k];
    }
}

cudaError_t scan_rec(const Launch &L, const uint32_t *in, uint32_t *out, int64_t n, const int64_t *ndyn,
                     uint32_t *tmp, int64_t tmp_cap) {
    int64_t tiles = (n + kScanTile - 1) / kScanTile;
    if (tiles > 1 && n <= int64_t(kSingleThreads) * kSingleItems) {
        k_scan_single<<<1, kSingleThreads, 0, L.stream>>>(in, out, n, ndyn);
        ++*L.count;
        return cudaGetLastError();
    }
    if (tiles <= 1) {
        k_scan_apply<<<1, kScanThreads, 0, L.stream>>>(in, out, n, ndyn, nullptr);
        ++*L.count;
        return cudaGetLastError();
    }
    if (tiles > tmp_cap) return cudaErrorInvalidValue;
    k_scan_reduce<<<unsigned(tiles), kScanThreads, 0, L.stream>>>(in, n, ndyn, tmp);
    ++*L.count;
    cudaError_t e = scan_rec(L, tmp, tmp, tiles, nullptr, tmp + tiles, tmp_cap - tiles);
    if (e != cudaSuccess) return e;
    k_scan_apply<<<unsigned(tiles), kScanThreads, 0, L.stream>>>(in, out, n, ndyn, tmp);
    ++*L.count;
    return cudaGetLastError();
}

// Polls of a look-back wait (the one-sweep sort's and the single-pass scan's) before the block
// gives up and records an error: far beyond any wait of a running predecessor.
constexpr int kOsSpinLimit = 1 << 22;

// Look-back words are read and written whole (count and flag in one word); nothing else is
// passed through them, so volatile (uncached, untorn) accesses suffice.
__device__ __forceinline__ uint32_t ld_volatile(const uint32_t *p) { return *reinterpret_cast<const volatile uint32_t *>(p); }
__device__ __forceinline__ void st_volatile(uint32_t *p, uint32_t v) { *reinterpret_cast<volatile uint32_t *>(p) = v; }
__device__ __forceinline__ unsigned long long ld_volatile64(const unsigned long long *p) {
    return *reinterpret_cast<const volatile unsigned long long *>(p);
}
__device__ __forceinline__ void st_volatile64(unsigned long long *p, unsigned long long v) {
    *reinterpret_cast<volatile unsigned long long *>(p) = v;
}

// Single-pass exclusive scan with decoupled look-back (one launch; every scan of tree_build, in
// place of a reduce, a scan of the tile sums and an apply): a block takes the next tile
// from *ctr, publishes its sum, adds its predecessors' (their inclusive prefix, or their sums
// back to one that has published a prefix) and publishes its own inclusive prefix. Waits are
// bounded as in the one-sweep sort. status: one 64-bit word per tile (flag in the top 2 bits).
__global__ __launch_bounds__(kScanThreads) void k_scan_lb(const uint32_t *in, uint32_t *out, int64_t n,
                                                          const int64_t *ndyn, uint32_t *ctr,
                                                          unsigned long long *status, DevInfo *info) {
    __shared__ uint32_t s_warp[kScanThreads / 32 + 1];
    __shared__ uint32_t s_tile;
    __shared__ unsigned long long s_prefix;
    if (threadIdx.x == 0) s_tile = atomicAdd(ctr, 1u);
    __syncthreads();
    const uint32_t tile = s_tile;
    const int64_t ne = dyn_len(n, ndyn);
    if (int64_t(tile) * kScanTile >= ne) return;  // uniform
    const int64_t base = int64_t(tile) * kScanTile + int64_t(threadIdx.x) * kScanItems;
    uint32_t v[kScanItems];
    uint32_t sum = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        v[k] = base + k < ne ? in[base + k] : 0;
        sum += v[k];
    }
    uint32_t total;
    uint32_t run = block_excl_scan(sum, s_warp, total);
    if (threadIdx.x < 32) {
        // warp 0 publishes the tile's sum, then reads its predecessors' words 32 at a time (lane j
        // the (j+1)-th tile back) and adds them down to the nearest published prefix
        constexpr unsigned long long kAgg = 1ull << 62, kPre = 2ull << 62, kVal = (1ull << 62) - 1;
        const int lane = threadIdx.x;
        unsigned long long excl = 0;
        if (tile == 0) {
            if (lane == 0) st_volatile64(status, kPre | total);
        } else {
            if (lane == 0) st_volatile64(status + tile, kAgg | total);
            int64_t t = int64_t(tile) - 1;
            int spins = 0;
            bool bad = false;
            for (;;) {
                const int64_t idx = t - lane;
                unsigned long long w = idx >= 0 ? ld_volatile64(status + idx) : kPre;  // before tile 0: prefix 0
                // every word up to the nearest prefix must be published; wait for the others
                for (;;) {
                    const unsigned pre = __ballot_sync(0xffffffffu, (w >> 62) == 2);
                    const unsigned upto = pre ? (pre & (0u - pre)) * 2u - 1u : 0xffffffffu;  // lanes to the first prefix
                    const unsigned wait = __ballot_sync(0xffffffffu, !(w >> 62)) & upto;
                    if (!wait) break;
                    if (++spins > kOsSpinLimit) {
                        bad = true;
                        break;
                    }
                    if ((wait >> lane) & 1u) w = ld_volatile64(status + idx);
                }
                if (bad) break;
                const unsigned pre = __ballot_sync(0xffffffffu, (w >> 62) == 2);
                const unsigned upto = pre ? (pre & (0u - pre)) * 2u - 1u : 0xffffffffu;
                unsigned long long v = ((upto >> lane) & 1u) ? (w & kVal) : 0ull;
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
                excl += v;
                if (pre) break;
                t -= 32;
            }
            if (lane == 0) {
                if (bad) dev_error(info, kErrScanWait);
                st_volatile64(status + tile, kPre | ((excl + total) & kVal));
            }
        }
        if (lane == 0) s_prefix = excl;
    }
    __syncthreads();
    run += uint32_t(s_prefix);
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        if (base + k < ne) out[base + k] = run;
        run += v[k];
    }
}

// ---------------------------------------------------------------- collect + bbox + keys

__device__ __forceinline__ bool is_star(uint8_t alive, uint8_t kind) { return alive && kind != GBH_BLACK_HOLE; }

// Order-preserving map of a double to a signed 64-bit integer (an involution): min and max of
// the keys are the keys of the min and max, computed on the integer ALU instead of the slow
// FP64 pipe. (-0 orders before +0; the coordinates are not NaN.)
__device__ __forceinline__ long long ord_key(double v) {
    long long b = __double_as_longlong(v);
    return b ^ ((b >> 63) & 0x7fffffffffffffffll);
}
__device__ __forceinline__ double ord_val(long long k) { return __longlong_as_double(k ^ ((k >> 63) & 0x7fffffffffffffffll)); }

// Per-block min/max of the 6 ordered keys into part[6 * blockIdx.x ...] (as raw 64-bit words).
template <int kBlock>
__device__ __forceinline__ void block_minmax(long long mn[3], long long mx[3], double *part) {
    __shared__ long long s[6][kBlock / 32];
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        for (int o = 16; o > 0; o >>= 1) {
            mn[c] = min(mn[c], __shfl_xor_sync(0xffffffffu, mn[c], o));
            mx[c] = max(mx[c], __shfl_xor_sync(0xffffffffu, mx[c], o));
        }
        if (lane == 0) {
            s[c][warp] = mn[c];
            s[3 + c][warp] = mx[c];
        }
    }
    __syncthreads();
    if (threadIdx.x < 6) {
        bool isMin = threadIdx.x < 3;
        long long v = s[threadIdx.x][0];
        for (int w = 1; w < kBlock / 32; ++w) v = isMin ? min(v, s[threadIdx.x][w]) : max(v, s[threadIdx.x][w]);
        part[blockIdx.x * 6 + threadIdx.x] = __longlong_as_double(v);
    }
}

// Star flags, per-block bbox partials; alive holes get zero acceleration (bh.go:99-101).
// A non-finite coordinate of a star makes the bbox non-finite by itself (NaN and infinities map to
// keys beyond every finite one); a non-finite mass is folded in as the key of a NaN, so that
// k_bbox_final can reject the input before keys are formed (collect, build.go:62-113, would
// carry a NaN into the root cube and every key).
__global__ __launch_bounds__(kThreads) void k_flags_bbox(int64_t n, const double *__restrict__ px,
                                                         const double *__restrict__ py, const double *__restrict__ pz,
                                                         const double *__restrict__ mass,
                                                         const uint8_t *__restrict__ kind,
                                                         const uint8_t *__restrict__ alive, uint32_t *__restrict__ flag,
                                                         double *__restrict__ part, double *ax, double *ay, double *az,
                                                         DevInfo *info, Pos4 *__restrict__ pos4) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {  // the build's first kernel clears the error record
        info->err = 0;
        info->err_where = 0;
    }
    long long mn[3] = {LLONG_MAX, LLONG_MAX, LLONG_MAX}, mx[3] = {LLONG_MIN, LLONG_MIN, LLONG_MIN};
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
        uint8_t al = alive ? alive[i] : 1, kd = kind ? kind[i] : 0;
        bool st = is_star(al, kd);
        flag[i] = st;
        if (st) {
            const double vx = px[i], vy = py[i], vz = pz[i], m = mass ? mass[i] : 0.0;
            pos4[i] = Pos4{vx, vy, vz, m};  // one record for k_gather's reads through the sort order
            long long x = ord_key(vx), y = ord_key(vy), z = ord_key(vz);
            mn[0] = min(mn[0], x);
            mx[0] = max(mx[0], mass && !isfinite(m) ? LLONG_MAX : x);
            mn[1] = min(mn[1], y);
            mx[1] = max(mx[1], y);
            mn[2] = min(mn[2], z);
            mx[2] = max(mx[2], z);
        } else if (al && kd == GBH_BLACK_HOLE) {
            ax[i] = 0;
            ay[i] = 0;
            az[i] = 0;
        }
    }
    block_minmax<kThreads>(mn, mx, part);
}

// Root cube (build.go:19-21): side = max(max extent * (1+1e-9), 1e-12), scale = 2^21 / side.
// One block reduces the per-block partials (min/max are exact, so the order does not matter).
constexpr int kFinalThreads = 1024;
__global__ __launch_bounds__(kFinalThreads) void k_bbox_final(int nparts, const double *__restrict__ part, int64_t n,
                                                              const uint32_t *__restrict__ scan, const uint8_t *kind,
                                                              const uint8_t *alive, double theta, DevInfo *info,
                                                              SysGeo *geo) {
    long long kmn[3] = {LLONG_MAX, LLONG_MAX, LLONG_MAX}, kmx[3] = {LLONG_MIN, LLONG_MIN, LLONG_MIN};
    for (int b = threadIdx.x; b < nparts; b += blockDim.x)
        for (int c = 0; c < 3; ++c) {
            kmn[c] = min(kmn[c], __double_as_longlong(part[b * 6 + c]));
            kmx[c] = max(kmx[c], __double_as_longlong(part[b * 6 + 3 + c]));
        }
    __shared__ long long s[6][kFinalThreads / 32];
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int c = 0; c < 3; ++c) {
        for (int o = 16; o > 0; o >>= 1) {
            kmn[c] = min(kmn[c], __shfl_xor_sync(0xffffffffu, kmn[c], o));
            kmx[c] = max(kmx[c], __shfl_xor_sync(0xffffffffu, kmx[c], o));
        }
        if (lane == 0) {
            s[c][warp] = kmn[c];
            s[3 + c][warp] = kmx[c];
        }
    }
    __syncthreads();
    // warp 0 reduces the warps' values (lane w holds warp w's)
    if (warp != 0) return;
    static_assert(kFinalThreads / 32 == 32, "one value per lane");
    double mn[3], mx[3];
    for (int c = 0; c < 3; ++c) {
        long long a = s[c][lane], b = s[3 + c][lane];
        for (int o = 16; o > 0; o >>= 1) {
            a = min(a, __shfl_xor_sync(0xffffffffu, a, o));
            b = max(b, __shfl_xor_sync(0xffffffffu, b, o));
        }
        mn[c] = ord_val(a);
        mx[c] = ord_val(b);
    }
    double side = fmax(mx[0] - mn[0], fmax(mx[1] - mn[1], mx[2] - mn[2]));
    side = fmax(side * (1 + 1e-9), 1e-12);
    // opening bases 2 half_L / theta, half_L = side / 2^(L+1): halving is exact, so lane L forms its
    // own level's half with one exact scaling instead of L successive halvings
    if (lane <= kMaxLevel) {
        const double half = ldexp(side, -(lane + 1));
        info->crit_base[lane] = __double2float_rn(2 * half / theta);
        if (geo) geo[0].crit_base[lane] = info->crit_base[lane];
    }
    if (lane != 0) return;
    int64_t ns = 0;
    if (n > 0) ns = int64_t(scan[n - 1]) + (is_star(alive ? alive[n - 1] : 1, kind ? kind[n - 1] : 0) ? 1 : 0);
    info->minx = mn[0];
    info->miny = mn[1];
    info->minz = mn[2];
    info->side = side;
    info->scale = double(1 << kMortonBits) / side;
    info->theta = theta;
    info->nstars = ns;
    info->nnodes = 0;
    info->work = 0;
    info->nleaves = 0;
    if (ns > 0 && !(isfinite(mn[0]) && isfinite(mn[1]) && isfinite(mn[2]) && isfinite(mx[0]) && isfinite(mx[1]) &&
                    isfinite(mx[2]))) {
        info->err = 1;  // reported to the caller as GBH_ERR_ARG
        info->err_where = kErrNonFinite;
    }
    for (int c = 0; c < 3; ++c) {
        float h = __double2float_rn(mn[c]);
        info->min_hi[c] = h;
        info->min_lo[c] = __double2float_rn(mn[c] - double(h));
    }
    float sh = __double2float_rn(side);
    info->side_hi = sh;
    info->side_lo = __double2float_rn(side - double(sh));
    if (geo) {  // the single system of a plain state
        SysGeo &g = geo[0];
        g.minx = info->minx;
        g.miny = info->miny;
        g.minz = info->minz;
        g.side = side;
        g.scale = info->scale;
        for (int c = 0; c < 3; ++c) {
            g.min_hi[c] = info->min_hi[c];
            g.min_lo[c] = info->min_lo[c];
        }
        g.side_hi = info->side_hi;
        g.side_lo = info->side_lo;
        g.star_lo = 0;
        g.star_hi = int32_t(ns);
        g.root = 0;
        g.group_lo = 0;
        g.ngroups = int32_t((ns + 63) / 64);
    }
}

// morton.go:7-15.
__device__ __forceinline__ uint64_t spread(uint64_t v) {
    v &= (uint64_t(1) << kMortonBits) - 1;
    v = (v | v << 32) & 0x1f00000000ffffull;
    v = (v | v << 16) & 0x1f0000ff0000ffull;
    v = (v | v << 8) & 0x100f00f00f00f00full;
    v = (v | v << 4) & 0x10c30c30c30c30c3ull;
    v = (v | v << 2) & 0x1249249249249249ull;
    return v;
}

// cell(), build.go:23-25: uint64(min(2^21-1, max(0, (v-lo)*scale))).
__device__ __forceinline__ uint64_t cell(double v, double lo, double scale) {
    double t = fmin(double((1 << kMortonBits) - 1), fmax(0.0, (v - lo) * scale));
    return uint64_t(t);
}

// order[k] = i for the k-th star in state order; keys[k] = mortonKey(cells) (build.go:26-31).
__global__ __launch_bounds__(kThreads) void k_compact_keys(int64_t n, const double *__restrict__ px,
                                                           const double *__restrict__ py, const double *__restrict__ pz,
                                                           const uint8_t *__restrict__ kind,
                                                           const uint8_t *__restrict__ alive,
                                                           const uint32_t *__restrict__ scan, const DevInfo *info,
                                                           uint64_t *__restrict__ keys, int32_t *__restrict__ order) {
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (!is_star(alive ? alive[i] : 1, kind ? kind[i] : 0)) return;
    double sc = info->scale;
    uint64_t k = spread(cell(px[i], info->minx, sc)) << 2 | spread(cell(py[i], info->miny, sc)) << 1 |
                 spread(cell(pz[i], info->minz, sc));
    uint32_t pos = scan[i];
    keys[pos] = k;
    order[pos] = int32_t(i);
}

// ---------------------------------------------------------------- stable LSD radix sort

// kSid: the digit is taken from the system id of the element's body (forest sorts by system
// after the 8 key passes) instead of the key.
template <bool kSid>
__global__ __launch_bounds__(kRsThreads) void k_rs_hist(const uint64_t *__restrict__ keys, const int32_t *__restrict__ vals,
                                                        const uint16_t *__restrict__ sys_of, const DevInfo *info,
                                                        int shift, uint32_t ntiles, uint32_t *__restrict__ hist) {
    __shared__ uint32_t h[kRsBins];
    int64_t n = info->nstars;
    h[threadIdx.x] = 0;
    __syncthreads();
    int64_t base = int64_t(blockIdx.x) * kRsTile;
    if (base < n) {
#pragma unroll
        for (int it = 0; it < kRsItems; ++it) {
            int64_t idx = base + it * kRsThreads + threadIdx.x;
            if (idx < n) {
                uint32_t d = kSid ? uint32_t(sys_of[vals[idx]] >> shift) : uint32_t(keys[idx] >> shift);
                atomicAdd(&h[d & (kRsBins - 1)], 1u);
            }
        }
    }
    __syncthreads();
    hist[size_t(threadIdx.x) * ntiles + blockIdx.x] = h[threadIdx.x];
}

// Stable scatter of one tile. Rank of a key = keys of the same digit earlier in the tile, in
// the order (item round, warp, lane) used to load them; offs holds the digit-major exclusive
// scan of the tile histograms, so equal digits keep their input order across tiles too.
template <bool kSid>
__global__ __launch_bounds__(kRsThreads) void k_rs_scatter(const uint64_t *__restrict__ kin,
                                                           const int32_t *__restrict__ vin,
                                                           uint64_t *__restrict__ kout, int32_t *__restrict__ vout,
                                                           const uint16_t *__restrict__ sys_of, DevInfo *info, int shift,
                                                           uint32_t ntiles, const uint32_t *__restrict__ offs) {
    __shared__ uint32_t s_run[kRsBins];
    __shared__ uint32_t s_goff[kRsBins];
    __shared__ uint32_t s_w[2][kRsWarps][kRsBins];
    int64_t n = info->nstars;
    int64_t base = int64_t(blockIdx.x) * kRsTile;
    if (base >= n) return;  // uniform over the block
    int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    s_run[tid] = 0;
    s_goff[tid] = offs[size_t(tid) * ntiles + blockIdx.x];
#pragma unroll
    for (int w = 0; w < kRsWarps; ++w) {
        s_w[0][w][tid] = 0;
        s_w[1][w][tid] = 0;
    }
    uint64_t k[kRsItems];
    int32_t v[kRsItems];
#pragma unroll
    for (int it = 0; it < kRsItems; ++it) {
        int64_t idx = base + it * kRsThreads + tid;
        if (idx < n) {
            k[it] = kin[idx];
            v[it] = vin[idx];
        }
    }
    __syncthreads();
    const uint32_t lt = (1u << lane) - 1u;
#pragma unroll
    for (int it = 0; it < kRsItems; ++it) {
        const int buf = it & 1;
        int64_t idx = base + it * kRsThreads + tid;
        bool valid = idx < n;
        uint32_t d = 0u;
        if (valid) d = (kSid ? uint32_t(sys_of[v[it]] >> shift) : uint32_t(k[it] >> shift)) & (kRsBins - 1);
        uint32_t peers = __match_any_sync(0xffffffffu, valid ? d : uint32_t(kRsBins + lane));
        uint32_t rank = __popc(peers & lt);
        if (valid && rank == 0) s_w[buf][warp][d] = __popc(peers);
        __syncthreads();
        uint32_t run = s_run[tid];
#pragma unroll
        for (int w = 0; w < kRsWarps; ++w) {
            uint32_t c = s_w[buf][w][tid];
            s_w[buf][w][tid] = run;
            run += c;
            s_w[buf ^ 1][w][tid] = 0;  // readers of the other buffer finished before this round's first barrier
        }
        s_run[tid] = run;
        __syncthreads();
        if (valid) {
            uint32_t pos = s_goff[d] + s_w[buf][warp][d] + rank;
            if (pos < n) {
                kout[pos] = k[it];
                vout[pos] = v[it];
            } else {
                dev_error(info, 10);
            }
        }
    }
}

// ---------------------------------------------------------------- one-sweep radix sort
//
// The same stable LSD sort in one launch per pass after a single histogram launch. k_os_hist
// reads the keys once and counts every pass's digits (and, for a forest, the two system-id
// digits); a pass block takes the next tile from a counter, ranks its keys exactly as
// k_rs_scatter does, publishes its per-digit counts and then looks back over its predecessors'
// published counts (decoupled look-back: a predecessor's word holds either its own count or its
// inclusive prefix) to find where each of its digits starts. Tiles are taken in counter order, so
// every tile a block waits for belongs to a block that is already running. Each wait is bounded:
// past kOsSpinLimit polls the block records an error (reported as GBH_ERR_LIMIT), publishes what
// it has so that its successors are not held, and its output is not used.

constexpr int kOsPassesMax = 10;  // 8 key digits, then 2 system-id digits (forest)
constexpr uint32_t kOsAgg = 1u << 30, kOsPre = 2u << 30, kOsCount = (1u << 30) - 1u;
// States of up to kOsMaxN bodies (capacity) build with the one-sweep sort and single-pass scans;
// larger ones with the three-launch passes. Measured on the merger (CUDA events, whole build,
// one-sweep against three-launch): 16k bodies 0.29 / 0.36 ms, 64k 0.32 / 0.45, 131k 0.36 / 0.46,
// 262k 0.41 / 0.50, 1M 0.72 / 0.69. With every tile of a large pass resident at once, each
// tile's look-back walks back to the nearest published prefix while all of them are still
// aggregates, a chain of L2 round trips that outgrows the launches it saves.
constexpr int64_t kOsMaxN = int64_t(3) << 18;
static_assert(kOsMaxN * 8 < int64_t(kOsCount), "one-sweep counts are 30-bit");
constexpr int kOsHistBlocksPerSm = 2;
constexpr int kOsWindow = 8;  // predecessors' look-back words read per round trip

// Word offsets inside TreeBufs::os_state.
constexpr int64_t kOsHistWords = int64_t(kOsPassesMax) * kRsBins;  // [pass][digit]
constexpr int64_t kOsCtrWords = 32;                                 // tile counters: passes, then scans
constexpr int kOsScanCtr = kOsPassesMax;                            // first scan counter
constexpr int kOsScans = 3;                                         // flags, chain counts, child counts
__host__ __device__ inline int64_t os_scan_tiles(int64_t n) { return (n + kScanTile - 1) / kScanTile; }
// Keys a thread of a one-sweep pass ranks: the fewest of 4, 8, 12 that keep a state of `cap`
// bodies within 96 tiles (measured: more tiles spread a small sort over more SMs, fewer tiles
// shorten the look-back; against 8 keys a thread, 4 made the 16k build 6 % faster and 12 the
// 262k build 4 % faster).
inline int os_items(int64_t cap) { return cap <= 96 * 4 * kRsThreads ? 4 : cap <= 96 * 8 * kRsThreads ? 8 : 12; }
inline int64_t os_sort_tiles(int64_t n, int items) {
    const int64_t tile = int64_t(items) * kRsThreads;
    return (n + tile - 1) / tile;
}
inline int64_t rs_sort_tiles(int64_t n) { return (n + kRsTile - 1) / kRsTile; }

// Every pass's digit histogram in one read of the keys (warp-aggregated shared counters, then one
// global add per non-zero bin and block).
template <bool kSid>
__global__ __launch_bounds__(kRsThreads) void k_os_hist(const uint64_t *__restrict__ keys,
                                                        const int32_t *__restrict__ vals,
                                                        const uint16_t *__restrict__ sys_of, const DevInfo *info,
                                                        uint32_t *__restrict__ ghist) {
    constexpr int kPasses = kSid ? kOsPassesMax : 8;
    __shared__ uint32_t h[kPasses * kRsBins];
    for (int i = threadIdx.x; i < kPasses * kRsBins; i += blockDim.x) h[i] = 0;
    __syncthreads();
    const int64_t n = info->nstars;
    const int lane = threadIdx.x & 31;
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    // whole warps iterate together (the match below needs every lane)
    for (int64_t i0 = int64_t(blockIdx.x) * blockDim.x + (threadIdx.x & ~31); i0 < n; i0 += stride) {
        const int64_t i = i0 + lane;
        const bool valid = i < n;
        const uint64_t k = valid ? keys[i] : 0;
        const uint32_t sd = kSid && valid ? uint32_t(sys_of[vals[i]]) : 0u;
#pragma unroll
        for (int p = 0; p < kPasses; ++p) {
            const uint32_t d = p < 8 ? uint32_t(k >> (8 * p)) & 255u : (sd >> (8 * (p - 8))) & 255u;
            const uint32_t peers = __match_any_sync(0xffffffffu, valid ? d : 256u + lane);
            if (valid && (peers & ((1u << lane) - 1u)) == 0) atomicAdd(&h[p * kRsBins + d], __popc(peers));
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kPasses * kRsBins; i += blockDim.x)
        if (h[i]) atomicAdd(&ghist[i], h[i]);
}

// Ranks a tile's keys by digit, stably, for the one-sweep pass. Warp w holds the tile's keys
// [w, w + 1) x kItems x 32 (item it of lane l: position w kItems 32 + it 32 + l), so the
// order (warp, item, lane) is the input order. Each warp counts its own keys per digit in
// s_w[w][digit] (the lowest lane of each group of equal digits reads and advances the counter;
// no block barrier inside the loop), so a key's rank among its warp's earlier keys of the same
// digit is the counter before its group plus its place in the group. On return s_w holds the
// warp counts (the caller turns them into offsets after a barrier). Measured against the
// round-barrier ranking of k_rs_scatter: the one-sweep builds 2-4 % faster (16k-262k bodies);
// in k_rs_scatter it made the 1M and 4M builds 3-5 % slower, so that kernel keeps its own.
template <bool kSid, int kItems>
__device__ __forceinline__ void rank_tile(const uint64_t *__restrict__ kin, const int32_t *__restrict__ vin,
                                          const uint16_t *__restrict__ sys_of, int shift, int64_t base, int64_t n,
                                          uint32_t (&s_w)[kRsWarps][kRsBins], uint64_t (&k)[kItems],
                                          int32_t (&v)[kItems], uint32_t (&dig)[kItems], uint32_t (&rk)[kItems]) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
#pragma unroll
    for (int w = 0; w < kRsWarps; ++w) s_w[w][tid] = 0;
    const int64_t wbase = base + int64_t(warp) * (kItems * 32);
#pragma unroll
    for (int it = 0; it < kItems; ++it) {
        const int64_t idx = wbase + it * 32 + lane;
        if (idx < n) {
            k[it] = kin[idx];
            v[it] = vin[idx];
        }
    }
    __syncthreads();  // counters cleared
    const uint32_t lt = (1u << lane) - 1u;
#pragma unroll
    for (int it = 0; it < kItems; ++it) {
        const bool valid = wbase + it * 32 + lane < n;
        uint32_t d = 0u;
        if (valid) d = (kSid ? uint32_t(sys_of[v[it]] >> shift) : uint32_t(k[it] >> shift)) & (kRsBins - 1);
        const uint32_t peers = __match_any_sync(0xffffffffu, valid ? d : uint32_t(kRsBins + lane));
        const int leader = __ffs(peers) - 1;
        uint32_t old = 0;
        if (valid && lane == leader) old = s_w[warp][d];
        old = __shfl_sync(0xffffffffu, old, leader);
        rk[it] = old + __popc(peers & lt);
        dig[it] = d;
        if (valid && lane == leader) s_w[warp][d] = old + __popc(peers);
        __syncwarp();
    }
}

// One stable pass over the tile the block takes. status: [tile][digit] words of this pass.
template <bool kSid, int kItems>
__global__ __launch_bounds__(kRsThreads) void k_os_pass(const uint64_t *__restrict__ kin,
                                                        const int32_t *__restrict__ vin, uint64_t *__restrict__ kout,
                                                        int32_t *__restrict__ vout, const uint16_t *__restrict__ sys_of,
                                                        DevInfo *info, int shift, const uint32_t *__restrict__ ghist,
                                                        uint32_t *ctr, uint32_t *status) {
    __shared__ uint32_t s_goff[kRsBins];
    __shared__ uint32_t s_w[kRsWarps][kRsBins];
    __shared__ uint32_t s_warp[kScanThreads / 32 + 1];
    __shared__ uint32_t s_tile;
    static_assert(kRsThreads == kScanThreads && kRsThreads == kRsBins, "one thread per digit");
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) s_tile = atomicAdd(ctr, 1u);
    // where each digit starts in the output: exclusive scan of the pass's histogram
    uint32_t total;
    const uint32_t gstart = block_excl_scan(ghist[tid], s_warp, total);  // its barriers publish s_tile too
    const uint32_t tile = s_tile;
    const int64_t n = info->nstars;
    const int64_t base = int64_t(tile) * (kItems * kRsThreads);
    if (base >= n) return;  // uniform over the block
    uint64_t k[kItems];
    int32_t v[kItems];
    uint32_t dig[kItems], rk[kItems];
    rank_tile<kSid, kItems>(kin, vin, sys_of, shift, base, n, s_w, k, v, dig, rk);
    __syncthreads();
    // digit tid: each warp's start inside the tile, and the tile's count
    uint32_t run = 0;
#pragma unroll
    for (int w = 0; w < kRsWarps; ++w) {
        const uint32_t c = s_w[w][tid];
        s_w[w][tid] = run;
        run += c;
    }
    // look-back for digit tid: this tile's count is run. Predecessors' words are read kOsWindow
    // at a time (independent loads), then taken in order back to the first prefix.
    const uint32_t agg = run;
    uint32_t *mine = status + size_t(tile) * kRsBins + tid;
    uint32_t excl = 0;
    if (tile == 0) {
        st_volatile(mine, kOsPre | agg);
    } else {
        st_volatile(mine, kOsAgg | agg);
        int64_t t = int64_t(tile) - 1;
        int spins = 0;
        bool done = false, bad = false;
        while (!done && !bad) {
            uint32_t w[kOsWindow];
#pragma unroll
            for (int j = 0; j < kOsWindow; ++j)  // before tile 0: a prefix of 0
                w[j] = t - j >= 0 ? ld_volatile(status + size_t(t - j) * kRsBins + tid) : kOsPre;
#pragma unroll
            for (int j = 0; j < kOsWindow; ++j) {
                if (done || bad) continue;
                while (!(w[j] >> 30)) {  // not published yet: wait for this word
                    if (++spins > kOsSpinLimit) {
                        bad = true;
                        break;
                    }
                    w[j] = ld_volatile(status + size_t(t - j) * kRsBins + tid);
                }
                if (bad) continue;
                excl += w[j] & kOsCount;
                done = (w[j] >> 30) == (kOsPre >> 30);
            }
            t -= kOsWindow;
        }
        if (bad) dev_error(info, kErrSortWait);
        st_volatile(mine, kOsPre | ((excl + agg) & kOsCount));
    }
    s_goff[tid] = gstart + excl;
    __syncthreads();
    const int64_t wbase = base + int64_t(warp) * (kItems * 32);
#pragma unroll
    for (int it = 0; it < kItems; ++it) {
        if (wbase + it * 32 + lane < n) {
            const uint32_t pos = s_goff[dig[it]] + s_w[warp][dig[it]] + rk[it];
            if (pos < n) {
                kout[pos] = k[it];
                vout[pos] = v[it];
            } else {
                dev_error(info, 10);
            }
        }
    }
}

// ---------------------------------------------------------------- sorted copies

// build.go:34-41 with SourceMass (sim.go:93-98); FP32 hi/lo split for the walks. Each star's
// position and mass come from its 32-byte record written by the collect kernel: one sector read
// through the sort order instead of one sector per array.
__global__ __launch_bounds__(kThreads) void k_gather(const DevInfo *info, const int32_t *__restrict__ order,
                                                     const Pos4 *__restrict__ pos4,
                                                     const uint8_t *__restrict__ kind, int dm_off, int fp64_copies,
                                                     double *__restrict__ sx, double *__restrict__ sy,
                                                     double *__restrict__ sz, double *__restrict__ sm,
                                                     float4 *__restrict__ st_hi, float4 *__restrict__ st_lo,
                                                     const uint16_t *__restrict__ sys_of,
                                                     int32_t *__restrict__ sid_sorted) {
    int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (k >= info->nstars) return;
    int32_t i = order[k];
    if (sys_of) sid_sorted[k] = sys_of[i];
    const Pos4 p = pos4[i];
    const double x = p.x, y = p.y, z = p.z;
    double m = p.m;
    if (dm_off && kind && kind[i] == GBH_DARK_MATTER) m = 0;
    if (fp64_copies) {  // read by the FP64 upsweep, walk and potential only
        sx[k] = x;
        sy[k] = y;
        sz[k] = z;
        sm[k] = m;
    }
    float hx = __double2float_rn(x), hy = __double2float_rn(y), hz = __double2float_rn(z);
    st_hi[k] = make_float4(hx, hy, hz, __double2float_rn(m));
    st_lo[k] = make_float4(__double2float_rn(x - double(hx)), __double2float_rn(y - double(hy)),
                           __double2float_rn(z - double(hz)), 0.f);
}

// ---------------------------------------------------------------- node set (chains)

// Sorted star range [lo, hi) of the system that sorted position i belongs to (the whole array
// for a plain state).
struct SysRange {
    int64_t lo, hi;
};
__device__ __forceinline__ SysRange sys_range(const int32_t *__restrict__ sid_sorted, const SysGeo *__restrict__ geo,
                                              int64_t i, int64_t n) {
    if (!sid_sorted) return SysRange{0, n};
    const SysGeo &g = geo[sid_sorted[i]];
    return SysRange{g.star_lo, g.star_hi};
}

// Shallowest level at which sorted position i starts a new cell (0 at the first star of its
// system, kNoCell if its key equals the previous one).
__device__ __forceinline__ int start_level(const uint64_t *__restrict__ keys, int64_t i, int64_t lo = 0) {
    if (i == lo) return 0;
    uint64_t x = keys[i] ^ keys[i - 1];
    if (x == 0) return kNoCell;
    int h = 63 - __clzll(static_cast<long long>(x));
    return kMaxLevel - h / 3;
}

__device__ __forceinline__ uint64_t prefix(uint64_t k, int L) { return L == 0 ? 0 : k >> (3 * (kMaxLevel - L)); }

// First position after i whose level-L cell differs from i's (galloping, then binary search).
__device__ int64_t cell_end(const uint64_t *__restrict__ keys, int64_t n, int64_t i, int L) {
    if (L == 0) return n;
    uint64_t P = prefix(keys[i], L);
    int64_t lo = i + 1, hi = n, step = 1;
    for (;;) {
        int64_t probe = i + step;
        if (probe >= n) break;
        if (prefix(keys[probe], L) != P) {
            hi = probe;
            break;
        }
        lo = probe + 1;
        step <<= 1;
    }
    while (lo < hi) {
        int64_t mid = (lo + hi) >> 1;
        if (prefix(keys[mid], L) == P) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// First position of i's level-L cell (not before lo_bound, the first star of its system).
__device__ int64_t cell_start(const uint64_t *__restrict__ keys, int64_t lo_bound, int64_t i, int L) {
    if (L == 0) return lo_bound;
    uint64_t P = prefix(keys[i], L);
    int64_t lo = lo_bound, hi = i, step = 1;
    for (;;) {
        int64_t probe = i - step;
        if (probe < lo_bound) break;
        if (prefix(keys[probe], L) != P) {
            lo = probe + 1;
            break;
        }
        hi = probe;
        step <<= 1;
    }
    while (lo < hi) {
        int64_t mid = (lo + hi) >> 1;
        if (prefix(keys[mid], L) == P) hi = mid;
        else lo = mid + 1;
    }
    return lo;
}

// Number of nodes that start at sorted position i.
__global__ __launch_bounds__(kThreads) void k_chain_count(const uint64_t *__restrict__ keys, const DevInfo *info,
                                                          const int32_t *__restrict__ sid_sorted,
                                                          const SysGeo *__restrict__ geo, int leaf,
                                                          uint32_t *__restrict__ cnt) {
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    int64_t n = info->nstars;
    if (i >= n) return;
    const SysRange R = sys_range(sid_sorted, geo, i, n);
    int L0 = start_level(keys, i, R.lo);
    uint32_t c = 0;
    if (L0 <= kMaxLevel) {
        // A level-L cell starting at i holds more than leaf stars exactly when the star leaf
        // positions on is still inside it (cells are contiguous runs of the sorted keys).
        const uint64_t ki = keys[i];
        const bool ahead = i + leaf < R.hi;
        const uint64_t ka = ahead ? keys[i + leaf] : 0;
        bool exists = true;
        if (i > R.lo) {  // the parent cell (level L0-1) contains i-1 and i; it splits iff it holds > leaf stars
            int Lp = L0 - 1;
            exists = (ahead && prefix(ka, Lp) == prefix(ki, Lp)) ||
                     cell_end(keys, R.hi, i, Lp) - cell_start(keys, R.lo, i, Lp) > leaf;
        }
        if (exists) {
            for (int L = L0;; ++L) {
                ++c;
                if (!(ahead && prefix(ka, L) == prefix(ki, L) && L < kMaxLevel)) break;
            }
        }
    }
    cnt[i] = c;
}

// Pre-order node arrays: parent (pre-order index), level | octant << 8 | child mask << 16,
// child count. base = exclusive scan of cnt: the pre-order index of the first node at i.
__global__ __launch_bounds__(kThreads) void k_chain_emit(const uint64_t *__restrict__ keys, DevInfo *info,
                                                         const uint32_t *__restrict__ cnt,
                                                         const uint32_t *__restrict__ base,
                                                         int32_t *__restrict__ pre_parent,
                                                         uint32_t *__restrict__ pre_info,
                                                         uint32_t *__restrict__ pre_nchild,
                                                         uint32_t *__restrict__ pre_mask,
                                                         int32_t *__restrict__ pre_star,
                                                         int32_t *__restrict__ leaves,
                                                         const int32_t *__restrict__ sid_sorted,
                                                         const SysGeo *__restrict__ geo) {
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    int64_t n = info->nstars;
    uint32_t c = i < n ? cnt[i] : 0;
    // every position with nodes ends its chain in exactly one leaf: append it to the leaf list
    unsigned m = __ballot_sync(0xffffffffu, c > 0);
    if (m) {
        int lane = threadIdx.x & 31;
        uint32_t off = 0;
        if (lane == __ffs(m) - 1) off = atomicAdd(&info->nleaves, uint32_t(__popc(m)));
        off = __shfl_sync(0xffffffffu, off, __ffs(m) - 1);
        if (c > 0) leaves[off + __popc(m & ((1u << lane) - 1u))] = int32_t(i);
    }
    if (i >= n) return;
    if (i == n - 1) info->nnodes = int64_t(base[i]) + c;
    if (c == 0) return;
    const SysRange R = sys_range(sid_sorted, geo, i, n);
    int L0 = start_level(keys, i, R.lo);
    int32_t parent_pre = -1;
    if (i > R.lo) {
        int Lp = L0 - 1;
        int64_t ps = cell_start(keys, R.lo, i, Lp);
        int Lps = start_level(keys, ps, R.lo);  // ps starts its chain at this level; the parent is Lp - Lps deeper
        parent_pre = int32_t(base[ps]) + (Lp - Lps);
    }
    uint64_t key = keys[i];
    uint32_t p = base[i];
    for (uint32_t t = 0; t < c; ++t, ++p) {
        int L = L0 + int(t);
        uint32_t oct = L == 0 ? 0u : uint32_t(key >> (3 * (kMaxLevel - L))) & 7u;
        int32_t par = t == 0 ? parent_pre : int32_t(p) - 1;
        pre_parent[p] = par;
        pre_info[p] = uint32_t(L) | oct << 8;
        pre_star[p] = int32_t(i);
        if (par >= 0) {  // every node marks its octant in its parent's child mask (both zeroed first)
            atomicOr(&pre_mask[par], 1u << oct);
            atomicAdd(&pre_nchild[par], 1u);
        }
    }
}

// Grid of the per-node kernels below: they loop over the nodes, whose count only the device knows.
inline unsigned node_blocks(int64_t cap_nodes) {
    const unsigned nb = blocks_for(cap_nodes, kThreads);
    return nb < 4096u ? nb : 4096u;
}

// Reference index of every node: 1 + (children allocated before its parent's block) + rank
// among the parent's non-empty octants. child_base = exclusive scan of child counts. One thread
// per node (pre-order index p).
__global__ __launch_bounds__(kThreads) void k_ref_index(DevInfo *info, const uint32_t *__restrict__ base,
                                                        const int32_t *__restrict__ pre_star,
                                                        const int32_t *__restrict__ pre_parent,
                                                        const uint32_t *__restrict__ pre_info,
                                                        const uint32_t *__restrict__ pre_mask,
                                                        const uint32_t *__restrict__ child_base,
                                                        int32_t *__restrict__ pre_ref,
                                                        const int32_t *__restrict__ sid_sorted,
                                                        const SysGeo *__restrict__ geo, int64_t cap_nodes) {
    const int64_t n = info->nstars, nn = info->nnodes < cap_nodes ? info->nnodes : cap_nodes;
    if (blockIdx.x == 0 && threadIdx.x == 0 && info->nnodes > cap_nodes) dev_error(info, 11);
    for (int64_t p = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; p < nn; p += int64_t(gridDim.x) * blockDim.x) {
        const int64_t i = pre_star[p];
        if (i < 0 || i >= n) {
            dev_error(info, 11);
            continue;
        }
        // a system's nodes are the pre-order block starting at its root (pre-order index of its
        // first star's chain); its reference layout fills the same block
        const uint32_t root = base[sys_range(sid_sorted, geo, i, n).lo];
        const int32_t pp = pre_parent[p];
        if (pp < 0) {
            pre_ref[p] = int32_t(root);
            continue;
        }
        const uint32_t oct = (pre_info[p] >> 8) & 0xffu;
        const uint32_t pmask = pre_mask[pp];
        pre_ref[p] = int32_t(root + 1 + (child_base[pp] - child_base[root]) + __popc(pmask & ((1u << oct) - 1u)));
    }
}

// Links and ranges of every node in the reference layout (bh.go:59-67). One thread per node: the
// search for the end of its cell runs beside the other nodes' searches, not after those of the
// shallower nodes of its chain.
__global__ __launch_bounds__(kThreads) void k_emit_nodes(const uint64_t *__restrict__ keys, DevInfo *info,
                                                         const uint32_t *__restrict__ cnt,
                                                         const uint32_t *__restrict__ base,
                                                         const int32_t *__restrict__ pre_star,
                                                         const int32_t *__restrict__ pre_parent,
                                                         const uint32_t *__restrict__ pre_info,
                                                         const uint32_t *__restrict__ pre_mask,
                                                         const uint32_t *__restrict__ child_base,
                                                         const int32_t *__restrict__ pre_ref, gbh_node *__restrict__ nodes,
                                                         int32_t *__restrict__ n_parent, uint32_t *__restrict__ n_info,
                                                         int32_t *__restrict__ n_arrive,
                                                         const int32_t *__restrict__ sid_sorted,
                                                         const SysGeo *__restrict__ geo, int64_t cap_nodes) {
    const int64_t n = info->nstars, nn = info->nnodes < cap_nodes ? info->nnodes : cap_nodes;
    for (int64_t p = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; p < nn; p += int64_t(gridDim.x) * blockDim.x) {
        const int64_t i = pre_star[p];
        const int32_t r = pre_ref[p];
        if (i < 0 || i >= n || r < 0 || r >= nn) {
            dev_error(info, 11);
            continue;
        }
        const SysRange R = sys_range(sid_sorted, geo, i, n);
        const uint32_t root = base[R.lo];
        const uint32_t inf = pre_info[p];
        const int L = int(inf & 0xffu);
        const uint32_t mask = pre_mask[p];
        const int64_t hi = cell_end(keys, R.hi, i, L);
        gbh_node &nd = nodes[r];
        nd.first = mask ? int32_t(root + 1 + (child_base[p] - child_base[root])) : -1;
        int32_t nx = hi == R.hi ? -1 : pre_ref[base[hi]];  // a system's walk ends at its own last node
        if (nx >= nn || (hi < R.hi && cnt[hi] == 0)) {
            dev_error(info, 12);
            nx = -1;
        }
        nd.next = nx;
        nd.lo = int32_t(i);
        nd.hi = int32_t(hi);
        const int32_t pp = pre_parent[p];
        n_parent[r] = pp < 0 ? -1 : pre_ref[pp];
        n_info[r] = uint32_t(L) | uint32_t(__popc(mask)) << 8;
        n_arrive[r] = 0;
    }
}

// ---------------------------------------------------------------- moments (finish, build.go:176-217)

struct Moments {
    double x, y, z, m, qxx, qyy, qzz, qxy, qxz, qyz;
};

// quadrupole.add, build.go:329-337.
__device__ __forceinline__ void quad_add(Moments &q, double m, double dx, double dy, double dz) {
    double r2 = dx * dx + dy * dy + dz * dz;
    q.qxx += m * (3 * dx * dx - r2);
    q.qyy += m * (3 * dy * dy - r2);
    q.qzz += m * (3 * dz * dz - r2);
    q.qxy += m * 3 * dx * dy;
    q.qxz += m * 3 * dx * dz;
    q.qyz += m * 3 * dy * dz;
}

// Geometric centre and half side of the level-L cell containing key, through the same
// rounded additions as the recursion c_child = c + offset(oct, bit) * half/2 (build.go:142-152).
__device__ __forceinline__ void cell_center(const SysGeo &inf, uint64_t key, int L, double &cx, double &cy,
                                            double &cz, double &half) {
    double h = inf.side / 2;
    cx = inf.minx + h;
    cy = inf.miny + h;
    cz = inf.minz + h;
    for (int l = 1; l <= L; ++l) {
        h = h / 2;
        uint32_t oct = uint32_t(key >> (3 * (kMaxLevel - l))) & 7u;
        cx = cx + ((oct >> 2 & 1u) ? h : -h);
        cy = cy + ((oct >> 1 & 1u) ? h : -h);
        cz = cz + ((oct & 1u) ? h : -h);
    }
    half = h;
}

__device__ __forceinline__ void write_node(gbh_node *nodes, PNode *pn, MNode *mn, int2 *mr, int32_t r, const Moments &q,
                                           double crit2) {
    gbh_node &nd = nodes[r];
    nd.x = q.x;
    nd.y = q.y;
    nd.z = q.z;
    nd.m = q.m;
    nd.qxx = q.qxx;
    nd.qyy = q.qyy;
    nd.qzz = q.qzz;
    nd.qxy = q.qxy;
    nd.qxz = q.qxz;
    nd.qyz = q.qyz;
    nd.crit2 = crit2;
    int32_t first = nd.first, next = nd.next, lo = nd.lo, hi = nd.hi;
    float fx = __double2float_rn(q.x), fy = __double2float_rn(q.y), fz = __double2float_rn(q.z);
    float fm = __double2float_rn(q.m), fc = __double2float_rn(crit2);
    PNode p;
    p.com = make_float4(fx, fy, fz, fm);
    p.q1 = make_float4(__double2float_rn(q.qxx), __double2float_rn(q.qyy), __double2float_rn(q.qzz),
                       __double2float_rn(q.qxy));
    p.q2 = make_float4(__double2float_rn(q.qxz), __double2float_rn(q.qyz), fc, 0.f);
    p.links = make_int4(first, next, lo, hi);
    pn[r] = p;
    MNode m;
    m.a = make_float4(fx, fy, fz, fc);
    m.b = make_float4(__double2float_rn(q.x - double(fx)), __double2float_rn(q.y - double(fy)),
                      __double2float_rn(q.z - double(fz)), fm);
    m.c = p.q1;
    m.d = make_float4(p.q2.x, p.q2.y, __int_as_float(first), __int_as_float(next));
    mn[r] = m;
    mr[r] = make_int2(lo, hi);
}

__device__ __forceinline__ double crit2_of(double theta, const Moments &q, double cx, double cy, double cz,
                                           double half) {
    double delta = sqrt((q.x - cx) * (q.x - cx) + (q.y - cy) * (q.y - cy) + (q.z - cz) * (q.z - cz));
    double crit = 2 * half / theta + delta;
    return crit * crit;
}

// Bottom-up moments: one thread per leaf; the last child to finish computes its parent.
__global__ __launch_bounds__(kThreads) void k_upsweep(const uint64_t *__restrict__ keys, const DevInfo *info,
                                                      const uint32_t *__restrict__ cnt, const uint32_t *__restrict__ base,
                                                      const int32_t *__restrict__ pre_ref, const double *__restrict__ sx,
                                                      const double *__restrict__ sy, const double *__restrict__ sz,
                                                      const double *__restrict__ sm, gbh_node *nodes,
                                                      const int32_t *__restrict__ n_parent,
                                                      const uint32_t *__restrict__ n_info, int32_t *n_arrive, PNode *pn,
                                                      MNode *mn, int2 *mr, const int32_t *__restrict__ sid_sorted,
                                                      const SysGeo *__restrict__ geo, DevInfo *err_info) {
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= info->nstars) return;
    uint32_t c = cnt[i];
    if (c == 0) return;
    const DevInfo inf = *info;
    int32_t r = pre_ref[base[i] + c - 1];  // the last node of a chain never splits: a leaf
    {
        int32_t lo = nodes[r].lo, hi = nodes[r].hi;
        int L = int(n_info[r] & 0xffu);
        Moments q = {};
        for (int32_t j = lo; j < hi; ++j) {
            double mj = sm[j];
            q.x = q.x + mj * sx[j];
            q.y = q.y + mj * sy[j];
            q.z = q.z + mj * sz[j];
            q.m = q.m + mj;
        }
        double cx, cy, cz, half;
        const SysGeo &g = geo[sid_sorted ? sid_sorted[lo] : 0];
        cell_center(g, keys[lo], L, cx, cy, cz, half);
        if (q.m > 0) {
            q.x = q.x / q.m;
            q.y = q.y / q.m;
            q.z = q.z / q.m;
        } else {
            q.x = cx;
            q.y = cy;
            q.z = cz;
        }
        for (int32_t j = lo; j < hi; ++j) quad_add(q, sm[j], sx[j] - q.x, sy[j] - q.y, sz[j] - q.z);
        write_node(nodes, pn, mn, mr, r, q, crit2_of(inf.theta, q, cx, cy, cz, half));
    }
    int32_t cur = r;
    for (int guard = 0; guard <= kMaxLevel + 1; ++guard) {
        int32_t par = n_parent[cur];
        if (par < 0) break;
        uint32_t nch = (n_info[par] >> 8) & 0xffu;
        __threadfence();
        int old = atomicAdd(&n_arrive[par], 1);
        if (old != int(nch) - 1) break;
        __threadfence();
        int32_t first = nodes[par].first;
        if (first < 0 || int64_t(first) + nch > inf.nnodes) {
            dev_error(err_info, 13);
            break;
        }
        Moments q = {};
        for (int32_t ch = first; ch < first + int32_t(nch); ++ch) {
            double cm = __ldcg(&nodes[ch].m);
            q.x = q.x + cm * __ldcg(&nodes[ch].x);
            q.y = q.y + cm * __ldcg(&nodes[ch].y);
            q.z = q.z + cm * __ldcg(&nodes[ch].z);
            q.m = q.m + cm;
        }
        int L = int(n_info[par] & 0xffu);
        double cx, cy, cz, half;
        const int32_t plo = nodes[par].lo;
        cell_center(geo[sid_sorted ? sid_sorted[plo] : 0], keys[plo], L, cx, cy, cz, half);
        if (q.m > 0) {
            q.x = q.x / q.m;
            q.y = q.y / q.m;
            q.z = q.z / q.m;
        } else {
            q.x = cx;
            q.y = cy;
            q.z = cz;
        }
        for (int32_t ch = first; ch < first + int32_t(nch); ++ch) {
            q.qxx = q.qxx + __ldcg(&nodes[ch].qxx);
            q.qyy = q.qyy + __ldcg(&nodes[ch].qyy);
            q.qzz = q.qzz + __ldcg(&nodes[ch].qzz);
            q.qxy = q.qxy + __ldcg(&nodes[ch].qxy);
            q.qxz = q.qxz + __ldcg(&nodes[ch].qxz);
            q.qyz = q.qyz + __ldcg(&nodes[ch].qyz);
            quad_add(q, __ldcg(&nodes[ch].m), __ldcg(&nodes[ch].x) - q.x, __ldcg(&nodes[ch].y) - q.y,
                     __ldcg(&nodes[ch].z) - q.z);
        }
        write_node(nodes, pn, mn, mr, par, q, crit2_of(inf.theta, q, cx, cy, cz, half));
        cur = par;
    }
}

// ---------------------------------------------------------------- FP64 walk (bh.go:106-155)

__global__ __launch_bounds__(kThreads) void k_walk_fp64(const DevInfo *info, const gbh_node *__restrict__ nodes,
                                                        const double *__restrict__ sx, const double *__restrict__ sy,
                                                        const double *__restrict__ sz, const double *__restrict__ sm,
                                                        const int32_t *__restrict__ order, double eps2, int quad,
                                                        double *ax, double *ay, double *az,
                                                        const int32_t *__restrict__ targets,
                                                        const int32_t *__restrict__ sid_sorted,
                                                        const SysGeo *__restrict__ geo, DevInfo *err_info) {
    int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    int64_t ns = info->nstars;
    if (t >= (targets ? int64_t(info->ntargets) : ns)) return;
    int64_t k = targets ? int64_t(targets[t]) : t;
    int64_t nn = info->nnodes;
    double x = sx[k], y = sy[k], z = sz[k];
    double fax = 0, fay = 0, faz = 0;
    int64_t steps = 0;
    const int32_t root = sid_sorted ? geo[sid_sorted[k]].root : 0;  // the star's own system
    for (int32_t i = nn > 0 ? root : -1; i >= 0;) {
        if (++steps > nn || i >= nn) {  // each node is visited at most once
            dev_error(err_info, 1);
            break;
        }
        const gbh_node &nd = nodes[i];
        double dx = nd.x - x, dy = nd.y - y, dz = nd.z - z;
        double d2 = dx * dx + dy * dy + dz * dz;
        if (d2 >= nd.crit2) {
            double inv = 1 / (d2 + eps2);
            double inv3 = inv * sqrt(inv);
            double f = nd.m * inv3;
            if (quad) {
                double qx = nd.qxx * dx + nd.qxy * dy + nd.qxz * dz;
                double qy = nd.qxy * dx + nd.qyy * dy + nd.qyz * dz;
                double qz = nd.qxz * dx + nd.qyz * dy + nd.qzz * dz;
                double inv5 = inv3 * inv;
                f += 2.5 * (dx * qx + dy * qy + dz * qz) * inv5 * inv;
                fax -= qx * inv5;
                fay -= qy * inv5;
                faz -= qz * inv5;
            }
            fax += f * dx;
            fay += f * dy;
            faz += f * dz;
            i = nd.next;
            continue;
        }
        if (nd.first >= 0) {
            i = nd.first;
            continue;
        }
        if (nd.lo < 0 || nd.hi > ns || nd.lo > nd.hi) {
            dev_error(err_info, 7);
            break;
        }
        for (int32_t j = nd.lo; j < nd.hi; ++j) {
            if (j == k) continue;
            double ddx = sx[j] - x, ddy = sy[j] - y, ddz = sz[j] - z;
            double r2 = ddx * ddx + ddy * ddy + ddz * ddz + eps2;
            double f = sm[j] / (r2 * sqrt(r2));
            fax += f * ddx;
            fay += f * ddy;
            faz += f * ddz;
        }
        i = nd.next;
    }
    int32_t o = order[k];
    ax[o] = fax;
    ay[o] = fay;
    az[o] = faz;
}

// ---------------------------------------------------------------- KDK (sim.go:302-343)

__global__ __launch_bounds__(kThreads) void k_kick(int64_t n, double h, double *vx, double *vy, double *vz,
                                                   const double *__restrict__ ax, const double *__restrict__ ay,
                                                   const double *__restrict__ az) {
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    vx[i] += h * ax[i];
    vy[i] += h * ay[i];
    vz[i] += h * az[i];
}

// kick (sim.go:305-313) then drift (sim.go:315-343): x += dt u for c <= 0 (inv_c2 == 0), else
// x += dt u / sqrt(1 + u^2 / c^2) with the reference's 1 / c^2 factor inv_c2.
__global__ __launch_bounds__(kThreads) void k_kick_drift(int64_t n, double h, double dt, double inv_c2, double *px,
                                                         double *py, double *pz, double *vx, double *vy, double *vz,
                                                         const double *__restrict__ ax, const double *__restrict__ ay,
                                                         const double *__restrict__ az) {
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double x = vx[i] + h * ax[i], y = vy[i] + h * ay[i], z = vz[i] + h * az[i];
    vx[i] = x;
    vy[i] = y;
    vz[i] = z;
    double f = dt;
    if (inv_c2 > 0) f = dt / sqrt(1 + (x * x + y * y + z * z) * inv_c2);
    px[i] += f * x;
    py[i] += f * y;
    pz[i] += f * z;
}

// ---------------------------------------------------------------- direct sum (direct.go:18-48)

constexpr int kDirThreads = 128;

__global__ __launch_bounds__(kDirThreads) void k_direct_fp64(int64_t n, const double *__restrict__ px,
                                                             const double *__restrict__ py, const double *__restrict__ pz,
                                                             const double *__restrict__ mass,
                                                             const uint8_t *__restrict__ kind, double eps2, int dm_off,
                                                             const int64_t *__restrict__ targets, int64_t ntargets,
                                                             double *ax, double *ay, double *az) {
    __shared__ double s_x[kDirThreads], s_y[kDirThreads], s_z[kDirThreads], s_m[kDirThreads];
    __shared__ uint8_t s_skip[kDirThreads];
    int64_t q = int64_t(blockIdx.x) * kDirThreads + threadIdx.x;
    bool valid = q < ntargets;
    int64_t i = valid ? (targets ? targets[q] : q) : 0;
    double xi = px[i], yi = py[i], zi = pz[i];
    double fax = 0, fay = 0, faz = 0;
    for (int64_t j0 = 0; j0 < n; j0 += kDirThreads) {
        int64_t j = j0 + threadIdx.x;
        if (j < n) {
            uint8_t kd = kind ? kind[j] : 0;
            s_x[threadIdx.x] = px[j];
            s_y[threadIdx.x] = py[j];
            s_z[threadIdx.x] = pz[j];
            s_m[threadIdx.x] = mass[j];
            s_skip[threadIdx.x] = kd == GBH_BLACK_HOLE || (dm_off && kd == GBH_DARK_MATTER);
        }
        __syncthreads();
        int64_t cnt = n - j0 < kDirThreads ? n - j0 : kDirThreads;
        for (int t = 0; t < cnt; ++t) {
            if (j0 + t == i || s_skip[t]) continue;
            double dx = s_x[t] - xi, dy = s_y[t] - yi, dz = s_z[t] - zi;
            double re2 = dx * dx + dy * dy + dz * dz + eps2;
            double f = s_m[t] / (re2 * sqrt(re2));
            fax += f * dx;
            fay += f * dy;
            faz += f * dz;
        }
        __syncthreads();
    }
    if (!valid) return;
    bool hole = kind && kind[i] == GBH_BLACK_HOLE;
    ax[q] = hole ? 0 : fax;
    ay[q] = hole ? 0 : fay;
    az[q] = hole ? 0 : faz;
}

// ---------------------------------------------------------------- potential (potential.go:16-81)

__device__ __forceinline__ double schwarzschild(double m, double c) { return c <= 0 ? 0 : 2 * m / (c * c); }

__device__ __forceinline__ double pair_rs(uint8_t ki, double mi, uint8_t kj, double mj, double c) {
    bool hi = ki == GBH_BLACK_HOLE, hj = kj == GBH_BLACK_HOLE;
    if (c <= 0 || hi == hj) return 0;
    return hi ? schwarzschild(mi, c) : schwarzschild(mj, c);
}

__device__ __forceinline__ double pair_potential(double mi, double mj, double r2, double eps2, double rs) {
    double re = sqrt(r2 + eps2);
    if (rs == 0) return -mi * mj / re;
    if (re >= 1.5 * rs) return -mi * mj / (re - rs);
    return mi * mj * (-2 / rs + 4 / (rs * rs) * (re - 1.5 * rs));
}

// PotentialEnergyParallel (diag.go:42-64): row i of the exact pair sum, sum over j > i of the
// pair model's potential in ascending j, kinds and liveness as the reference reads them (all
// bodies). The rows are then added in ascending i (the reference adds its ParallelFor chunks
// in completion order, so only round-off may differ).
__global__ __launch_bounds__(kDirThreads) void k_pot_exact_rows(int64_t n, const double *__restrict__ px,
                                                                const double *__restrict__ py,
                                                                const double *__restrict__ pz,
                                                                const double *__restrict__ mass,
                                                                const uint8_t *__restrict__ kind, double eps2, double c,
                                                                int dm_off, double *rows) {
    __shared__ double s_x[kDirThreads], s_y[kDirThreads], s_z[kDirThreads], s_m[kDirThreads];
    __shared__ uint8_t s_k[kDirThreads];
    const int64_t i0 = int64_t(blockIdx.x) * kDirThreads;
    const int64_t i = i0 + threadIdx.x;
    const bool act = i < n;
    const uint8_t ki = act && kind ? kind[i] : 0;
    const double xi = act ? px[i] : 0, yi = act ? py[i] : 0, zi = act ? pz[i] : 0, mi = act ? mass[i] : 0;
    const double smi = dm_off && ki == GBH_DARK_MATTER ? 0.0 : mi;
    double part = 0;
    for (int64_t j0 = i0 + 1; j0 < n; j0 += kDirThreads) {
        int64_t j = j0 + threadIdx.x;
        if (j < n) {
            s_x[threadIdx.x] = px[j];
            s_y[threadIdx.x] = py[j];
            s_z[threadIdx.x] = pz[j];
            s_m[threadIdx.x] = mass[j];
            s_k[threadIdx.x] = kind ? kind[j] : 0;
        }
        __syncthreads();
        int cnt = n - j0 < kDirThreads ? int(n - j0) : kDirThreads;
        for (int t = 0; t < cnt; ++t) {
            if (j0 + t <= i) continue;
            double dx = s_x[t] - xi, dy = s_y[t] - yi, dz = s_z[t] - zi;
            uint8_t kj = s_k[t];
            double rs = pair_rs(ki, mi, kj, s_m[t], c);
            double smj = dm_off && kj == GBH_DARK_MATTER ? 0.0 : s_m[t];
            part += pair_potential(smi, smj, dx * dx + dy * dy + dz * dz, eps2, rs);
        }
        __syncthreads();
    }
    if (act) rows[i] = part;
}

__global__ void k_pot_exact_final(int64_t n, const double *__restrict__ rows, double *out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double sum = 0;
    for (int64_t i = 0; i < n; ++i) sum += rows[i];
    *out = sum;
}

// holePotential, potential.go:84-96.
__device__ double hole_potential(int64_t i, const double *px, const double *py, const double *pz, const double *mass,
                                 const uint8_t *kind, const int32_t *holes, int32_t nholes, double eps2, double c,
                                 int dm_off) {
    double x = px[i], y = py[i], z = pz[i], u = 0;
    uint8_t ki = kind ? kind[i] : 0;
    double smi = (dm_off && ki == GBH_DARK_MATTER) ? 0.0 : mass[i];
    for (int32_t t = 0; t < nholes; ++t) {
        int32_t h = holes[t];
        if (h == i) continue;
        double dx = px[h] - x, dy = py[h] - y, dz = pz[h] - z;
        double rs = pair_rs(ki, mass[i], GBH_BLACK_HOLE, mass[h], c);
        u += pair_potential(smi, mass[h], dx * dx + dy * dy + dz * dz, eps2, rs);
    }
    return u;
}

// Per sorted star: sm[k] * walkPotential(k) - holePotential(order[k]); block partial sums.
__global__ __launch_bounds__(kThreads) void k_potential_walk(const DevInfo *info, const gbh_node *__restrict__ nodes,
                                                             const double *__restrict__ sx, const double *__restrict__ sy,
                                                             const double *__restrict__ sz, const double *__restrict__ sm,
                                                             const int32_t *__restrict__ order, const double *px,
                                                             const double *py, const double *pz, const double *mass,
                                                             const uint8_t *kind, const int32_t *holes, int32_t nholes,
                                                             double eps2, double c, int dm_off, int quad, double *part,
                                                             const int32_t *__restrict__ sid_sorted,
                                                             const SysGeo *__restrict__ geo, DevInfo *err_info) {
    int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    int64_t ns = info->nstars, nn = info->nnodes;
    double v = 0;
    if (k < ns) {
        double x = sx[k], y = sy[k], z = sz[k], psi = 0;
        int64_t steps = 0;
        const int32_t root = sid_sorted ? geo[sid_sorted[k]].root : 0;
        for (int32_t i = nn > 0 ? root : -1; i >= 0;) {
            if (++steps > nn || i >= nn) {
                dev_error(err_info, 2);
                break;
            }
            const gbh_node &nd = nodes[i];
            double dx = nd.x - x, dy = nd.y - y, dz = nd.z - z;
            double d2 = dx * dx + dy * dy + dz * dz;
            if (d2 >= nd.crit2) {
                double inv = 1 / (d2 + eps2);
                psi += nd.m * sqrt(inv);
                if (quad) {
                    double dqd = nd.qxx * dx * dx + nd.qyy * dy * dy + nd.qzz * dz * dz +
                                 2 * (nd.qxy * dx * dy + nd.qxz * dx * dz + nd.qyz * dy * dz);
                    psi += 0.5 * dqd * inv * inv * sqrt(inv);
                }
                i = nd.next;
                continue;
            }
            if (nd.first >= 0) {
                i = nd.first;
                continue;
            }
            for (int32_t j = nd.lo; j < nd.hi; ++j) {
                if (j == k) continue;
                double ddx = sx[j] - x, ddy = sy[j] - y, ddz = sz[j] - z;
                psi += sm[j] / sqrt(ddx * ddx + ddy * ddy + ddz * ddz + eps2);
            }
            i = nd.next;
        }
        v = sm[k] * psi - (nholes ? hole_potential(order[k], px, py, pz, mass, kind, holes, nholes, eps2, c, dm_off) : 0.0);
    }
    // Deterministic block sum (tree order over threads).
    __shared__ double s[kThreads];
    s[threadIdx.x] = v;
    __syncthreads();
    for (int o = kThreads / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = s[0];
}

// Sum of the block parts plus the hole terms (potential.go:31-41); U = -sum / 2.
__global__ void k_potential_final(int64_t nparts, const double *part, const DevInfo *info,
                                  const double *__restrict__ sx, const double *__restrict__ sy,
                                  const double *__restrict__ sz, const double *__restrict__ sm, const double *px,
                                  const double *py, const double *pz, const double *mass, const uint8_t *kind,
                                  const int32_t *holes, int32_t nholes, double eps2, double c, int dm_off, double *u) {
    __shared__ double s[kThreads];
    double v = 0;
    for (int64_t b = threadIdx.x; b < nparts; b += blockDim.x) v += part[b];
    int64_t ns = info->nstars;
    for (int32_t t = 0; t < nholes; ++t) {
        int32_t i = holes[t];
        double x = px[i], y = py[i], z = pz[i];
        double rs = schwarzschild(mass[i], c);
        for (int64_t k = threadIdx.x; k < ns; k += blockDim.x) {
            double dx = sx[k] - x, dy = sy[k] - y, dz = sz[k] - z;
            v -= pair_potential(mass[i], sm[k], dx * dx + dy * dy + dz * dz, eps2, rs);
        }
        if (threadIdx.x == 0) v -= hole_potential(i, px, py, pz, mass, kind, holes, nholes, eps2, c, dm_off);
    }
    s[threadIdx.x] = v;
    __syncthreads();
    for (int o = kThreads / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) *u = -s[0] / 2;
}

constexpr int kFlagBlocksMax = 1024;

}  // namespace

// ---------------------------------------------------------------- forests (many systems)

namespace {

__global__ void k_sys_init(int32_t nsys, SysGeo *geo, DevInfo *info) {
    int32_t s = int32_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (s == 0) {  // cleared before k_sys_final may report a non-finite system
        info->err = 0;
        info->err_where = 0;
    }
    if (s >= nsys) return;
    for (int c = 0; c < 3; ++c) {
        geo[s].kmin[c] = LLONG_MAX;
        geo[s].kmax[c] = LLONG_MIN;
    }
}

// Star flags, alive holes' accelerations zeroed, and each system's bbox (ordered keys, one
// warp-wide atomic per quantity when the warp's stars share a system).
__global__ __launch_bounds__(kThreads) void k_flags_sys(int64_t n, const double *__restrict__ px,
                                                        const double *__restrict__ py, const double *__restrict__ pz,
                                                        const double *__restrict__ mass,
                                                        const uint8_t *__restrict__ kind,
                                                        const uint8_t *__restrict__ alive,
                                                        const uint16_t *__restrict__ sys_of, uint32_t *__restrict__ flag,
                                                        SysGeo *geo, double *ax, double *ay, double *az,
                                                        Pos4 *__restrict__ pos4) {
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    bool st = false;
    int s = -1;
    long long k[3] = {LLONG_MAX, LLONG_MAX, LLONG_MAX};
    if (i < n) {
        uint8_t al = alive ? alive[i] : 1, kd = kind ? kind[i] : 0;
        st = is_star(al, kd);
        flag[i] = st;
        if (st) {
            s = sys_of[i];
            const double vx = px[i], vy = py[i], vz = pz[i], m = mass ? mass[i] : 0.0;
            pos4[i] = Pos4{vx, vy, vz, m};
            k[0] = mass && !isfinite(m) ? LLONG_MAX : ord_key(vx);  // as in k_flags_bbox
            k[1] = ord_key(vy);
            k[2] = ord_key(vz);
        } else if (al && kd == GBH_BLACK_HOLE) {
            ax[i] = 0;
            ay[i] = 0;
            az[i] = 0;
        }
    }
    unsigned m = __match_any_sync(0xffffffffu, s);
    int lane = threadIdx.x & 31;
    bool uniform = m == 0xffffffffu;
    if (uniform) {
        if (s < 0) return;
        long long mn[3] = {k[0], k[1], k[2]}, mx[3] = {k[0], k[1], k[2]};
        for (int c = 0; c < 3; ++c)
            for (int o = 16; o > 0; o >>= 1) {
                mn[c] = min(mn[c], __shfl_xor_sync(0xffffffffu, mn[c], o));
                mx[c] = max(mx[c], __shfl_xor_sync(0xffffffffu, mx[c], o));
            }
        if (lane == 0)
            for (int c = 0; c < 3; ++c) {
                atomicMin(&geo[s].kmin[c], mn[c]);
                atomicMax(&geo[s].kmax[c], mx[c]);
            }
    } else if (s >= 0) {
        for (int c = 0; c < 3; ++c) {
            atomicMin(&geo[s].kmin[c], k[c]);
            atomicMax(&geo[s].kmax[c], k[c]);
        }
    }
}

// Per system: root cube (build.go:19-21), FP32 views, opening bases, sorted star range.
// Thread 0 also resets the per-build scalars.
__global__ void k_sys_final(int32_t nsys, int64_t n, const int64_t *__restrict__ sys_off,
                            const uint32_t *__restrict__ scan, const uint8_t *kind, const uint8_t *alive, double theta,
                            SysGeo *geo, DevInfo *info) {
    int32_t s = int32_t(blockIdx.x) * blockDim.x + threadIdx.x;
    int64_t total = n > 0 ? int64_t(scan[n - 1]) + (is_star(alive ? alive[n - 1] : 1, kind ? kind[n - 1] : 0) ? 1 : 0)
                          : 0;
    if (s == 0) {
        info->theta = theta;
        info->nstars = total;
        info->nnodes = 0;
        info->work = 0;
        info->nleaves = 0;
    }
    if (s >= nsys) return;
    SysGeo &g = geo[s];
    double mn[3], mx[3];
    for (int c = 0; c < 3; ++c) {
        mn[c] = ord_val(g.kmin[c]);
        mx[c] = ord_val(g.kmax[c]);
    }

    double side = fmax(mx[0] - mn[0], fmax(mx[1] - mn[1], mx[2] - mn[2]));
    side = fmax(side * (1 + 1e-9), 1e-12);
    g.minx = mn[0];
    g.miny = mn[1];
    g.minz = mn[2];
    g.side = side;
    g.scale = double(1 << kMortonBits) / side;
    for (int c = 0; c < 3; ++c) {
        float h = __double2float_rn(mn[c]);
        g.min_hi[c] = h;
        g.min_lo[c] = __double2float_rn(mn[c] - double(h));
    }
    float sh = __double2float_rn(side);
    g.side_hi = sh;
    g.side_lo = __double2float_rn(side - double(sh));
    double half = side / 2;
    for (int L = 0; L <= kMaxLevel; ++L, half = half / 2) g.crit_base[L] = __double2float_rn(2 * half / theta);
    int64_t a = sys_off[s], b = sys_off[s + 1];
    g.star_lo = int32_t(a < n ? int64_t(scan[a]) : total);
    g.star_hi = int32_t(b < n ? int64_t(scan[b]) : total);
    // an empty system keeps its initial keys (a NaN box); a system with stars must be finite
    if (g.star_hi > g.star_lo && !(isfinite(mn[0]) && isfinite(mn[1]) && isfinite(mn[2]) && isfinite(mx[0]) &&
                                   isfinite(mx[1]) && isfinite(mx[2])))
        dev_error(info, kErrNonFinite);
}

// Each star's Morton key in its own system's cube (build.go:19-31).
__global__ __launch_bounds__(kThreads) void k_compact_keys_sys(int64_t n, const double *__restrict__ px,
                                                               const double *__restrict__ py,
                                                               const double *__restrict__ pz,
                                                               const uint8_t *__restrict__ kind,
                                                               const uint8_t *__restrict__ alive,
                                                               const uint16_t *__restrict__ sys_of,
                                                               const uint32_t *__restrict__ scan,
                                                               const SysGeo *__restrict__ geo,
                                                               uint64_t *__restrict__ keys, int32_t *__restrict__ order) {
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (!is_star(alive ? alive[i] : 1, kind ? kind[i] : 0)) return;
    const SysGeo &g = geo[sys_of[i]];
    double sc = g.scale;
    uint64_t k = spread(cell(px[i], g.minx, sc)) << 2 | spread(cell(py[i], g.miny, sc)) << 1 |
                 spread(cell(pz[i], g.minz, sc));
    uint32_t pos = scan[i];
    keys[pos] = k;
    order[pos] = int32_t(i);
}

// Roots (the pre-order index of a system's first star chain) and the gsize-star groups of the
// mixed walk, which never straddle two systems.
__global__ void k_sys_layout(int32_t nsys, int32_t gsize, const uint32_t *__restrict__ base, SysGeo *geo,
                             DevInfo *info) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    int32_t groups = 0;
    for (int32_t s = 0; s < nsys; ++s) {
        SysGeo &g = geo[s];
        int32_t cnt = g.star_hi - g.star_lo;
        g.root = cnt > 0 ? int32_t(base[g.star_lo]) : -1;
        g.group_lo = groups;
        g.ngroups = (cnt + gsize - 1) / gsize;
        groups += g.ngroups;
    }
    info->ngroups = uint32_t(groups);
}

__global__ void k_sys_groups(int32_t nsys, int32_t gsize, const SysGeo *__restrict__ geo, int4 *__restrict__ groups) {
    int32_t s = int32_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (s >= nsys) return;
    const SysGeo &g = geo[s];
    for (int32_t q = 0; q < g.ngroups; ++q) {
        int32_t start = g.star_lo + gsize * q;
        int32_t cnt = g.star_hi - start < gsize ? g.star_hi - start : gsize;
        groups[g.group_lo + q] = make_int4(start, cnt, g.root, 0);
    }
}

}  // namespace

int64_t scan_tmp_size(int64_t n) {
    int64_t total = 0;
    for (int64_t t = (n + kScanTile - 1) / kScanTile; t > 1; t = (t + kScanTile - 1) / kScanTile) total += t;
    return total + 64;
}

cudaError_t scan_u32(const Launch &L, const uint32_t *in, uint32_t *out, int64_t n, uint32_t *tmp, int64_t tmp_cap) {
    return scan_rec(L, in, out, n, nullptr, tmp, tmp_cap);
}

static cudaError_t scan_dyn(const Launch &L, const uint32_t *in, uint32_t *out, int64_t n, const int64_t *ndyn,
                            uint32_t *tmp, int64_t tmp_cap) {
    return scan_rec(L, in, out, n, ndyn, tmp, tmp_cap);
}

void tree_free(TreeBufs &b) {
    void *ptrs[] = {b.flag, b.pos4, b.bbox_part, b.keys, b.keys_alt, b.order, b.order_alt, b.hist, b.os_state, b.hs_state, b.sx, b.sy, b.sz, b.sm,
                    b.st_hi, b.st_lo, b.st_off, b.chain_cnt, b.leaves, b.targets, b.geo, b.sid_sorted, b.groups, b.gcost, b.gperm, b.pre_parent, b.pre_info, b.pre_nchild, b.pre_mask, b.pre_ref, b.pre_star, b.nodes,
                    b.n_parent, b.n_info, b.n_arrive, b.pnodes, b.mnodes, b.mrange, b.lnode, b.walk_ctr, b.scan_tmp, b.info, b.part_acc};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    b = TreeBufs{};
}

// Worst-case node count: at most n leaves, and at each of the 22 levels at most n/(leaf+1)
// cells hold more than leaf stars (only those have children).
static int64_t node_capacity(int64_t n, int leaf) { return n + 22 * (n / (leaf + 1) + 1) + 1; }

cudaError_t tree_alloc(TreeBufs &b, int64_t n, int leaf, int32_t nsys) {
    int64_t need_nodes = node_capacity(n, leaf);
    if (nsys < 1) nsys = 1;
    if (n <= b.cap_n && need_nodes <= b.cap_nodes && nsys <= b.cap_sys && n / 32 + nsys + 1 <= b.cap_groups) {
        b.nsys = nsys;
        return split_reserve(b, n);
    }
    if (nsys > b.cap_sys) b.cap_sys = 0;
    int64_t cn = n > b.cap_n ? n + n / 4 : b.cap_n;  // grow by 1.25x like gpuBuffers.ensure (gpu_darwin.go:164-177)
    int64_t cnodes = need_nodes > b.cap_nodes ? node_capacity(cn, leaf) : b.cap_nodes;
    if (cnodes < need_nodes) cnodes = need_nodes;
    const int64_t gen = b.generation + 1;
    tree_free(b);
    b.generation = gen;
    cn = cn < 1 ? 1 : cn;
    int64_t rs_tiles = (cn + kRsTile - 1) / kRsTile;
    int64_t scan_cap = scan_tmp_size(cnodes > cn * 1 ? cnodes : cn);
    int64_t scan_cap2 = scan_tmp_size(rs_tiles * kRsBins);
    if (scan_cap2 > scan_cap) scan_cap = scan_cap2;
    b.scan_tmp_cap = scan_cap;
    cudaError_t e = cudaSuccess;
#define GBH_ALLOC(ptr, count)                                                     \
    do {                                                                          \
        if (e == cudaSuccess) e = dev_alloc(&(ptr), sizeof(*(ptr)) * size_t(count)); \
    } while (0)
    GBH_ALLOC(b.flag, cn);
    GBH_ALLOC(b.pos4, cn);
    GBH_ALLOC(b.bbox_part, kFlagBlocksMax * 6);
    GBH_ALLOC(b.keys, cn);
    GBH_ALLOC(b.keys_alt, cn);
    GBH_ALLOC(b.order, cn);
    GBH_ALLOC(b.order_alt, cn);
    GBH_ALLOC(b.hist, rs_tiles * kRsBins);
    GBH_ALLOC(b.sx, cn);
    GBH_ALLOC(b.sy, cn);
    GBH_ALLOC(b.sz, cn);
    GBH_ALLOC(b.sm, cn);
    GBH_ALLOC(b.st_hi, cn);
    GBH_ALLOC(b.st_lo, cn);
    GBH_ALLOC(b.st_off, cn);
    GBH_ALLOC(b.chain_cnt, cn * 2);  // counts, then their scan
    GBH_ALLOC(b.leaves, cn);
    GBH_ALLOC(b.targets, cn);
    const int32_t csys = nsys + nsys / 4 + 1;
    const int64_t cgroups = cn / 32 + csys + 1;  // groups of 32 or 64 stars
    GBH_ALLOC(b.geo, csys);
    GBH_ALLOC(b.sid_sorted, cn);
    GBH_ALLOC(b.groups, cgroups);
    GBH_ALLOC(b.gcost, cgroups);
    GBH_ALLOC(b.gperm, cgroups + 1);
    GBH_ALLOC(b.pre_parent, cnodes);
    GBH_ALLOC(b.pre_info, cnodes);
    GBH_ALLOC(b.pre_nchild, cnodes);
    GBH_ALLOC(b.pre_mask, cnodes);
    GBH_ALLOC(b.pre_ref, cnodes);
    GBH_ALLOC(b.pre_star, cnodes);
    GBH_ALLOC(b.nodes, cnodes);
    GBH_ALLOC(b.n_parent, cnodes);
    GBH_ALLOC(b.n_info, cnodes);
    GBH_ALLOC(b.n_arrive, cnodes);
    GBH_ALLOC(b.pnodes, cnodes);
    GBH_ALLOC(b.mnodes, cnodes);
    GBH_ALLOC(b.mrange, cnodes);
    GBH_ALLOC(b.lnode, cnodes);
    GBH_ALLOC(b.walk_ctr, 16);
    GBH_ALLOC(b.scan_tmp, scan_cap);
    // single-pass scans of larger states: the digit tables of the three-launch passes (10 with a
    // forest's system digits) and the build's three other scans, each 2 words of counter and the
    // 64-bit look-back words of its tiles
    const int64_t hs_words = kOsPassesMax * (2 + 2 * os_scan_tiles(rs_tiles * kRsBins)) +
                             kOsScans * (2 + 2 * os_scan_tiles(cn > cnodes ? cn : cnodes));
    GBH_ALLOC(b.hs_state, hs_words);
    int64_t os_words = 0;
    if (cn <= kOsMaxN) {  // node capacity stays below 2^30 too (at most 12 nodes a body)
        const int64_t stiles = os_scan_tiles(cn > cnodes ? cn : cnodes);
        os_words = kOsHistWords + kOsCtrWords + 2 * kOsScans * stiles +
                   kOsPassesMax * os_sort_tiles(cn, os_items(cn)) * kRsBins;
        GBH_ALLOC(b.os_state, os_words);
    }
    GBH_ALLOC(b.info, 1);
#undef GBH_ALLOC
    if (e != cudaSuccess) {
        tree_free(b);
        return e;
    }
    b.cap_n = cn;
    b.cap_nodes = cnodes;
    b.os_words = os_words;
    b.hs_words = hs_words;
    b.cap_sys = csys;
    b.cap_groups = cgroups;
    b.nsys = nsys;
    // no launch order yet: gperm[cap_groups] = -1 matches no group count
    if ((e = cudaMemset(b.gperm, 0xff, sizeof(int32_t) * size_t(cgroups + 1))) != cudaSuccess) return e;
    if ((e = cudaMemset(b.info, 0, sizeof(DevInfo))) != cudaSuccess) return e;
    return split_reserve(b, n);
}

#define GBH_LAUNCH_CHECK()                         \
    do {                                           \
        ++*L.count;                                \
        cudaError_t e_ = cudaGetLastError();       \
        if (e_ != cudaSuccess) return e_;          \
    } while (0)

// Word offset of the sort's look-back words in os_state (after the histograms, the counters and
// the scans' 64-bit words).
static int64_t os_scan_cap(const TreeBufs &b) { return os_scan_tiles(b.cap_n > b.cap_nodes ? b.cap_n : b.cap_nodes); }
static int64_t os_sort_base(const TreeBufs &b) { return kOsHistWords + kOsCtrWords + 2 * kOsScans * os_scan_cap(b); }

// Single-pass exclusive scan `which` (0 flags, 1 chain counts, 2 child counts) of a build.
static cudaError_t scan_lb(const Launch &L, TreeBufs &b, int which, const uint32_t *in, uint32_t *out, int64_t n,
                           const int64_t *ndyn) {
    const int64_t tiles = os_scan_tiles(n);
    if (tiles < 1) return cudaSuccess;
    uint32_t *ctr = b.os_state + kOsHistWords + kOsScanCtr + which;
    unsigned long long *st =
        reinterpret_cast<unsigned long long *>(b.os_state + kOsHistWords + kOsCtrWords) + which * os_scan_cap(b);
    k_scan_lb<<<unsigned(tiles), kScanThreads, 0, L.stream>>>(in, out, n, ndyn, ctr, st, b.info);
    ++*L.count;
    return cudaGetLastError();
}

// Single-pass scans of larger states (hs_state), in place of the three-launch scans: pass p's
// digit table (rs_tiles x 256 entries: at 1M bodies 81 tiles, a look-back of three round trips),
// and scan `which` (0 flags, 1 chain counts, 2 child counts) of n entries.
static cudaError_t scan_hs(const Launch &L, TreeBufs &b, uint32_t *base, const uint32_t *in, uint32_t *out, int64_t n,
                           const int64_t *ndyn) {
    const int64_t tiles = os_scan_tiles(n);
    if (tiles < 1) return cudaSuccess;
    k_scan_lb<<<unsigned(tiles), kScanThreads, 0, L.stream>>>(in, out, n, ndyn, base,
                                                              reinterpret_cast<unsigned long long *>(base + 2), b.info);
    ++*L.count;
    return cudaGetLastError();
}
static int64_t hs_pass_words(const TreeBufs &b) { return 2 + 2 * os_scan_tiles(rs_sort_tiles(b.cap_n) * kRsBins); }
static cudaError_t scan_hist(const Launch &L, TreeBufs &b, int p, uint32_t ntiles) {
    return scan_hs(L, b, b.hs_state + int64_t(p) * hs_pass_words(b), b.hist, b.hist, int64_t(ntiles) * kRsBins,
                   nullptr);
}
static cudaError_t scan_big(const Launch &L, TreeBufs &b, int which, const uint32_t *in, uint32_t *out, int64_t n,
                            const int64_t *ndyn) {
    const int64_t stiles = os_scan_tiles(b.cap_n > b.cap_nodes ? b.cap_n : b.cap_nodes);
    uint32_t *base = b.hs_state + kOsPassesMax * hs_pass_words(b) + int64_t(which) * (2 + 2 * stiles);
    return scan_hs(L, b, base, in, out, n, ndyn);
}

cudaError_t tree_build(const Launch &L, TreeBufs &b, int64_t n, const double *px, const double *py, const double *pz,
                       const double *mass, const uint8_t *kind, const uint8_t *alive, double *ax, double *ay,
                       double *az, double theta, int leaf, int dm_off, bool exact, bool plain_records,
                       const uint16_t *sys_of, const int64_t *sys_off) {
    cudaStream_t s = L.stream;
    const int64_t cap = b.cap_n;
    const bool forest = b.nsys > 1;
    if (forest && (!sys_of || !sys_off)) return cudaErrorInvalidValue;
    cudaError_t e;
    // one-sweep sort and single-pass scans (capacity up to kOsMaxN bodies): histograms, tile
    // counters and the look-back words of the passes this tree build runs start at zero
    const bool os = b.os_state != nullptr;
    // a forest then sorts stably by system id, one pass per byte: up to 256 systems the high
    // byte is 0 everywhere, and that pass (a stable pass over equal digits) is left out
    const int sid_passes = forest ? (b.nsys > 256 ? 2 : 1) : 0;
    const int npass = 8 + sid_passes;
    // the passes ping-pong between the two buffers and end in keys / order: with an odd count
    // the keys are formed in the other pair
    uint64_t *const keys0 = (npass & 1) ? b.keys_alt : b.keys;
    int32_t *const order0 = (npass & 1) ? b.order_alt : b.order;
    const int os_k = os_items(cap);  // keys a thread of a one-sweep pass ranks
    const int64_t os_tiles = os_sort_tiles(cap, os_k);
    if (os) {
        const int64_t words = os_sort_base(b) + int64_t(npass) * os_tiles * kRsBins;
        if ((e = cudaMemsetAsync(b.os_state, 0, sizeof(uint32_t) * size_t(words), s)) != cudaSuccess) return e;
    } else if ((e = cudaMemsetAsync(b.hs_state, 0, sizeof(uint32_t) * size_t(b.hs_words), s)) != cudaSuccess) {
        return e;
    }
    if (!forest) {
        // collect + bbox (build.go:62-113)
        unsigned fb = blocks_for(n, kThreads);
        if (fb > unsigned(kFlagBlocksMax)) fb = kFlagBlocksMax;
        k_flags_bbox<<<fb, kThreads, 0, s>>>(n, px, py, pz, mass, kind, alive, b.flag, b.bbox_part, ax, ay, az,
                                             b.info, b.pos4);
        GBH_LAUNCH_CHECK();
        e = os ? scan_lb(L, b, 0, b.flag, b.flag, n, nullptr) : scan_big(L, b, 0, b.flag, b.flag, n, nullptr);
        if (e != cudaSuccess) return e;
        k_bbox_final<<<1, kFinalThreads, 0, s>>>(int(fb), b.bbox_part, n, b.flag, kind, alive, theta, b.info, b.geo);
        GBH_LAUNCH_CHECK();
        k_compact_keys<<<blocks_for(n, kThreads), kThreads, 0, s>>>(n, px, py, pz, kind, alive, b.flag, b.info, keys0,
                                                                    order0);
        GBH_LAUNCH_CHECK();
    } else {
        // collect per system: each system gets its own root cube and keys (build.go:11-31)
        const unsigned sb = blocks_for(b.nsys, 128);
        k_sys_init<<<sb, 128, 0, s>>>(b.nsys, b.geo, b.info);
        GBH_LAUNCH_CHECK();
        k_flags_sys<<<blocks_for(n, kThreads), kThreads, 0, s>>>(n, px, py, pz, mass, kind, alive, sys_of, b.flag,
                                                                 b.geo, ax, ay, az, b.pos4);
        GBH_LAUNCH_CHECK();
        e = os ? scan_lb(L, b, 0, b.flag, b.flag, n, nullptr) : scan_big(L, b, 0, b.flag, b.flag, n, nullptr);
        if (e != cudaSuccess) return e;
        k_sys_final<<<sb, 128, 0, s>>>(b.nsys, n, sys_off, b.flag, kind, alive, theta, b.geo, b.info);
        GBH_LAUNCH_CHECK();
        k_compact_keys_sys<<<blocks_for(n, kThreads), kThreads, 0, s>>>(n, px, py, pz, kind, alive, sys_of, b.flag,
                                                                        b.geo, keys0, order0);
        GBH_LAUNCH_CHECK();
    }
    // radix sort (morton.go:25-49): 8 stable passes, ping-pong, result back in keys/order
    const uint32_t ntiles = uint32_t((cap + kRsTile - 1) / kRsTile);
    uint64_t *kin = keys0, *kout = keys0 == b.keys ? b.keys_alt : b.keys;
    int32_t *vin = order0, *vout = order0 == b.order ? b.order_alt : b.order;
    if (os) {
        // forest: then stably by system, (system, key) order, each system's stars contiguous
        uint32_t *ghist = b.os_state, *ctr = b.os_state + kOsHistWords;
        unsigned hb = unsigned(L.num_sms > 0 ? L.num_sms : 152) * kOsHistBlocksPerSm;
        if (int64_t(hb) * kRsThreads > cap) hb = blocks_for(cap, kRsThreads);
        if (forest) k_os_hist<true><<<hb, kRsThreads, 0, s>>>(kin, vin, sys_of, b.info, ghist);
        else k_os_hist<false><<<hb, kRsThreads, 0, s>>>(kin, vin, nullptr, b.info, ghist);
        GBH_LAUNCH_CHECK();
        for (int p = 0; p < npass; ++p) {
            uint32_t *st = b.os_state + os_sort_base(b) + int64_t(p) * os_tiles * kRsBins;
            const uint16_t *so = p < 8 ? nullptr : sys_of;
            const int shift = p < 8 ? 8 * p : 8 * (p - 8);
            const unsigned g = unsigned(os_tiles);
            const uint32_t *gh = ghist + p * kRsBins;
            if (p < 8) {
                if (os_k == 4) k_os_pass<false, 4><<<g, kRsThreads, 0, s>>>(kin, vin, kout, vout, so, b.info, shift, gh, ctr + p, st);
                else if (os_k == 8) k_os_pass<false, 8><<<g, kRsThreads, 0, s>>>(kin, vin, kout, vout, so, b.info, shift, gh, ctr + p, st);
                else k_os_pass<false, 12><<<g, kRsThreads, 0, s>>>(kin, vin, kout, vout, so, b.info, shift, gh, ctr + p, st);
            } else {
                if (os_k == 4) k_os_pass<true, 4><<<g, kRsThreads, 0, s>>>(kin, vin, kout, vout, so, b.info, shift, gh, ctr + p, st);
                else if (os_k == 8) k_os_pass<true, 8><<<g, kRsThreads, 0, s>>>(kin, vin, kout, vout, so, b.info, shift, gh, ctr + p, st);
                else k_os_pass<true, 12><<<g, kRsThreads, 0, s>>>(kin, vin, kout, vout, so, b.info, shift, gh, ctr + p, st);
            }
            GBH_LAUNCH_CHECK();
            uint64_t *tk = kin;
            kin = kout;
            kout = tk;
            int32_t *tv = vin;
            vin = vout;
            vout = tv;
        }
    }
    for (int shift = 0; shift < 64 && !os; shift += 8) {
        k_rs_hist<false><<<ntiles, kRsThreads, 0, s>>>(kin, vin, nullptr, b.info, shift, ntiles, b.hist);
        GBH_LAUNCH_CHECK();
        if ((e = scan_hist(L, b, shift / 8, ntiles)) != cudaSuccess) return e;
        k_rs_scatter<false><<<ntiles, kRsThreads, 0, s>>>(kin, vin, kout, vout, nullptr, b.info, shift, ntiles, b.hist);
        GBH_LAUNCH_CHECK();
        uint64_t *tk = kin;
        kin = kout;
        kout = tk;
        int32_t *tv = vin;
        vin = vout;
        vout = tv;
    }
    if (forest && !os) {  // then stably by system: (system, key) order, each system's stars contiguous
        for (int shift = 0; shift < 8 * sid_passes; shift += 8) {
            k_rs_hist<true><<<ntiles, kRsThreads, 0, s>>>(kin, vin, sys_of, b.info, shift, ntiles, b.hist);
            GBH_LAUNCH_CHECK();
            if ((e = scan_hist(L, b, 8 + shift / 8, ntiles)) != cudaSuccess) return e;
            k_rs_scatter<true><<<ntiles, kRsThreads, 0, s>>>(kin, vin, kout, vout, sys_of, b.info, shift, ntiles,
                                                             b.hist);
            GBH_LAUNCH_CHECK();
            uint64_t *tk = kin;
            kin = kout;
            kout = tk;
            int32_t *tv = vin;
            vin = vout;
            vout = tv;
        }
    }
    // sorted copies (build.go:34-41)
    const unsigned nb = blocks_for(cap, kThreads);
    k_gather<<<nb, kThreads, 0, s>>>(b.info, b.order, b.pos4, kind, dm_off, exact ? 1 : 0, b.sx, b.sy, b.sz,
                                     b.sm, b.st_hi, b.st_lo, forest ? sys_of : nullptr, b.sid_sorted);
    GBH_LAUNCH_CHECK();
    // node set
    uint32_t *cnt = b.chain_cnt, *base = b.chain_cnt + cap;
    const int32_t *sid = forest ? b.sid_sorted : nullptr;
    k_chain_count<<<nb, kThreads, 0, s>>>(b.keys, b.info, sid, b.geo, leaf, cnt);
    GBH_LAUNCH_CHECK();
    e = os ? scan_lb(L, b, 1, cnt, base, cap, &b.info->nstars) : scan_big(L, b, 1, cnt, base, cap, &b.info->nstars);
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(b.pre_mask, 0, sizeof(uint32_t) * size_t(b.cap_nodes), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(b.pre_nchild, 0, sizeof(uint32_t) * size_t(b.cap_nodes), s);
    if (e != cudaSuccess) return e;
    k_chain_emit<<<nb, kThreads, 0, s>>>(b.keys, b.info, cnt, base, b.pre_parent, b.pre_info, b.pre_nchild, b.pre_mask,
                                         b.pre_star, b.leaves, sid, b.geo);
    GBH_LAUNCH_CHECK();
    e = os ? scan_lb(L, b, 2, b.pre_nchild, b.pre_nchild, b.cap_nodes, &b.info->nnodes)
           : scan_big(L, b, 2, b.pre_nchild, b.pre_nchild, b.cap_nodes, &b.info->nnodes);
    if (e != cudaSuccess) return e;
    const unsigned nbn = node_blocks(b.cap_nodes);
    k_ref_index<<<nbn, kThreads, 0, s>>>(b.info, base, b.pre_star, b.pre_parent, b.pre_info, b.pre_mask, b.pre_nchild,
                                         b.pre_ref, sid, b.geo, b.cap_nodes);
    GBH_LAUNCH_CHECK();
    k_emit_nodes<<<nbn, kThreads, 0, s>>>(b.keys, b.info, cnt, base, b.pre_star, b.pre_parent, b.pre_info, b.pre_mask,
                                          b.pre_nchild, b.pre_ref, b.nodes, b.n_parent, b.n_info, b.n_arrive, sid,
                                          b.geo, b.cap_nodes);
    GBH_LAUNCH_CHECK();
    if (forest) {
        k_sys_layout<<<1, 32, 0, s>>>(b.nsys, b.group == 32 ? 32 : 64, base, b.geo, b.info);
        GBH_LAUNCH_CHECK();
        k_sys_groups<<<blocks_for(b.nsys, 128), 128, 0, s>>>(b.nsys, b.group == 32 ? 32 : 64, b.geo, b.groups);
        GBH_LAUNCH_CHECK();
    }
    b.moments_exact = exact;
    if (!exact) return upsweep_fast(L, b, plain_records);
    k_upsweep<<<nb, kThreads, 0, s>>>(b.keys, b.info, cnt, base, b.pre_ref, b.sx, b.sy, b.sz, b.sm, b.nodes,
                                      b.n_parent, b.n_info, b.n_arrive, b.pnodes, b.mnodes, b.mrange, sid, b.geo,
                                      b.info);
    GBH_LAUNCH_CHECK();
    return cudaSuccess;
}

namespace {
__global__ __launch_bounds__(kThreads) void k_fault_link(const DevInfo *info, gbh_node *nodes, PNode *pnodes,
                                                         MNode *mnodes, LNode *lnode, int64_t cap) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= info->nnodes || i >= cap) return;
    if (nodes[i].next != -1 || nodes[i].first != -1) return;
    nodes[i].next = 0;
    pnodes[i].links.y = 0;
    mnodes[i].d.w = __int_as_float(0);
    lnode[i].a.w = fabsf(lnode[i].a.w);  // the list walk: the leaf becomes an inner node whose child is node 0
    lnode[i].b.w = __int_as_float(0);
}
}  // namespace

cudaError_t fault_link(const Launch &L, TreeBufs &b) {
    k_fault_link<<<blocks_for(b.cap_nodes, kThreads), kThreads, 0, L.stream>>>(b.info, b.nodes, b.pnodes, b.mnodes,
                                                                               b.lnode, b.cap_nodes);
    GBH_LAUNCH_CHECK();
    return cudaSuccess;
}

cudaError_t walk_fp64(const Launch &L, const TreeBufs &b, int64_t n, double eps2, int quad, double *ax, double *ay,
                      double *az, bool targets) {
    (void)n;
    k_walk_fp64<<<blocks_for(b.cap_n, kThreads), kThreads, 0, L.stream>>>(
        b.info, b.nodes, b.sx, b.sy, b.sz, b.sm, b.order, eps2, quad, ax, ay, az, targets ? b.targets : nullptr,
        b.nsys > 1 ? b.sid_sorted : nullptr, b.geo, b.info);
    GBH_LAUNCH_CHECK();
    return cudaSuccess;
}

cudaError_t kick(const Launch &L, int64_t n, double h, double *vx, double *vy, double *vz, const double *ax,
                 const double *ay, const double *az) {
    if (n == 0) return cudaSuccess;
    k_kick<<<blocks_for(n, kThreads), kThreads, 0, L.stream>>>(n, h, vx, vy, vz, ax, ay, az);
    GBH_LAUNCH_CHECK();
    return cudaSuccess;
}

cudaError_t kick_drift(const Launch &L, int64_t n, double h, double dt, double c, double *px, double *py, double *pz,
                       double *vx, double *vy, double *vz, const double *ax, const double *ay, const double *az) {
    if (n == 0) return cudaSuccess;
    const double inv_c2 = c > 0 ? 1 / (c * c) : 0.0;  // sim.go:335 (invC2)
    k_kick_drift<<<blocks_for(n, kThreads), kThreads, 0, L.stream>>>(n, h, dt, inv_c2, px, py, pz, vx, vy, vz, ax, ay,
                                                                     az);
    GBH_LAUNCH_CHECK();
    return cudaSuccess;
}

cudaError_t direct_fp64(const Launch &L, int64_t n, const double *px, const double *py, const double *pz,
                        const double *mass, const uint8_t *kind, double eps2, int dm_off, const int64_t *targets,
                        int64_t ntargets, double *ax, double *ay, double *az) {
    if (ntargets == 0 || n == 0) return cudaSuccess;
    k_direct_fp64<<<blocks_for(ntargets, kDirThreads), kDirThreads, 0, L.stream>>>(n, px, py, pz, mass, kind, eps2,
                                                                                  dm_off, targets, ntargets, ax, ay, az);
    GBH_LAUNCH_CHECK();
    return cudaSuccess;
}

// Potential from the mixed walk's psi (sorted order): the block sums of m_k psi_k minus each
// star's hole pairs, as k_potential_walk forms them from the FP64 walk.
__global__ __launch_bounds__(kThreads) void k_potential_parts_psi(const DevInfo *info, const int32_t *__restrict__ order,
                                                                  const double *__restrict__ psi, const double *px,
                                                                  const double *py, const double *pz,
                                                                  const double *mass, const uint8_t *kind,
                                                                  const int32_t *holes, int32_t nholes, double eps2,
                                                                  double c, int dm_off, double *part) {
    int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    double v = 0;
    if (k < info->nstars) {
        int32_t i = order[k];
        double smi = (dm_off && kind && kind[i] == GBH_DARK_MATTER) ? 0.0 : mass[i];
        v = smi * psi[k] - (nholes ? hole_potential(i, px, py, pz, mass, kind, holes, nholes, eps2, c, dm_off) : 0.0);
    }
    __shared__ double s[kThreads];
    s[threadIdx.x] = v;
    __syncthreads();
    for (int o = kThreads / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = s[0];
}

// U = -(parts - hole pairs) / 2, the hole-star pairs taken over the alive non-hole bodies in
// state order (k_potential_final takes them over the sorted copies).
__global__ void k_potential_final_state(int64_t nparts, const double *part, int64_t n, const double *px,
                                        const double *py, const double *pz, const double *mass, const uint8_t *kind,
                                        const uint8_t *alive, const int32_t *holes, int32_t nholes, double eps2,
                                        double c, int dm_off, double *u) {
    __shared__ double s[kThreads];
    double v = 0;
    for (int64_t b = threadIdx.x; b < nparts; b += blockDim.x) v += part[b];
    for (int32_t t = 0; t < nholes; ++t) {
        int32_t i = holes[t];
        double x = px[i], y = py[i], z = pz[i];
        double rs = schwarzschild(mass[i], c);
        for (int64_t j = threadIdx.x; j < n; j += blockDim.x) {
            uint8_t kj = kind ? kind[j] : 0;
            if (kj == GBH_BLACK_HOLE || (alive && !alive[j])) continue;
            double smj = (dm_off && kj == GBH_DARK_MATTER) ? 0.0 : mass[j];
            double dx = px[j] - x, dy = py[j] - y, dz = pz[j] - z;
            v -= pair_potential(mass[i], smj, dx * dx + dy * dy + dz * dz, eps2, rs);
        }
        if (threadIdx.x == 0) v -= hole_potential(i, px, py, pz, mass, kind, holes, nholes, eps2, c, dm_off);
    }
    s[threadIdx.x] = v;
    __syncthreads();
    for (int o = kThreads / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) *u = -s[0] / 2;
}

cudaError_t potential_exact_fp64(const Launch &L, int64_t n, const double *px, const double *py, const double *pz,
                                 const double *mass, const uint8_t *kind, double eps2, double c, int dm_off,
                                 double *rows, double *u_dev) {
    k_pot_exact_rows<<<blocks_for(n, kDirThreads), kDirThreads, 0, L.stream>>>(n, px, py, pz, mass, kind, eps2, c,
                                                                               dm_off, rows);
    GBH_LAUNCH_CHECK();
    k_pot_exact_final<<<1, 32, 0, L.stream>>>(n, rows, u_dev);
    GBH_LAUNCH_CHECK();
    return cudaSuccess;
}

cudaError_t potential_mixed(const Launch &L, const TreeBufs &b, int64_t n, const double *px, const double *py,
                            const double *pz, const double *mass, const uint8_t *kind, const uint8_t *alive,
                            const int32_t *holes, int32_t nholes, double eps2, double c, int dm_off, int quad,
                            double *psi, double *part, double *u_dev) {
    cudaError_t e = walk_mixed_potential(L, b, b.cap_n, float(eps2), quad, psi);
    if (e != cudaSuccess) return e;
    unsigned nb = blocks_for(b.cap_n, kThreads);
    k_potential_parts_psi<<<nb, kThreads, 0, L.stream>>>(b.info, b.order, psi, px, py, pz, mass, kind, holes, nholes,
                                                         eps2, c, dm_off, part);
    GBH_LAUNCH_CHECK();
    k_potential_final_state<<<1, kThreads, 0, L.stream>>>(nb, part, n, px, py, pz, mass, kind, alive, holes, nholes,
                                                          eps2, c, dm_off, u_dev);
    GBH_LAUNCH_CHECK();
    return cudaSuccess;
}

cudaError_t potential_fp64(const Launch &L, const TreeBufs &b, int64_t n, const double *px, const double *py,
                           const double *pz, const double *mass, const uint8_t *kind, const uint8_t *alive,
                           const int32_t *holes, int32_t nholes, double eps2, double c, int dm_off, int quad,
                           double *part, double *u_dev) {
    (void)n;
    (void)alive;
    unsigned nb = blocks_for(b.cap_n, kThreads);
    k_potential_walk<<<nb, kThreads, 0, L.stream>>>(b.info, b.nodes, b.sx, b.sy, b.sz, b.sm, b.order, px, py, pz, mass,
                                                    kind, holes, nholes, eps2, c, dm_off, quad, part,
                                                    b.nsys > 1 ? b.sid_sorted : nullptr, b.geo, b.info);
    GBH_LAUNCH_CHECK();
    k_potential_final<<<1, kThreads, 0, L.stream>>>(nb, part, b.info, b.sx, b.sy, b.sz, b.sm, px, py, pz, mass, kind,
                                                    holes, nholes, eps2, c, dm_off, u_dev);
    GBH_LAUNCH_CHECK();
    return cudaSuccess;
}

}  // namespace gbh

namespace gbh {

// ---------------------------------------------------------------- Morton order into caller-owned scratch

namespace {
inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// Star flags and per-block bbox partials, as k_flags_bbox but writing no accelerations.
__global__ __launch_bounds__(kThreads) void k_flags_bbox_noacc(int64_t n, const double *__restrict__ px,
                                                               const double *__restrict__ py,
                                                               const double *__restrict__ pz,
                                                               const uint8_t *__restrict__ kind,
                                                               const uint8_t *__restrict__ alive,
                                                               uint32_t *__restrict__ flag, double *__restrict__ part) {
    long long mn[3] = {LLONG_MAX, LLONG_MAX, LLONG_MAX}, mx[3] = {LLONG_MIN, LLONG_MIN, LLONG_MIN};
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
        bool st = is_star(alive ? alive[i] : 1, kind ? kind[i] : 0);
        flag[i] = st;
        if (st) {
            long long x = ord_key(px[i]), y = ord_key(py[i]), z = ord_key(pz[i]);
            mn[0] = min(mn[0], x);
            mx[0] = max(mx[0], x);
            mn[1] = min(mn[1], y);
            mx[1] = max(mx[1], y);
            mn[2] = min(mn[2], z);
            mx[2] = max(mx[2], z);
        }
    }
    block_minmax<kThreads>(mn, mx, part);
}
}  // namespace

size_t morton_sort_scratch_bytes(int64_t nmax) {
    int64_t tiles = (nmax + kRsTile - 1) / kRsTile;
    size_t b = align256(sizeof(DevInfo));
    b += align256(sizeof(double) * kFlagBlocksMax * 6);
    b += align256(sizeof(uint32_t) * size_t(nmax));
    b += align256(sizeof(uint64_t) * size_t(nmax));
    b += align256(sizeof(int32_t) * size_t(nmax));
    b += align256(sizeof(uint32_t) * size_t(tiles) * kRsBins);
    b += align256(sizeof(uint32_t) * size_t(scan_tmp_size(nmax > tiles * kRsBins ? nmax : tiles * kRsBins)));
    return b;
}

// The collect, key and stable-sort stages of tree_build (the same kernels), with every
// temporary carved out of one caller-provided device block instead of TreeBufs.
cudaError_t morton_sort(const Launch &L, int64_t n, const double *px, const double *py, const double *pz,
                        const uint8_t *kind, const uint8_t *alive, uint64_t *keys, int32_t *order, void *scratch,
                        size_t scratch_bytes, DevInfo **info_out) {
    if (morton_sort_scratch_bytes(n) > scratch_bytes) return cudaErrorInvalidValue;
    char *p = static_cast<char *>(scratch);
    DevInfo *info = reinterpret_cast<DevInfo *>(p);
    p += align256(sizeof(DevInfo));
    double *bbox_part = reinterpret_cast<double *>(p);
    p += align256(sizeof(double) * kFlagBlocksMax * 6);
    uint32_t *flag = reinterpret_cast<uint32_t *>(p);
    p += align256(sizeof(uint32_t) * size_t(n));
    uint64_t *keys_alt = reinterpret_cast<uint64_t *>(p);
    p += align256(sizeof(uint64_t) * size_t(n));
    int32_t *order_alt = reinterpret_cast<int32_t *>(p);
    p += align256(sizeof(int32_t) * size_t(n));
    const uint32_t ntiles = uint32_t((n + kRsTile - 1) / kRsTile);
    uint32_t *hist = reinterpret_cast<uint32_t *>(p);
    p += align256(sizeof(uint32_t) * size_t(ntiles) * kRsBins);
    uint32_t *tmp = reinterpret_cast<uint32_t *>(p);
    int64_t tmp_cap = int64_t((static_cast<char *>(scratch) + scratch_bytes - p) / sizeof(uint32_t));
    *info_out = info;
    cudaStream_t s = L.stream;
    cudaError_t e = cudaMemsetAsync(info, 0, sizeof(DevInfo), s);
    if (e != cudaSuccess || n == 0) return e;
    unsigned fb = blocks_for(n, kThreads);
    if (fb > unsigned(kFlagBlocksMax)) fb = kFlagBlocksMax;
    k_flags_bbox_noacc<<<fb, kThreads, 0, s>>>(n, px, py, pz, kind, alive, flag, bbox_part);
    GBH_LAUNCH_CHECK();
    if ((e = scan_u32(L, flag, flag, n, tmp, tmp_cap)) != cudaSuccess) return e;
    k_bbox_final<<<1, kFinalThreads, 0, s>>>(int(fb), bbox_part, n, flag, kind, alive, 0.9, info, nullptr);
    GBH_LAUNCH_CHECK();
    k_compact_keys<<<blocks_for(n, kThreads), kThreads, 0, s>>>(n, px, py, pz, kind, alive, flag, info, keys, order);
    GBH_LAUNCH_CHECK();
    uint64_t *kin = keys, *kout = keys_alt;
    int32_t *vin = order, *vout = order_alt;
    for (int shift = 0; shift < 64; shift += 8) {
        k_rs_hist<false><<<ntiles ? ntiles : 1, kRsThreads, 0, s>>>(kin, vin, nullptr, info, shift, ntiles ? ntiles : 1,
                                                                    hist);
        GBH_LAUNCH_CHECK();
        if ((e = scan_u32(L, hist, hist, int64_t(ntiles ? ntiles : 1) * kRsBins, tmp, tmp_cap)) != cudaSuccess) return e;
        k_rs_scatter<false><<<ntiles ? ntiles : 1, kRsThreads, 0, s>>>(kin, vin, kout, vout, nullptr, info, shift,
                                                                        ntiles ? ntiles : 1, hist);
        GBH_LAUNCH_CHECK();
        uint64_t *tk = kin;
        kin = kout;
        kout = tk;
        int32_t *tv = vin;
        vin = vout;
        vout = tv;
    }
    return cudaSuccess;  // eight passes: the result is back in keys/order
}

}  // namespace gbh

namespace gbh {

// ---------------------------------------------------------------- diagnostics (diag.go:31-135)

namespace {

constexpr int kDiagSums = 11;  // kinetic, p(3), L(3), m x (3), m

// Per-block sums over bodies i (all bodies, as Momentum/AngularMomentum/CenterOfMass iterate
// s.Len(); kinetic over the bodies that gravitate, sourceKinetic diag.go:66-76).
__global__ __launch_bounds__(kThreads) void k_diag_partial(int64_t n, const double *__restrict__ px,
                                                           const double *__restrict__ py, const double *__restrict__ pz,
                                                           const double *__restrict__ vx, const double *__restrict__ vy,
                                                           const double *__restrict__ vz,
                                                           const double *__restrict__ mass,
                                                           const uint8_t *__restrict__ kind, double c, int dm_off,
                                                           double *__restrict__ part) {
    double acc[kDiagSums] = {};
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
        double m = mass[i], x = px[i], y = py[i], z = pz[i], ux = vx[i], uy = vy[i], uz = vz[i];
        uint8_t kd = kind ? kind[i] : 0;
        bool source = !(dm_off && kd == GBH_DARK_MATTER);
        double u2 = ux * ux + uy * uy + uz * uz;
        double g = c <= 0 ? 1.0 : sqrt(1 + u2 / (c * c));  // gamma, relativity.go:15-20
        if (source) acc[0] += m * u2 / (g + 1);           // kinetic, relativity.go:22-26
        acc[1] += m * ux;
        acc[2] += m * uy;
        acc[3] += m * uz;
        acc[4] += m * (y * uz - z * uy);
        acc[5] += m * (z * ux - x * uz);
        acc[6] += m * (x * uy - y * ux);
        acc[7] += m * x;
        acc[8] += m * y;
        acc[9] += m * z;
        acc[10] += m;
    }
    __shared__ double s[kThreads];
    for (int q = 0; q < kDiagSums; ++q) {
        s[threadIdx.x] = acc[q];
        __syncthreads();
        for (int o = kThreads / 2; o > 0; o >>= 1) {
            if (threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
            __syncthreads();
        }
        if (threadIdx.x == 0) part[blockIdx.x * kDiagSums + q] = s[0];
        __syncthreads();
    }
}

__global__ void k_diag_final(int nparts, const double *__restrict__ part, double *out) {
    if (threadIdx.x >= kDiagSums) return;
    double v = 0;
    for (int b = 0; b < nparts; ++b) v += part[b * kDiagSums + threadIdx.x];
    out[threadIdx.x] = v;
}

}  // namespace

int diag_parts() { return kFlagBlocksMax; }

cudaError_t diagnostics(const Launch &L, int64_t n, const double *px, const double *py, const double *pz,
                        const double *vx, const double *vy, const double *vz, const double *mass, const uint8_t *kind,
                        double c, int dm_off, double *part, double *out) {
    unsigned nb = blocks_for(n, kThreads);
    if (nb > unsigned(kFlagBlocksMax)) nb = kFlagBlocksMax;
    k_diag_partial<<<nb, kThreads, 0, L.stream>>>(n, px, py, pz, vx, vy, vz, mass, kind, c, dm_off, part);
    GBH_LAUNCH_CHECK();
    k_diag_final<<<1, 32, 0, L.stream>>>(int(nb), part, out);
    GBH_LAUNCH_CHECK();
    return cudaSuccess;
}

}  // namespace gbh

namespace gbh {

// ---------------------------------------------------------------- active-star lists (block steps)

namespace {

__global__ __launch_bounds__(kThreads) void k_target_flags(const DevInfo *info, const int32_t *__restrict__ order,
                                                           const int32_t *__restrict__ end, int32_t tick,
                                                           uint32_t *__restrict__ flag) {
    int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (k >= info->nstars) return;
    flag[k] = end[order[k]] == tick;
}

__global__ __launch_bounds__(kThreads) void k_target_write(DevInfo *info, const int32_t *__restrict__ order,
                                                           const int32_t *__restrict__ end, int32_t tick,
                                                           const uint32_t *__restrict__ pos, int32_t *__restrict__ targets) {
    int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    int64_t ns = info->nstars;
    if (k >= ns) return;
    bool on = end[order[k]] == tick;
    if (on) targets[pos[k]] = int32_t(k);
    if (k == ns - 1) info->ntargets = pos[k] + (on ? 1u : 0u);
}

}  // namespace

cudaError_t select_targets(const Launch &L, TreeBufs &b, const int32_t *end, int32_t tick) {
    const unsigned nb = blocks_for(b.cap_n, kThreads);
    k_target_flags<<<nb, kThreads, 0, L.stream>>>(b.info, b.order, end, tick, b.flag);
    GBH_LAUNCH_CHECK();
    cudaError_t e = scan_dyn(L, b.flag, b.flag, b.cap_n, &b.info->nstars, b.scan_tmp, b.scan_tmp_cap);
    if (e != cudaSuccess) return e;
    k_target_write<<<nb, kThreads, 0, L.stream>>>(b.info, b.order, end, tick, b.flag, b.targets);
    GBH_LAUNCH_CHECK();
    return cudaSuccess;
}

}  // namespace gbh

namespace gbh {

// ---------------------------------------------------------------- block time steps
//
// Gravity has no block steps in the reference; these follow its gas block steps
// (internal/sim/blockstep.go:22-90): a global step T is split into 2^(levels-1) ticks, a body
// on rung r steps T / 2^r, its rung is the smallest r with T / 2^r <= dt_i (rungFor,
// blockstep.go:38-45) capped at levels - 1, with dt_i = eta sqrt(eps / |a_i|), and a step may
// start only at a multiple of its length (blockstep.go:84-86). Kick-drift-kick per body: an
// opening half kick when its step starts, all bodies drift together from event to event, and
// at the end of its step a body gets its new acceleration, the closing half kick, a new rung
// and the next opening kick. With one level this is exactly the global KDK of sim.go.

namespace {

__device__ __forceinline__ int rung_for(double dt, double T, int rmax) {
    int r = 0;
    double x = T;
    while (x > dt && r < rmax) {
        x *= 0.5;
        ++r;
    }
    return r;
}

__device__ __forceinline__ double body_dt(double ax, double ay, double az, double eta, double eps) {
    double a = sqrt(ax * ax + ay * ay + az * az);
    return a > 0 ? eta * sqrt(eps / a) : INFINITY;
}

// Tick 0 of a global step: every body starts a step (rung from its acceleration) with the
// opening half kick.
__global__ __launch_bounds__(kThreads) void k_block_open(int64_t n, double T, int32_t ticks, int levels, double eta,
                                                         double eps, const double *__restrict__ ax,
                                                         const double *__restrict__ ay, const double *__restrict__ az,
                                                         double *vx, double *vy, double *vz, uint8_t *rung,
                                                         int32_t *end, DevInfo *info) {
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double a0 = ax[i], a1 = ay[i], a2 = az[i];
    int r = rung_for(body_dt(a0, a1, a2, eta, eps), T, levels - 1);
    rung[i] = uint8_t(r);
    int32_t e = ticks >> r;
    end[i] = e;
    double h = 0.5 * (T / double(1 << r));
    vx[i] += h * a0;
    vy[i] += h * a1;
    vz[i] += h * a2;
    atomicMin(&info->next_tick, e);
}

// driftOne (sim.go:345-350): x += dt u / gamma(u, c), gamma = 1 for c <= 0 (relativity.go:15-20).
__global__ __launch_bounds__(kThreads) void k_block_drift(int64_t n, double dt, double c, double *px, double *py,
                                                          double *pz, const double *__restrict__ vx,
                                                          const double *__restrict__ vy, const double *__restrict__ vz) {
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double ux = vx[i], uy = vy[i], uz = vz[i];
    double f = dt / (c <= 0 ? 1.0 : sqrt(1 + (ux * ux + uy * uy + uz * uz) / (c * c)));
    px[i] += f * ux;
    py[i] += f * uy;
    pz[i] += f * uz;
}

// Bodies whose step ends at tick: closing half kick with the new acceleration, then (before
// the end of the global step) a new rung aligned to tick and the opening half kick.
__global__ __launch_bounds__(kThreads) void k_block_close(int64_t n, int32_t tick, int32_t ticks, double T, int levels,
                                                          double eta, double eps, const double *__restrict__ ax,
                                                          const double *__restrict__ ay, const double *__restrict__ az,
                                                          double *vx, double *vy, double *vz, uint8_t *rung,
                                                          int32_t *end, DevInfo *info) {
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int32_t e = end[i];
    if (e == tick) {
        double a0 = ax[i], a1 = ay[i], a2 = az[i];
        double h = 0.5 * (T / double(1 << rung[i]));
        vx[i] += h * a0;
        vy[i] += h * a1;
        vz[i] += h * a2;
        if (tick < ticks) {
            int r = rung_for(body_dt(a0, a1, a2, eta, eps), T, levels - 1);
            while (tick % (ticks >> r) != 0) ++r;
            rung[i] = uint8_t(r);
            e = tick + (ticks >> r);
            end[i] = e;
            double h2 = 0.5 * (T / double(1 << r));
            vx[i] += h2 * a0;
            vy[i] += h2 * a1;
            vz[i] += h2 * a2;
        }
    }
    atomicMin(&info->next_tick, e);
}

// The bodies whose step ends at the next event tick (the host sizes that event's walk by them).
__global__ __launch_bounds__(kThreads) void k_count_next(int64_t n, const int32_t *__restrict__ end, DevInfo *info) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    const int32_t tn = info->next_tick;
    const unsigned m = __ballot_sync(0xffffffffu, i < n && end[i] == tn);  // whole warps: no early return
    if ((threadIdx.x & 31) == 0 && m) atomicAdd(&info->next_count, uint32_t(__popc(m)));
}

cudaError_t count_next(const Launch &L, const TreeBufs &b, int64_t n, const int32_t *end) {
    cudaError_t e = cudaMemsetAsync(&b.info->next_count, 0, sizeof(uint32_t), L.stream);
    if (e != cudaSuccess) return e;
    k_count_next<<<blocks_for(n, kThreads), kThreads, 0, L.stream>>>(n, end, b.info);
    GBH_LAUNCH_CHECK();
    return cudaSuccess;
}

}  // namespace

cudaError_t block_open(const Launch &L, const TreeBufs &b, int64_t n, double T, int levels, double eta, double eps,
                       const double *ax, const double *ay, const double *az, double *vx, double *vy, double *vz,
                       uint8_t *rung, int32_t *end) {
    cudaError_t e = cudaMemsetAsync(&b.info->next_tick, 0x7f, sizeof(int32_t), L.stream);
    if (e != cudaSuccess) return e;
    k_block_open<<<blocks_for(n, kThreads), kThreads, 0, L.stream>>>(n, T, 1 << (levels - 1), levels, eta, eps, ax, ay,
                                                                     az, vx, vy, vz, rung, end, b.info);
    GBH_LAUNCH_CHECK();
    return count_next(L, b, n, end);
}

cudaError_t block_drift(const Launch &L, int64_t n, double dt, double c, double *px, double *py, double *pz,
                        const double *vx, const double *vy, const double *vz) {
    k_block_drift<<<blocks_for(n, kThreads), kThreads, 0, L.stream>>>(n, dt, c, px, py, pz, vx, vy, vz);
    GBH_LAUNCH_CHECK();
    return cudaSuccess;
}

cudaError_t block_close(const Launch &L, const TreeBufs &b, int64_t n, int32_t tick, double T, int levels, double eta,
                        double eps, const double *ax, const double *ay, const double *az, double *vx, double *vy,
                        double *vz, uint8_t *rung, int32_t *end) {
    cudaError_t e = cudaMemsetAsync(&b.info->next_tick, 0x7f, sizeof(int32_t), L.stream);
    if (e != cudaSuccess) return e;
    k_block_close<<<blocks_for(n, kThreads), kThreads, 0, L.stream>>>(n, tick, 1 << (levels - 1), T, levels, eta, eps,
                                                                      ax, ay, az, vx, vy, vz, rung, end, b.info);
    GBH_LAUNCH_CHECK();
    return count_next(L, b, n, end);
}

}  // namespace gbh
