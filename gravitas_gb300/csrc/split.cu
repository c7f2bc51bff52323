// split.cu — the hole-aware step of internal/sim/split.go (stepSplit) without gas, instant gravity
// and no spins: star-star forces from the tree once per step (api.cu), every force involving an
// alive black hole summed here directly (O(N x holes), the pair model of pair.go: Paczynski-Wiita
// star-hole pairs for c > 0), and the stars near a hole plus the holes themselves advanced in
// power-of-two substeps, every drift by u / gamma (relativity.go). Built with -fmad=false: the pair terms, kicks and drifts
// round like the FP64 restatement (orc_split_kdk), so the FP64 walk's trajectories match it bit
// for bit. A hole's pull from the far stars is summed in 256-body chunks (sequential inside a
// chunk, chunks in index order), the fixed order the restatement uses.
#include <cuda_runtime.h>

#include <algorithm>

#include "gbh_internal.cuh"

namespace gbh {
namespace {

constexpr int kEw = 256;
constexpr int kHoleChunk = 256;

#define SPLIT_LAUNCH_CHECK()                 \
    do {                                     \
        ++*L.count;                          \
        cudaError_t e_ = cudaGetLastError(); \
        if (e_ != cudaSuccess) return e_;    \
    } while (0)

inline unsigned ew_blocks(int64_t n) { return unsigned(std::max<int64_t>(1, (n + kEw - 1) / kEw)); }

// pair.go:26-35 (PairForce): f such that the acceleration is f d; capped inside 1.5 rs.
__device__ __forceinline__ double pair_force(double m, double r2, double eps2, double rs) {
    double re2 = r2 + eps2;
    double re = sqrt(re2);
    if (rs == 0) return m / (re2 * re);
    double den = fmax(re - rs, rs / 2);
    return m / (den * den * re);
}

__device__ __forceinline__ double schwarzschild(double m, double c) { return c <= 0 ? 0 : 2 * m / (c * c); }

// PairRS (pair.go:14-23) of body i with hole h: the hole's radius unless i is a hole too.
__device__ __forceinline__ double hole_rs(int64_t i, int32_t h, const double *mass, const uint8_t *kind, double c) {
    return kind[i] == GBH_BLACK_HOLE ? 0.0 : schwarzschild(mass[h], c);
}

// dt / gamma (relativity.go:15-20, driftIdx / driftFar split.go:226-250).
__device__ __forceinline__ double drift_factor(double dt, double ux, double uy, double uz, double c) {
    return dt / (c <= 0 ? 1.0 : sqrt(1 + (ux * ux + uy * uy + uz * uz) / (c * c)));
}

// split.go:27-36 (holeTimescale): sqrt(r_eps / a) of body i in the field of hole h.
__device__ __forceinline__ double timescale(int64_t i, int64_t h, const double *px, const double *py,
                                            const double *pz, const double *mass, const uint8_t *kind, double eps2,
                                            double c) {
    double dx = px[i] - px[h], dy = py[i] - py[h], dz = pz[i] - pz[h];
    double r2 = dx * dx + dy * dy + dz * dz;
    double a = pair_force(mass[h], r2, eps2, hole_rs(i, int32_t(h), mass, kind, c)) * sqrt(r2);
    if (a == 0) return __longlong_as_double(0x7ff0000000000000LL);
    return sqrt(sqrt(r2 + eps2) / a);
}

// split.go:119-137 (holePull): the pull of every hole but i itself on body i, holes in order.
__device__ __forceinline__ void hole_pull(int64_t i, const int32_t *__restrict__ holes, int32_t nh,
                                          const double *px, const double *py, const double *pz,
                                          const double *mass, const uint8_t *kind, double eps2, double c, double &fx,
                                          double &fy, double &fz) {
    double x = px[i], y = py[i], z = pz[i];
    fx = fy = fz = 0;
    for (int32_t k = 0; k < nh; ++k) {
        int32_t h = holes[k];
        if (h == i) continue;
        double dx = px[h] - x, dy = py[h] - y, dz = pz[h] - z;
        double f = pair_force(mass[h], dx * dx + dy * dy + dz * dz, eps2, hole_rs(i, h, mass, kind, c));
        fx += f * dx;
        fy += f * dy;
        fz += f * dz;
    }
}

__device__ __forceinline__ double source_mass(int64_t i, const double *mass, const uint8_t *kind, int dm_off) {
    return dm_off && kind[i] == GBH_DARK_MATTER ? 0.0 : mass[i];  // Params.SourceMass, sim.go:93-98
}

// classify (split.go:39-85): near flags (byte and u32 for the scan) and the minimum timescale
// (as the bits of a positive double, ordered like the value) over near stars and hole pairs.
__global__ void k_classify(int64_t n, const double *__restrict__ px, const double *__restrict__ py,
                           const double *__restrict__ pz, const double *__restrict__ mass,
                           const uint8_t *__restrict__ kind, const int32_t *__restrict__ holes, int32_t nh,
                           double eps2, double c, double limit, uint8_t *near8, uint32_t *near32,
                           unsigned long long *tau_bits) {
    __shared__ double smin[kEw / 32];
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    double local = __longlong_as_double(0x7ff0000000000000LL);
    if (i < n) {
        bool nr = false;
        if (kind[i] != GBH_BLACK_HOLE)
            for (int32_t k = 0; k < nh; ++k) {
                double tau = timescale(i, holes[k], px, py, pz, mass, kind, eps2, c);
                if (tau < limit) {
                    nr = true;
                    local = fmin(local, tau);
                }
            }
        near8[i] = nr;
        near32[i] = nr;
    }
    for (int o = 16; o > 0; o >>= 1) local = fmin(local, __shfl_xor_sync(0xffffffffu, local, o));
    if ((threadIdx.x & 31) == 0) smin[threadIdx.x >> 5] = local;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < int(blockDim.x >> 5); ++w) local = fmin(local, smin[w]);
        if (blockIdx.x == 0)  // hole pairs: each with the mass of the later one (split.go:64-70)
            for (int32_t a = 0; a < nh; ++a)
                for (int32_t b = a + 1; b < nh; ++b) {
                    double tau = timescale(holes[a], holes[b], px, py, pz, mass, kind, eps2, c);
                    if (tau < limit) local = fmin(local, tau);
                }
        atomicMin(tau_bits, static_cast<unsigned long long>(__double_as_longlong(local)));
    }
}

// Near list in index order from the exclusive scan of the flags; out[1] = its length.
__global__ void k_near_list(int64_t n, const uint8_t *__restrict__ near8, const uint32_t *__restrict__ scan,
                            int32_t *near, unsigned long long *out) {
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (near8[i]) near[scan[i]] = int32_t(i);
    if (i == n - 1) out[1] = scan[i] + near8[i];
}

// outerHoleForces, far bodies (split.go:83-96): far stars feel every hole; near stars and holes
// get 0 here (the holes' sums come from k_far_holes_*).
__global__ void k_far_bodies(int64_t n, const double *__restrict__ px, const double *__restrict__ py,
                             const double *__restrict__ pz, const double *__restrict__ mass,
                             const uint8_t *__restrict__ kind, const uint8_t *__restrict__ near8,
                             const int32_t *__restrict__ holes, int32_t nh, double eps2, double c, double *fx,
                             double *fy, double *fz) {
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double x = 0, y = 0, z = 0;
    if (kind[i] != GBH_BLACK_HOLE && !near8[i]) hole_pull(i, holes, nh, px, py, pz, mass, kind, eps2, c, x, y, z);
    fx[i] = x;
    fy[i] = y;
    fz[i] = z;
}

// outerHoleForces, holes (split.go:97-116): partial sums of each hole's pull from the far stars
// of one 256-body chunk, sequential in index order.
__global__ void k_far_holes_part(int64_t n, const double *__restrict__ px, const double *__restrict__ py,
                                 const double *__restrict__ pz, const double *__restrict__ mass,
                                 const uint8_t *__restrict__ kind, const uint8_t *__restrict__ near8, int dm_off,
                                 const int32_t *__restrict__ holes, int32_t nh, double eps2, double c,
                                 double *part) {
    __shared__ double sx[kHoleChunk], sy[kHoleChunk], sz[kHoleChunk], sm[kHoleChunk];
    __shared__ uint8_t skip[kHoleChunk];
    const int64_t c0 = int64_t(blockIdx.x) * kHoleChunk;
    const int cnt = n - c0 < kHoleChunk ? int(n - c0) : kHoleChunk;
    for (int q = threadIdx.x; q < cnt; q += blockDim.x) {
        int64_t i = c0 + q;
        sx[q] = px[i];
        sy[q] = py[i];
        sz[q] = pz[i];
        sm[q] = source_mass(i, mass, kind, dm_off);
        skip[q] = kind[i] == GBH_BLACK_HOLE || near8[i];
    }
    __syncthreads();
    for (int32_t k = threadIdx.x; k < nh; k += blockDim.x) {
        int32_t h = holes[k];
        double x = px[h], y = py[h], z = pz[h];
        const double rs = schwarzschild(mass[h], c);
        double ax = 0, ay = 0, az = 0;
        for (int q = 0; q < cnt; ++q) {
            if (skip[q]) continue;
            double dx = sx[q] - x, dy = sy[q] - y, dz = sz[q] - z;
            double f = pair_force(sm[q], dx * dx + dy * dy + dz * dz, eps2, rs);
            ax += f * dx;
            ay += f * dy;
            az += f * dz;
        }
        double *p = part + (int64_t(blockIdx.x) * nh + k) * 3;
        p[0] = ax;
        p[1] = ay;
        p[2] = az;
    }
}

// Each hole's far-star pull: the chunk partials added in chunk order to 0.
__global__ void k_far_holes_final(int64_t nchunks, const int32_t *__restrict__ holes, int32_t nh,
                                  const double *__restrict__ part, double *fx, double *fy, double *fz) {
    int32_t k = int32_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (k >= nh) return;
    double ax = 0, ay = 0, az = 0;
    for (int64_t c = 0; c < nchunks; ++c) {
        const double *p = part + (c * nh + k) * 3;
        ax += p[0];
        ay += p[1];
        az += p[2];
    }
    int32_t h = holes[k];
    fx[h] = ax;
    fy[h] = ay;
    fz[h] = az;
}

// kickOuter (split.go:206-213): every body, v += h (a + far).
__global__ void k_kick_outer(int64_t n, double h, double *vx, double *vy, double *vz, const double *__restrict__ ax,
                             const double *__restrict__ ay, const double *__restrict__ az,
                             const double *__restrict__ fx, const double *__restrict__ fy,
                             const double *__restrict__ fz) {
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    vx[i] = vx[i] + h * (ax[i] + fx[i]);
    vy[i] = vy[i] + h * (ay[i] + fy[i]);
    vz[i] = vz[i] + h * (az[i] + fz[i]);
}

// fastForces, near stars (split.go:142-147): the pull of every hole.
__global__ void k_fast_near(int32_t nnear, const int32_t *__restrict__ near, const double *__restrict__ px,
                            const double *__restrict__ py, const double *__restrict__ pz,
                            const double *__restrict__ mass, const uint8_t *__restrict__ kind,
                            const int32_t *__restrict__ holes, int32_t nh, double eps2, double c, double *fx,
                            double *fy, double *fz) {
    int32_t q = int32_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (q >= nnear) return;
    int32_t i = near[q];
    double x, y, z;
    hole_pull(i, holes, nh, px, py, pz, mass, kind, eps2, c, x, y, z);
    fx[i] = x;
    fy[i] = y;
    fz[i] = z;
}

// fastForces, holes (split.go:148-158): the other holes, then the near stars in index order.
__global__ void k_fast_holes(int32_t nnear, const int32_t *__restrict__ near, const double *__restrict__ px,
                             const double *__restrict__ py, const double *__restrict__ pz,
                             const double *__restrict__ mass, const uint8_t *__restrict__ kind, int dm_off,
                             const int32_t *__restrict__ holes, int32_t nh, double eps2, double c, double *fx,
                             double *fy, double *fz) {
    int32_t k = int32_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (k >= nh) return;
    int32_t h = holes[k];
    double x = px[h], y = py[h], z = pz[h];
    const double rs = schwarzschild(mass[h], c);
    double ax, ay, az;
    hole_pull(h, holes, nh, px, py, pz, mass, kind, eps2, c, ax, ay, az);
    for (int32_t q = 0; q < nnear; ++q) {
        int32_t i = near[q];
        double dx = px[i] - x, dy = py[i] - y, dz = pz[i] - z;
        double f = pair_force(source_mass(i, mass, kind, dm_off), dx * dx + dy * dy + dz * dz, eps2, rs);
        ax += f * dx;
        ay += f * dy;
        az += f * dz;
    }
    fx[h] = ax;
    fy[h] = ay;
    fz[h] = az;
}

// kickFast (split.go:215-224) and driftIdx (split.go:226-234, c = 0) over the near stars, then
// the holes: entry q < nnear is near[q], the rest are the holes.
__global__ void k_fast_update(int32_t nnear, const int32_t *__restrict__ near, const int32_t *__restrict__ holes,
                              int32_t nh, int drift, double h, double c, double *px, double *py, double *pz,
                              double *vx, double *vy, double *vz, const double *__restrict__ fx,
                              const double *__restrict__ fy, const double *__restrict__ fz) {
    int32_t q = int32_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (q >= nnear + nh) return;
    int32_t i = q < nnear ? near[q] : holes[q - nnear];
    if (drift) {
        const double f = drift_factor(h, vx[i], vy[i], vz[i], c);
        px[i] = px[i] + f * vx[i];
        py[i] = py[i] + f * vy[i];
        pz[i] = pz[i] + f * vz[i];
    } else {
        vx[i] = vx[i] + h * fx[i];
        vy[i] = vy[i] + h * fy[i];
        vz[i] = vz[i] + h * fz[i];
    }
}

// driftFar (split.go:236-250, no gas): every body that is neither a hole nor near.
__global__ void k_drift_far(int64_t n, double dt, double c, const uint8_t *__restrict__ kind,
                            const uint8_t *__restrict__ near8, double *px, double *py, double *pz,
                            const double *__restrict__ vx, const double *__restrict__ vy,
                            const double *__restrict__ vz) {
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n || kind[i] == GBH_BLACK_HOLE || near8[i]) return;
    const double f = drift_factor(dt, vx[i], vy[i], vz[i], c);
    px[i] = px[i] + f * vx[i];
    py[i] = py[i] + f * vy[i];
    pz[i] = pz[i] + f * vz[i];
}

}  // namespace

void split_free(SplitBufs &s) {
    void *ptrs[] = {s.holes, s.near8, s.near32, s.near, s.scan_tmp, s.far, s.fast, s.part, s.scalars};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    s = SplitBufs{};
}

cudaError_t split_reserve(SplitBufs &s, int64_t n, const std::vector<int32_t> &holes) {
    cudaError_t e = cudaSuccess;
    const int32_t nh = int32_t(holes.size());
    if (n > s.cap_n) {
        void *ptrs[] = {s.near8, s.near32, s.near, s.scan_tmp, s.far, s.fast};
        for (void *p : ptrs)
            if (p) cudaFree(p);
        s.near8 = nullptr;
        s.near32 = nullptr;
        s.near = nullptr;
        s.scan_tmp = nullptr;
        s.far = s.fast = nullptr;
        s.cap_n = 0;
        int64_t cap = n + n / 4;
        s.scan_cap = scan_tmp_size(cap);
        if (e == cudaSuccess) e = dev_alloc(&s.near8, size_t(cap));
        if (e == cudaSuccess) e = dev_alloc(&s.near32, sizeof(uint32_t) * size_t(cap));
        if (e == cudaSuccess) e = dev_alloc(&s.near, sizeof(int32_t) * size_t(cap));
        if (e == cudaSuccess) e = dev_alloc(&s.scan_tmp, sizeof(uint32_t) * size_t(s.scan_cap));
        if (e == cudaSuccess) e = dev_alloc(&s.far, sizeof(double) * 3 * size_t(cap));
        if (e == cudaSuccess) e = dev_alloc(&s.fast, sizeof(double) * 3 * size_t(cap));
        if (e != cudaSuccess) return e;
        s.cap_n = cap;
    }
    int64_t need_part = ((n + kHoleChunk - 1) / kHoleChunk) * std::max(nh, 1) * 3;
    if (need_part > s.cap_part) {
        if (s.part) cudaFree(s.part);
        s.part = nullptr;
        s.cap_part = 0;
        if ((e = dev_alloc(&s.part, sizeof(double) * size_t(need_part + need_part / 4)))) return e;
        s.cap_part = need_part + need_part / 4;
    }
    if (nh > s.cap_holes) {
        if (s.holes) cudaFree(s.holes);
        s.holes = nullptr;
        s.cap_holes = 0;
        if ((e = dev_alloc(&s.holes, sizeof(int32_t) * size_t(nh)))) return e;
        s.cap_holes = nh;
    }
    if (!s.scalars && (e = dev_alloc(&s.scalars, 2 * sizeof(unsigned long long)))) return e;
    s.nholes = nh;
    return cudaSuccess;
}

cudaError_t split_classify(const Launch &L, SplitBufs &s, int64_t n, const double *px, const double *py,
                           const double *pz, const double *mass, const uint8_t *kind, double eps2, double c,
                           double limit) {
    static const unsigned long long kInit[2] = {0x7ff0000000000000ULL, 0};  // +inf, no near stars
    cudaError_t e = cudaMemcpyAsync(s.scalars, kInit, sizeof kInit, cudaMemcpyHostToDevice, L.stream);
    if (e != cudaSuccess) return e;
    k_classify<<<ew_blocks(n), kEw, 0, L.stream>>>(n, px, py, pz, mass, kind, s.holes, s.nholes, eps2, c, limit,
                                                   s.near8, s.near32, s.scalars);
    SPLIT_LAUNCH_CHECK();
    if ((e = scan_u32(L, s.near32, s.near32, n, s.scan_tmp, s.scan_cap))) return e;
    k_near_list<<<ew_blocks(n), kEw, 0, L.stream>>>(n, s.near8, s.near32, s.near, s.scalars);
    SPLIT_LAUNCH_CHECK();
    return cudaSuccess;
}

cudaError_t split_outer(const Launch &L, SplitBufs &s, int64_t n, const double *px, const double *py,
                        const double *pz, const double *mass, const uint8_t *kind, int dm_off, double eps2, double c) {
    double *fx = s.far, *fy = fx + n, *fz = fy + n;
    k_far_bodies<<<ew_blocks(n), kEw, 0, L.stream>>>(n, px, py, pz, mass, kind, s.near8, s.holes, s.nholes, eps2, c,
                                                     fx, fy, fz);
    SPLIT_LAUNCH_CHECK();
    int64_t nchunks = (n + kHoleChunk - 1) / kHoleChunk;
    k_far_holes_part<<<unsigned(nchunks), 64, 0, L.stream>>>(n, px, py, pz, mass, kind, s.near8, dm_off, s.holes,
                                                            s.nholes, eps2, c, s.part);
    SPLIT_LAUNCH_CHECK();
    k_far_holes_final<<<unsigned((s.nholes + 63) / 64), 64, 0, L.stream>>>(nchunks, s.holes, s.nholes, s.part, fx,
                                                                          fy, fz);
    SPLIT_LAUNCH_CHECK();
    return cudaSuccess;
}

cudaError_t split_kick_outer(const Launch &L, SplitBufs &s, int64_t n, double h, double *vx, double *vy, double *vz,
                             const double *ax, const double *ay, const double *az) {
    k_kick_outer<<<ew_blocks(n), kEw, 0, L.stream>>>(n, h, vx, vy, vz, ax, ay, az, s.far, s.far + n, s.far + 2 * n);
    SPLIT_LAUNCH_CHECK();
    return cudaSuccess;
}

cudaError_t split_fast(const Launch &L, SplitBufs &s, int64_t n, int32_t nnear, const double *px, const double *py,
                       const double *pz, const double *mass, const uint8_t *kind, int dm_off, double eps2, double c) {
    double *fx = s.fast, *fy = fx + n, *fz = fy + n;
    if (nnear > 0) {
        k_fast_near<<<ew_blocks(nnear), kEw, 0, L.stream>>>(nnear, s.near, px, py, pz, mass, kind, s.holes, s.nholes,
                                                            eps2, c, fx, fy, fz);
        SPLIT_LAUNCH_CHECK();
    }
    k_fast_holes<<<unsigned((s.nholes + 31) / 32), 32, 0, L.stream>>>(nnear, s.near, px, py, pz, mass, kind, dm_off,
                                                                      s.holes, s.nholes, eps2, c, fx, fy, fz);
    SPLIT_LAUNCH_CHECK();
    return cudaSuccess;
}

cudaError_t split_fast_update(const Launch &L, SplitBufs &s, int64_t n, int32_t nnear, bool drift, double h,
                              double c, double *px, double *py, double *pz, double *vx, double *vy, double *vz) {
    k_fast_update<<<ew_blocks(int64_t(nnear) + s.nholes), kEw, 0, L.stream>>>(
        nnear, s.near, s.holes, s.nholes, drift ? 1 : 0, h, c, px, py, pz, vx, vy, vz, s.fast, s.fast + n,
        s.fast + 2 * n);
    SPLIT_LAUNCH_CHECK();
    return cudaSuccess;
}

cudaError_t split_drift_far(const Launch &L, SplitBufs &s, int64_t n, double dt, double c, const uint8_t *kind,
                            double *px, double *py, double *pz, const double *vx, const double *vy, const double *vz) {
    k_drift_far<<<ew_blocks(n), kEw, 0, L.stream>>>(n, dt, c, kind, s.near8, px, py, pz, vx, vy, vz);
    SPLIT_LAUNCH_CHECK();
    return cudaSuccess;
}

}  // namespace gbh
