// adjoint.cu — reverse-mode gradient of the KDK leapfrog (sim.go:302-343) with the softened
// direct-sum force (direct.go:27-47, every body a star). The forward saves (x, v, a) every K
// steps; the backward replays each segment from its checkpoint and runs the adjoint steps in
// reverse. Built with -fmad=false: the FP64 kernels are bit identical to the CPU restatement
// (j ascending, IEEE divide and square root, no contraction); the FP32 kernels use explicit
// fmaf, rsqrtf and double-float separations.
//
// The adjoint of one step x' = x + dt (v + h a(x)), v' = v + h a(x) + h a(x'), h = dt/2:
//   lambda_v += dt lambda_x                               (drift)
//   lambda_x += c J(x)^T lambda_v,  lambda_m += c (da/dm)^T lambda_v   (kicks at x)
// where c = dt for the closing kick of step s-1 and the opening kick of step s together
// (both act at x_s with the same lambda_v), h at x_0 and at x_T. For the softened pair force
//   (J^T w)_i = sum_{j != i} K(d_ij) (m_i w_j - m_j w_i),   K(d) = I / s^3 - 3 d d^T / s^5,
//   (da/dm)^T w)_i = -sum_{j != i} (w_j . d_ij) / s^3,      d_ij = x_j - x_i, s^2 = |d|^2 + eps^2.
#include <cuda_runtime.h>

#include <algorithm>

#include "gbh_internal.cuh"

namespace gbh {
namespace {

constexpr int kPairThreads = 128;  // targets per block of the pair kernels, and the j tile
constexpr int kEwThreads = 256;

#define ADJ_LAUNCH_CHECK()                   \
    do {                                     \
        ++*L.count;                          \
        cudaError_t e_ = cudaGetLastError(); \
        if (e_ != cudaSuccess) return e_;    \
    } while (0)

inline unsigned ew_blocks(int64_t n) { return unsigned(std::max<int64_t>(1, (n + kEwThreads - 1) / kEwThreads)); }

// ---- FP64 pair kernels (the oracle's loop order, j ascending) ----

__global__ void __launch_bounds__(kPairThreads) k_force64(int64_t n, const double *__restrict__ px,
                                                          const double *__restrict__ py,
                                                          const double *__restrict__ pz,
                                                          const double *__restrict__ m, double eps2, double *ax,
                                                          double *ay, double *az) {
    __shared__ double sx[kPairThreads], sy[kPairThreads], sz[kPairThreads], sm[kPairThreads];
    int64_t i = int64_t(blockIdx.x) * kPairThreads + threadIdx.x;
    bool act = i < n;
    double xi = act ? px[i] : 0, yi = act ? py[i] : 0, zi = act ? pz[i] : 0;
    double fx = 0, fy = 0, fz = 0;
    for (int64_t j0 = 0; j0 < n; j0 += kPairThreads) {
        int64_t j = j0 + threadIdx.x;
        if (j < n) {
            sx[threadIdx.x] = px[j];
            sy[threadIdx.x] = py[j];
            sz[threadIdx.x] = pz[j];
            sm[threadIdx.x] = m[j];
        }
        __syncthreads();
        int cnt = n - j0 < kPairThreads ? int(n - j0) : kPairThreads;
        for (int q = 0; q < cnt; ++q) {
            if (j0 + q == i) continue;
            double dx = sx[q] - xi, dy = sy[q] - yi, dz = sz[q] - zi;
            double re2 = dx * dx + dy * dy + dz * dz + eps2;
            double f = sm[q] / (re2 * sqrt(re2));
            fx += f * dx;
            fy += f * dy;
            fz += f * dz;
        }
        __syncthreads();
    }
    if (act) {
        ax[i] = fx;
        ay[i] = fy;
        az[i] = fz;
    }
}

// lambda_x += c J^T w, lambda_m += c (da/dm)^T w, w = lambda_v (read only here).
__global__ void __launch_bounds__(kPairThreads) k_vjp64(int64_t n, const double *__restrict__ px,
                                                        const double *__restrict__ py,
                                                        const double *__restrict__ pz,
                                                        const double *__restrict__ m, const double *__restrict__ wx,
                                                        const double *__restrict__ wy,
                                                        const double *__restrict__ wz, double eps2, double c,
                                                        double *gx, double *gy, double *gz, double *gm) {
    __shared__ double sx[kPairThreads], sy[kPairThreads], sz[kPairThreads], sm[kPairThreads];
    __shared__ double swx[kPairThreads], swy[kPairThreads], swz[kPairThreads];
    int64_t i = int64_t(blockIdx.x) * kPairThreads + threadIdx.x;
    bool act = i < n;
    double xi = act ? px[i] : 0, yi = act ? py[i] : 0, zi = act ? pz[i] : 0, mi = act ? m[i] : 0;
    double wix = act ? wx[i] : 0, wiy = act ? wy[i] : 0, wiz = act ? wz[i] : 0;
    double ax = 0, ay = 0, az = 0, am = 0;
    for (int64_t j0 = 0; j0 < n; j0 += kPairThreads) {
        int64_t j = j0 + threadIdx.x;
        if (j < n) {
            sx[threadIdx.x] = px[j];
            sy[threadIdx.x] = py[j];
            sz[threadIdx.x] = pz[j];
            sm[threadIdx.x] = m[j];
            swx[threadIdx.x] = wx[j];
            swy[threadIdx.x] = wy[j];
            swz[threadIdx.x] = wz[j];
        }
        __syncthreads();
        int cnt = n - j0 < kPairThreads ? int(n - j0) : kPairThreads;
        for (int q = 0; q < cnt; ++q) {
            if (j0 + q == i) continue;
            double dx = sx[q] - xi, dy = sy[q] - yi, dz = sz[q] - zi;
            double s2 = dx * dx + dy * dy + dz * dz + eps2;
            double inv3 = 1 / (s2 * sqrt(s2));
            double inv5 = inv3 / s2;
            double ux = mi * swx[q] - sm[q] * wix, uy = mi * swy[q] - sm[q] * wiy, uz = mi * swz[q] - sm[q] * wiz;
            double du = dx * ux + dy * uy + dz * uz;
            ax += ux * inv3 - 3 * dx * du * inv5;
            ay += uy * inv3 - 3 * dy * du * inv5;
            az += uz * inv3 - 3 * dz * du * inv5;
            am -= (swx[q] * dx + swy[q] * dy + swz[q] * dz) * inv3;
        }
        __syncthreads();
    }
    if (act) {
        gx[i] += c * ax;
        gy[i] += c * ay;
        gz[i] += c * az;
        gm[i] += c * am;
    }
}

// ---- FP32 pair kernels: double-float positions, plain FP32 sums over one j tile folded into
// compensated (TwoSum) accumulators, one partial per j split. ----

__device__ __forceinline__ void fold(float &s, float &comp, float x) {
    float t = s + x;
    float bp = t - s;
    comp += (s - (t - bp)) + (x - bp);
    s = t;
}

// hi = (x, y, z, m) rounded to FP32, lo = the FP32 remainders; w = lambda_v in FP32 (optional).
__global__ void k_prep32(int64_t n, const double *__restrict__ px, const double *__restrict__ py,
                         const double *__restrict__ pz, const double *__restrict__ m, const double *__restrict__ wx,
                         const double *__restrict__ wy, const double *__restrict__ wz, float4 *hi, float4 *lo,
                         float4 *w) {
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double x = px[i], y = py[i], z = pz[i];
    float hx = __double2float_rn(x), hy = __double2float_rn(y), hz = __double2float_rn(z);
    hi[i] = make_float4(hx, hy, hz, __double2float_rn(m[i]));
    lo[i] = make_float4(__double2float_rn(x - double(hx)), __double2float_rn(y - double(hy)),
                        __double2float_rn(z - double(hz)), 0.f);
    if (w) w[i] = make_float4(__double2float_rn(wx[i]), __double2float_rn(wy[i]), __double2float_rn(wz[i]), 0.f);
}

__device__ __forceinline__ float2 f2(float v) { return make_float2(v, v); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

__device__ __forceinline__ void fold2(float2 &s, float2 &comp, float2 x) {
    fold(s.x, comp.x, x.x);
    fold(s.y, comp.y, x.y);
}

// Each thread owns two targets, i0 and i0 + kPairThreads, whose arithmetic runs as one packed
// FP32x2 operation (__fadd2_rn / __fmul2_rn / __ffma2_rn); a block covers kPairTargets targets.
constexpr int kPairTargets = 2 * kPairThreads;

// part[(split * 3 + axis) * n + i]: the accelerations of target i from the sources of one split.
__global__ void __launch_bounds__(kPairThreads) k_force32(int64_t n, int64_t chunk, const float4 *__restrict__ hi,
                                                          const float4 *__restrict__ lo, float eps2,
                                                          double *part) {
    __shared__ float4 shi[kPairThreads], slo[kPairThreads];
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
    const int64_t i0 = int64_t(blockIdx.x) * kPairTargets + threadIdx.x, i1 = i0 + kPairThreads;
    const bool a0 = i0 < n, a1 = i1 < n;
    const float4 h0 = a0 ? hi[i0] : z4, h1 = a1 ? hi[i1] : z4, l0 = a0 ? lo[i0] : z4, l1 = a1 ? lo[i1] : z4;
    // negated target coordinates, so separations are sums
    const float2 nhx = make_float2(-h0.x, -h1.x), nhy = make_float2(-h0.y, -h1.y), nhz = make_float2(-h0.z, -h1.z);
    const float2 nlx = make_float2(-l0.x, -l1.x), nly = make_float2(-l0.y, -l1.y), nlz = make_float2(-l0.z, -l1.z);
    const float2 e2 = f2(eps2);
    float2 ax = f2(0.f), ay = f2(0.f), az = f2(0.f), cx = f2(0.f), cy = f2(0.f), cz = f2(0.f);
    int64_t jb = int64_t(blockIdx.y) * chunk, je = jb + chunk < n ? jb + chunk : n;
    for (int64_t j0 = jb; j0 < je; j0 += kPairThreads) {
        int64_t j = j0 + threadIdx.x;
        // padding sources have zero mass at the origin: s^2 >= eps^2 > 0, so they add exactly 0
        shi[threadIdx.x] = j < je ? hi[j] : z4;
        slo[threadIdx.x] = j < je ? lo[j] : z4;
        __syncthreads();
        float2 tx = f2(0.f), ty = f2(0.f), tz = f2(0.f);
#pragma unroll 8
        for (int q = 0; q < kPairThreads; ++q) {
            const float4 sh = shi[q], sl = slo[q];
            // j == i gives d == 0 exactly and adds nothing
            const float2 dx = add2(add2(f2(sh.x), nhx), add2(f2(sl.x), nlx));
            const float2 dy = add2(add2(f2(sh.y), nhy), add2(f2(sl.y), nly));
            const float2 dz = add2(add2(f2(sh.z), nhz), add2(f2(sl.z), nlz));
            const float2 s2 = fma2(dx, dx, fma2(dy, dy, fma2(dz, dz, e2)));
            const float2 r = make_float2(rsqrtf(s2.x), rsqrtf(s2.y));
            const float2 f = mul2(mul2(f2(sh.w), r), mul2(r, r));
            tx = fma2(f, dx, tx);
            ty = fma2(f, dy, ty);
            tz = fma2(f, dz, tz);
        }
        __syncthreads();
        fold2(ax, cx, tx);
        fold2(ay, cy, ty);
        fold2(az, cz, tz);
    }
    double *p = part + int64_t(blockIdx.y) * 3 * n;
    if (a0) {
        p[i0] = double(ax.x) + double(cx.x);
        p[n + i0] = double(ay.x) + double(cy.x);
        p[2 * n + i0] = double(az.x) + double(cz.x);
    }
    if (a1) {
        p[i1] = double(ax.y) + double(cx.y);
        p[n + i1] = double(ay.y) + double(cy.y);
        p[2 * n + i1] = double(az.y) + double(cz.y);
    }
}

// part[(split * 4 + k) * n + i]: (J^T w)_i (k = 0..2) and ((da/dm)^T w)_i (k = 3) of one split.
__global__ void __launch_bounds__(kPairThreads) k_vjp32(int64_t n, int64_t chunk, const float4 *__restrict__ hi,
                                                        const float4 *__restrict__ lo,
                                                        const float4 *__restrict__ w, float eps2, double *part) {
    __shared__ float4 shi[kPairThreads], slo[kPairThreads], sw[kPairThreads];
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
    const int64_t i0 = int64_t(blockIdx.x) * kPairTargets + threadIdx.x, i1 = i0 + kPairThreads;
    const bool a0 = i0 < n, a1 = i1 < n;
    const float4 h0 = a0 ? hi[i0] : z4, h1 = a1 ? hi[i1] : z4, l0 = a0 ? lo[i0] : z4, l1 = a1 ? lo[i1] : z4;
    const float4 w0 = a0 ? w[i0] : z4, w1 = a1 ? w[i1] : z4;
    const float2 nhx = make_float2(-h0.x, -h1.x), nhy = make_float2(-h0.y, -h1.y), nhz = make_float2(-h0.z, -h1.z);
    const float2 nlx = make_float2(-l0.x, -l1.x), nly = make_float2(-l0.y, -l1.y), nlz = make_float2(-l0.z, -l1.z);
    const float2 mi = make_float2(h0.w, h1.w);
    const float2 wix = make_float2(w0.x, w1.x), wiy = make_float2(w0.y, w1.y), wiz = make_float2(w0.z, w1.z);
    const float2 e2 = f2(eps2);
    float2 gx = f2(0.f), gy = f2(0.f), gz = f2(0.f), gm = f2(0.f);
    float2 cx = f2(0.f), cy = f2(0.f), cz = f2(0.f), cm = f2(0.f);
    int64_t jb = int64_t(blockIdx.y) * chunk, je = jb + chunk < n ? jb + chunk : n;
    for (int64_t j0 = jb; j0 < je; j0 += kPairThreads) {
        int64_t j = j0 + threadIdx.x;
        // padding sources: zero mass and zero weight, so u == 0 and w_j . d == 0
        shi[threadIdx.x] = j < je ? hi[j] : z4;
        slo[threadIdx.x] = j < je ? lo[j] : z4;
        sw[threadIdx.x] = j < je ? w[j] : z4;
        __syncthreads();
        float2 tx = f2(0.f), ty = f2(0.f), tz = f2(0.f), tm = f2(0.f);
#pragma unroll 4
        for (int q = 0; q < kPairThreads; ++q) {
            const float4 sh = shi[q], sl = slo[q], wj = sw[q];
            const float2 dx = add2(add2(f2(sh.x), nhx), add2(f2(sl.x), nlx));
            const float2 dy = add2(add2(f2(sh.y), nhy), add2(f2(sl.y), nly));
            const float2 dz = add2(add2(f2(sh.z), nhz), add2(f2(sl.z), nlz));
            const float2 s2 = fma2(dx, dx, fma2(dy, dy, fma2(dz, dz, e2)));
            const float2 r = make_float2(rsqrtf(s2.x), rsqrtf(s2.y));
            const float2 r2 = mul2(r, r);
            const float2 inv3 = mul2(r2, r);
            const float2 inv5 = mul2(inv3, r2);
            // u = m_i w_j - m_j w_i from two rounded products: for j == i they cancel exactly
            const float2 nmj = f2(-sh.w);
            const float2 ux = add2(mul2(mi, f2(wj.x)), mul2(nmj, wix));
            const float2 uy = add2(mul2(mi, f2(wj.y)), mul2(nmj, wiy));
            const float2 uz = add2(mul2(mi, f2(wj.z)), mul2(nmj, wiz));
            const float2 du = fma2(dx, ux, fma2(dy, uy, mul2(dz, uz)));
            const float2 nt = mul2(mul2(f2(-3.f), du), inv5);
            tx = fma2(dx, nt, fma2(ux, inv3, tx));
            ty = fma2(dy, nt, fma2(uy, inv3, ty));
            tz = fma2(dz, nt, fma2(uz, inv3, tz));
            const float2 pw = fma2(f2(wj.x), dx, fma2(f2(wj.y), dy, mul2(f2(wj.z), dz)));
            tm = fma2(pw, inv3, tm);  // the mass term is -sum pw inv3: negated at the end
        }
        __syncthreads();
        fold2(gx, cx, tx);
        fold2(gy, cy, ty);
        fold2(gz, cz, tz);
        fold2(gm, cm, tm);
    }
    double *p = part + int64_t(blockIdx.y) * 4 * n;
    if (a0) {
        p[i0] = double(gx.x) + double(cx.x);
        p[n + i0] = double(gy.x) + double(cy.x);
        p[2 * n + i0] = double(gz.x) + double(cz.x);
        p[3 * n + i0] = -(double(gm.x) + double(cm.x));
    }
    if (a1) {
        p[i1] = double(gx.y) + double(cx.y);
        p[n + i1] = double(gy.y) + double(cy.y);
        p[2 * n + i1] = double(gz.y) + double(cz.y);
        p[3 * n + i1] = -(double(gm.y) + double(cm.y));
    }
}

// ---- FP64 elementwise steps ----

enum : int { kReduce = 1, kClose = 2, kOpen = 4, kDrift = 8 };

// One fused integrator update of body i: a = sum of the splits (kReduce), v += h a (kClose),
// checkpoint (x, v, a) (ck != NULL), v += h a (kOpen), xout = xin + dt v (kDrift).
__global__ void k_update(int64_t n, int nsplit, const double *__restrict__ part, int flags, double h, double dt,
                         double *ax, double *ay, double *az, const double *xin, const double *yin,
                         const double *zin, double *xout, double *yout, double *zout, double *vx, double *vy,
                         double *vz, double *ck) {
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double a0, a1, a2;
    if (flags & kReduce) {
        a0 = a1 = a2 = 0;
        for (int s = 0; s < nsplit; ++s) {
            const double *p = part + int64_t(s) * 3 * n;
            a0 += p[i];
            a1 += p[n + i];
            a2 += p[2 * n + i];
        }
        ax[i] = a0;
        ay[i] = a1;
        az[i] = a2;
    } else {
        a0 = ax[i];
        a1 = ay[i];
        a2 = az[i];
    }
    double u = vx[i], v = vy[i], w = vz[i];
    if (flags & kClose) {
        u = u + h * a0;
        v = v + h * a1;
        w = w + h * a2;
    }
    if (ck) {
        ck[i] = xin[i];
        ck[n + i] = yin[i];
        ck[2 * n + i] = zin[i];
        ck[3 * n + i] = u;
        ck[4 * n + i] = v;
        ck[5 * n + i] = w;
        ck[6 * n + i] = a0;
        ck[7 * n + i] = a1;
        ck[8 * n + i] = a2;
    }
    if (flags & kOpen) {
        u = u + h * a0;
        v = v + h * a1;
        w = w + h * a2;
    }
    vx[i] = u;
    vy[i] = v;
    vz[i] = w;
    if (flags & kDrift) {
        xout[i] = xin[i] + dt * u;
        yout[i] = yin[i] + dt * v;
        zout[i] = zin[i] + dt * w;
    }
}

// Restores (x, v, a) of a checkpoint into (x, v, a) working arrays.
__global__ void k_restore(int64_t n, const double *__restrict__ ck, double *x, double *y, double *z, double *vx,
                          double *vy, double *vz, double *ax, double *ay, double *az) {
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    x[i] = ck[i];
    y[i] = ck[n + i];
    z[i] = ck[2 * n + i];
    vx[i] = ck[3 * n + i];
    vy[i] = ck[4 * n + i];
    vz[i] = ck[5 * n + i];
    ax[i] = ck[6 * n + i];
    ay[i] = ck[7 * n + i];
    az[i] = ck[8 * n + i];
}

// Adjoint drift: lambda_v += dt lambda_x.
__global__ void k_adj_drift(int64_t n, double dt, const double *lx, const double *ly, const double *lz, double *lu,
                            double *lv, double *lw) {
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    lu[i] = lu[i] + dt * lx[i];
    lv[i] = lv[i] + dt * ly[i];
    lw[i] = lw[i] + dt * lz[i];
}

// lambda_x += c sum of the splits, lambda_m likewise; then (drift) lambda_v += dt lambda_x, the
// adjoint drift of the step before.
__global__ void k_vjp_reduce(int64_t n, int nsplit, const double *__restrict__ part, double c, int drift, double dt,
                             double *lam) {
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double s0 = 0, s1 = 0, s2 = 0, s3 = 0;
    for (int s = 0; s < nsplit; ++s) {
        const double *p = part + int64_t(s) * 4 * n;
        s0 += p[i];
        s1 += p[n + i];
        s2 += p[2 * n + i];
        s3 += p[3 * n + i];
    }
    double lx = lam[i] + c * s0, ly = lam[n + i] + c * s1, lz = lam[2 * n + i] + c * s2;
    lam[i] = lx;
    lam[n + i] = ly;
    lam[2 * n + i] = lz;
    lam[6 * n + i] = lam[6 * n + i] + c * s3;
    if (drift) {
        lam[3 * n + i] = lam[3 * n + i] + dt * lx;
        lam[4 * n + i] = lam[4 * n + i] + dt * ly;
        lam[5 * n + i] = lam[5 * n + i] + dt * lz;
    }
}

// ---- host helpers ----

// Stars per group of the tree force's list walk. 64 (two a lane, each lane adding its two stars'
// terms before the adjoint walk's reduce-scatter) measured 5 % faster at N = 32,768 (1.73 against
// 1.82 s per 1,000-step gradient), but the tree forward's own dynamics then jump more often: its
// central differences over 1,000 steps disagree more (median 2.3e-3 against 8e-4 on 8 coordinates),
// since a star's move shifts the box of 64 stars' opening tests. 32 keeps them smoother.
constexpr int kAdjGroup = 32;

inline cudaError_t mark(AdjTape &t) { return t.mark ? t.mark(t.mark_arg) : cudaSuccess; }

// The tree at (x, y, z) for the tree force: FP32 moments, kAdjGroup-star groups of the list walk
// (the forward and the adjoint walk take the same groups, and both split among warps when the
// groups are few).
cudaError_t tree_at(const Launch &L, AdjTape &t, const double *x, const double *y, const double *z, double *ax,
                    double *ay, double *az) {
    TreeBufs &b = *t.tb;
    b.group = kAdjGroup;
    b.list_depth = 0;
    b.lpt = true;
    b.split = true;  // few groups: the forward walk shares each among several warps (the same lists)
    return tree_build(L, b, t.n, x, y, z, t.m, nullptr, nullptr, ax, ay, az, t.theta, t.leaf, 0, false, false,
                      nullptr, nullptr);
}

// Accelerations at (x, y, z): FP64 and the tree force straight into (ax, ay, az); FP32 pairs
// into t.part (summed by k_update).
cudaError_t force(const Launch &L, AdjTape &t, const double *x, const double *y, const double *z, double *ax,
                  double *ay, double *az) {
    cudaError_t e;
    if ((e = mark(t))) return e;
    if (t.tree) {
        if ((e = tree_at(L, t, x, y, z, ax, ay, az))) return e;
        if ((e = mark(t))) return e;
        if ((e = walk_lists(L, *t.tb, t.n, float(t.eps2), 1, ax, ay, az, 0, false, kAdjGroup / 32))) return e;
        return mark(t);
    }
    if (!t.fp32) {
        if ((e = mark(t))) return e;
        k_force64<<<unsigned((t.n + kPairThreads - 1) / kPairThreads), kPairThreads, 0, L.stream>>>(
            t.n, x, y, z, t.m, t.eps2, ax, ay, az);
        ADJ_LAUNCH_CHECK();
        return mark(t);
    }
    k_prep32<<<ew_blocks(t.n), kEwThreads, 0, L.stream>>>(t.n, x, y, z, t.m, nullptr, nullptr, nullptr, t.hi, t.lo,
                                                          nullptr);
    ADJ_LAUNCH_CHECK();
    if ((e = mark(t))) return e;
    dim3 grid(unsigned((t.n + kPairTargets - 1) / kPairTargets), unsigned(t.nsplit));
    k_force32<<<grid, kPairThreads, 0, L.stream>>>(t.n, t.chunk, t.hi, t.lo, float(t.eps2), t.part);
    ADJ_LAUNCH_CHECK();
    return mark(t);
}

cudaError_t update(const Launch &L, AdjTape &t, int flags, const double *xin, double *xout, double *v, double *a,
                   double *ck) {
    int64_t n = t.n;
    if (!t.fp32 || t.tree) flags &= ~kReduce;
    k_update<<<ew_blocks(n), kEwThreads, 0, L.stream>>>(n, t.nsplit, t.part, flags, 0.5 * t.dt, t.dt, a, a + n,
                                                        a + 2 * n, xin, xin + n, xin + 2 * n, xout, xout + n,
                                                        xout + 2 * n, v, v + n, v + 2 * n, ck);
    ADJ_LAUNCH_CHECK();
    return cudaSuccess;
}

// lambda_x, lambda_m += c (kicks at positions x with weights lambda_v); then, when drift, the
// adjoint drift of the step before.
cudaError_t vjp(const Launch &L, AdjTape &t, const double *x, double c, bool drift) {
    int64_t n = t.n;
    double *lam = t.lam;
    cudaError_t e;
    if ((e = mark(t))) return e;
    if (t.tree) {  // the tree at x again (the forward's lists), then its transposed Jacobian
        if ((e = tree_at(L, t, x, x + n, x + 2 * n, t.ra, t.ra + n, t.ra + 2 * n))) return e;
        if ((e = mark(t))) return e;
        if ((e = walk_lists_adjoint(L, *t.tb, float(t.eps2), x, x + n, x + 2 * n, t.m, lam + 3 * n, lam + 4 * n,
                                    lam + 5 * n, n, t.tbs, t.part)))
            return e;
        if ((e = mark(t))) return e;
        k_vjp_reduce<<<ew_blocks(n), kEwThreads, 0, L.stream>>>(n, 1, t.part, c, drift ? 1 : 0, t.dt, lam);
        ADJ_LAUNCH_CHECK();
        return cudaSuccess;
    }
    if (!t.fp32) {
        if ((e = mark(t))) return e;
        k_vjp64<<<unsigned((n + kPairThreads - 1) / kPairThreads), kPairThreads, 0, L.stream>>>(
            n, x, x + n, x + 2 * n, t.m, lam + 3 * n, lam + 4 * n, lam + 5 * n, t.eps2, c, lam, lam + n, lam + 2 * n,
            lam + 6 * n);
        ADJ_LAUNCH_CHECK();
        if ((e = mark(t))) return e;
        if (drift) {
            k_adj_drift<<<ew_blocks(n), kEwThreads, 0, L.stream>>>(n, t.dt, lam, lam + n, lam + 2 * n, lam + 3 * n,
                                                                   lam + 4 * n, lam + 5 * n);
            ADJ_LAUNCH_CHECK();
        }
        return cudaSuccess;
    }
    k_prep32<<<ew_blocks(n), kEwThreads, 0, L.stream>>>(n, x, x + n, x + 2 * n, t.m, lam + 3 * n, lam + 4 * n,
                                                        lam + 5 * n, t.hi, t.lo, t.w);
    ADJ_LAUNCH_CHECK();
    if ((e = mark(t))) return e;
    dim3 grid(unsigned((n + kPairTargets - 1) / kPairTargets), unsigned(t.nsplit));
    k_vjp32<<<grid, kPairThreads, 0, L.stream>>>(n, t.chunk, t.hi, t.lo, t.w, float(t.eps2), t.part);
    ADJ_LAUNCH_CHECK();
    if ((e = mark(t))) return e;
    k_vjp_reduce<<<ew_blocks(n), kEwThreads, 0, L.stream>>>(n, t.nsplit, t.part, c, drift ? 1 : 0, t.dt, lam);
    ADJ_LAUNCH_CHECK();
    return cudaSuccess;
}

}  // namespace

void adj_free(AdjTape &t) {
    if (t.block) cudaFree(t.block);
    adj_tree_free(t.tbs);
    t = AdjTape{};
}

cudaError_t adj_reserve(AdjTape &t, int64_t n, int64_t nsteps, int64_t every, double dt, double eps, bool fp32,
                        int num_sms) {
    t.valid = false;
    int64_t nck = (nsteps + every - 1) / every;
    int64_t seg = std::min(every, nsteps);
    // j splits: about 8 blocks per SM, each split at least 4 tiles long
    int64_t nb = (n + kPairTargets - 1) / kPairTargets;
    int64_t ns = fp32 ? std::max<int64_t>(1, (8 * int64_t(num_sms) + nb - 1) / nb) : 1;
    ns = std::min<int64_t>(ns, std::max<int64_t>(1, n / (4 * kPairThreads)));
    ns = std::min<int64_t>(ns, 64);
    int64_t chunk = (n + ns - 1) / ns;
    chunk = (chunk + kPairThreads - 1) / kPairThreads * kPairThreads;
    ns = (n + chunk - 1) / chunk;
    // doubles: x v a (9n), mass (n), lambda (7n), checkpoints (9n each), segment positions (3n
    // each), replay v and a (6n), splits (4n each); floats: hi lo w (12n)
    int64_t nd = 9 * n + n + 7 * n + 9 * n * nck + 3 * n * seg + 6 * n + (fp32 ? 4 * n * ns : 0);
    size_t bytes = sizeof(double) * size_t(nd) + (fp32 ? sizeof(float4) * 3 * size_t(n) : 0) + 256;
    if (bytes > t.bytes) {
        if (t.block) cudaFree(t.block);
        t.block = nullptr;
        t.bytes = 0;
        size_t want = bytes + bytes / 4;
        cudaError_t e = dev_alloc(&t.block, want);
        if (e != cudaSuccess) return e;
        t.bytes = want;
    }
    double *p = static_cast<double *>(t.block);
    auto take = [&](int64_t cnt) {
        double *q = p;
        p += cnt;
        return q;
    };
    t.x = take(3 * n);
    t.v = take(3 * n);
    t.a = take(3 * n);
    t.m = take(n);
    t.lam = take(7 * n);
    t.ck = take(9 * n * nck);
    t.seg = take(3 * n * seg);
    t.rv = take(3 * n);
    t.ra = take(3 * n);
    t.part = fp32 ? take(4 * n * ns) : nullptr;
    float4 *f = reinterpret_cast<float4 *>((reinterpret_cast<uintptr_t>(p) + 15) & ~uintptr_t(15));
    t.hi = fp32 ? f : nullptr;
    t.lo = fp32 ? f + n : nullptr;
    t.w = fp32 ? f + 2 * n : nullptr;
    t.n = n;
    t.nsteps = nsteps;
    t.every = every;
    t.nck = nck;
    t.nsplit = int(ns);
    t.chunk = chunk;
    t.dt = dt;
    t.eps2 = eps * eps;
    t.fp32 = fp32;
    return cudaSuccess;
}

cudaError_t adj_forward(const Launch &L, AdjTape &t) {
    cudaError_t e;
    const int64_t T = t.nsteps;
    double *x = t.x;
    if ((e = force(L, t, x, x + t.n, x + 2 * t.n, t.a, t.a + t.n, t.a + 2 * t.n))) return e;
    for (int64_t s = 0; s < T; ++s) {
        int flags = kReduce | kOpen | kDrift | (s > 0 ? kClose : 0);
        double *ck = s % t.every == 0 ? t.ck + 9 * t.n * (s / t.every) : nullptr;
        if ((e = update(L, t, flags, x, x, t.v, t.a, ck))) return e;
        if ((e = force(L, t, x, x + t.n, x + 2 * t.n, t.a, t.a + t.n, t.a + 2 * t.n))) return e;
    }
    if ((e = update(L, t, kReduce | kClose, x, x, t.v, t.a, nullptr))) return e;
    t.valid = true;
    return cudaSuccess;
}

cudaError_t adj_backward(const Launch &L, AdjTape &t) {
    cudaError_t e;
    const int64_t n = t.n, T = t.nsteps;
    const double h = 0.5 * t.dt;
    // closing kick of the last step, at x_T
    if ((e = vjp(L, t, t.x, h, true))) return e;
    for (int64_t c = t.nck - 1; c >= 0; --c) {
        int64_t s0 = c * t.every, k = std::min(t.every, T - s0);
        // replay: seg[q] = x_{s0 + q}
        k_restore<<<ew_blocks(n), kEwThreads, 0, L.stream>>>(n, t.ck + 9 * n * c, t.seg, t.seg + n, t.seg + 2 * n,
                                                             t.rv, t.rv + n, t.rv + 2 * n, t.ra, t.ra + n,
                                                             t.ra + 2 * n);
        ADJ_LAUNCH_CHECK();
        for (int64_t q = 0; q + 1 < k; ++q) {
            double *xq = t.seg + 3 * n * q, *xn = t.seg + 3 * n * (q + 1);
            if (q > 0 && (e = force(L, t, xq, xq + n, xq + 2 * n, t.ra, t.ra + n, t.ra + 2 * n))) return e;
            int flags = kOpen | kDrift | (q > 0 ? kReduce | kClose : 0);
            if ((e = update(L, t, flags, xq, xn, t.rv, t.ra, nullptr))) return e;
        }
        // adjoint steps s = s0 + k - 1 .. s0; the drift of step s was applied by the call before
        for (int64_t q = k - 1; q >= 0; --q) {
            int64_t s = s0 + q;
            if ((e = vjp(L, t, t.seg + 3 * n * q, s > 0 ? t.dt : h, s > 0))) return e;
        }
    }
    return cudaSuccess;
}

}  // namespace gbh
