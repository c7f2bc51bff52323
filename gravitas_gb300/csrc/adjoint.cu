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

// ---- FP64 pair kernels (the checker's loops, j ascending) ----

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

// part[(split * 3 + axis) * n + i]: the accelerations of target i from the sources of one split.
__global__ void __launch_bounds__(kPairThreads) k_force32(int64_t n, int64_t chunk, const float4 *__restrict__ hi,
                                                          const float4 *__restrict__ lo, float eps2,
                                                          double *part) {
    __shared__ float4 shi[kPairThreads], slo[kPairThreads];
    int64_t i = int64_t(blockIdx.x) * kPairThreads + threadIdx.x;
    bool act = i < n;
    float4 h = act ? hi[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    float4 l = act ? lo[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    float ax = 0.f, ay = 0.f, az = 0.f, cx = 0.f, cy = 0.f, cz = 0.f;
    int64_t jb = int64_t(blockIdx.y) * chunk, je = jb + chunk < n ? jb + chunk : n;
    for (int64_t j0 = jb; j0 < je; j0 += kPairThreads) {
        int64_t j = j0 + threadIdx.x;
        // padding sources have zero mass at the origin: s^2 >= eps^2 > 0, so they add exactly 0
        shi[threadIdx.x] = j < je ? hi[j] : make_float4(0.f, 0.f, 0.f, 0.f);
        slo[threadIdx.x] = j < je ? lo[j] : make_float4(0.f, 0.f, 0.f, 0.f);
        __syncthreads();
        float tx = 0.f, ty = 0.f, tz = 0.f;
#pragma unroll 8
        for (int q = 0; q < kPairThreads; ++q) {
            float4 sh = shi[q], sl = slo[q];
            // j == i gives d == 0 exactly and adds nothing
            float dx = (sh.x - h.x) + (sl.x - l.x);
            float dy = (sh.y - h.y) + (sl.y - l.y);
            float dz = (sh.z - h.z) + (sl.z - l.z);
            float s2 = fmaf(dx, dx, fmaf(dy, dy, fmaf(dz, dz, eps2)));
            float r = rsqrtf(s2);
            float f = (sh.w * r) * (r * r);
            tx = fmaf(f, dx, tx);
            ty = fmaf(f, dy, ty);
            tz = fmaf(f, dz, tz);
        }
        __syncthreads();
        fold(ax, cx, tx);
        fold(ay, cy, ty);
        fold(az, cz, tz);
    }
    if (act) {
        double *p = part + int64_t(blockIdx.y) * 3 * n;
        p[i] = double(ax) + double(cx);
        p[n + i] = double(ay) + double(cy);
        p[2 * n + i] = double(az) + double(cz);
    }
}

// part[(split * 4 + k) * n + i]: (J^T w)_i (k = 0..2) and ((da/dm)^T w)_i (k = 3) of one split.
__global__ void __launch_bounds__(kPairThreads) k_vjp32(int64_t n, int64_t chunk, const float4 *__restrict__ hi,
                                                        const float4 *__restrict__ lo,
                                                        const float4 *__restrict__ w, float eps2, double *part) {
    __shared__ float4 shi[kPairThreads], slo[kPairThreads], sw[kPairThreads];
    int64_t i = int64_t(blockIdx.x) * kPairThreads + threadIdx.x;
    bool act = i < n;
    float4 h = act ? hi[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    float4 l = act ? lo[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    float4 wi = act ? w[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    float gx = 0.f, gy = 0.f, gz = 0.f, gm = 0.f, cx = 0.f, cy = 0.f, cz = 0.f, cm = 0.f;
    int64_t jb = int64_t(blockIdx.y) * chunk, je = jb + chunk < n ? jb + chunk : n;
    for (int64_t j0 = jb; j0 < je; j0 += kPairThreads) {
        int64_t j = j0 + threadIdx.x;
        // padding sources: zero mass and zero weight, so u == 0 and w_j . d == 0
        shi[threadIdx.x] = j < je ? hi[j] : make_float4(0.f, 0.f, 0.f, 0.f);
        slo[threadIdx.x] = j < je ? lo[j] : make_float4(0.f, 0.f, 0.f, 0.f);
        sw[threadIdx.x] = j < je ? w[j] : make_float4(0.f, 0.f, 0.f, 0.f);
        __syncthreads();
        float tx = 0.f, ty = 0.f, tz = 0.f, tm = 0.f;
#pragma unroll 4
        for (int q = 0; q < kPairThreads; ++q) {
            float4 sh = shi[q], sl = slo[q], wj = sw[q];
            float dx = (sh.x - h.x) + (sl.x - l.x);
            float dy = (sh.y - h.y) + (sl.y - l.y);
            float dz = (sh.z - h.z) + (sl.z - l.z);
            float s2 = fmaf(dx, dx, fmaf(dy, dy, fmaf(dz, dz, eps2)));
            float r = rsqrtf(s2);
            float r2 = r * r;
            float inv3 = r2 * r;
            float inv5 = inv3 * r2;
            // separate products: for j == i both are equal and u is exactly 0
            float ux = h.w * wj.x - sh.w * wi.x;
            float uy = h.w * wj.y - sh.w * wi.y;
            float uz = h.w * wj.z - sh.w * wi.z;
            float du = fmaf(dx, ux, fmaf(dy, uy, dz * uz));
            float t = 3.f * du * inv5;
            tx = fmaf(-dx, t, fmaf(ux, inv3, tx));
            ty = fmaf(-dy, t, fmaf(uy, inv3, ty));
            tz = fmaf(-dz, t, fmaf(uz, inv3, tz));
            float pw = fmaf(wj.x, dx, fmaf(wj.y, dy, wj.z * dz));
            tm = fmaf(-pw, inv3, tm);
        }
        __syncthreads();
        fold(gx, cx, tx);
        fold(gy, cy, ty);
        fold(gz, cz, tz);
        fold(gm, cm, tm);
    }
    if (act) {
        double *p = part + int64_t(blockIdx.y) * 4 * n;
        p[i] = double(gx) + double(cx);
        p[n + i] = double(gy) + double(cy);
        p[2 * n + i] = double(gz) + double(cz);
        p[3 * n + i] = double(gm) + double(cm);
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

inline cudaError_t mark(AdjTape &t) { return t.mark ? t.mark(t.mark_arg) : cudaSuccess; }

// Accelerations at (x, y, z): FP64 straight into (ax, ay, az); FP32 into t.part (summed by k_update).
cudaError_t force(const Launch &L, AdjTape &t, const double *x, const double *y, const double *z, double *ax,
                  double *ay, double *az) {
    cudaError_t e;
    if ((e = mark(t))) return e;
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
    dim3 grid(unsigned((t.n + kPairThreads - 1) / kPairThreads), unsigned(t.nsplit));
    k_force32<<<grid, kPairThreads, 0, L.stream>>>(t.n, t.chunk, t.hi, t.lo, float(t.eps2), t.part);
    ADJ_LAUNCH_CHECK();
    return mark(t);
}

cudaError_t update(const Launch &L, AdjTape &t, int flags, const double *xin, double *xout, double *v, double *a,
                   double *ck) {
    int64_t n = t.n;
    if (!t.fp32) flags &= ~kReduce;
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
    dim3 grid(unsigned((n + kPairThreads - 1) / kPairThreads), unsigned(t.nsplit));
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
    t = AdjTape{};
}

cudaError_t adj_reserve(AdjTape &t, int64_t n, int64_t nsteps, int64_t every, double dt, double eps, bool fp32,
                        int num_sms) {
    t.valid = false;
    int64_t nck = (nsteps + every - 1) / every;
    int64_t seg = std::min(every, nsteps);
    // j splits: about 8 blocks of kPairThreads per SM, each split at least 4 tiles long
    int64_t nb = (n + kPairThreads - 1) / kPairThreads;
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
        cudaError_t e = cudaMalloc(&t.block, want);
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
