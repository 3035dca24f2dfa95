// common.cuh - device building blocks of the rod step.
//
// Arithmetic specification shared with the CPU oracle: every FP64 expression
// on the FP64 path is written in one fixed evaluation order, the FP64
// translation units are compiled with --fmad=false (no contraction), and the
// only operations used are IEEE +,-,*,/,sqrt plus the log / sincos below,
// which are built from those.  Sums over constraints use the fixed tree of
// block_tree_sum / chunk reduction.  With identical inputs the FP64 GPU path
// therefore reproduces the oracle bit for bit.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace alens {

constexpr double kPi = 3.141592653589793;
constexpr double kTwoPi = 6.283185307179586;
constexpr double kLn2 = 0.6931471805599453;
constexpr double kParallelEps = 1e-12;
constexpr int kTile = 64;         // level-1 reduction tile (constraints)
constexpr int kChunk = 1024;      // level-2+ reduction chunk (one warp)
constexpr int kImageNone = 13;    // image code of the zero periodic shift
constexpr int kImageBoundary = 27; // keys (i, b, 27 + point): rod i against boundary b

// error flag bits (DevCtl::errFlags)
constexpr int kErrOverflow = 1;
constexpr int kErrNaN = 2;
constexpr int kErrTimeout = 4;
constexpr int kErrSolverFit = 8;  // the cluster-resident solver could not hold the
                                  // problem; the host reruns the step in grid form
// flags after which the solve and the update of a step are skipped
constexpr int kErrStepAbort = kErrOverflow | kErrNaN | kErrTimeout | kErrSolverFit;

// ------------------------------------------------------------------ math
// Natural logarithm: x = m 2^e, m in [sqrt(1/2), sqrt(2)),
// log m = 2 atanh((m-1)/(m+1)) by its power series to the 23rd power.
__host__ __device__ inline double det_log(double x) {
#ifdef __CUDA_ARCH__
    unsigned long long bits = (unsigned long long)__double_as_longlong(x);
#else
    unsigned long long bits;
    __builtin_memcpy(&bits, &x, 8);
#endif
    int e = (int)((bits >> 52) & 0x7ff);
    if (e == 0) {
        x = x * 18014398509481984.0;  // 2^54, exact
#ifdef __CUDA_ARCH__
        bits = (unsigned long long)__double_as_longlong(x);
#else
        __builtin_memcpy(&bits, &x, 8);
#endif
        e = (int)((bits >> 52) & 0x7ff) - 54;
    }
    e -= 1023;
    bits = (bits & 0x800fffffffffffffULL) | (0x3ffULL << 52);
    double m;
#ifdef __CUDA_ARCH__
    m = __longlong_as_double((long long)bits);
#else
    __builtin_memcpy(&m, &bits, 8);
#endif
    if (m > 1.4142135623730951) {
        m = m * 0.5;
        e += 1;
    }
    const double u = (m - 1.0) / (m + 1.0);
    const double u2 = u * u;
    double p = 1.0 / 23.0;
    p = p * u2 + 1.0 / 21.0;
    p = p * u2 + 1.0 / 19.0;
    p = p * u2 + 1.0 / 17.0;
    p = p * u2 + 1.0 / 15.0;
    p = p * u2 + 1.0 / 13.0;
    p = p * u2 + 1.0 / 11.0;
    p = p * u2 + 1.0 / 9.0;
    p = p * u2 + 1.0 / 7.0;
    p = p * u2 + 1.0 / 5.0;
    p = p * u2 + 1.0 / 3.0;
    p = p * u2 + 1.0;
    return (double)e * kLn2 + 2.0 * u * p;
}

// sin and cos by halving to |x| <= 1, Taylor polynomials (to x^19 and
// x^20), then the double-angle identities.
__host__ __device__ inline void det_sincos(double x, double *s_out, double *c_out) {
    int k = 0;
    while (fabs(x) > 1.0 && k < 64) {
        x = x * 0.5;
        k++;
    }
    const double x2 = x * x;
    double s = -1.0 / 121645100408832000.0;
    s = s * x2 + 1.0 / 355687428096000.0;
    s = s * x2 - 1.0 / 1307674368000.0;
    s = s * x2 + 1.0 / 6227020800.0;
    s = s * x2 - 1.0 / 39916800.0;
    s = s * x2 + 1.0 / 362880.0;
    s = s * x2 - 1.0 / 5040.0;
    s = s * x2 + 1.0 / 120.0;
    s = s * x2 - 1.0 / 6.0;
    s = s * x2 + 1.0;
    s = s * x;
    double c = 1.0 / 2432902008176640000.0;
    c = c * x2 - 1.0 / 6402373705728000.0;
    c = c * x2 + 1.0 / 20922789888000.0;
    c = c * x2 - 1.0 / 87178291200.0;
    c = c * x2 + 1.0 / 479001600.0;
    c = c * x2 - 1.0 / 3628800.0;
    c = c * x2 + 1.0 / 40320.0;
    c = c * x2 - 1.0 / 720.0;
    c = c * x2 + 1.0 / 24.0;
    c = c * x2 - 0.5;
    c = c * x2 + 1.0;
    for (int i = 0; i < k; i++) {
        const double s2 = 2.0 * s * c;
        const double c2 = c * c - s * s;
        s = s2;
        c = c2;
    }
    *s_out = s;
    *c_out = c;
}

// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11).
__host__ __device__ inline void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
    uint32_t c0 = c[0], c1 = c[1], c2 = c[2], c3 = c[3];
#pragma unroll
    for (int r = 0; r < 10; r++) {
        const unsigned long long p0 = (unsigned long long)0xD2511F53u * c0;
        const unsigned long long p1 = (unsigned long long)0xCD9E8D57u * c2;
        const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        c0 = hi1 ^ c1 ^ k0;
        c1 = lo1;
        c2 = hi0 ^ c3 ^ k1;
        c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    c[0] = c0;
    c[1] = c1;
    c[2] = c2;
    c[3] = c3;
}

// Six standard normals keyed by (seed, gid, step): Philox blocks with
// counter (gid_lo, gid_hi, step, b), b = 0,1,2; uniforms with 53 bits from
// word pairs; Box-Muller with the project's log and sincos.
// FP32 natural log for x in (0, inf) normal: x = m 2^e, m in [sqrt(1/2),
// sqrt(2)), log m = 2 atanh(u), u = (m-1)/(m+1), series to u^13.
__host__ __device__ inline float det_logf(float x) {
#ifdef __CUDA_ARCH__
    unsigned int bits = (unsigned int)__float_as_int(x);
#else
    unsigned int bits;
    __builtin_memcpy(&bits, &x, 4);
#endif
    int e = (int)((bits >> 23) & 0xffu) - 127;
    bits = (bits & 0x807fffffu) | (127u << 23);
    float m;
#ifdef __CUDA_ARCH__
    m = __int_as_float((int)bits);
#else
    __builtin_memcpy(&m, &bits, 4);
#endif
    if (m > 1.41421356f) {
        m = m * 0.5f;
        e += 1;
    }
    const float u = (m - 1.0f) / (m + 1.0f);
    const float u2 = u * u;
    float p = 1.0f / 13.0f;
    p = p * u2 + 1.0f / 11.0f;
    p = p * u2 + 1.0f / 9.0f;
    p = p * u2 + 1.0f / 7.0f;
    p = p * u2 + 1.0f / 5.0f;
    p = p * u2 + 1.0f / 3.0f;
    p = p * u2 + 1.0f;
    return (float)e * 0.693147181f + 2.0f * u * p;
}

// FP32 sin and cos for |x| <= pi: halve until |x| <= 1, Taylor polynomials
// to x^11 / x^12, then the double-angle identities.
__host__ __device__ inline void det_sincosf(float x, float *s_out, float *c_out) {
    int k = 0;
    while ((x < 0.0f ? -x : x) > 1.0f && k < 8) {
        x = x * 0.5f;
        k++;
    }
    const float x2 = x * x;
    float s = -1.0f / 39916800.0f;
    s = s * x2 + 1.0f / 362880.0f;
    s = s * x2 - 1.0f / 5040.0f;
    s = s * x2 + 1.0f / 120.0f;
    s = s * x2 - 1.0f / 6.0f;
    s = s * x2 + 1.0f;
    s = s * x;
    float c = 1.0f / 479001600.0f;
    c = c * x2 - 1.0f / 3628800.0f;
    c = c * x2 + 1.0f / 40320.0f;
    c = c * x2 - 1.0f / 720.0f;
    c = c * x2 + 1.0f / 24.0f;
    c = c * x2 - 0.5f;
    c = c * x2 + 1.0f;
    for (int i = 0; i < k; i++) {
        const float s2 = 2.0f * s * c;
        const float c2 = c * c - s * s;
        s = s2;
        c = c2;
    }
    *s_out = s;
    *c_out = c;
}

// Six standard normals for (seed, gid, step): two Philox blocks, six 24-bit
// uniforms in (0,1), three Box-Muller pairs in FP32 (the noise needs no
// more; FP64 transcendentals cost 64x more issue on GB300).
__host__ __device__ inline void normals6(unsigned long long seed, long long gid, long long step,
                                         double z[6]) {
    uint32_t w[8];
    for (uint32_t b = 0; b < 2; b++) {
        uint32_t c[4] = {(uint32_t)(unsigned long long)gid,
                         (uint32_t)((unsigned long long)gid >> 32),
                         (uint32_t)(unsigned long long)step, b};
        philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
        w[4 * b] = c[0];
        w[4 * b + 1] = c[1];
        w[4 * b + 2] = c[2];
        w[4 * b + 3] = c[3];
    }
    float u[6];
#pragma unroll
    for (int i = 0; i < 6; i++) u[i] = ((float)(w[i] >> 8) + 0.5f) * 5.9604644775390625e-08f;  // 2^-24
#pragma unroll
    for (int p = 0; p < 3; p++) {
        const float r = sqrtf(-2.0f * det_logf(u[2 * p]));
        const float ang = u[2 * p + 1] * 6.28318531f - 3.14159265f;
        float sn, cs;
        det_sincosf(ang, &sn, &cs);
        // angle + pi: cos -> -cos, sin -> -sin
        z[2 * p] = (double)(r * -cs);
        z[2 * p + 1] = (double)(r * -sn);
    }
}

// ------------------------------------------------------------ boundaries
// Boundary with a unit axis (normalised on the host); the oracle states the
// same arithmetic.
struct BoundaryDev {
    int type, inside;
    double c[3], a[3], R;
};

// Contact points of a rod with a boundary: both ends for walls and for
// inside spheres/tubes (one point, the centre, for sphere-shaped rods); the
// point nearest the centre for outside spheres.
__host__ __device__ inline int boundary_npoints(const BoundaryDev &B, double h) {
    if (B.type == 1 && !B.inside) return 1;
    return h > 0.0 ? 2 : 1;
}

// Contact point e of rod (centre x, unit axis u, collision half-length h):
// Q, the signed distance s of Q to the boundary (positive on the allowed
// side) and the unit normal n pointing into the allowed region.
__host__ __device__ inline void boundary_contact(const BoundaryDev &B, const double x[3], const double u[3],
                                                 double h, int e, double Q[3], double &s, double n[3]) {
    double t;
    if (B.type == 1 && !B.inside) {
        t = (B.c[0] - x[0]) * u[0] + (B.c[1] - x[1]) * u[1] + (B.c[2] - x[2]) * u[2];
        t = t < -h ? -h : (t > h ? h : t);
    } else {
        t = e == 0 ? -h : h;
    }
    Q[0] = x[0] + t * u[0];
    Q[1] = x[1] + t * u[1];
    Q[2] = x[2] + t * u[2];
    const double v[3] = {Q[0] - B.c[0], Q[1] - B.c[1], Q[2] - B.c[2]};
    if (B.type == 0) {  // wall
        s = v[0] * B.a[0] + v[1] * B.a[1] + v[2] * B.a[2];
        n[0] = B.a[0];
        n[1] = B.a[1];
        n[2] = B.a[2];
        return;
    }
    double w[3];
    if (B.type == 2) {  // tube: radial part of v
        const double p = v[0] * B.a[0] + v[1] * B.a[1] + v[2] * B.a[2];
        w[0] = v[0] - p * B.a[0];
        w[1] = v[1] - p * B.a[1];
        w[2] = v[2] - p * B.a[2];
    } else {
        w[0] = v[0];
        w[1] = v[1];
        w[2] = v[2];
    }
    const double rho = sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
    double d[3] = {1.0, 0.0, 0.0};
    if (rho > 0.0) {
        d[0] = w[0] / rho;
        d[1] = w[1] / rho;
        d[2] = w[2] / rho;
    }
    if (B.inside) {
        s = B.R - rho;
        n[0] = -d[0];
        n[1] = -d[1];
        n[2] = -d[2];
    } else {
        s = rho - B.R;
        n[0] = d[0];
        n[1] = d[1];
        n[2] = d[2];
    }
}

// ------------------------------------------------------------ rod geometry
__host__ __device__ inline void quat_axis(double qx, double qy, double qz, double qw, double a[3]) {
    a[0] = 2.0 * (qx * qz + qw * qy);
    a[1] = 2.0 * (qy * qz - qw * qx);
    a[2] = 1.0 - 2.0 * (qx * qx + qy * qy);
}

// Drag mobilities (1/zeta_par, 1/zeta_perp, 1/zeta_rot) of a straight rod
// from the local slender-body operator (Tornberg & Shelley 2004):
// b = -(1 + 2 ln(r/L)); zeta_par = 4 pi mu L / b; zeta_perp = 8 pi mu L /
// (b+2); zeta_rot = 2 pi mu L^3 / (3 (b+2)).  Spheres (L < 2r): Stokes drag.
__host__ __device__ inline void mobility_coeffs(double L, double r, double mu, bool sphere,
                                                double out[3]) {
    if (sphere) {
        const double mt = 1.0 / (6.0 * kPi * mu * r);
        out[0] = mt;
        out[1] = mt;
        out[2] = 1.0 / (8.0 * kPi * mu * r * r * r);
    } else {
        const double eps = r / L;
        const double b = -(1.0 + 2.0 * det_log(eps));
        out[0] = b / (4.0 * kPi * mu * L);
        out[1] = (b + 2.0) / (8.0 * kPi * mu * L);
        out[2] = 3.0 * (b + 2.0) / (2.0 * kPi * mu * L * L * L);
    }
}

// U = M F for one rod; monolayer projects out z force/velocity and x,y
// torque/rotation on both sides.
template <class T>
__host__ __device__ inline void mobility_apply(const T a[3], const T m[3], bool sphere, bool mono,
                                               const T F[6], T U[6]) {
    T f0 = F[0], f1 = F[1], f2 = F[2];
    T t0 = F[3], t1 = F[4], t2 = F[5];
    if (mono) {
        f2 = T(0);
        t0 = T(0);
        t1 = T(0);
    }
    if (sphere) {
        U[0] = m[0] * f0;
        U[1] = m[0] * f1;
        U[2] = m[0] * f2;
        U[3] = m[2] * t0;
        U[4] = m[2] * t1;
        U[5] = m[2] * t2;
    } else {
        const T fa = a[0] * f0 + a[1] * f1 + a[2] * f2;
        U[0] = m[0] * fa * a[0] + m[1] * (f0 - fa * a[0]);
        U[1] = m[0] * fa * a[1] + m[1] * (f1 - fa * a[1]);
        U[2] = m[0] * fa * a[2] + m[1] * (f2 - fa * a[2]);
        const T ta = a[0] * t0 + a[1] * t1 + a[2] * t2;
        U[3] = m[2] * (t0 - ta * a[0]);
        U[4] = m[2] * (t1 - ta * a[1]);
        U[5] = m[2] * (t2 - ta * a[2]);
    }
    if (mono) {
        U[2] = T(0);
        U[3] = T(0);
        U[4] = T(0);
    }
}

__host__ __device__ inline double clampd(double x, double lo, double hi) {
    return x < lo ? lo : (x > hi ? hi : x);
}

__host__ __device__ inline void cross3(const double a[3], const double b[3], double c[3]) {
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}

// Closest points of segments c1 + s u1 (|s| <= h1) and c2 + t u2 (|t| <= h2)
// with unit axes (Ericson, Real-Time Collision Detection, sec. 5.1.9,
// centred parameterisation); parallel overlapping segments take the middle
// of the overlap.
struct DcpResult {
    double s, t, dist;
    double P[3], Q[3];
};

__host__ __device__ inline DcpResult dcp_segseg(const double c1[3], const double u1[3], double h1,
                                                const double c2[3], const double u2[3], double h2) {
    DcpResult R;
    const double w0 = c1[0] - c2[0], w1 = c1[1] - c2[1], w2 = c1[2] - c2[2];
    const double b = u1[0] * u2[0] + u1[1] * u2[1] + u1[2] * u2[2];
    const double d = u1[0] * w0 + u1[1] * w1 + u1[2] * w2;
    const double e = u2[0] * w0 + u2[1] * w1 + u2[2] * w2;
    const double det = 1.0 - b * b;
    double s, t;
    if (det > kParallelEps) {
        s = clampd((b * e - d) / det, -h1, h1);
    } else {
        const double ab = fabs(b);
        const double l1 = -d - ab * h2;
        const double l2 = -d + ab * h2;
        const double lo = (-h1 < l1) ? l1 : -h1;   // max(-h1, l1)
        const double hi = (l2 < h1) ? l2 : h1;     // min(h1, l2)
        if (lo <= hi)
            s = 0.5 * (lo + hi);
        else
            s = clampd(-d, -h1, h1);
    }
    t = b * s + e;
    if (t < -h2) {
        t = -h2;
        s = clampd(b * t - d, -h1, h1);
    } else if (t > h2) {
        t = h2;
        s = clampd(b * t - d, -h1, h1);
    }
    R.P[0] = c1[0] + s * u1[0];
    R.P[1] = c1[1] + s * u1[1];
    R.P[2] = c1[2] + s * u1[2];
    R.Q[0] = c2[0] + t * u2[0];
    R.Q[1] = c2[1] + t * u2[1];
    R.Q[2] = c2[2] + t * u2[2];
    const double x0 = R.P[0] - R.Q[0], x1 = R.P[1] - R.Q[1], x2 = R.P[2] - R.Q[2];
    R.dist = sqrt(x0 * x0 + x1 * x1 + x2 * x2);
    R.s = s;
    R.t = t;
    return R;
}

// Unit normal pointing from Q (rod J) to P (rod I); when the axes touch
// (distance 0) a direction perpendicular to both axes is used.
__host__ __device__ inline void contact_normal(const DcpResult &R, const double u1[3],
                                               const double u2[3], double n[3]) {
    if (R.dist > 0.0) {
        n[0] = (R.P[0] - R.Q[0]) / R.dist;
        n[1] = (R.P[1] - R.Q[1]) / R.dist;
        n[2] = (R.P[2] - R.Q[2]) / R.dist;
        return;
    }
    double c[3];
    cross3(u1, u2, c);
    double cn = sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
    if (!(cn > 0.0)) {
        const double ax = fabs(u1[0]);
        const double ay = fabs(u1[1]);
        const double az = fabs(u1[2]);
        double e[3] = {0.0, 0.0, 0.0};
        if (ax <= ay && ax <= az)
            e[0] = 1.0;
        else if (ay <= az)
            e[1] = 1.0;
        else
            e[2] = 1.0;
        cross3(u1, e, c);
        cn = sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
    }
    n[0] = c[0] / cn;
    n[1] = c[1] / cn;
    n[2] = c[2] / cn;
}

__host__ __device__ inline unsigned long long pair_key(int i, int j, int img) {
    return ((unsigned long long)(unsigned)i << 32) | ((unsigned long long)(unsigned)j << 5) |
           (unsigned long long)img;
}

// ----------------------------------------------------- reduction trees
// Warp tree: lane l accumulates v[l] + v[l+off] for off = 16, 8, 4, 2, 1;
// lane 0 holds the result.
__device__ __forceinline__ double warp_tree_sum(double v) {
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) {
        const double o = __shfl_down_sync(0xffffffffu, v, off);
        v = v + o;
    }
    return v;
}

template <class T>
__device__ __forceinline__ T warp_tree_sum_t(T v) {
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) {
        const T o = __shfl_down_sync(0xffffffffu, v, off);
        v = v + o;
    }
    return v;
}

__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) {
        const double o = __shfl_down_sync(0xffffffffu, v, off);
        v = (o > v) ? o : v;
    }
    return v;
}

// Block tree over a 256-thread block: warp trees, then the same tree over
// the 8 warp sums with offsets 4,2,1.  Result valid in thread 0.
// scratch: 8 doubles of shared memory per value.
template <int NV>
__device__ __forceinline__ void block_tree_sum256(double (&v)[NV], double (*scratch)[8]) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < NV; q++) v[q] = warp_tree_sum(v[q]);
    if (lane == 0) {
#pragma unroll
        for (int q = 0; q < NV; q++) scratch[q][warp] = v[q];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int q = 0; q < NV; q++) {
            double w[8];
#pragma unroll
            for (int i = 0; i < 8; i++) w[i] = scratch[q][i];
#pragma unroll
            for (int off = 4; off >= 1; off >>= 1)
#pragma unroll
                for (int i = 0; i < off; i++) w[i] = w[i] + w[i + off];
            v[q] = w[0];
        }
    }
    __syncthreads();
}

__device__ __forceinline__ double block_max256(double v, double *scratch8) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    v = warp_max(v);
    if (lane == 0) scratch8[warp] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double m = scratch8[0];
        for (int i = 1; i < 8; i++) m = (scratch8[i] > m) ? scratch8[i] : m;
        v = m;
    }
    __syncthreads();
    return v;
}

// Reduce m level-1 partials (stride `stride` between value kinds) to one
// value per kind with the chunk tree: chunks of 2048, lane t adds chunk
// entries t, t+256, ..., t+1792 in order, then the block tree; repeated
// until one value remains.  Runs in one 256-thread block; `work` must hold
// ceil(m/2048) doubles per kind.  Result valid in thread 0.
template <int NV>
__device__ inline void chunk_reduce(const double *const (&src)[NV], int m, double *const (&work)[NV],
                                    double (&out)[NV], double (*scratch)[8]) {
    if (m <= 0) {
#pragma unroll
        for (int q = 0; q < NV; q++) out[q] = 0.0;
        return;
    }
    const double *cur[NV];
#pragma unroll
    for (int q = 0; q < NV; q++) cur[q] = src[q];
    while (true) {
        const int mc = (m + kChunk - 1) / kChunk;
        for (int c = 0; c < mc; c++) {
            double v[NV];
#pragma unroll
            for (int q = 0; q < NV; q++) {
                double acc = 0.0;
#pragma unroll
                for (int k = 0; k < 8; k++) {
                    const int i = c * kChunk + (int)threadIdx.x + 256 * k;
                    if (i < m) acc = acc + cur[q][i];
                }
                v[q] = acc;
            }
            block_tree_sum256<NV>(v, scratch);
            if (threadIdx.x == 0) {
#pragma unroll
                for (int q = 0; q < NV; q++) work[q][c] = v[q];
            }
        }
        __syncthreads();
        if (mc == 1) {
#pragma unroll
            for (int q = 0; q < NV; q++) out[q] = work[q][0];
            return;
        }
        // next level reads the chunk sums (in-place is safe: chunk c only
        // writes work[c] after reading entries >= c*2048 >= c)
#pragma unroll
        for (int q = 0; q < NV; q++) cur[q] = work[q];
        m = mc;
    }
}

// ------------------------------------------------------------ grid barrier
// Arrival counter and release flag live on separate 128-byte lines so that
// spinning readers do not contend with arriving atomics.
struct GridBarrier {
    unsigned int count;
    unsigned int pad0[31];
    unsigned int gen;
    unsigned int pad1[31];
    unsigned int pass[3][32];  // BBPGD pass counters (pass p uses pass[p % 3][0])
};

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ unsigned int ld_acquire_u32(const unsigned int *p) {
    unsigned int v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long *p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ unsigned int atom_add_release_u32(unsigned int *p, unsigned int v) {
    unsigned int old;
    asm volatile("atom.release.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}

__device__ __forceinline__ unsigned int atom_add_acqrel_u32(unsigned int *p, unsigned int v) {
    unsigned int old;
    asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}

__device__ __forceinline__ void st_relaxed_u32(unsigned int *p, unsigned int v) {
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ int ld_volatile_i32(const int *p) {
    return *(const volatile int *)p;
}

// Barrier over all blocks of a cooperative launch (release/acquire at GPU
// scope).  The wait is bounded: after `timeout_ns` (or when another block
// has already given up) the block sets kErrTimeout in *err and returns
// false; callers then leave the kernel.
__device__ inline bool grid_sync(GridBarrier *bar, unsigned int nblocks, int *err,
                                 unsigned long long timeout_ns) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        const unsigned int g = ld_acquire_u32(&bar->gen);
        const unsigned int arrived = atom_add_acqrel_u32(&bar->count, 1u);
        if (arrived == nblocks - 1) {
            st_relaxed_u32(&bar->count, 0u);
            atom_add_release_u32(&bar->gen, 1u);
        } else {
            unsigned long long t0 = 0;
            unsigned int spins = 0;
            while (ld_acquire_u32(&bar->gen) == g) {
                if (++spins > 64) {
                    __nanosleep(spins > 1024 ? 256 : 32);
                    if ((spins & 255) == 0) {
                        if (t0 == 0) t0 = global_ns();
                        if (ld_volatile_i32(err) & kErrTimeout) {
                            ok = 0;
                            break;
                        }
                        if (global_ns() - t0 > timeout_ns) {
                            atomicOr(err, kErrTimeout);
                            ok = 0;
                            break;
                        }
                    }
                }
            }
        }
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// Barrier ending pass p of the BBPGD kernel.  Pass p has its own counter
// (three in rotation); each block adds 1 + (act << kBarActShift) to it with
// one release reduction (act = the replicas it owns that iterated in this
// pass) and then polls it until all nblocks arrivals are in.  The final
// value also gives the pass's total active count, hence "continue or
// stop", so no block waits on a last arriver's second store.  Block 0
// clears the counter of pass p + 1 during pass p (its last use was pass
// p - 2, which every block has left).  Bounded like grid_sync.
constexpr int kBarActShift = 12;  // arrivals in the low 12 bits (up to 4095 blocks)

__device__ __forceinline__ void red_add_release_u32(unsigned int *p, unsigned int v) {
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ inline bool grid_sync_pass(GridBarrier *bar, unsigned int nblocks, int *err,
                                      unsigned long long timeout_ns, int p, int act, int &stop) {
    __shared__ int s_ok, s_stop;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        unsigned int *c = &bar->pass[p % 3][0];
        red_add_release_u32(c, 1u + ((unsigned int)act << kBarActShift));
        unsigned long long t0 = 0;
        unsigned int spins = 0;
        unsigned int v;
        while (((v = ld_acquire_u32(c)) & ((1u << kBarActShift) - 1u)) < nblocks) {
            if (++spins > 64) {
                __nanosleep(spins > 1024 ? 256 : 32);
                if ((spins & 255) == 0) {
                    if (t0 == 0) t0 = global_ns();
                    if (ld_volatile_i32(err) & kErrTimeout) {
                        ok = 0;
                        break;
                    }
                    if (global_ns() - t0 > timeout_ns) {
                        atomicOr(err, kErrTimeout);
                        ok = 0;
                        break;
                    }
                }
            }
        }
        s_ok = ok;
        s_stop = (v >> kBarActShift) == 0u ? 1 : 0;
    }
    __syncthreads();
    stop = s_stop;
    return s_ok != 0;
}

}  // namespace alens
