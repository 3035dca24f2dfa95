// oracle.cpp - FP64 C++/OpenMP CPU oracle of the rod collision-and-constraint
// step.  TEST INFRASTRUCTURE ONLY (tests, smoke check and the benchmark's CPU
// baseline leg); the GPU library never links or calls it.
//
// What it restates, and from where:
//   * the step order of SimToolbox SylinderSystem::runStep as aLENS drives it
//     (SRC/TubuleSystem.cpp:214-224: protein blocks queued, then runStep,
//     then calcConStress; restart path calls stepEuler, :55);
//   * the rod record (Sylinder: gid, radius, length, pos, orientation; axis =
//     q*(0,0,1), SRC/TubuleBind.hpp:54-67) and the sphere convention
//     length < 2*radius (SRC/TubuleBind.hpp:99);
//   * the ConstraintBlock contract (SRC/TubuleSystem.cpp:714-742);
//   * near-pair search with sylinderColBuf (docs/source/quickstart.md:346-348);
//   * segment-segment closest points (the DCPQuery role; method of
//     C. Ericson, "Real-Time Collision Detection" (2005) sec. 5.1.9, with the
//     parallel-overlap case resolved at the overlap midpoint);
//   * the complementarity formulation and BBPGD with alternating
//     Barzilai-Borwein steps (Yan, Zhang, Shelley, J. Chem. Phys. 150:064109
//     (2019); Barzilai & Borwein, IMA J. Numer. Anal. 8:141 (1988)); the
//     operator dt D^T M D is assembled explicitly once per step (the
//     Delassus matrix of contact mechanics) and applied as a sparse product;
//   * slender-body drag of a straight rod from the local slender-body
//     operator of Tornberg & Shelley, J. Comput. Phys. 196:8 (2004):
//     b = -(1 + 2 ln(r/L)), zeta_par = 4 pi mu L / b,
//     zeta_perp = 8 pi mu L / (b + 2), zeta_rot = 2 pi mu L^3 / (3 (b + 2));
//     spheres use Stokes drag 6 pi mu r and 8 pi mu r^3;
//   * Brownian velocity sqrt(2 kT / dt) M^(1/2) xi (fluctuation-dissipation),
//     xi from Philox4x32-10 (Salmon et al., SC'11) + Box-Muller.
//
// SimToolbox's own source is absent from the reference checkout, so parity
// with it is UNPINNED; these formulas are the project's documented choices.
//
// Canonical arithmetic: every floating-point expression below is written in
// a fixed evaluation order, compiled with -ffp-contract=off (no FMA), uses
// only IEEE +,-,*,/,sqrt plus the project's own log / sincos built from
// those, and every sum over constraints or rods uses the fixed reduction
// tree of canon_sum().  The GPU FP64 path follows the same specification,
// so for identical inputs the two agree bit for bit.

#include "oracle.h"
#include "oracle_ctx.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr double kPi = 3.141592653589793;
constexpr double kTwoPi = 6.283185307179586;
constexpr double kLn2 = 0.6931471805599453;
constexpr double kParallelEps = 1e-12;

// ---------------------------------------------------------------- det. math
// Natural log: x = m 2^e with m in [sqrt(1/2), sqrt(2)), log m = 2 atanh(u),
// u = (m-1)/(m+1), atanh series to u^23.
double det_log(double x) {
    uint64_t bits;
    std::memcpy(&bits, &x, 8);
    int e = (int)((bits >> 52) & 0x7ff);
    if (e == 0) {  // subnormal: scale up exactly
        x = x * 18014398509481984.0;  // 2^54
        std::memcpy(&bits, &x, 8);
        e = (int)((bits >> 52) & 0x7ff) - 54;
    }
    e -= 1023;
    bits = (bits & 0x800fffffffffffffULL) | (0x3ffULL << 52);
    double m;
    std::memcpy(&m, &bits, 8);  // m in [1, 2)
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

// sin and cos: halve until |x| <= 1, Taylor polynomials to x^19 / x^20,
// then double-angle formulas.
void det_sincos(double x, double *s_out, double *c_out) {
    int k = 0;
    while (std::fabs(x) > 1.0 && k < 64) {
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

// Philox4x32-10.
void philox(const uint32_t ctr_in[4], const uint32_t key_in[2],
            uint32_t out[4]) {
    uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
    uint32_t k0 = key_in[0], k1 = key_in[1];
    for (int r = 0; r < 10; r++) {
        const uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        const uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        c0 = hi1 ^ c1 ^ k0;
        c1 = lo1;
        c2 = hi0 ^ c3 ^ k1;
        c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0;
    out[1] = c1;
    out[2] = c2;
    out[3] = c3;
}

// FP32 natural log of a normal x > 0: x = m 2^e, m in [sqrt(1/2), sqrt(2)),
// log m = 2 atanh(u), u = (m-1)/(m+1), atanh series to u^13.
float det_logf(float x) {
    uint32_t bits;
    std::memcpy(&bits, &x, 4);
    int e = (int)((bits >> 23) & 0xffu) - 127;
    bits = (bits & 0x807fffffu) | (127u << 23);
    float m;
    std::memcpy(&m, &bits, 4);  // m in [1, 2)
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
// to x^11 / x^12, then double-angle formulas.
void det_sincosf(float x, float *s_out, float *c_out) {
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

// Six standard normals for (seed, gid, step): two Philox blocks, six
// 24-bit uniforms in (0,1), three Box-Muller pairs in FP32.
void normals6(uint64_t seed, int64_t gid, int64_t step, double z[6]) {
    const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    uint32_t w[8];
    for (uint32_t b = 0; b < 2; b++) {
        const uint32_t ctr[4] = {(uint32_t)(uint64_t)gid,
                                 (uint32_t)((uint64_t)gid >> 32),
                                 (uint32_t)(uint64_t)step, b};
        philox(ctr, key, w + 4 * b);
    }
    float u[6];
    for (int i = 0; i < 6; i++) u[i] = ((float)(w[i] >> 8) + 0.5f) * 5.9604644775390625e-08f;  // 2^-24
    for (int p = 0; p < 3; p++) {
        const float r = std::sqrt(-2.0f * det_logf(u[2 * p]));
        const float ang = u[2 * p + 1] * 6.28318531f - 3.14159265f;
        float sn, cs;
        det_sincosf(ang, &sn, &cs);
        // angle + pi: cos -> -cos, sin -> -sin
        z[2 * p] = (double)(r * -cs);
        z[2 * p + 1] = (double)(r * -sn);
    }
}

// ------------------------------------------------------- canonical reduction
// Level 1: tiles of 64 elements held by two warps; in each warp the tree
// v[l] = v[l] + v[l+off] for off = 16..1, then tile = warp0 + warp1.
// Level 2+: chunks of 1024 partials reduced by one warp: lane l adds
// partials l, l+32, ..., l+992 in order (from 0.0), then the warp tree;
// repeated until one value remains.
double warp_tree(double *v) {
    for (int off = 16; off >= 1; off >>= 1)
        for (int l = 0; l < off; l++) v[l] = v[l] + v[l + off];
    return v[0];
}

template <class F>
double tile_sum(F &&val, int64_t base, int64_t n) {
    double lanes[64];
    for (int l = 0; l < 64; l++) {
        const int64_t i = base + l;
        lanes[l] = (i < n) ? val(i) : 0.0;
    }
    const double w0 = warp_tree(lanes);
    const double w1 = warp_tree(lanes + 32);
    return w0 + w1;
}

double chunk_sum(const double *T, int64_t base, int64_t m) {
    double lanes[32];
    for (int l = 0; l < 32; l++) {
        double acc = 0.0;
        for (int j = 0; j < 32; j++) {
            const int64_t i = base + l + 32 * j;
            if (i < m) acc = acc + T[i];
        }
        lanes[l] = acc;
    }
    return warp_tree(lanes);
}

double reduce_partials(std::vector<double> T) {
    int64_t m = (int64_t)T.size();
    if (m == 0) return 0.0;
    while (true) {
        const int64_t mc = (m + 1023) / 1024;
        std::vector<double> R(mc);
        for (int64_t c = 0; c < mc; c++) R[c] = chunk_sum(T.data(), 1024 * c, m);
        if (mc == 1) return R[0];
        T.swap(R);
        m = mc;
    }
}

template <class F>
double canon_sum_f(F &&val, int64_t n) {
    const int64_t m = (n + 63) / 64;
    std::vector<double> T(m);
#pragma omp parallel for schedule(static)
    for (int64_t t = 0; t < m; t++) T[t] = tile_sum(val, 64 * t, n);
    return reduce_partials(std::move(T));
}

// ------------------------------------------------------------- rod geometry
inline void quat_axis(const double *q, double a[3]) {
    const double qx = q[0], qy = q[1], qz = q[2], qw = q[3];
    a[0] = 2.0 * (qx * qz + qw * qy);
    a[1] = 2.0 * (qy * qz - qw * qx);
    a[2] = 1.0 - 2.0 * (qx * qx + qy * qy);
}

// out = (1/zeta_par, 1/zeta_perp, 1/zeta_rot); sphere: (mt, mt, mr)
void mobility_coeffs(double L, double r, double mu, bool sphere,
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

// U6 = M F6 for one rod
void mobility_apply(const double a[3], const double m[3], bool sphere,
                    bool mono, const double F[6], double U[6]) {
    double f0 = F[0], f1 = F[1], f2 = F[2];
    double t0 = F[3], t1 = F[4], t2 = F[5];
    if (mono) {
        f2 = 0.0;
        t0 = 0.0;
        t1 = 0.0;
    }
    if (sphere) {
        U[0] = m[0] * f0;
        U[1] = m[0] * f1;
        U[2] = m[0] * f2;
        U[3] = m[2] * t0;
        U[4] = m[2] * t1;
        U[5] = m[2] * t2;
    } else {
        const double fa = a[0] * f0 + a[1] * f1 + a[2] * f2;
        U[0] = m[0] * fa * a[0] + m[1] * (f0 - fa * a[0]);
        U[1] = m[0] * fa * a[1] + m[1] * (f1 - fa * a[1]);
        U[2] = m[0] * fa * a[2] + m[1] * (f2 - fa * a[2]);
        const double ta = a[0] * t0 + a[1] * t1 + a[2] * t2;
        U[3] = m[2] * (t0 - ta * a[0]);
        U[4] = m[2] * (t1 - ta * a[1]);
        U[5] = m[2] * (t2 - ta * a[2]);
    }
    if (mono) {
        U[2] = 0.0;
        U[3] = 0.0;
        U[4] = 0.0;
    }
}

inline double clampd(double x, double lo, double hi) {
    return x < lo ? lo : (x > hi ? hi : x);
}

inline void cross3(const double a[3], const double b[3], double c[3]) {
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}

// Closest points between segments c1 + s u1 (|s| <= h1) and c2 + t u2
// (|t| <= h2), unit axes.
void dcp(const double c1[3], const double u1[3], double h1, const double c2[3],
         const double u2[3], double h2, double *s_out, double *t_out,
         double P[3], double Q[3], double *dist) {
    const double w0 = c1[0] - c2[0], w1 = c1[1] - c2[1], w2 = c1[2] - c2[2];
    const double b = u1[0] * u2[0] + u1[1] * u2[1] + u1[2] * u2[2];
    const double d = u1[0] * w0 + u1[1] * w1 + u1[2] * w2;
    const double e = u2[0] * w0 + u2[1] * w1 + u2[2] * w2;
    const double det = 1.0 - b * b;
    double s, t;
    if (det > kParallelEps) {
        s = clampd((b * e - d) / det, -h1, h1);
    } else {
        const double ab = std::fabs(b);
        const double lo = std::max(-h1, -d - ab * h2);
        const double hi = std::min(h1, -d + ab * h2);
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
    P[0] = c1[0] + s * u1[0];
    P[1] = c1[1] + s * u1[1];
    P[2] = c1[2] + s * u1[2];
    Q[0] = c2[0] + t * u2[0];
    Q[1] = c2[1] + t * u2[1];
    Q[2] = c2[2] + t * u2[2];
    const double x0 = P[0] - Q[0], x1 = P[1] - Q[1], x2 = P[2] - Q[2];
    *dist = std::sqrt(x0 * x0 + x1 * x1 + x2 * x2);
    *s_out = s;
    *t_out = t;
}

// Unit normal from Q to P; degenerate contacts fall back to a direction
// perpendicular to the axes.
void contact_normal(const double P[3], const double Q[3], double dist,
                    const double u1[3], const double u2[3], double n[3]) {
    if (dist > 0.0) {
        n[0] = (P[0] - Q[0]) / dist;
        n[1] = (P[1] - Q[1]) / dist;
        n[2] = (P[2] - Q[2]) / dist;
        return;
    }
    double c[3];
    cross3(u1, u2, c);
    double cn = std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
    if (!(cn > 0.0)) {
        const double ax = std::fabs(u1[0]), ay = std::fabs(u1[1]),
                     az = std::fabs(u1[2]);
        double e[3] = {0.0, 0.0, 0.0};
        if (ax <= ay && ax <= az)
            e[0] = 1.0;
        else if (ay <= az)
            e[1] = 1.0;
        else
            e[2] = 1.0;
        cross3(u1, e, c);
        cn = std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
    }
    n[0] = c[0] / cn;
    n[1] = c[1] / cn;
    n[2] = c[2] / cn;
}

inline double dot6(const double *J, const double *U) {
    return J[0] * U[0] + J[1] * U[1] + J[2] * U[2] + J[3] * U[3] +
           J[4] * U[4] + J[5] * U[5];
}

inline uint64_t pair_key(int64_t i, int64_t j, int img) {
    return ((uint64_t)i << 32) | ((uint64_t)j << 5) | (uint64_t)img;
}

}  // namespace

// ------------------------------------------------------------------ context
// struct OrcCtx: oracle_ctx.h

namespace {

bool box_ok(const AlensConfig &c) {
    for (int d = 0; d < 3; d++)
        if (!(c.simBoxHigh[d] > c.simBoxLow[d])) return false;
    return c.dt > 0 && c.viscosity > 0 && c.sylinderColBuf >= 0 &&
           c.sylinderDiameterColRatio > 0 && c.sylinderLengthColRatio > 0 &&
           c.conMaxIte >= 0 && c.conResTol > 0;
}

int setup_grid(OrcCtx *x) {
    double mx = 0.0;
    for (int i = 0; i < x->n; i++) {
        const bool sphere = x->len[i] < 2.0 * x->rad[i];
        const double h =
            sphere ? 0.0 : 0.5 * (x->len[i] * x->cfg.sylinderLengthColRatio);
        const double rc = x->rad[i] * x->cfg.sylinderDiameterColRatio;
        mx = std::max(mx, 2.0 * h + 2.0 * rc);
    }
    x->cutoff = mx + x->cfg.sylinderColBuf;
    for (int d = 0; d < 3; d++) {
        const double Lb = x->cfg.simBoxHigh[d] - x->cfg.simBoxLow[d];
        if (x->cfg.simBoxPBC[d] && Lb < x->cutoff) return ALENS_INVALID_ARG;
        int nc = (int)std::floor(Lb / x->cutoff);
        nc = std::max(1, std::min(nc, 1024));
        x->ncell[d] = nc;
        x->cellsz[d] = Lb / nc;
    }
    return ALENS_OK;
}

void wrap_positions(OrcCtx *x) {
    for (int i = 0; i < x->n; i++) {
        for (int d = 0; d < 3; d++) {
            if (!x->cfg.simBoxPBC[d]) continue;
            const double lo = x->cfg.simBoxLow[d], hi = x->cfg.simBoxHigh[d];
            const double Lb = hi - lo;
            double v = x->pos[3 * i + d];
            for (int k = 0; k < 64; k++) {
                if (v < lo)
                    v = v + Lb;
                else if (v >= hi)
                    v = v - Lb;
                else
                    break;
            }
            x->pos[3 * i + d] = v;
        }
    }
}

int cell_coord(const OrcCtx *x, int d, double v) {
    const double f = std::floor((v - x->cfg.simBoxLow[d]) / x->cellsz[d]);
    int c = f < 0.0 ? 0 : (f > (double)(x->ncell[d] - 1) ? x->ncell[d] - 1 : (int)f);
    return c;
}

void rod_prepare(OrcCtx *x) {
    const int n = x->n;
    const AlensConfig &c = x->cfg;
    x->axis.assign(3 * n, 0.0);
    x->hcol.assign(n, 0.0);
    x->rcol.assign(n, 0.0);
    x->mob.assign(3 * n, 0.0);
    x->unc.assign(6 * n, 0.0);
    x->sph.assign(n, 0);
    const bool mono = c.monolayer != 0;
    const double bc = c.KBT > 0.0 ? std::sqrt(2.0 * c.KBT / c.dt) : 0.0;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; i++) {
        double a[3];
        quat_axis(&x->quat[4 * i], a);
        x->axis[3 * i] = a[0];
        x->axis[3 * i + 1] = a[1];
        x->axis[3 * i + 2] = a[2];
        const bool sphere = x->len[i] < 2.0 * x->rad[i];
        x->sph[i] = sphere;
        x->hcol[i] = sphere ? 0.0 : 0.5 * (x->len[i] * c.sylinderLengthColRatio);
        x->rcol[i] = x->rad[i] * c.sylinderDiameterColRatio;
        double m[3] = {0.0, 0.0, 0.0};
        if (!x->imm[i]) mobility_coeffs(x->len[i], x->rad[i], c.viscosity, sphere, m);
        x->mob[3 * i] = m[0];
        x->mob[3 * i + 1] = m[1];
        x->mob[3 * i + 2] = m[2];
        if (c.KBT > 0.0 && !x->imm[i]) {
            double z[6];
            normals6(c.rngSeed, x->gid[i], x->step, z);
            if (mono) {
                z[2] = 0.0;
                z[3] = 0.0;
                z[4] = 0.0;
            }
            double u[6];
            if (sphere) {
                const double st = std::sqrt(m[0]), sr = std::sqrt(m[2]);
                u[0] = st * z[0];
                u[1] = st * z[1];
                u[2] = st * z[2];
                u[3] = sr * z[3];
                u[4] = sr * z[4];
                u[5] = sr * z[5];
            } else {
                const double sp = std::sqrt(m[0]), sq = std::sqrt(m[1]),
                             sr = std::sqrt(m[2]);
                const double za = a[0] * z[0] + a[1] * z[1] + a[2] * z[2];
                u[0] = sp * za * a[0] + sq * (z[0] - za * a[0]);
                u[1] = sp * za * a[1] + sq * (z[1] - za * a[1]);
                u[2] = sp * za * a[2] + sq * (z[2] - za * a[2]);
                const double ra = a[0] * z[3] + a[1] * z[4] + a[2] * z[5];
                u[3] = sr * (z[3] - ra * a[0]);
                u[4] = sr * (z[4] - ra * a[1]);
                u[5] = sr * (z[5] - ra * a[2]);
            }
            if (mono) {
                u[2] = 0.0;
                u[3] = 0.0;
                u[4] = 0.0;
            }
            for (int k = 0; k < 6; k++) x->unc[6 * i + k] = bc * u[k];
        }
    }
}

// image code of shift (sx, sy, sz) in {-1,0,1}^3
inline int img_code(int sx, int sy, int sz) {
    return (sx + 1) * 9 + (sy + 1) * 3 + (sz + 1);
}

void image_shift(const OrcCtx *x, int img, double S[3]) {
    const int sx = img / 9 - 1, sy = (img / 3) % 3 - 1, sz = img % 3 - 1;
    const int sv[3] = {sx, sy, sz};
    for (int d = 0; d < 3; d++)
        S[d] = (double)sv[d] * (x->cfg.simBoxHigh[d] - x->cfg.simBoxLow[d]);
}

// Rod-boundary contact points: both rod ends for walls and inside
// spheres/tubes (the centre alone for sphere-shaped rods); the point
// nearest the centre for outside spheres.  Q, the signed distance s to the
// boundary (positive on the allowed side) and the unit normal n into the
// allowed region.
int boundary_npoints(const OrcCtx::Bnd &B, double h) {
    if (B.type == 1 && !B.inside) return 1;
    return h > 0.0 ? 2 : 1;
}

void boundary_contact(const OrcCtx::Bnd &B, const double x[3], const double u[3], double h, int e,
                      double Q[3], double &s, double n[3]) {
    double t;
    if (B.type == 1 && !B.inside) {
        t = (B.c[0] - x[0]) * u[0] + (B.c[1] - x[1]) * u[1] + (B.c[2] - x[2]) * u[2];
        t = t < -h ? -h : (t > h ? h : t);
    } else {
        t = e == 0 ? -h : h;
    }
    for (int d = 0; d < 3; d++) Q[d] = x[d] + t * u[d];
    const double v[3] = {Q[0] - B.c[0], Q[1] - B.c[1], Q[2] - B.c[2]};
    if (B.type == 0) {
        s = v[0] * B.a[0] + v[1] * B.a[1] + v[2] * B.a[2];
        for (int d = 0; d < 3; d++) n[d] = B.a[d];
        return;
    }
    double w[3];
    if (B.type == 2) {
        const double p = v[0] * B.a[0] + v[1] * B.a[1] + v[2] * B.a[2];
        for (int d = 0; d < 3; d++) w[d] = v[d] - p * B.a[d];
    } else {
        for (int d = 0; d < 3; d++) w[d] = v[d];
    }
    const double rho = std::sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
    double dir[3] = {1.0, 0.0, 0.0};
    if (rho > 0.0)
        for (int d = 0; d < 3; d++) dir[d] = w[d] / rho;
    if (B.inside) {
        s = B.R - rho;
        for (int d = 0; d < 3; d++) n[d] = -dir[d];
    } else {
        s = rho - B.R;
        for (int d = 0; d < 3; d++) n[d] = dir[d];
    }
}

void find_pairs(OrcCtx *x, std::vector<std::vector<uint64_t>> &perRod) {
    const int n = x->n;
    const AlensConfig &c = x->cfg;
    const int nx = x->ncell[0], ny = x->ncell[1], nz = x->ncell[2];
    const int64_t ncells = (int64_t)nx * ny * nz;
    std::vector<int> cellOf(n);
    std::vector<int64_t> start(ncells + 1, 0);
    for (int i = 0; i < n; i++) {
        const int cx = cell_coord(x, 0, x->pos[3 * i]);
        const int cy = cell_coord(x, 1, x->pos[3 * i + 1]);
        const int cz = cell_coord(x, 2, x->pos[3 * i + 2]);
        cellOf[i] = (cz * ny + cy) * nx + cx;
        start[cellOf[i] + 1]++;
    }
    for (int64_t k = 0; k < ncells; k++) start[k + 1] += start[k];
    std::vector<int> members(n);
    {
        std::vector<int64_t> cur(start.begin(), start.end() - 1);
        for (int i = 0; i < n; i++) members[cur[cellOf[i]]++] = i;
    }
    const double colBuf = c.sylinderColBuf;
    perRod.assign(n, {});
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < n; i++) {
        const int ci0 = cellOf[i];
        const int cx = ci0 % nx, cy = (ci0 / nx) % ny, cz = ci0 / (nx * ny);
        const double *pi = &x->pos[3 * i];
        const double *ai = &x->axis[3 * i];
        const double hi_ = x->hcol[i], ri = x->rcol[i];
        std::vector<uint64_t> &out = perRod[i];
        for (int oz = -1; oz <= 1; oz++) {
            int z = cz + oz, sz = 0;
            if (z < 0 || z >= nz) {
                if (!c.simBoxPBC[2]) continue;
                if (z < 0) { z += nz; sz = -1; } else { z -= nz; sz = 1; }
            }
            for (int oy = -1; oy <= 1; oy++) {
                int y = cy + oy, sy = 0;
                if (y < 0 || y >= ny) {
                    if (!c.simBoxPBC[1]) continue;
                    if (y < 0) { y += ny; sy = -1; } else { y -= ny; sy = 1; }
                }
                for (int ox = -1; ox <= 1; ox++) {
                    int xx = cx + ox, sx = 0;
                    if (xx < 0 || xx >= nx) {
                        if (!c.simBoxPBC[0]) continue;
                        if (xx < 0) { xx += nx; sx = -1; } else { xx -= nx; sx = 1; }
                    }
                    const int img = img_code(sx, sy, sz);
                    double S[3];
                    image_shift(x, img, S);
                    const int64_t cell = ((int64_t)z * ny + y) * nx + xx;
                    for (int64_t m = start[cell]; m < start[cell + 1]; m++) {
                        const int j = members[m];
                        if (j < i) continue;
                        if (j == i && img <= 13) continue;
                        const double *pj = &x->pos[3 * j];
                        const double c2[3] = {pj[0] + S[0], pj[1] + S[1], pj[2] + S[2]};
                        const double d0 = pi[0] - c2[0], d1 = pi[1] - c2[1],
                                     d2 = pi[2] - c2[2];
                        const double dd = d0 * d0 + d1 * d1 + d2 * d2;
                        const double lim = hi_ + x->hcol[j] + ri + x->rcol[j] + colBuf;
                        if (dd > lim * lim * (1.0 + 1e-10) + 1e-300) continue;
                        double s, t, P[3], Q[3], dist;
                        dcp(pi, ai, hi_, c2, &x->axis[3 * j], x->hcol[j], &s, &t, P, Q, &dist);
                        const double sep = dist - ri - x->rcol[j];
                        if (sep < colBuf) out.push_back(pair_key(i, j, img));
                    }
                }
            }
        }
        // contacts with the boundaries: keys (i, b, 27 + point)
        for (size_t b = 0; b < x->bnd.size(); b++) {
            const int np = boundary_npoints(x->bnd[b], hi_);
            for (int e = 0; e < np; e++) {
                double Q[3], sd, nn[3];
                boundary_contact(x->bnd[b], pi, ai, hi_, e, Q, sd, nn);
                if (sd - ri < colBuf) out.push_back(pair_key(i, (int64_t)b, 27 + e));
            }
        }
        std::sort(out.begin(), out.end());
    }
}

void build_constraints(OrcCtx *x) {
    const int n = x->n;
    const AlensConfig &c = x->cfg;
    std::vector<std::vector<uint64_t>> perRod;
    find_pairs(x, perRod);
    std::vector<uint64_t> keys;
    for (int i = 0; i < n; i++) keys.insert(keys.end(), perRod[i].begin(), perRod[i].end());
    x->ncoll = (int)keys.size();
    x->blocks = x->queue;
    x->queue.clear();
    // link blocks after the queued ones (the alens_set_links links, then the
    // springs of doubly bound proteins): anchors P = c_I + sI a_I,
    // Q = c_J + sJ a_J, d = P - Q reduced to the minimum image
    auto add_link = [&](int I, int J, double sI, double sJ, double rest, double kappa) {
        const double *aI = &x->axis[3 * I], *aJ = &x->axis[3 * J];
        const double pI[3] = {x->pos[3 * I] + sI * aI[0], x->pos[3 * I + 1] + sI * aI[1],
                              x->pos[3 * I + 2] + sI * aI[2]};
        const double pJ[3] = {x->pos[3 * J] + sJ * aJ[0], x->pos[3 * J + 1] + sJ * aJ[1],
                              x->pos[3 * J + 2] + sJ * aJ[2]};
        double d[3];
        for (int cc = 0; cc < 3; cc++) {
            d[cc] = pI[cc] - pJ[cc];
            if (c.simBoxPBC[cc]) {
                const double Lb = c.simBoxHigh[cc] - c.simBoxLow[cc];
                d[cc] = d[cc] - Lb * std::floor(d[cc] / Lb + 0.5);
            }
        }
        const double len = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
        double nn[3] = {0.0, 0.0, 1.0};
        if (len > 0.0) {
            nn[0] = d[0] / len;
            nn[1] = d[1] / len;
            nn[2] = d[2] / len;
        }
        AlensBlock B;
        std::memset(&B, 0, sizeof(B));
        const double delta0 = len - rest;
        B.delta0 = delta0;
        B.gamma = -delta0 * kappa;
        B.gidI = x->gid[I];
        B.gidJ = x->gid[J];
        B.globalIndexI = I;
        B.globalIndexJ = J;
        for (int cc = 0; cc < 3; cc++) {
            B.normI[cc] = nn[cc];
            B.normJ[cc] = -nn[cc];
            B.posI[cc] = sI * aI[cc];
            B.posJ[cc] = sJ * aJ[cc];
            B.labI[cc] = pI[cc];
            B.labJ[cc] = pI[cc] - d[cc];
        }
        B.bilateral = 1;
        B.kappa = kappa;
        x->blocks.push_back(B);
    };
    for (size_t L = 0; L < x->linkI.size(); L++)
        add_link(x->linkI[L], x->linkJ[L], x->linkSI[L], x->linkSJ[L], x->linkRest[L], x->linkKappa[L]);
    for (size_t L = 0; L < x->springI.size(); L++)
        if (x->springI[L] < n && x->springJ[L] < n)
            add_link(x->springI[L], x->springJ[L], x->springSI[L], x->springSJ[L], x->springRest[L],
                 x->springKappa[L]);
    x->nbil = (int)x->blocks.size();
    const int nc = x->ncoll + x->nbil;
    x->ci.assign(nc, -1);
    x->cj.assign(nc, -1);
    x->cimg.assign(nc, -1);
    x->jac.assign(12 * (size_t)nc, 0.0);
    x->phi0.assign(nc, 0.0);
    x->q.assign(nc, 0.0);
    x->gamma.assign(nc, 0.0);
    x->cinv.assign(nc, 0.0);
    x->lb.assign(nc, 0.0);
    x->lab.assign(6 * (size_t)nc, 0.0);
    x->unil.assign(nc, 1);
    const bool warmPrev = c.warmStart == ALENS_WARM_PREV || c.warmStart == ALENS_WARM_MLP;
#pragma omp parallel for schedule(static)
    for (int k = 0; k < x->ncoll; k++) {
        const uint64_t key = keys[k];
        const int i = (int)(key >> 32), j = (int)((key >> 5) & 0x7ffffff),
                  img = (int)(key & 31);
        double g0 = 0.0;
        if (warmPrev && !x->prevKeys.empty()) {
            auto it = std::lower_bound(x->prevKeys.begin(), x->prevKeys.end(), key);
            if (it != x->prevKeys.end() && *it == key)
                g0 = x->prevGamma[it - x->prevKeys.begin()];
        }
        if (img >= 27) {
            // rod i against boundary j: one-sided, force along the normal
            const double *xi = &x->pos[3 * i], *ai = &x->axis[3 * i];
            double Q[3], sd, nn[3];
            boundary_contact(x->bnd[j], xi, ai, x->hcol[i], img - 27, Q, sd, nn);
            double *J = &x->jac[12 * (size_t)k];
            const double r[3] = {Q[0] - xi[0], Q[1] - xi[1], Q[2] - xi[2]};
            J[0] = nn[0];
            J[1] = nn[1];
            J[2] = nn[2];
            cross3(r, nn, J + 3);
            x->ci[k] = i;
            x->cj[k] = -1;
            x->cimg[k] = img;
            x->phi0[k] = sd - x->rcol[i];
            for (int d = 0; d < 3; d++) {
                x->lab[6 * (size_t)k + d] = Q[d];
                x->lab[6 * (size_t)k + 3 + d] = Q[d] - sd * nn[d];
            }
            x->gamma[k] = g0;
            continue;
        }
        double S[3];
        image_shift(x, img, S);
        const double *pj = &x->pos[3 * j];
        const double c2[3] = {pj[0] + S[0], pj[1] + S[1], pj[2] + S[2]};
        const double *ai = &x->axis[3 * i], *aj = &x->axis[3 * j];
        double s, t, P[3], Q[3], dist, nrm[3];
        dcp(&x->pos[3 * i], ai, x->hcol[i], c2, aj, x->hcol[j], &s, &t, P, Q, &dist);
        contact_normal(P, Q, dist, ai, aj, nrm);
        const double sep = dist - x->rcol[i] - x->rcol[j];
        double *J = &x->jac[12 * (size_t)k];
        const double rI[3] = {s * ai[0], s * ai[1], s * ai[2]};
        const double rJ[3] = {t * aj[0], t * aj[1], t * aj[2]};
        const double nJ[3] = {-nrm[0], -nrm[1], -nrm[2]};
        J[0] = nrm[0];
        J[1] = nrm[1];
        J[2] = nrm[2];
        cross3(rI, nrm, J + 3);
        J[6] = nJ[0];
        J[7] = nJ[1];
        J[8] = nJ[2];
        cross3(rJ, nJ, J + 9);
        x->ci[k] = i;
        x->cj[k] = j;
        x->cimg[k] = img;
        x->phi0[k] = sep;
        for (int d = 0; d < 3; d++) {
            x->lab[6 * (size_t)k + d] = P[d];
            x->lab[6 * (size_t)k + 3 + d] = Q[d];
        }
        x->gamma[k] = g0;
    }
    for (int b = 0; b < x->nbil; b++) {
        const AlensBlock &B = x->blocks[b];
        const int k = x->ncoll + b;
        double *J = &x->jac[12 * (size_t)k];
        J[0] = B.normI[0];
        J[1] = B.normI[1];
        J[2] = B.normI[2];
        cross3(B.posI, B.normI, J + 3);
        x->ci[k] = B.globalIndexI;
        if (!B.oneSide) {
            J[6] = B.normJ[0];
            J[7] = B.normJ[1];
            J[8] = B.normJ[2];
            cross3(B.posJ, B.normJ, J + 9);
            x->cj[k] = B.globalIndexJ;
        }
        x->phi0[k] = B.delta0;
        x->gamma[k] = B.gamma;
        x->unil[k] = B.bilateral ? 0 : 1;
        x->lb[k] = B.bilateral ? 0.0 : B.gammaLB;
        x->cinv[k] = (B.bilateral && B.kappa > 0.0) ? 1.0 / B.kappa : 0.0;
        for (int d = 0; d < 3; d++) {
            x->lab[6 * (size_t)k + d] = B.labI[d];
            x->lab[6 * (size_t)k + 3 + d] = B.labJ[d];
        }
    }
    if (!x->initGammaOverride.empty() && (int)x->initGammaOverride.size() == nc) {
        x->gamma = x->initGammaOverride;
    }
    x->initGammaOverride.clear();
    // rod-major rows, entries 2k + side in ascending order
    x->rowptr.assign(n + 1, 0);
    for (int k = 0; k < nc; k++) {
        x->rowptr[x->ci[k] + 1]++;
        if (x->cj[k] >= 0) x->rowptr[x->cj[k] + 1]++;
    }
    for (int i = 0; i < n; i++) x->rowptr[i + 1] += x->rowptr[i];
    x->rowent.assign(x->rowptr[n], 0);
    {
        std::vector<int64_t> cur(x->rowptr.begin(), x->rowptr.end() - 1);
        for (int k = 0; k < nc; k++) {
            x->rowent[cur[x->ci[k]]++] = 2 * (int64_t)k;
            if (x->cj[k] >= 0) x->rowent[cur[x->cj[k]]++] = 2 * (int64_t)k + 1;
        }
    }
    // q = phi0 + dt * D^T U_nc
    const double dt = c.dt;
#pragma omp parallel for schedule(static)
    for (int k = 0; k < nc; k++) {
        const double *J = &x->jac[12 * (size_t)k];
        const double dI = dot6(J, &x->unc[6 * (size_t)x->ci[k]]);
        const double dJ = x->cj[k] >= 0 ? dot6(J + 6, &x->unc[6 * (size_t)x->cj[k]]) : 0.0;
        x->q[k] = x->phi0[k] + dt * (dI + dJ);
    }
}

// Delassus operator A = dt D^T M D, assembled explicitly per step.
// W_k,side = M_rod J_k,side (mobility-weighted Jacobian).  Row k lists the
// constraints l that share a rod with k, in ascending l; its value is
// dt * (sum of J_k,sk . W_l,sl over shared rods), contributions ordered by
// k's side (rod I first), then by the rod row (entry 2l+sl ascending).
void build_delassus(OrcCtx *x) {
    const int nc = x->ncoll + x->nbil;
    const bool mono = x->cfg.monolayer != 0;
    const double dt = x->cfg.dt;
    std::vector<double> W(12 * (size_t)nc, 0.0);
#pragma omp parallel for schedule(static)
    for (int k = 0; k < nc; k++) {
        for (int side = 0; side < 2; side++) {
            const int r = side == 0 ? x->ci[k] : x->cj[k];
            if (r < 0 || x->imm[r]) continue;
            mobility_apply(&x->axis[3 * r], &x->mob[3 * r], x->sph[r], mono,
                           &x->jac[12 * (size_t)k + 6 * side], &W[12 * (size_t)k + 6 * side]);
        }
    }
    std::vector<std::vector<std::pair<int, double>>> rows(nc);
#pragma omp parallel for schedule(dynamic, 256)
    for (int k = 0; k < nc; k++) {
        const int rI = x->ci[k], rJ = x->cj[k];
        const int64_t *LI = &x->rowent[x->rowptr[rI]];
        const int64_t nI = x->rowptr[rI + 1] - x->rowptr[rI];
        const int64_t *LJ = rJ >= 0 ? &x->rowent[x->rowptr[rJ]] : nullptr;
        const int64_t nJ = rJ >= 0 ? x->rowptr[rJ + 1] - x->rowptr[rJ] : 0;
        const double *JkI = &x->jac[12 * (size_t)k];
        const double *JkJ = JkI + 6;
        int64_t a = 0, b = 0;
        auto &row = rows[k];
        while (a < nI || b < nJ) {
            const int64_t la = a < nI ? (LI[a] >> 1) : INT64_MAX;
            const int64_t lb = b < nJ ? (LJ[b] >> 1) : INT64_MAX;
            const int64_t l = la < lb ? la : lb;
            double acc = 0.0;
            while (a < nI && (LI[a] >> 1) == l) {
                acc = acc + dot6(JkI, &W[12 * (size_t)l + 6 * (LI[a] & 1)]);
                a++;
            }
            while (b < nJ && (LJ[b] >> 1) == l) {
                acc = acc + dot6(JkJ, &W[12 * (size_t)l + 6 * (LJ[b] & 1)]);
                b++;
            }
            row.emplace_back((int)l, dt * acc);
        }
    }
    x->aptr.assign(nc + 1, 0);
    for (int k = 0; k < nc; k++) x->aptr[k + 1] = x->aptr[k] + (int64_t)rows[k].size();
    x->acol.resize(x->aptr[nc]);
    x->aval.resize(x->aptr[nc]);
#pragma omp parallel for schedule(static)
    for (int k = 0; k < nc; k++) {
        int64_t o = x->aptr[k];
        for (auto &e : rows[k]) {
            x->acol[o] = e.first;
            x->aval[o] = e.second;
            o++;
        }
    }
}

// y_k = sum_l A_kl x_l (ascending l, fused multiply-adds) + cinv_k x_k
// (+ q_k when withQ)
void spmv_A(OrcCtx *x, const std::vector<double> &xin, std::vector<double> &y, bool withQ) {
    const int nc = x->ncoll + x->nbil;
    y.assign(nc, 0.0);
#pragma omp parallel for schedule(static)
    for (int k = 0; k < nc; k++) {
        double v = 0.0;
        for (int64_t e = x->aptr[k]; e < x->aptr[k + 1]; e++) v = std::fma(x->aval[e], xin[x->acol[e]], v);
        v = std::fma(x->cinv[k], xin[k], v);
        if (withQ) v = v + x->q[k];
        y[k] = v;
    }
}

inline double proj(double v, bool unil, double lb) {
    return (unil && v < lb) ? lb : v;
}

int solve_bbpgd(OrcCtx *x, AlensStepStats *st) {
    const int nc = x->ncoll + x->nbil;
    const double tol = x->cfg.conResTol;
    std::vector<double> &gam = x->gamma;
    for (int k = 0; k < nc; k++) gam[k] = proj(gam[k], x->unil[k], x->lb[k]);
    st->iterations = 0;
    st->refineIterations = 0;
    st->residual = 0.0;
    st->converged = 1;
    if (nc == 0) return ALENS_OK;
    std::vector<double> g, Ag, gn, gamn(nc);
    spmv_A(x, gam, g, true);
    auto residual = [&](const std::vector<double> &gm, const std::vector<double> &gg) {
        double res = 0.0;
        bool bad = false;
#pragma omp parallel for reduction(max : res) reduction(|| : bad)
        for (int k = 0; k < nc; k++) {
            const double r = std::fabs(gm[k] - proj(gm[k] - gg[k], x->unil[k], x->lb[k]));
            if (!(r == r)) bad = true;
            res = std::max(res, r);
        }
        return bad ? NAN : res;
    };
    double res = residual(gam, g);
    if (std::isnan(res)) {
        st->residual = res;
        st->converged = 0;
        return ALENS_NAN_DETECTED;
    }
    if (res <= tol) {
        st->residual = res;
        return ALENS_OK;
    }
    spmv_A(x, g, Ag, false);
    const double gg = canon_sum_f([&](int64_t k) { return g[k] * g[k]; }, nc);
    const double gAg = canon_sum_f([&](int64_t k) { return g[k] * Ag[k]; }, nc);
    double alpha = (gAg > 0.0) ? gg / gAg : 1.0;
    if (!(alpha > 0.0) || std::isinf(alpha)) alpha = 1.0;
    int it = 0;
    bool conv = false;
    for (it = 1; it <= x->cfg.conMaxIte; it++) {
#pragma omp parallel for schedule(static)
        for (int k = 0; k < nc; k++)
            gamn[k] = proj(std::fma(-alpha, g[k], gam[k]), x->unil[k], x->lb[k]);
        spmv_A(x, gamn, gn, true);
        const double ss = canon_sum_f(
            [&](int64_t k) { const double s = gamn[k] - gam[k]; return s * s; }, nc);
        const double sy = canon_sum_f(
            [&](int64_t k) { return (gamn[k] - gam[k]) * (gn[k] - g[k]); }, nc);
        const double yy = canon_sum_f(
            [&](int64_t k) { const double y = gn[k] - g[k]; return y * y; }, nc);
        res = residual(gamn, gn);
        gam.swap(gamn);
        g.swap(gn);
        if (std::isnan(res)) break;
        if (res <= tol) {
            conv = true;
            break;
        }
        if (sy > 0.0) {
            const double a = (it & 1) ? ss / sy : sy / yy;
            if (a > 0.0 && !std::isinf(a)) alpha = a;
        }
    }
    st->iterations = conv ? it : std::min(it, x->cfg.conMaxIte);
    st->residual = res;
    st->converged = conv ? 1 : 0;
    if (std::isnan(res)) return ALENS_NAN_DETECTED;
    return conv ? ALENS_OK : ALENS_NOT_CONVERGED;
}

void advance(OrcCtx *x) {
    const int n = x->n;
    const AlensConfig &c = x->cfg;
    const bool mono = c.monolayer != 0;
    const double dt = c.dt;
    x->vel.assign(6 * (size_t)n, 0.0);
#pragma omp parallel for schedule(static)
    for (int r = 0; r < n; r++) {
        if (x->imm[r]) continue;
        double F[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
        for (int64_t e = x->rowptr[r]; e < x->rowptr[r + 1]; e++) {
            const int64_t ent = x->rowent[e];
            const int64_t k = ent >> 1;
            const double *J = &x->jac[12 * k + 6 * (ent & 1)];
            const double g = x->gamma[k];
            for (int cc = 0; cc < 6; cc++) F[cc] = F[cc] + g * J[cc];
        }
        double Uc[6], U[6];
        mobility_apply(&x->axis[3 * r], &x->mob[3 * r], x->sph[r], mono, F, Uc);
        for (int cc = 0; cc < 6; cc++) U[cc] = Uc[cc] + x->unc[6 * (size_t)r + cc];
        for (int cc = 0; cc < 6; cc++) x->vel[6 * (size_t)r + cc] = U[cc];
        double *p = &x->pos[3 * r];
        p[0] = p[0] + dt * U[0];
        p[1] = p[1] + dt * U[1];
        p[2] = p[2] + dt * U[2];
        const double w0 = U[3], w1 = U[4], w2 = U[5];
        const double wn2 = w0 * w0 + w1 * w1 + w2 * w2;
        if (wn2 > 0.0) {
            const double wn = std::sqrt(wn2);
            const double half = 0.5 * dt * wn;
            double sh, ch;
            det_sincos(half, &sh, &ch);
            const double kk = sh / wn;
            const double v0 = kk * w0, v1 = kk * w1, v2 = kk * w2;
            double *qq = &x->quat[4 * r];
            const double qx = qq[0], qy = qq[1], qz = qq[2], qw = qq[3];
            const double nw = ch * qw - (v0 * qx + v1 * qy + v2 * qz);
            const double nx = (ch * qx + qw * v0) + (v1 * qz - v2 * qy);
            const double ny = (ch * qy + qw * v1) + (v2 * qx - v0 * qz);
            const double nz = (ch * qz + qw * v2) + (v0 * qy - v1 * qx);
            const double nn = std::sqrt(nx * nx + ny * ny + nz * nz + nw * nw);
            qq[0] = nx / nn;
            qq[1] = ny / nn;
            qq[2] = nz / nn;
            qq[3] = nw / nn;
        }
        for (int d = 0; d < 3; d++) {
            if (!c.simBoxPBC[d]) continue;
            const double lo = c.simBoxLow[d], hi = c.simBoxHigh[d];
            const double Lb = hi - lo;
            double v = p[d];
            for (int k = 0; k < 64; k++) {
                if (v < lo)
                    v = v + Lb;
                else if (v >= hi)
                    v = v - Lb;
                else
                    break;
            }
            p[d] = v;
        }
    }
    // keep collision keys and gamma for the next step's warm start
    x->prevKeys.resize(x->ncoll);
    x->prevGamma.resize(x->ncoll);
    for (int k = 0; k < x->ncoll; k++) {
        x->prevKeys[k] = pair_key(x->ci[k], x->cj[k], x->cimg[k]);
        x->prevGamma[k] = x->gamma[k];
    }
    x->step++;
}

bool rods_finite(const OrcCtx *x) {
    for (size_t i = 0; i < x->pos.size(); i++)
        if (!std::isfinite(x->pos[i])) return false;
    for (size_t i = 0; i < x->quat.size(); i++)
        if (!std::isfinite(x->quat[i])) return false;
    return true;
}

}  // namespace

// -------------------------------------------------------------------- C ABI
extern "C" {

int orc_set_threads(int nthreads) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
    return omp_get_max_threads();
#else
    (void)nthreads;
    return 1;
#endif
}

int orc_create(const AlensConfig *cfg, OrcCtx **out) {
    if (!cfg || !out) return ALENS_INVALID_ARG;
    if (!box_ok(*cfg)) return ALENS_INVALID_ARG;
    OrcCtx *x = new OrcCtx();
    x->cfg = *cfg;
    *out = x;
    return ALENS_OK;
}

int orc_destroy(OrcCtx *ctx) {
    delete ctx;
    return ALENS_OK;
}

int orc_set_rods(OrcCtx *x, int n, const int64_t *gid, const double *pos,
                 const double *orientation, const double *length,
                 const double *radius, const int32_t *immovable) {
    if (!x || n < 0 || (n > 0 && (!gid || !pos || !orientation || !length || !radius)))
        return ALENS_INVALID_ARG;
    if (n >= (1 << 27)) return ALENS_INVALID_ARG;
    for (int i = 0; i < n; i++)
        if (!(length[i] >= 0.0) || !(radius[i] > 0.0)) return ALENS_INVALID_ARG;
    x->n = n;
    x->gid.assign(gid, gid + n);
    x->pos.assign(pos, pos + 3 * (size_t)n);
    x->quat.assign(orientation, orientation + 4 * (size_t)n);
    x->len.assign(length, length + n);
    x->rad.assign(radius, radius + n);
    x->imm.assign(n, 0);
    if (immovable)
        for (int i = 0; i < n; i++) x->imm[i] = immovable[i] ? 1 : 0;
    x->prevKeys.clear();
    x->prevGamma.clear();
    x->detected = x->solved = false;
    const int rc = setup_grid(x);
    kmc_springs(x);  // the protein springs are rebuilt from the new rods
    return rc;
}

int orc_update_rods(OrcCtx *x, int n, const double *pos, const double *orientation) {
    if (!x || n != x->n || !pos || !orientation) return ALENS_INVALID_ARG;
    x->pos.assign(pos, pos + 3 * (size_t)n);
    x->quat.assign(orientation, orientation + 4 * (size_t)n);
    return ALENS_OK;
}

int orc_get_rods(OrcCtx *x, int n, double *pos, double *orientation) {
    if (!x || n != x->n) return ALENS_INVALID_ARG;
    if (pos) std::copy(x->pos.begin(), x->pos.end(), pos);
    if (orientation) std::copy(x->quat.begin(), x->quat.end(), orientation);
    return ALENS_OK;
}

int orc_get_velocity(OrcCtx *x, int n, double *vel, double *omega) {
    if (!x || n != x->n) return ALENS_INVALID_ARG;
    if (x->vel.size() != 6 * (size_t)n) return ALENS_NOT_READY;
    for (int i = 0; i < n; i++)
        for (int d = 0; d < 3; d++) {
            if (vel) vel[3 * i + d] = x->vel[6 * (size_t)i + d];
            if (omega) omega[3 * i + d] = x->vel[6 * (size_t)i + 3 + d];
        }
    return ALENS_OK;
}

int orc_get_known_velocity(OrcCtx *x, int n, double *vel6) {
    if (!x || n != x->n || !vel6) return ALENS_INVALID_ARG;
    if (x->unc.size() != 6 * (size_t)n) return ALENS_NOT_READY;
    std::copy(x->unc.begin(), x->unc.end(), vel6);
    return ALENS_OK;
}

int orc_add_bilateral(OrcCtx *x, int n, const AlensBlock *blocks) {
    if (!x || n < 0 || (n > 0 && !blocks)) return ALENS_INVALID_ARG;
    for (int b = 0; b < n; b++) {
        const AlensBlock &B = blocks[b];
        if (B.globalIndexI < 0 || B.globalIndexI >= x->n) return ALENS_INVALID_ARG;
        if (!B.oneSide && (B.globalIndexJ < 0 || B.globalIndexJ >= x->n))
            return ALENS_INVALID_ARG;
    }
    x->queue.insert(x->queue.end(), blocks, blocks + n);
    return ALENS_OK;
}

int orc_set_links(OrcCtx *x, int n, const int32_t *idxI, const int32_t *idxJ, const double *sI,
                  const double *sJ, const double *rest, const double *kappa) {
    if (!x || n < 0) return ALENS_INVALID_ARG;
    for (int k = 0; k < n; k++)
        if (idxI[k] < 0 || idxI[k] >= x->n || idxJ[k] < 0 || idxJ[k] >= x->n || !(kappa[k] > 0.0))
            return ALENS_INVALID_ARG;
    x->linkI.assign(idxI, idxI + n);
    x->linkJ.assign(idxJ, idxJ + n);
    x->linkSI.assign(sI, sI + n);
    x->linkSJ.assign(sJ, sJ + n);
    x->linkRest.assign(rest, rest + n);
    x->linkKappa.assign(kappa, kappa + n);
    kmc_springs(x);  // the library rebuilds the protein springs with its link rows
    return ALENS_OK;
}

int orc_set_boundaries(OrcCtx *x, int n, const AlensBoundary *b) {
    if (!x || n < 0 || n > ALENS_MAX_BOUNDARIES || (n > 0 && !b)) return ALENS_INVALID_ARG;
    std::vector<OrcCtx::Bnd> v;
    for (int k = 0; k < n; k++) {
        OrcCtx::Bnd d{};
        d.type = b[k].type;
        d.inside = b[k].inside ? 1 : 0;
        if (d.type < 0 || d.type > 2 || (d.type == 2 && !d.inside)) return ALENS_INVALID_ARG;
        const double an = std::sqrt(b[k].axis[0] * b[k].axis[0] + b[k].axis[1] * b[k].axis[1] +
                                    b[k].axis[2] * b[k].axis[2]);
        if (d.type != 1 && !(an > 0.0)) return ALENS_INVALID_ARG;
        if (d.type != 0 && !(b[k].radius > 0.0)) return ALENS_INVALID_ARG;
        for (int c = 0; c < 3; c++) {
            d.c[c] = b[k].center[c];
            d.a[c] = an > 0.0 ? b[k].axis[c] / an : 0.0;
        }
        d.R = b[k].radius;
        v.push_back(d);
    }
    x->bnd = v;
    return ALENS_OK;
}

int orc_set_initial_gamma(OrcCtx *x, int n, const double *gamma) {
    if (!x || n < 0 || (n > 0 && !gamma)) return ALENS_INVALID_ARG;
    x->initGammaOverride.assign(gamma, gamma + n);
    return ALENS_OK;
}

int orc_detect(OrcCtx *x, AlensStepStats *st) {
    if (!x) return ALENS_INVALID_ARG;
    if (x->n == 0 && x->queue.empty()) {
        // an empty system still steps
    }
    if (!rods_finite(x)) return ALENS_NAN_DETECTED;
    wrap_positions(x);
    rod_prepare(x);
    build_constraints(x);
    build_delassus(x);
    x->detected = true;
    x->solved = false;
    x->last = AlensStepStats{};
    x->last.step = x->step;
    x->last.nRods = x->n;
    x->last.nCollision = x->ncoll;
    x->last.nBilateral = x->nbil;
    if (st) *st = x->last;
    return ALENS_OK;
}

int orc_solve(OrcCtx *x, AlensStepStats *st) {
    if (!x) return ALENS_INVALID_ARG;
    if (!x->detected) return ALENS_NOT_READY;
    int rc = solve_bbpgd(x, &x->last);
    x->last.status = rc;
    x->solved = true;
    if (st) *st = x->last;
    return rc;
}

int orc_advance(OrcCtx *x, AlensStepStats *st) {
    if (!x) return ALENS_INVALID_ARG;
    if (!x->solved) return ALENS_NOT_READY;
    advance(x);
    x->detected = x->solved = false;
    if (st) *st = x->last;
    return ALENS_OK;
}

int orc_step(OrcCtx *x, AlensStepStats *st) {
    int rc = orc_detect(x, st);
    if (rc != ALENS_OK) return rc;
    const int src = orc_solve(x, st);
    if (src != ALENS_OK && src != ALENS_NOT_CONVERGED) return src;
    rc = orc_advance(x, st);
    if (rc != ALENS_OK) return rc;
    return src;
}

int orc_get_num_constraints(OrcCtx *x, int *nCollision, int *nBilateral) {
    if (!x) return ALENS_INVALID_ARG;
    if (nCollision) *nCollision = x->ncoll;
    if (nBilateral) *nBilateral = x->nbil;
    return ALENS_OK;
}

int orc_get_constraints(OrcCtx *x, int cap, int32_t *indexI, int32_t *indexJ,
                        int32_t *image, double *delta0, double *gamma, double *jac) {
    if (!x) return ALENS_INVALID_ARG;
    const int nc = x->ncoll + x->nbil;
    if (cap < nc) return ALENS_CAPACITY;
    for (int k = 0; k < nc; k++) {
        if (indexI) indexI[k] = x->ci[k];
        if (indexJ) indexJ[k] = x->cj[k];
        if (image) image[k] = x->cimg[k];
        if (delta0) delta0[k] = x->phi0[k];
        if (gamma) gamma[k] = x->gamma[k];
        if (jac)
            for (int c = 0; c < 12; c++) jac[12 * (size_t)k + c] = x->jac[12 * (size_t)k + c];
    }
    return ALENS_OK;
}

int orc_get_con_stress(OrcCtx *x, double *stress9) {
    if (!x || !stress9) return ALENS_INVALID_ARG;
    const int64_t nc = x->ncoll + x->nbil;
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) {
            stress9[3 * a + b] = canon_sum_f(
                [&](int64_t k) {
                    const double r = x->lab[6 * k + a] - x->lab[6 * k + 3 + a];
                    return x->gamma[k] * r * x->jac[12 * k + b];
                },
                nc);
        }
    return ALENS_OK;
}

int orc_get_solver_data(OrcCtx *x, int cap, double *q, double *diag) {
    if (!x) return ALENS_INVALID_ARG;
    const int nc = x->ncoll + x->nbil;
    if (cap < nc) return ALENS_CAPACITY;
    for (int k = 0; k < nc; k++) {
        if (q) q[k] = x->q[k];
        if (diag) {
            double d = 0.0;
            for (int64_t e = x->aptr[k]; e < x->aptr[k + 1]; e++)
                if (x->acol[e] == k) d = x->aval[e];
            diag[k] = d + x->cinv[k];
        }
    }
    return ALENS_OK;
}

int orc_get_operator(OrcCtx *x, int capNnz, int *nnz, int32_t *rowPtr, int32_t *cols, double *vals) {
    if (!x) return ALENS_INVALID_ARG;
    const int nc = x->ncoll + x->nbil;
    if (!x->detected && !x->solved) return ALENS_NOT_READY;
    const int64_t total = x->aptr[nc];
    if (nnz) *nnz = (int)total;
    if ((cols || vals) && capNnz < total) return ALENS_CAPACITY;
    if (rowPtr)
        for (int k = 0; k <= nc; k++) rowPtr[k] = (int32_t)x->aptr[k];
    for (int64_t e = 0; e < total; e++) {
        if (cols) cols[e] = x->acol[e];
        if (vals) vals[e] = x->aval[e];
    }
    return ALENS_OK;
}

int orc_get_step_count(OrcCtx *x, int64_t *count) {
    if (!x || !count) return ALENS_INVALID_ARG;
    *count = x->step;
    return ALENS_OK;
}

void orc_dcp(const double c1[3], const double u1[3], double h1, const double c2[3],
             const double u2[3], double h2, double *s, double *t, double P[3],
             double Q[3], double *dist) {
    dcp(c1, u1, h1, c2, u2, h2, s, t, P, Q, dist);
}

double orc_log(double x) { return det_log(x); }

void orc_sincos(double x, double *s, double *c) { det_sincos(x, s, c); }

void orc_normal_pair(uint32_t wa, uint32_t wb, double *z0, double *z1) {
    // one Box-Muller pair of normals6 on two Philox words
    const float ua = ((float)(wa >> 8) + 0.5f) * 5.9604644775390625e-08f;
    const float ub = ((float)(wb >> 8) + 0.5f) * 5.9604644775390625e-08f;
    const float r = std::sqrt(-2.0f * det_logf(ua));
    const float ang = ub * 6.28318531f - 3.14159265f;
    float sn, cs;
    det_sincosf(ang, &sn, &cs);
    *z0 = (double)(r * -cs);
    *z1 = (double)(r * -sn);
}

void orc_philox4x32(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    philox(ctr, key, out);
}

void orc_normals6(uint64_t seed, int64_t gid, int64_t step, double z[6]) {
    normals6(seed, gid, step, z);
}

double orc_canon_sum(const double *v, int64_t n) {
    return canon_sum_f([&](int64_t k) { return v[k]; }, n);
}

void orc_mobility(double length, double radius, double viscosity, double out3[3]) {
    mobility_coeffs(length, radius, viscosity, length < 2.0 * radius, out3);
}

}  // extern "C"
