// oracle_kmc.cpp - CPU oracle of the protein binding step (two-stage KMC
// model: unbound U, singly bound S, doubly bound D).  TEST INFRASTRUCTURE
// ONLY (tests, smoke check, benchmark CPU baseline); the GPU library never
// links or calls it.
//
// What it restates, and from where:
//   * the rates of Protein/ProteinModel.md ("Between Unbound and Singly
//     Bound Stages", "Between Singly Bound and Doubly Bound Stages", "The
//     (dimensionless) S->D probability integral") and the factors of
//     Protein/ProteinData.hpp:90-140 (getBindingFactorUS/SD,
//     getUnbindingFactorSU/DS with the PtoAPratio prefactor and the
//     lambda load sensitivity), with ProteinType::readFromYaml's unit
//     conversion (Protein/ProteinType.hpp:121-127) and the fixedEnd0 rule;
//   * the per-protein step of CalcProteinBind::operator()
//     (SRC/CalcProteinBind.hpp:77-170: stage by bound heads; one roll for
//     U and D, three for S) and KMC_U / KMC_S / KMC_D
//     (SRC/kmc_step_funcs.hpp:35-230: two stacked probabilities, one per
//     head, chosen by the roll; within the head the shifted roll picks the
//     rod and the binding point);
//   * the springs of setProteinConstraints (SRC/TubuleSystem.cpp:694-745).
//
// The reference delegates the probability sums, the chooser and the S->D
// lookup table to the KMC submodule (lamsoa729/KMC, .gitmodules:4-6), which
// is absent from the checkout with no recorded commit.  This file restates
// its published role from Protein/ProteinModel.md:
//   * P = rate x dt per candidate; candidates in ascending rod index;
//   * choose(p0, p1, roll): head 0 if roll < p0, head 1 if roll < p0 + p1
//     (roll shifted by p0), else no event;
//   * U->S: binding point uniform on the chord L_c of the rod's axis inside
//     the capture sphere, radius max(rc, sqrt(6 diffUnbound dt));
//   * S->U: the protein is released uniformly inside that sphere around the
//     head (rejection sampling on Philox words);
//   * S->D: the integral of exp(-(1-lambda) kappa / (2 kT) (l_f(s) - ell0)^2)
//     over the rod, l_f = sqrt(d^2 + s^2) - D (lookupType 0), by composite
//     8-point Gauss-Legendre quadrature over the support where the exponent
//     is above -36 (instead of the table; the integrand in FP32, edges and
//     sums in FP64), the binding point by inverting the cumulative integral
//     (panel search, then 40 bisections).
// Rolls: Philox4x32-10 with key = rngSeed and counter (gid, step,
// 0x6B6D6300 + block), a 53-bit uniform from the first two words of block 0.
//
// PARITY: the PtoAPratio known-answer test of Protein/ProteinTest.hpp:33-71
// pins the S->D binding factor.  The rest of the step (the KMC submodule's
// part) is UNPINNED: no golden outputs exist for it.
//
// Canonical arithmetic as in oracle.cpp: fixed evaluation order, no FMA
// contraction, IEEE +,-,*,/,sqrt in FP64 and FP32 and the project's own exp.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>

#include "oracle_ctx.h"

namespace {

constexpr double kPi = 3.141592653589793;
// 8-point Gauss-Legendre nodes and weights on [-1, 1], rounded to FP32
const float kX8[8] = {
    -0.9602898359298706f, -0.7966665029525757f, -0.5255324244499207f, -0.1834346354007721f,
    0.1834346354007721f,  0.5255324244499207f,  0.7966665029525757f,  0.9602898359298706f};
const float kW8[8] = {
    0.10122853517532349f, 0.22238104045391083f, 0.313706636428833f, 0.3626837730407715f,
    0.3626837730407715f,  0.313706636428833f,   0.22238104045391083f, 0.10122853517532349f};

double bits_to_double(uint64_t b) {
    double d;
    std::memcpy(&d, &b, 8);
    return d;
}

// e^x by Cody-Waite reduction (x = k ln2 + r; ln2 = 0.693147182464599609375
// - 1.904654299957768e-09, the head exact in 24 bits) and the Taylor
// polynomial of e^r to r^13, then exact scaling by 2^k
double kexp(double x) {
    if (!(x == x)) return x;
    if (x > 709.78) return std::numeric_limits<double>::infinity();
    if (x < -745.2) return 0.0;
    const double k = std::floor(x * 1.4426950408889634 + 0.5);
    const double r = (x - k * 0.693147182464599609375) - k * -1.904654299957768e-09;
    double p = 1.0 / 6227020800.0;
    p = p * r + 1.0 / 479001600.0;
    p = p * r + 1.0 / 39916800.0;
    p = p * r + 1.0 / 3628800.0;
    p = p * r + 1.0 / 362880.0;
    p = p * r + 1.0 / 40320.0;
    p = p * r + 1.0 / 5040.0;
    p = p * r + 1.0 / 720.0;
    p = p * r + 1.0 / 120.0;
    p = p * r + 1.0 / 24.0;
    p = p * r + 1.0 / 6.0;
    p = p * r + 0.5;
    p = p * r + 1.0;
    p = p * r + 1.0;
    int ki = (int)k;
    if (ki > 1000) {
        p = p * 0x1p1000;
        ki -= 1000;
    }
    if (ki < -1000) {
        p = p * 0x1p-1000;
        ki += 1000;
    }
    return p * bits_to_double((uint64_t)(int64_t)(ki + 1023) << 52);
}

float bits_to_float(uint32_t b) {
    float f;
    std::memcpy(&f, &b, 4);
    return f;
}

// FP32 e^x of the S->D integrand: ln2 = 0.693145751953125 + 1.428606765330187e-06
// (head exact for |k| < 2^9), Taylor polynomial of e^r to r^8; below e^-87
// the result is zero
float kexpf(float x) {
    if (!(x == x)) return x;
    if (x < -87.0f) return 0.0f;
    if (x > 88.0f) return std::numeric_limits<float>::infinity();
    const float k = std::floor(x * 1.4426950216293335f + 0.5f);
    const float r = (x - k * 0.693145751953125f) - k * 1.428606765330187e-06f;
    float p = 2.4801587642286904e-05f;
    p = p * r + 0.00019841270113829523f;
    p = p * r + 0.0013888889225199819f;
    p = p * r + 0.008333333767950535f;
    p = p * r + 0.0416666679084301f;
    p = p * r + 0.1666666716337204f;
    p = p * r + 0.5f;
    p = p * r + 1.0f;
    p = p * r + 1.0f;
    return p * bits_to_float((unsigned)((int)k + 127) << 23);
}

// species constants (the same folding of dt as the library's table)
struct Kt {
    double ell0, c, A, w, rOuter, Ads, rcap, PtoAP;
    double usCoef[2], suProb[2], sdCoef[2], koD[2];
    double dt, kappa;
    // FP32 copies used by the unbound / singly bound stages
    float rcapf, rOuterf, wf, Af, cf;
    float usCoeff[2], suProbf[2], sdCoeff[2];
    float prefPar, prefAnti;
    float Df;
    int lookup;
    // motion step
    int walkOff, vdrag[2];
    double fstall, vmax[2], vmaxAP[2], diffS[2], diffD[2], diffU, dragD[2], KBT;
};

double bind_volume(double a, double c) {
    const double G = 0.5 * std::sqrt(kPi / a) * (1.0 + std::erf(c * std::sqrt(a)));
    const double e = std::exp(-(a * (c * c)));
    return 4.0 * kPi * ((c * e) / (2.0 * a) + G * (1.0 / (2.0 * a) + c * c));
}

Kt make_type(const AlensProteinType &in, double KBT, double D, double dt) {
    Kt T{};
    double koS[2] = {in.ko_s[0], in.ko_s[1]}, koD[2] = {in.ko_d[0], in.ko_d[1]};
    if (in.fixedEnd0) {
        koS[0] = 0.0;
        koD[0] = 0.0;
    }
    const double Ka[2] = {in.Ka[0] / 602.0, in.Ka[1] / 602.0};
    const double Ke[2] = {in.useBindVol ? in.Ke[0] / 602.0 : in.Ke[0], in.useBindVol ? in.Ke[1] / 602.0 : in.Ke[1]};
    T.ell0 = in.freeLength;
    T.lookup = in.lookupType;
    // centre of the S->D exponent: the head distance less D equals ell0
    // (lookupType 0), or the scaled distance (1 - D/d) r equals ell0 (1)
    T.c = in.lookupType == 0 ? in.freeLength + D : in.freeLength;
    T.A = ((1.0 - in.lambda) * in.kappa) / (2.0 * KBT);
    T.w = 6.0 / std::sqrt(T.A);
    T.rOuter = (in.freeLength + D) + T.w;
    T.Ads = (in.lambda * in.kappa) / (2.0 * KBT);
    const double rd = std::sqrt((6.0 * in.diffUnbound) * dt);
    T.rcap = in.rc > rd ? in.rc : rd;
    T.PtoAP = in.PtoAPratio;
    const double vol = 3.0 / (4.0 * kPi * ((T.rcap * T.rcap) * T.rcap));
    const double Vb = in.useBindVol ? bind_volume(T.A, T.c) : 1.0;
    for (int e = 0; e < 2; e++) {
        T.usCoef[e] = (((koS[e] * Ka[e]) * in.eps) * vol) * dt;
        T.suProb[e] = koS[e] * dt;
        T.sdCoef[e] = (((koD[e] * Ke[e]) * in.eps) * dt) / Vb;
        T.koD[e] = koD[e];
    }
    T.dt = dt;
    T.kappa = in.kappa;
    T.rcapf = (float)T.rcap;
    T.rOuterf = (float)T.rOuter;
    T.wf = (float)T.w;
    T.Af = (float)T.A;
    T.cf = (float)T.c;
    for (int e = 0; e < 2; e++) {
        T.usCoeff[e] = (float)T.usCoef[e];
        T.suProbf[e] = (float)T.suProb[e];
        T.sdCoeff[e] = (float)T.sdCoef[e];
    }
    // Protein/ProteinData.hpp:110-124: the prefactor never exceeds 1
    const float r = (float)in.PtoAPratio;
    T.prefPar = r < 1.0f ? r : 1.0f;
    T.prefAnti = r > 1.0f ? 1.0f / r : 1.0f;
    T.Df = (float)D;
    T.walkOff = in.walkOff ? 1 : 0;
    T.fstall = in.fstall;
    for (int e = 0; e < 2; e++) {
        T.vdrag[e] = in.vdrag[e] ? 1 : 0;
        T.vmax[e] = in.vmax[e];
        T.vmaxAP[e] = in.vmaxAP[e];
        // sqrt(dt D 2) as ProteinData::updatePosWalk / updatePosDiffuse
        T.diffS[e] = std::sqrt((dt * in.diffBoundS[e]) * 2.0);
        T.diffD[e] = std::sqrt((dt * in.diffBoundD[e]) * 2.0);
        T.dragD[e] = in.diffBoundD[e];
    }
    T.diffU = std::sqrt((dt * in.diffUnbound) * 2.0);
    T.KBT = KBT;
    return T;
}

// ---- the S->D integral in FP32: support, panels, sums in a fixed order
float fmaxf_(float a, float b) { return a > b ? a : b; }
float fminf_(float a, float b) { return a < b ? a : b; }

float panel(float a, float b, float d2, float A, float c, float sc) {
    const float h = 0.5f * (b - a), m = 0.5f * (a + b);
    float acc = 0.0f;
    for (int k = 0; k < 8; k++) {
        const float s = m + h * kX8[k];
        const float x = sc * std::sqrt(d2 + s * s) - c;
        acc = acc + kW8[k] * kexpf(-(A * (x * x)));
    }
    return h * acc;
}

// support of the integrand within [sA, sB]: head distances within w of
// c = ell0 + D, i.e. |s| in [sl, sh]; at most two arcs of at most 64
// panels of width <= w/4 each
// lookupType 1 (stretch (1 - D/d) r, d the distance from the axis): the
// exponent -A (k r - c)^2 with k = 1 - D/d, head distances up to
// ell0 + D + w as for lookupType 0, no support when d <= D
struct SdGeom {
    float d2, A, c, k;
    float lo[2], hi[2], step[2];
    int n[2];
};

SdGeom sd_geom(float d2, float sA, float sB, const Kt &T) {
    SdGeom G{};
    const float rO = T.rOuterf, w = T.wf;
    G.d2 = d2;
    G.A = T.Af;
    G.c = T.cf;
    G.k = 1.0f;
    float ro2 = rO * rO;
    if (!(d2 < ro2)) return G;
    float ri = G.c - w;
    if (T.lookup == 1) {
        G.k = 1.0f - T.Df / std::sqrt(d2);
        if (!(G.k > 0.0f)) return G;
        const float rh = (G.c + w) / G.k;
        if (rh < rO) ro2 = rh * rh;
        if (!(d2 < ro2)) return G;
        ri = (G.c - w) / G.k;
    }
    const float sh = std::sqrt(ro2 - d2);
    const float sl = (ri > 0.0f && ri * ri > d2) ? std::sqrt(ri * ri - d2) : 0.0f;
    int k = 0;
    float l = fmaxf_(sA, -sh), h = fminf_(sB, -sl);
    if (h > l) {
        G.lo[k] = l;
        G.hi[k] = h;
        k++;
    }
    l = fmaxf_(sA, sl);
    h = fminf_(sB, sh);
    if (h > l) {
        G.lo[k] = l;
        G.hi[k] = h;
        k++;
    }
    for (int i = 0; i < k; i++) {
        const float q = std::ceil((G.hi[i] - G.lo[i]) / (0.25f * w));
        G.n[i] = q < 1.0f ? 1 : (q > 64.0f ? 64 : (int)q);
        G.step[i] = (G.hi[i] - G.lo[i]) / (float)G.n[i];
    }
    return G;
}

void sd_edges(const SdGeom &G, int j, float *a, float *b) {
    const int i = j < G.n[0] ? 0 : 1;
    const int k = i == 0 ? j : j - G.n[0];
    *a = G.lo[i] + G.step[i] * (float)k;
    *b = k == G.n[i] - 1 ? G.hi[i] : G.lo[i] + G.step[i] * (float)(k + 1);
}

// the integral: panel k into partial sum k mod 32 (in panel order), then
// the 32 partial sums by a fixed pairwise tree (offsets 16, 8, 4, 2, 1)
float sd_integral(const SdGeom &G) {
    float s[32];
    for (int l = 0; l < 32; l++) s[l] = 0.0f;
    const int m = G.n[0] + G.n[1];
    for (int k = 0; k < m; k++) {
        float a, b;
        sd_edges(G, k, &a, &b);
        s[k % 32] = s[k % 32] + panel(a, b, G.d2, G.A, G.c, G.k);
    }
    for (int off = 16; off >= 1; off >>= 1)
        for (int l = 0; l < off; l++) s[l] = s[l] + s[l + off];
    return s[0];
}

// s where the integral from the support start reaches target: the panel
// by the running sum in panel order, then four rounds of a 32-way search of
// that panel's partial integral (the first of 32 equal sub-steps whose
// partial integral is not below the remainder)
float sd_invert(const SdGeom &G, float target) {
    const int m = G.n[0] + G.n[1];
    int kp = m - 1;
    float t = -1.0f, cum = 0.0f;
    for (int k = 0; k < m; k++) {
        float a, b;
        sd_edges(G, k, &a, &b);
        const float P = panel(a, b, G.d2, G.A, G.c, G.k);
        if (target < cum + P) {
            kp = k;
            t = target - cum;
            break;
        }
        cum = cum + P;
    }
    float a, b;
    sd_edges(G, kp, &a, &b);
    if (!(t >= 0.0f)) return b;
    float x0 = a, x1 = b;
    for (int round = 0; round < 4; round++) {
        const float step = (x1 - x0) / 32.0f;
        float xk[32];
        int first = 31;
        for (int k = 0; k < 32; k++) xk[k] = k == 31 ? x1 : x0 + step * (float)(k + 1);
        for (int k = 0; k < 32; k++)
            if (!(panel(a, xk[k], G.d2, G.A, G.c, G.k) < t)) {
                first = k;
                break;
            }
        x0 = first > 0 ? xk[first - 1] : x0;
        x1 = xk[first];
    }
    return 0.5f * (x0 + x1);
}

void words(uint64_t seed, int64_t gid, int64_t step, uint32_t b, uint32_t out[4]) {
    const uint32_t ctr[4] = {(uint32_t)(uint64_t)gid, (uint32_t)((uint64_t)gid >> 32), (uint32_t)(uint64_t)step,
                             0x6B6D6300u + b};
    const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    orc_philox4x32(ctr, key, out);
}

double u53(uint32_t hi, uint32_t lo) {
    return ((double)(hi >> 5) * 67108864.0 + (double)(lo >> 6)) * (1.0 / 9007199254740992.0);
}

// Decisions of the U and S stages in fixed point: an FP32 probability p
// becomes floor(p 2^53) (2^53 for p >= 1); the roll is the 53-bit integer
// of the first two Philox words; the event is the stacked slice holding it
uint64_t fix53(float p) {
    if (!(p > 0.0f)) return 0;
    if (p >= 1.0f) return 1ull << 53;
    uint32_t bits;
    std::memcpy(&bits, &p, 4);
    const int ex = (int)((bits >> 23) & 0xffu);
    if (ex == 0) return 0;
    const uint64_t man = (uint64_t)((bits & 0x7fffffu) | 0x800000u);
    const int sh = ex - 97;
    return sh >= 0 ? man << sh : (-sh >= 64 ? 0 : man >> (-sh));
}

uint64_t roll53(const uint32_t w[4]) { return ((uint64_t)(w[0] >> 5) << 26) | (uint64_t)(w[1] >> 6); }

int choose_fix(uint64_t F0, uint64_t F1, uint64_t *roll) {
    const uint64_t u = *roll;
    if (u < F0) return 0;
    if (u < F0 + F1) {
        *roll = u - F0;
        return 1;
    }
    return -1;
}

int pick_fix(const std::vector<uint64_t> &F, uint64_t roll, float *frac) {
    uint64_t cum = 0;
    int last = -1;
    for (int j = 0; j < (int)F.size(); j++) {
        if (F[j] == 0) continue;
        last = j;
        if (roll < cum + F[j]) {
            *frac = (float)(roll - cum) / (float)F[j];
            return j;
        }
        cum = cum + F[j];
    }
    *frac = 1.0f;
    return last;
}

int choose(double p0, double p1, double *roll) {
    const double u = *roll;
    if (u < p0) return 0;
    if (u < p0 + p1) {
        *roll = u - p0;
        return 1;
    }
    return -1;
}

double wrap1(double v, double lo, double hi, double L) {
    for (int k = 0; k < 64; k++) {
        if (v < lo)
            v = v + L;
        else if (v >= hi)
            v = v - L;
        else
            break;
    }
    return v;
}

void wrap_point(const AlensConfig &c, double p[3]) {
    for (int d = 0; d < 3; d++)
        if (c.simBoxPBC[d]) p[d] = wrap1(p[d], c.simBoxLow[d], c.simBoxHigh[d], c.simBoxHigh[d] - c.simBoxLow[d]);
}

double min_image(const AlensConfig &c, int d, double v) {
    if (!c.simBoxPBC[d]) return v;
    const double L = c.simBoxHigh[d] - c.simBoxLow[d];
    return v - L * std::floor(v / L + 0.5);
}

// The binding grid: cells of edge >= reach (largest rod half-length plus
// the largest capture distance), at most max(64, 2 n) cells with two per
// periodic side at least, so that every rod within reach of a point lies
// in one of the 27 cells around it, each offset naming one image.
struct Grid {
    int nc[3] = {1, 1, 1};
    double cs[3] = {1, 1, 1};
    std::vector<int> start, rod;  // rods by cell, ascending within a cell
};

int cell_of(const AlensConfig &c, const Grid &G, int d, double v) {
    const double f = std::floor((v - c.simBoxLow[d]) / G.cs[d]);
    return f < 0.0 ? 0 : (f > (double)(G.nc[d] - 1) ? G.nc[d] - 1 : (int)f);
}

// per rod: wrapped centre, axis, half-length (FP64) and the FP32 screening
// geometry (centre relative to its cell origin, half-length, axis)
struct RodView {
    std::vector<double> c, a, hl;
    std::vector<uint8_t> sphere;
    std::vector<float> rel, af, hlf;
};

RodView rod_view(const OrcCtx *x) {
    RodView V;
    const int n = x->n;
    V.c.resize(3 * (size_t)n);
    V.a.resize(3 * (size_t)n);
    V.hl.resize(n);
    V.sphere.resize(n);
    for (int i = 0; i < n; i++) {
        double p[3] = {x->pos[3 * i], x->pos[3 * i + 1], x->pos[3 * i + 2]};
        wrap_point(x->cfg, p);
        const double *q = &x->quat[4 * i];
        V.c[3 * i] = p[0];
        V.c[3 * i + 1] = p[1];
        V.c[3 * i + 2] = p[2];
        V.a[3 * i] = 2.0 * (q[0] * q[2] + q[3] * q[1]);
        V.a[3 * i + 1] = 2.0 * (q[1] * q[2] - q[3] * q[0]);
        V.a[3 * i + 2] = 1.0 - 2.0 * (q[0] * q[0] + q[1] * q[1]);
        V.hl[i] = 0.5 * x->len[i];
        V.sphere[i] = x->len[i] < 2.0 * x->rad[i] ? 1 : 0;
    }
    return V;
}

Grid make_grid(const OrcCtx *x, RodView &V, double reach) {
    const AlensConfig &cf = x->cfg;
    Grid G;
    for (int d = 0; d < 3; d++) {
        const double L = cf.simBoxHigh[d] - cf.simBoxLow[d];
        const double f = reach > 0.0 ? std::floor(L / reach) : 1.0;
        G.nc[d] = f < 1.0 ? 1 : (f > 512.0 ? 512 : (int)f);
    }
    const long long limit = std::max<long long>(64, 2LL * x->n);
    while ((long long)G.nc[0] * G.nc[1] * G.nc[2] > limit) {
        int d = -1;
        for (int e = 0; e < 3; e++)
            if (G.nc[e] > (cf.simBoxPBC[e] ? 2 : 1) && (d < 0 || G.nc[e] > G.nc[d])) d = e;
        if (d < 0) break;
        G.nc[d] = std::max(cf.simBoxPBC[d] ? 2 : 1, G.nc[d] / 2);
    }
    for (int d = 0; d < 3; d++) G.cs[d] = (cf.simBoxHigh[d] - cf.simBoxLow[d]) / G.nc[d];
    const int ncell = G.nc[0] * G.nc[1] * G.nc[2];
    std::vector<int> cnt(ncell + 1, 0), cell(x->n);
    V.rel.resize(3 * (size_t)x->n);
    V.af.resize(3 * (size_t)x->n);
    V.hlf.resize(x->n);
    for (int r = 0; r < x->n; r++) {
        int c[3];
        for (int d = 0; d < 3; d++) {
            c[d] = cell_of(cf, G, d, V.c[3 * r + d]);
            V.rel[3 * r + d] = (float)(V.c[3 * r + d] - (cf.simBoxLow[d] + (double)c[d] * G.cs[d]));
            V.af[3 * r + d] = (float)V.a[3 * r + d];
        }
        V.hlf[r] = (float)V.hl[r];
        cell[r] = (c[2] * G.nc[1] + c[1]) * G.nc[0] + c[0];
        cnt[cell[r] + 1]++;
    }
    for (int k = 0; k < ncell; k++) cnt[k + 1] += cnt[k];
    G.start = cnt;
    G.rod.resize(x->n);
    for (int r = 0; r < x->n; r++) G.rod[cnt[cell[r]]++] = r;
    return G;
}

// distance from P to the axis segment of rod r (minimum image)
double dist_point_seg(const OrcCtx *x, const RodView &V, const double P[3], int r) {
    double u[3];
    for (int d = 0; d < 3; d++) u[d] = min_image(x->cfg, d, P[d] - V.c[3 * r + d]);
    const double *a = &V.a[3 * r];
    double t = u[0] * a[0] + u[1] * a[1] + u[2] * a[2];
    t = t > V.hl[r] ? V.hl[r] : (t < -V.hl[r] ? -V.hl[r] : t);
    const double q0 = u[0] - t * a[0], q1 = u[1] - t * a[1], q2 = u[2] - t * a[2];
    return std::sqrt(q0 * q0 + q1 * q1 + q2 * q2);
}

// ProteinData::getProteinForceLength (Protein/ProteinData.hpp:171-195): the
// heads' distance ell less D (lookupType 0), or scaled by 1 - D/d with d the
// distance of head 0 from the segment of head 1's rod (lookupType 1)
double force_length(const OrcCtx *x, const RodView &V, const Kt &T, const double P0[3], int r1, double ell) {
    if (T.lookup == 0) return ell - x->kmcD;
    return (1.0 - x->kmcD / dist_point_seg(x, V, P0, r1)) * ell;
}

struct Cand {
    int li;
    float v0, v1, v2, v3;  // U: Lc, lo, hl; S: t0, d2, hl, axis dot
};

// the rods of the 27 stencil cells around X that pass the stage's distance
// test, ascending rod index
std::vector<Cand> gather(const OrcCtx *x, const RodView &V, const Grid &G, const Kt &T, const double X[3],
                         int stage, int idb, const float ab[3]) {
    const AlensConfig &cf = x->cfg;
    int c[3], lo[3], hi[3];
    float rx[3], csf[3];
    for (int d = 0; d < 3; d++) {
        c[d] = cell_of(cf, G, d, X[d]);
        rx[d] = (float)(X[d] - (cf.simBoxLow[d] + (double)c[d] * G.cs[d]));
        csf[d] = (float)G.cs[d];
        if (cf.simBoxPBC[d]) {
            lo[d] = -1;
            hi[d] = 1;
        } else {
            lo[d] = c[d] > 0 ? -1 : 0;
            hi[d] = c[d] < G.nc[d] - 1 ? 1 : 0;
        }
    }
    const float r2 = T.rcapf * T.rcapf;
    const float ro2 = T.rOuterf * T.rOuterf;
    std::vector<Cand> C;
    for (int oz = lo[2]; oz <= hi[2]; oz++)
        for (int oy = lo[1]; oy <= hi[1]; oy++)
            for (int ox = lo[0]; ox <= hi[0]; ox++) {
                const int o[3] = {ox, oy, oz};
                int cc[3];
                for (int d = 0; d < 3; d++) {
                    cc[d] = c[d] + o[d];
                    if (cf.simBoxPBC[d]) cc[d] = (cc[d] + G.nc[d]) % G.nc[d];
                }
                const int k = (cc[2] * G.nc[1] + cc[1]) * G.nc[0] + cc[0];
                const float sh[3] = {(float)o[0] * csf[0], (float)o[1] * csf[1], (float)o[2] * csf[2]};
                for (int s = G.start[k]; s < G.start[k + 1]; s++) {
                    const int r = G.rod[s];
                    if (V.sphere[r]) continue;
                    const float *R = &V.rel[3 * r], *A = &V.af[3 * r];
                    const float hl = V.hlf[r];
                    const float v0 = (rx[0] - R[0]) - sh[0];
                    const float v1 = (rx[1] - R[1]) - sh[1];
                    const float v2 = (rx[2] - R[2]) - sh[2];
                    const float t0 = (v0 * A[0] + v1 * A[1]) + v2 * A[2];
                    const float q0 = v0 - t0 * A[0], q1 = v1 - t0 * A[1], q2 = v2 - t0 * A[2];
                    const float d2 = (q0 * q0 + q1 * q1) + q2 * q2;
                    if (stage == 0) {
                        if (!(d2 < r2)) continue;
                        const float hc = std::sqrt(r2 - d2);
                        const float l = fmaxf_(-hl, t0 - hc), h = fminf_(hl, t0 + hc);
                        const float Lc = h - l;
                        if (!(Lc > 0.0f)) continue;
                        C.push_back(Cand{r, Lc, l, hl, 0.0f});
                    } else {
                        if (r == idb || !(d2 < ro2)) continue;
                        C.push_back(Cand{r, t0, d2, hl, (A[0] * ab[0] + A[1] * ab[1]) + A[2] * ab[2]});
                    }
                }
            }
    std::sort(C.begin(), C.end(), [](const Cand &a, const Cand &b) { return a.li < b.li; });
    return C;
}

// one protein's binding step; returns the transition (0 none, 1 U->S,
// 2 S->U, 3 S->D, 4 D->S) and the number of candidate rods
int protein_step(const OrcCtx *x, const RodView &V, const Grid &G, const Kt &T, AlensProtein &pr, int *ncand) {
    const AlensConfig &cf = x->cfg;
    const double qnan = std::numeric_limits<double>::quiet_NaN();
    for (int e = 0; e < 2; e++)
        if (pr.idBind[e] < 0 || pr.idBind[e] >= x->n) pr.idBind[e] = -1;
    double P[2][3];
    for (int e = 0; e < 2; e++) {
        if (pr.idBind[e] < 0) continue;
        const int r = pr.idBind[e];
        for (int d = 0; d < 3; d++) P[e][d] = V.c[3 * r + d] + pr.distBind[e] * V.a[3 * r + d];
    }
    const int nb = (pr.idBind[0] >= 0 ? 1 : 0) + (pr.idBind[1] >= 0 ? 1 : 0);
    uint32_t w[4];
    words(cf.rngSeed, pr.gid, x->step, 0, w);
    double roll = u53(w[0], w[1]);
    int trans = 0;
    *ncand = 0;
    if (nb == 0) {
        double X[3] = {pr.pos[0], pr.pos[1], pr.pos[2]};
        wrap_point(cf, X);
        pr.pos[0] = X[0];
        pr.pos[1] = X[1];
        pr.pos[2] = X[2];
        const float ab[3] = {0.0f, 0.0f, 0.0f};
        const std::vector<Cand> C = gather(x, V, G, T, X, 0, -1, ab);
        *ncand = (int)C.size();
        uint64_t R = roll53(w);
        uint64_t S0 = 0, S1 = 0;
        for (const Cand &k : C) S0 = S0 + fix53(k.v0 * T.usCoeff[0]);
        for (const Cand &k : C) S1 = S1 + fix53(k.v0 * T.usCoeff[1]);
        const int e = choose_fix(S0, S1, &R);
        if (e >= 0) {
            std::vector<uint64_t> F;
            for (const Cand &k : C) F.push_back(fix53(k.v0 * T.usCoeff[e]));
            float frac;
            const int j = pick_fix(F, R, &frac);
            if (j >= 0) {
                const double hl = V.hl[C[j].li];
                const double s = (double)(C[j].v1 + frac * C[j].v0);
                pr.idBind[e] = C[j].li;
                pr.distBind[e] = s > hl ? hl : (s < -hl ? -hl : s);
                trans = 1;
            }
        }
    } else if (nb == 1) {
        const int b = pr.idBind[0] >= 0 ? 0 : 1, f = 1 - b;
        double X[3] = {P[b][0], P[b][1], P[b][2]};
        wrap_point(cf, X);
        const int rb = pr.idBind[b];
        const float ab[3] = {(float)V.a[3 * rb], (float)V.a[3 * rb + 1], (float)V.a[3 * rb + 2]};
        const std::vector<Cand> C = gather(x, V, G, T, X, 1, rb, ab);
        *ncand = (int)C.size();
        std::vector<uint64_t> F(C.size());
        std::vector<float> I(C.size());
        for (size_t j = 0; j < C.size(); j++) {
            I[j] = sd_integral(sd_geom(C[j].v1, -C[j].v2 - C[j].v0, C[j].v2 - C[j].v0, T));
            // parallel when the axes' dot product is positive
            const float pref = C[j].v3 > 0.0f ? T.prefPar : T.prefAnti;
            F[j] = fix53((pref * T.sdCoeff[f]) * I[j]);
        }
        uint64_t Sb = 0;
        for (uint64_t v : F) Sb = Sb + v;
        const uint64_t FU = fix53(T.suProbf[b]);
        uint64_t R = roll53(w);
        const int e = choose_fix(b == 0 ? FU : Sb, b == 0 ? Sb : FU, &R);
        if (e == b) {
            double off[3] = {0.0, 0.0, 0.0};
            for (uint32_t k = 0; k < 32; k++) {
                uint32_t v[4];
                words(cf.rngSeed, pr.gid, x->step, 2 + k, v);
                const double xx = 2.0 * (((double)v[0] + 0.5) * 2.3283064365386963e-10) - 1.0;
                const double yy = 2.0 * (((double)v[1] + 0.5) * 2.3283064365386963e-10) - 1.0;
                const double zz = 2.0 * (((double)v[2] + 0.5) * 2.3283064365386963e-10) - 1.0;
                if ((xx * xx + yy * yy) + zz * zz <= 1.0) {
                    off[0] = xx;
                    off[1] = yy;
                    off[2] = zz;
                    break;
                }
            }
            for (int d = 0; d < 3; d++) pr.pos[d] = P[b][d] + T.rcap * off[d];
            pr.idBind[b] = -1;
            trans = 2;
        } else if (e == f) {
            float frac;
            const int j = pick_fix(F, R, &frac);
            if (j >= 0) {
                const SdGeom Gj = sd_geom(C[j].v1, -C[j].v2 - C[j].v0, C[j].v2 - C[j].v0, T);
                const float sStar = sd_invert(Gj, frac * I[j]);
                const double hl = V.hl[C[j].li];
                const double s = (double)(C[j].v0 + sStar);
                pr.idBind[f] = C[j].li;
                pr.distBind[f] = s > hl ? hl : (s < -hl ? -hl : s);
                trans = 3;
            }
        }
    } else {
        double dv[3];
        for (int d = 0; d < 3; d++) dv[d] = min_image(cf, d, P[1][d] - P[0][d]);
        const double ell = std::sqrt(dv[0] * dv[0] + dv[1] * dv[1] + dv[2] * dv[2]);
        const double xx = force_length(x, V, T, P[0], pr.idBind[1], ell) - T.ell0;
        const double M = T.Ads * (xx * xx);
        const double g = kexp(M);
        const double p0 = (T.koD[0] * g) * T.dt, p1 = (T.koD[1] * g) * T.dt;
        const int e = choose(p0, p1, &roll);
        if (e >= 0) {
            pr.idBind[e] = -1;
            trans = 4;
        }
    }
    for (int e = 0; e < 2; e++) {
        if (pr.idBind[e] < 0) {
            pr.distBind[e] = qnan;
            pr.posEnd[e][0] = pr.posEnd[e][1] = pr.posEnd[e][2] = qnan;
            continue;
        }
        const int r = pr.idBind[e];
        for (int d = 0; d < 3; d++) pr.posEnd[e][d] = V.c[3 * r + d] + pr.distBind[e] * V.a[3 * r + d];
    }
    const int nb2 = (pr.idBind[0] >= 0 ? 1 : 0) + (pr.idBind[1] >= 0 ? 1 : 0);
    if (nb2 == 1) {
        const int b = pr.idBind[0] >= 0 ? 0 : 1;
        for (int d = 0; d < 3; d++) pr.pos[d] = pr.posEnd[b][d];
    } else if (nb2 == 2) {
        for (int d = 0; d < 3; d++) {
            const double dv = min_image(cf, d, pr.posEnd[1][d] - pr.posEnd[0][d]);
            pr.pos[d] = pr.posEnd[0][d] + 0.5 * dv;
        }
    }
    wrap_point(cf, pr.pos);
    return trans;
}

// a point outside a boundary is moved onto it: wall, sphere (inside /
// outside), tube (inside)
void project(const OrcCtx::Bnd &B, double x[3]) {
    const double v[3] = {x[0] - B.c[0], x[1] - B.c[1], x[2] - B.c[2]};
    if (B.type == 0) {
        const double s = v[0] * B.a[0] + v[1] * B.a[1] + v[2] * B.a[2];
        if (s < 0.0)
            for (int d = 0; d < 3; d++) x[d] = x[d] - s * B.a[d];
    } else if (B.type == 1) {
        const double r = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        const bool out = B.inside ? r > B.R : r < B.R;
        if (out && r > 0.0)
            for (int d = 0; d < 3; d++) x[d] = B.c[d] + (B.R / r) * v[d];
    } else {
        const double s = v[0] * B.a[0] + v[1] * B.a[1] + v[2] * B.a[2];
        const double q[3] = {v[0] - s * B.a[0], v[1] - s * B.a[1], v[2] - s * B.a[2]};
        const double r = std::sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2]);
        if (r > B.R)
            for (int d = 0; d < 3; d++) x[d] = (B.c[d] + s * B.a[d]) + (B.R / r) * q[d];
    }
}

// one protein's motion step (ProteinData::updatePosWalk / updatePosDiffuse,
// Protein/ProteinData.hpp:318-406; walk velocity :459-478; drag :489-498;
// spring load of updateForceTorqueBind :418-440); returns the transition
// (0 none, 2 S->U, 4 D->S by walking off a rod end)
int protein_motion(const OrcCtx *x, const RodView &V, const Kt &T, AlensProtein &pr) {
    const AlensConfig &cf = x->cfg;
    int id[2] = {pr.idBind[0], pr.idBind[1]};
    for (int e = 0; e < 2; e++)
        if (id[e] < 0 || id[e] >= x->n) id[e] = -1;
    const int nb = (id[0] >= 0 ? 1 : 0) + (id[1] >= 0 ? 1 : 0);
    const uint32_t key[2] = {(uint32_t)cf.rngSeed, (uint32_t)(cf.rngSeed >> 32)};
    const uint32_t c0[4] = {(uint32_t)(uint64_t)pr.gid, (uint32_t)((uint64_t)pr.gid >> 32), (uint32_t)(uint64_t)x->step,
                            0x6D6F7400u};
    const uint32_t c1[4] = {c0[0], c0[1], c0[2], 0x6D6F7401u};
    uint32_t w[4], v[4];
    orc_philox4x32(c0, key, w);
    orc_philox4x32(c1, key, v);
    const double u01 = u53(w[0], w[1]);
    double z0, z1, z2, z3;
    orc_normal_pair(w[2], w[3], &z0, &z1);
    orc_normal_pair(v[0], v[1], &z2, &z3);
    int trans = 0;
    if (nb == 0) {
        pr.idBind[0] = pr.idBind[1] = -1;
        pr.pos[0] = pr.pos[0] + T.diffU * z0;
        pr.pos[1] = pr.pos[1] + T.diffU * z1;
        pr.pos[2] = pr.pos[2] + T.diffU * z2;
    } else {
        double dist[2] = {pr.distBind[0], pr.distBind[1]};
        if (nb == 2) {
            double P[2][3];
            for (int e = 0; e < 2; e++)
                for (int d = 0; d < 3; d++) P[e][d] = V.c[3 * id[e] + d] + dist[e] * V.a[3 * id[e] + d];
            double rv[3];
            for (int d = 0; d < 3; d++) rv[d] = min_image(cf, d, P[0][d] - P[1][d]);
            const double ell = std::sqrt(rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2]);
            const double force = (force_length(x, V, T, P[0], id[1], ell) - T.ell0) * T.kappa;
            const double f0[3] = {-force * (rv[0] / ell), -force * (rv[1] / ell), -force * (rv[2] / ell)};
            const double *a0 = &V.a[3 * id[0]], *a1 = &V.a[3 * id[1]];
            const double par = a0[0] * a1[0] + a0[1] * a1[1] + a0[2] * a1[2];
            const double z[2] = {z0, z1};
            for (int e = 0; e < 2; e++) {
                const double *a = e == 0 ? a0 : a1;
                const double sg = e == 0 ? 1.0 : -1.0;  // the other head's load is -f0
                const double fdir = sg * (f0[0] * a[0] + f0[1] * a[1] + f0[2] * a[2]);
                const double sgn = T.vmax[e] > 0.0 ? 1.0 : (T.vmax[e] < 0.0 ? -1.0 : 0.0);
                const double fproj = (sgn * fdir) / std::fabs(T.fstall);
                const double one = 1.0 + fproj;
                const double vfrac = one < 0.0 ? 0.0 : (one > 1.0 ? 1.0 : one);
                const double vel = (par > 0.0 ? T.vmax[e] : T.vmaxAP[e]) * vfrac;
                const double drag = T.vdrag[e] ? (fdir * T.dragD[e]) / T.KBT : 0.0;
                dist[e] = dist[e] + ((vel + drag) * T.dt + T.diffD[e] * z[e]);
            }
        } else {
            const int b = id[0] >= 0 ? 0 : 1;
            dist[b] = dist[b] + (T.vmax[b] * T.dt + T.diffS[b] * (b == 0 ? z0 : z1));
        }
        bool off[2] = {false, false};
        double half[2] = {0.0, 0.0};
        for (int e = 0; e < 2; e++) {
            if (id[e] < 0) continue;
            half[e] = V.hl[id[e]];
            off[e] = dist[e] > half[e] || dist[e] < -half[e];
        }
        auto clamp = [](double d, double h) { return d > h ? h : (d < -h ? -h : d); };
        if (T.walkOff) {
            if (off[0] && off[1]) {
                const int e = u01 < 0.5 ? 0 : 1;
                id[e] = -1;
                dist[1 - e] = clamp(dist[1 - e], half[1 - e]);
            } else if (off[0]) {
                id[0] = -1;
            } else if (off[1]) {
                id[1] = -1;
            }
        } else {
            for (int e = 0; e < 2; e++)
                if (id[e] >= 0) dist[e] = clamp(dist[e], half[e]);
        }
        const int nb2 = (id[0] >= 0 ? 1 : 0) + (id[1] >= 0 ? 1 : 0);
        if (nb2 < nb) trans = nb == 2 ? 4 : 2;
        for (int e = 0; e < 2; e++) {
            pr.idBind[e] = id[e];
            pr.distBind[e] = dist[e];
        }
    }
    if (pr.idBind[0] < 0 && pr.idBind[1] < 0)
        for (const OrcCtx::Bnd &B : x->bnd) project(B, pr.pos);
    return trans;
}

// head positions and centre of a protein's state, wrapped
void protein_geometry(const OrcCtx *x, const RodView &V, AlensProtein &pr) {
    const AlensConfig &cf = x->cfg;
    const double qnan = std::numeric_limits<double>::quiet_NaN();
    for (int e = 0; e < 2; e++) {
        if (pr.idBind[e] < 0) {
            pr.distBind[e] = qnan;
            pr.posEnd[e][0] = pr.posEnd[e][1] = pr.posEnd[e][2] = qnan;
            continue;
        }
        const int r = pr.idBind[e];
        for (int d = 0; d < 3; d++) pr.posEnd[e][d] = V.c[3 * r + d] + pr.distBind[e] * V.a[3 * r + d];
    }
    const int nb = (pr.idBind[0] >= 0 ? 1 : 0) + (pr.idBind[1] >= 0 ? 1 : 0);
    if (nb == 1) {
        const int b = pr.idBind[0] >= 0 ? 0 : 1;
        for (int d = 0; d < 3; d++) pr.pos[d] = pr.posEnd[b][d];
    } else if (nb == 2) {
        for (int d = 0; d < 3; d++) {
            const double dv = min_image(cf, d, pr.posEnd[1][d] - pr.posEnd[0][d]);
            pr.pos[d] = pr.posEnd[0][d] + 0.5 * dv;
        }
    }
    wrap_point(cf, pr.pos);
}

bool nonneg(double v) { return std::isfinite(v) && v >= 0.0; }

bool type_ok(const AlensProteinType &p) {
    bool ok = (p.lookupType == 0 || p.lookupType == 1) && std::isfinite(p.kappa) && p.kappa > 0.0 && std::isfinite(p.lambda) &&
              p.lambda >= 0.0 && p.lambda < 1.0 && nonneg(p.freeLength) && std::isfinite(p.rc) && p.rc > 0.0 &&
              nonneg(p.eps) && nonneg(p.diffUnbound) && std::isfinite(p.PtoAPratio) && p.PtoAPratio > 0.0;
    ok = ok && std::isfinite(p.fstall) && p.fstall != 0.0;
    for (int e = 0; e < 2; e++)
        ok = ok && nonneg(p.ko_s[e]) && nonneg(p.ko_d[e]) && nonneg(p.Ka[e]) && nonneg(p.Ke[e]) &&
             std::isfinite(p.vmax[e]) && std::isfinite(p.vmaxAP[e]) && nonneg(p.diffBoundS[e]) &&
             nonneg(p.diffBoundD[e]);
    return ok;
}

}  // namespace

void kmc_springs(OrcCtx *x) {
    x->springI.clear();
    x->springJ.clear();
    x->springSI.clear();
    x->springSJ.clear();
    x->springRest.clear();
    x->springKappa.clear();
    if (x->prot.empty() || x->ptypes.empty()) return;
    const RodView V = rod_view(x);
    for (const AlensProtein &p : x->prot) {
        if (p.idBind[0] < 0 || p.idBind[0] >= x->n || p.idBind[1] < 0 || p.idBind[1] >= x->n) continue;
        const AlensProteinType &t = x->ptypes[p.type];
        double rest = t.freeLength + x->kmcD;
        if (t.lookupType == 1) {
            // rest length so that head distance - rest is the lookupType 1
            // stretch at the current geometry
            const int r0 = p.idBind[0], r1 = p.idBind[1];
            double P0[3], dv[3];
            for (int d = 0; d < 3; d++) P0[d] = V.c[3 * r0 + d] + p.distBind[0] * V.a[3 * r0 + d];
            for (int d = 0; d < 3; d++)
                dv[d] = min_image(x->cfg, d, (V.c[3 * r1 + d] + p.distBind[1] * V.a[3 * r1 + d]) - P0[d]);
            const double ell = std::sqrt(dv[0] * dv[0] + dv[1] * dv[1] + dv[2] * dv[2]);
            rest = t.freeLength + (x->kmcD * ell) / dist_point_seg(x, V, P0, r1);
        }
        x->springI.push_back(p.idBind[0]);
        x->springJ.push_back(p.idBind[1]);
        x->springSI.push_back(p.distBind[0]);
        x->springSJ.push_back(p.distBind[1]);
        x->springRest.push_back(rest);
        x->springKappa.push_back(t.kappa);
    }
}

extern "C" {

int orc_set_protein_types(OrcCtx *x, int n, const AlensProteinType *t, double KBT, double D) {
    if (!x || n < 0 || (n > 0 && !t) || !(KBT > 0.0) || !std::isfinite(KBT) || !nonneg(D)) return ALENS_INVALID_ARG;
    for (int k = 0; k < n; k++)
        if (!type_ok(t[k])) return ALENS_INVALID_ARG;
    for (const AlensProtein &p : x->prot)
        if (p.type >= n) return ALENS_INVALID_ARG;
    x->ptypes.assign(t, t + n);
    x->kmcKBT = KBT;
    x->kmcD = D;
    kmc_springs(x);
    return ALENS_OK;
}

int orc_set_proteins(OrcCtx *x, int n, const AlensProtein *p) {
    if (!x || n < 0 || (n > 0 && !p)) return ALENS_INVALID_ARG;
    if (n > 0 && x->ptypes.empty()) return ALENS_NOT_READY;
    for (int k = 0; k < n; k++) {
        const AlensProtein &q = p[k];
        if (q.type < 0 || q.type >= (int)x->ptypes.size()) return ALENS_INVALID_ARG;
        int nb = 0;
        for (int e = 0; e < 2; e++) {
            if (q.idBind[e] == -1) continue;
            if (q.idBind[e] < 0 || q.idBind[e] >= x->n || !std::isfinite(q.distBind[e])) return ALENS_INVALID_ARG;
            nb++;
        }
        if (nb == 0 && !(std::isfinite(q.pos[0]) && std::isfinite(q.pos[1]) && std::isfinite(q.pos[2])))
            return ALENS_INVALID_ARG;
    }
    x->prot.assign(p, p + n);
    kmc_springs(x);
    return ALENS_OK;
}

int orc_get_proteins(OrcCtx *x, int cap, int *n, AlensProtein *out) {
    if (!x || !n || cap < 0) return ALENS_INVALID_ARG;
    *n = (int)x->prot.size();
    if (cap < *n) return ALENS_CAPACITY;
    if (*n > 0) std::memcpy(out, x->prot.data(), sizeof(AlensProtein) * x->prot.size());
    return ALENS_OK;
}

int orc_protein_bind_step(OrcCtx *x, AlensKmcStats *st) {
    if (!x) return ALENS_INVALID_ARG;
    AlensKmcStats s{};
    if (!x->prot.empty()) {
        if (x->ptypes.empty()) return ALENS_NOT_READY;
        RodView V = rod_view(x);
        std::vector<Kt> T;
        double reach = 0.0, hl = 0.0;
        for (const AlensProteinType &t : x->ptypes) {
            T.push_back(make_type(t, x->kmcKBT, x->kmcD, x->cfg.dt));
            reach = std::max(reach, std::max(T.back().rcap, T.back().rOuter));
        }
        for (int r = 0; r < x->n; r++) hl = std::max(hl, V.hl[r]);
        reach += hl;
        for (int d = 0; d < 3; d++)
            if (x->cfg.simBoxPBC[d] && !(x->cfg.simBoxHigh[d] - x->cfg.simBoxLow[d] >= 2.0 * reach))
                return ALENS_INVALID_ARG;
        const Grid G = make_grid(x, V, reach);
        const int np = (int)x->prot.size();
        std::vector<int> trans(np), nc(np);
#pragma omp parallel for schedule(dynamic, 64)
        for (int p = 0; p < np; p++) trans[p] = protein_step(x, V, G, T[x->prot[p].type], x->prot[p], &nc[p]);
        for (int p = 0; p < np; p++) {
            const AlensProtein &q = x->prot[p];
            const int nb = (q.idBind[0] >= 0 ? 1 : 0) + (q.idBind[1] >= 0 ? 1 : 0);
            (nb == 0 ? s.nU : nb == 1 ? s.nS : s.nD)++;
            if (trans[p] == 1) s.nUS++;
            if (trans[p] == 2) s.nSU++;
            if (trans[p] == 3) s.nSD++;
            if (trans[p] == 4) s.nDS++;
            s.maxCandidates = std::max(s.maxCandidates, nc[p]);
        }
    }
    kmc_springs(x);
    if (st) *st = s;
    return ALENS_OK;
}

int orc_protein_motion_step(OrcCtx *x, AlensKmcStats *st) {
    if (!x) return ALENS_INVALID_ARG;
    AlensKmcStats s{};
    if (!x->prot.empty()) {
        if (x->ptypes.empty()) return ALENS_NOT_READY;
        const RodView V = rod_view(x);
        std::vector<Kt> T;
        for (const AlensProteinType &t : x->ptypes) T.push_back(make_type(t, x->kmcKBT, x->kmcD, x->cfg.dt));
        const int np = (int)x->prot.size();
        std::vector<int> trans(np);
#pragma omp parallel for schedule(static)
        for (int p = 0; p < np; p++) {
            trans[p] = protein_motion(x, V, T[x->prot[p].type], x->prot[p]);
            protein_geometry(x, V, x->prot[p]);
        }
        for (int p = 0; p < np; p++) {
            const AlensProtein &q = x->prot[p];
            const int nb = (q.idBind[0] >= 0 ? 1 : 0) + (q.idBind[1] >= 0 ? 1 : 0);
            (nb == 0 ? s.nU : nb == 1 ? s.nS : s.nD)++;
            if (trans[p] == 2) s.nSU++;
            if (trans[p] == 4) s.nDS++;
        }
    }
    kmc_springs(x);
    if (st) *st = s;
    return ALENS_OK;
}

double orc_kmc_exp(double x) { return kexp(x); }

float orc_kmc_expf(float x) { return kexpf(x); }

double orc_kmc_sd_integral(const AlensProteinType *t, double KBT, double D, double dt, double d2, double sA,
                           double sB) {
    return (double)sd_integral(sd_geom((float)d2, (float)sA, (float)sB, make_type(*t, KBT, D, dt)));
}

double orc_kmc_sd_invert(const AlensProteinType *t, double KBT, double D, double dt, double d2, double sA,
                         double sB, double target) {
    return (double)sd_invert(sd_geom((float)d2, (float)sA, (float)sB, make_type(*t, KBT, D, dt)), (float)target);
}

double orc_kmc_bind_volume(const AlensProteinType *t, double KBT, double D) {
    const Kt T = make_type(*t, KBT, D, 1.0);
    return bind_volume(T.A, T.c);
}

// prefact * ko_d[e] * Ke[e] * eps (Ke after readFromYaml's conversion):
// getBindingFactorSD of Protein/ProteinData.hpp:110-124 for free end e,
// bound head on a rod along dirBound, candidate rod along dirRod
double orc_kmc_binding_factor_sd(const AlensProteinType *t, int e, const double dirBound[3],
                                 const double dirRod[3]) {
    const bool par = dirRod[0] * dirBound[0] + dirRod[1] * dirBound[1] + dirRod[2] * dirBound[2] > 0.0;
    double pref = 1.0;
    if (par && t->PtoAPratio < 1.0)
        pref = t->PtoAPratio;
    else if (!par && t->PtoAPratio > 1.0)
        pref = 1.0 / t->PtoAPratio;
    double koD = t->ko_d[e];
    if (t->fixedEnd0 && e == 0) koD = 0.0;
    const double Ke = t->useBindVol ? t->Ke[e] / 602.0 : t->Ke[e];
    return pref * ((koD * Ke) * t->eps);
}

// the U->S capture radius, the S->D reach and the four per-step
// probabilities' coefficients of species t (for known-answer tests)
void orc_kmc_type_constants(const AlensProteinType *t, double KBT, double D, double dt, double out[12]) {
    const Kt T = make_type(*t, KBT, D, dt);
    const double v[12] = {T.rcap,      T.rOuter,    T.A,         T.w,         T.usCoef[0], T.usCoef[1],
                          T.suProb[0], T.suProb[1], T.sdCoef[0], T.sdCoef[1], T.koD[0],    T.koD[1]};
    std::memcpy(out, v, sizeof(v));
}

}  // extern "C"
