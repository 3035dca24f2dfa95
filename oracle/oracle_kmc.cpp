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
//     is above -36 (instead of the table), the binding point by inverting
//     the cumulative integral (panel search, then 60 bisections).
// Rolls: Philox4x32-10 with key = rngSeed and counter (gid, step,
// 0x6B6D6300 + block), a 53-bit uniform from the first two words of block 0.
//
// PARITY: the PtoAPratio known-answer test of Protein/ProteinTest.hpp:33-71
// pins the S->D binding factor.  The rest of the step (the KMC submodule's
// part) is UNPINNED: no golden outputs exist for it.
//
// Canonical arithmetic as in oracle.cpp: fixed evaluation order, no FMA
// contraction, IEEE +,-,*,/,sqrt and the project's own exp.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>

#include "oracle_ctx.h"

namespace {

constexpr double kPi = 3.141592653589793;
const double kX8[8] = {-0.9602898564975362, -0.7966664774136267, -0.525532409916329, -0.18343464249564978,
                       0.18343464249564978, 0.525532409916329,   0.7966664774136267, 0.9602898564975362};
const double kW8[8] = {0.10122853629037706, 0.22238103445337443, 0.3137066458778869, 0.36268378337836166,
                       0.36268378337836166, 0.3137066458778869,  0.22238103445337443, 0.10122853629037706};

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

// species constants (the same folding of dt as the library's table)
struct Kt {
    double ell0, c, A, w, rOuter, Ads, rcap, PtoAP;
    double usCoef[2], suProb[2], sdCoef[2], koD[2];
    double dt, kappa;
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
    T.c = in.freeLength + D;
    T.A = ((1.0 - in.lambda) * in.kappa) / (2.0 * KBT);
    T.w = 6.0 / std::sqrt(T.A);
    T.rOuter = T.c + T.w;
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
    return T;
}

double panel(double a, double b, double d2, double A, double c) {
    const double h = 0.5 * (b - a), m = 0.5 * (a + b);
    double acc = 0.0;
    for (int k = 0; k < 8; k++) {
        const double s = m + h * kX8[k];
        const double x = std::sqrt(d2 + s * s) - c;
        acc = acc + kW8[k] * kexp(-(A * (x * x)));
    }
    return h * acc;
}

int support(double d2, double sA, double sB, const Kt &T, double lo[2], double hi[2]) {
    const double ro2 = T.rOuter * T.rOuter;
    if (!(d2 < ro2)) return 0;
    const double sh = std::sqrt(ro2 - d2);
    const double ri = T.c - T.w;
    const double sl = (ri > 0.0 && ri * ri > d2) ? std::sqrt(ri * ri - d2) : 0.0;
    int n = 0;
    double l = sA > -sh ? sA : -sh, h = sB < -sl ? sB : -sl;
    if (h > l) {
        lo[n] = l;
        hi[n] = h;
        n++;
    }
    l = sA > sl ? sA : sl;
    h = sB < sh ? sB : sh;
    if (h > l) {
        lo[n] = l;
        hi[n] = h;
        n++;
    }
    return n;
}

int npanel(double len, double w) {
    const double q = std::ceil(len / (0.25 * w));
    return q < 1.0 ? 1 : (q > 64.0 ? 64 : (int)q);
}

double edge(double lo, double hi, int k, int n) { return k == n ? hi : lo + ((hi - lo) * (double)k) / (double)n; }

double sd_integral(double d2, double sA, double sB, const Kt &T) {
    double lo[2], hi[2];
    const int ni = support(d2, sA, sB, T, lo, hi);
    double Q = 0.0;
    for (int i = 0; i < ni; i++) {
        const int n = npanel(hi[i] - lo[i], T.w);
        double a = lo[i];
        for (int k = 1; k <= n; k++) {
            const double b = edge(lo[i], hi[i], k, n);
            Q = Q + panel(a, b, d2, T.A, T.c);
            a = b;
        }
    }
    return Q;
}

double sd_invert(double d2, double sA, double sB, const Kt &T, double target) {
    double lo[2], hi[2];
    const int ni = support(d2, sA, sB, T, lo, hi);
    double cum = 0.0, last = sA;
    for (int i = 0; i < ni; i++) {
        const int n = npanel(hi[i] - lo[i], T.w);
        double a = lo[i];
        for (int k = 1; k <= n; k++) {
            const double b = edge(lo[i], hi[i], k, n);
            const double P = panel(a, b, d2, T.A, T.c);
            if (target < cum + P) {
                const double t = target - cum;
                double x0 = a, x1 = b;
                for (int it = 0; it < 60; it++) {
                    const double xm = 0.5 * (x0 + x1);
                    if (panel(a, xm, d2, T.A, T.c) < t)
                        x0 = xm;
                    else
                        x1 = xm;
                }
                return 0.5 * (x0 + x1);
            }
            cum = cum + P;
            a = b;
            last = b;
        }
    }
    return last;
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

int choose(double p0, double p1, double *roll) {
    const double u = *roll;
    if (u < p0) return 0;
    if (u < p0 + p1) {
        *roll = u - p0;
        return 1;
    }
    return -1;
}

// the rod view of a binding step: wrapped centre, axis, half-length
struct RodView {
    std::vector<double> c, a, hl;
    std::vector<uint8_t> sphere;
};

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

struct Cand {
    int li;
    double v0, v1, v2, v3;
};

int pick(const std::vector<Cand> &C, double scale, double roll, double *frac) {
    double cum = 0.0;
    const int n = (int)C.size();
    for (int j = 0; j < n; j++) {
        const double pj = C[j].v0 * scale;
        const double nc = cum + pj;
        if (roll < nc || j == n - 1) {
            const double f = pj > 0.0 ? (roll - cum) / pj : 0.0;
            *frac = f < 0.0 ? 0.0 : (f > 1.0 ? 1.0 : f);
            return j;
        }
        cum = nc;
    }
    *frac = 0.0;
    return -1;
}

// one protein's binding step; returns the transition (0 none, 1 U->S,
// 2 S->U, 3 S->D, 4 D->S) and the number of candidate rods
int protein_step(const OrcCtx *x, const RodView &V, const Kt &T, AlensProtein &pr, int *ncand) {
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
    std::vector<Cand> C;
    if (nb == 0) {
        double X[3] = {pr.pos[0], pr.pos[1], pr.pos[2]};
        wrap_point(cf, X);
        pr.pos[0] = X[0];
        pr.pos[1] = X[1];
        pr.pos[2] = X[2];
        const double r2 = T.rcap * T.rcap;
        for (int r = 0; r < x->n; r++) {
            if (V.sphere[r]) continue;
            const double *c = &V.c[3 * r], *a = &V.a[3 * r];
            double u[3];
            for (int d = 0; d < 3; d++) u[d] = min_image(cf, d, X[d] - c[d]);
            const double t0 = u[0] * a[0] + u[1] * a[1] + u[2] * a[2];
            const double q0 = u[0] - t0 * a[0], q1 = u[1] - t0 * a[1], q2 = u[2] - t0 * a[2];
            const double d2 = q0 * q0 + q1 * q1 + q2 * q2;
            if (!(d2 < r2)) continue;
            const double hc = std::sqrt(r2 - d2);
            const double hl = V.hl[r];
            const double lo = -hl > t0 - hc ? -hl : t0 - hc;
            const double hi = hl < t0 + hc ? hl : t0 + hc;
            const double Lc = hi - lo;
            if (!(Lc > 0.0)) continue;
            C.push_back(Cand{r, Lc, lo, hl, 0.0});
        }
        double P0 = 0.0, P1 = 0.0;
        for (const Cand &k : C) P0 = P0 + k.v0 * T.usCoef[0];
        for (const Cand &k : C) P1 = P1 + k.v0 * T.usCoef[1];
        const int e = choose(P0, P1, &roll);
        if (e >= 0) {
            double frac;
            const int j = pick(C, T.usCoef[e], roll, &frac);
            double s = C[j].v1 + frac * C[j].v0;
            s = s > C[j].v2 ? C[j].v2 : s;
            s = s < -C[j].v2 ? -C[j].v2 : s;
            pr.idBind[e] = C[j].li;
            pr.distBind[e] = s;
            trans = 1;
        }
    } else if (nb == 1) {
        const int b = pr.idBind[0] >= 0 ? 0 : 1, f = 1 - b;
        double X[3] = {P[b][0], P[b][1], P[b][2]};
        wrap_point(cf, X);
        const double ro2 = T.rOuter * T.rOuter;
        const double *ab = &V.a[3 * pr.idBind[b]];
        for (int r = 0; r < x->n; r++) {
            if (r == pr.idBind[b] || V.sphere[r]) continue;
            const double *c = &V.c[3 * r], *a = &V.a[3 * r];
            double u[3];
            for (int d = 0; d < 3; d++) u[d] = min_image(cf, d, X[d] - c[d]);
            const double t0 = u[0] * a[0] + u[1] * a[1] + u[2] * a[2];
            const double q0 = u[0] - t0 * a[0], q1 = u[1] - t0 * a[1], q2 = u[2] - t0 * a[2];
            const double d2 = q0 * q0 + q1 * q1 + q2 * q2;
            if (!(d2 < ro2)) continue;
            const double hl = V.hl[r];
            const double I = sd_integral(d2, -hl - t0, hl - t0, T);
            if (!(I > 0.0)) continue;
            // Protein/ProteinData.hpp:110-124: parallel when the axes' dot
            // product is positive; the prefactor never exceeds 1
            const bool par = a[0] * ab[0] + a[1] * ab[1] + a[2] * ab[2] > 0.0;
            double pref = 1.0;
            if (par && T.PtoAP < 1.0)
                pref = T.PtoAP;
            else if (!par && T.PtoAP > 1.0)
                pref = 1.0 / T.PtoAP;
            C.push_back(Cand{r, (pref * T.sdCoef[f]) * I, t0, d2, I});
        }
        double Pb = 0.0;
        for (const Cand &k : C) Pb = Pb + k.v0;
        const double pU = T.suProb[b];
        const int e = choose(b == 0 ? pU : Pb, b == 0 ? Pb : pU, &roll);
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
            double frac;
            const int j = pick(C, 1.0, roll, &frac);
            const int r = C[j].li;
            const double hl = V.hl[r];
            const double t0 = C[j].v1;
            const double sStar = sd_invert(C[j].v2, -hl - t0, hl - t0, T, frac * C[j].v3);
            double s = t0 + sStar;
            s = s > hl ? hl : s;
            s = s < -hl ? -hl : s;
            pr.idBind[f] = r;
            pr.distBind[f] = s;
            trans = 3;
        }
    } else {
        double dv[3];
        for (int d = 0; d < 3; d++) dv[d] = min_image(cf, d, P[1][d] - P[0][d]);
        const double ell = std::sqrt(dv[0] * dv[0] + dv[1] * dv[1] + dv[2] * dv[2]);
        const double xx = (ell - x->kmcD) - T.ell0;
        const double M = T.Ads * (xx * xx);
        const double g = kexp(M);
        const double p0 = (T.koD[0] * g) * T.dt, p1 = (T.koD[1] * g) * T.dt;
        const int e = choose(p0, p1, &roll);
        if (e >= 0) {
            pr.idBind[e] = -1;
            trans = 4;
        }
    }
    *ncand = (int)C.size();
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

bool nonneg(double v) { return std::isfinite(v) && v >= 0.0; }

bool type_ok(const AlensProteinType &p) {
    bool ok = p.lookupType == 0 && std::isfinite(p.kappa) && p.kappa > 0.0 && std::isfinite(p.lambda) &&
              p.lambda >= 0.0 && p.lambda < 1.0 && nonneg(p.freeLength) && std::isfinite(p.rc) && p.rc > 0.0 &&
              nonneg(p.eps) && nonneg(p.diffUnbound) && std::isfinite(p.PtoAPratio) && p.PtoAPratio > 0.0;
    for (int e = 0; e < 2; e++)
        ok = ok && nonneg(p.ko_s[e]) && nonneg(p.ko_d[e]) && nonneg(p.Ka[e]) && nonneg(p.Ke[e]);
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
    for (const AlensProtein &p : x->prot) {
        if (p.idBind[0] < 0 || p.idBind[0] >= x->n || p.idBind[1] < 0 || p.idBind[1] >= x->n) continue;
        const AlensProteinType &t = x->ptypes[p.type];
        x->springI.push_back(p.idBind[0]);
        x->springJ.push_back(p.idBind[1]);
        x->springSI.push_back(p.distBind[0]);
        x->springSJ.push_back(p.distBind[1]);
        x->springRest.push_back(t.freeLength + x->kmcD);
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
        const RodView V = rod_view(x);
        std::vector<Kt> T;
        for (const AlensProteinType &t : x->ptypes) T.push_back(make_type(t, x->kmcKBT, x->kmcD, x->cfg.dt));
        const int np = (int)x->prot.size();
        std::vector<int> trans(np), nc(np);
#pragma omp parallel for schedule(dynamic, 64)
        for (int p = 0; p < np; p++) trans[p] = protein_step(x, V, T[x->prot[p].type], x->prot[p], &nc[p]);
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
    if (st) *st = s;
    return ALENS_OK;
}

double orc_kmc_exp(double x) { return kexp(x); }

double orc_kmc_sd_integral(const AlensProteinType *t, double KBT, double D, double dt, double d2, double sA,
                           double sB) {
    return sd_integral(d2, sA, sB, make_type(*t, KBT, D, dt));
}

double orc_kmc_sd_invert(const AlensProteinType *t, double KBT, double D, double dt, double d2, double sA,
                         double sB, double target) {
    return sd_invert(d2, sA, sB, make_type(*t, KBT, D, dt), target);
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
