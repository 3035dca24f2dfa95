// kernels_kmc.cu - the protein binding step of the two-stage KMC model on
// the device: one thread per protein.
//
// What it computes (Protein/ProteinModel.md, "The Binding/Unbinding
// probabilities and rates in KMC"; step structure of
// SRC/CalcProteinBind.hpp:59-173 and SRC/kmc_step_funcs.hpp:35-230):
//   U (no head bound): each rod within the capture radius rcap of the
//     protein offers P_j = L_c,j (3 Ka ε ko_s / (4 π rcap³)) dt per head,
//     L_c,j the length of the rod's axis inside the capture sphere; the
//     head and rod are drawn from the roll, the binding point uniformly on
//     that chord.
//   S (one head bound at P on rod b): unbinding with ko_s dt, or binding of
//     the free head to a rod j ≠ b with
//       P_j = prefact_j ko_d Ke ε dt ∫ exp(-A (sqrt(d² + s²) - ell0 - D)²) ds
//     (divided by the bind volume Vb when useBindVol), A = (1 - λ) κ / (2 kT),
//     d the distance of P from rod j's axis, s the arc coordinate from the
//     foot of P over rod j; prefact_j from PtoAPratio by the sign of
//     a_j · a_b (Protein/ProteinData.hpp:110-124); the binding point is
//     drawn from the integrand (inverse of the cumulative integral).  On
//     unbinding the protein is released uniformly in the capture sphere
//     around P.
//   D (both bound): each head unbinds with ko_d exp(λ κ (ℓ - D - ell0)² /
//     (2 kT)) dt, ℓ the head distance (Protein/ProteinData.hpp:132-140).
// The event is chosen as in the reference: the two heads' probabilities
// are stacked in head order on [0, 1) and one uniform roll picks a head
// (or nothing); within the head the same roll, shifted, picks the rod in
// ascending rod order and then the point.
//
// The reference tabulates the S->D integral in a lookup table (KMC
// submodule, absent from the checkout).  Here it is evaluated by composite
// 8-point Gauss-Legendre quadrature over the integrand's support: head
// distances within w = 6/sqrt(A) of ell0 + D (outside, the integrand is
// below e^-36), split into at most two arcs and into panels of w/4.
//
// Arithmetic: FP64 with IEEE +,-,*,/,sqrt only (no FMA contraction: this
// file is compiled with --fmad=false), the project's own exp (Cody-Waite
// reduction by ln 2, Taylor polynomial to r^13), Philox4x32-10 rolls keyed
// by (seed, protein gid, step).  The CPU oracle states the same operations,
// so both produce the same protein states bit for bit.
#include "kmc.cuh"

namespace alens {
namespace {

// Gauss-Legendre on [-1, 1], 8 points: roots of P_8 and their weights
__constant__ double kGLx[8] = {-0.9602898564975362, -0.7966664774136267, -0.525532409916329,
                               -0.18343464249564978, 0.18343464249564978, 0.525532409916329,
                               0.7966664774136267,  0.9602898564975362};
__constant__ double kGLw[8] = {0.10122853629037706, 0.22238103445337443, 0.3137066458778869,
                               0.36268378337836166, 0.36268378337836166, 0.3137066458778869,
                               0.22238103445337443, 0.10122853629037706};

// e^x: x = k ln2 + r, |r| <= ln2/2, ln2 split into a 24-bit head (k ln2_hi
// exact) and the tail; e^r by its Taylor polynomial to r^13 (remainder
// below 4e-18); scaling by 2^k in at most two exact steps.
__device__ double kmc_exp(double x) {
    if (!(x == x)) return x;
    if (x > 709.78) return __longlong_as_double(0x7ff0000000000000LL);
    if (x < -745.2) return 0.0;
    const double k = floor(x * 1.4426950408889634 + 0.5);
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
    return p * __longlong_as_double((long long)(ki + 1023) << 52);
}

__device__ __forceinline__ double dmax(double a, double b) { return a > b ? a : b; }
__device__ __forceinline__ double dmin(double a, double b) { return a < b ? a : b; }

// one Gauss-Legendre panel of the S->D integrand over s in [a, b]
__device__ double sd_panel(double a, double b, double d2, double A, double c) {
    const double h = 0.5 * (b - a), m = 0.5 * (a + b);
    double acc = 0.0;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        const double s = m + h * kGLx[k];
        const double x = sqrt(d2 + s * s) - c;
        acc = acc + kGLw[k] * kmc_exp(-(A * (x * x)));
    }
    return h * acc;
}

// the integrand's support within [sA, sB]: |s| in [sl, sh], at most two arcs
__device__ int sd_support(double d2, double sA, double sB, const KmcType &T, double lo[2], double hi[2]) {
    const double ro2 = T.rOuter * T.rOuter;
    if (!(d2 < ro2)) return 0;
    const double sh = sqrt(ro2 - d2);
    const double ri = T.c - T.w;
    const double sl = (ri > 0.0 && ri * ri > d2) ? sqrt(ri * ri - d2) : 0.0;
    int n = 0;
    double l = dmax(sA, -sh), h = dmin(sB, -sl);
    if (h > l) {
        lo[n] = l;
        hi[n] = h;
        n++;
    }
    l = dmax(sA, sl);
    h = dmin(sB, sh);
    if (h > l) {
        lo[n] = l;
        hi[n] = h;
        n++;
    }
    return n;
}

__device__ __forceinline__ int sd_npanel(double len, double w) {
    const double q = ceil(len / (0.25 * w));
    return q < 1.0 ? 1 : (q > 64.0 ? 64 : (int)q);
}

__device__ __forceinline__ double sd_edge(double lo, double hi, int k, int n) {
    return k == n ? hi : lo + ((hi - lo) * (double)k) / (double)n;
}

__device__ double sd_integral(double d2, double sA, double sB, const KmcType &T) {
    double lo[2], hi[2];
    const int ni = sd_support(d2, sA, sB, T, lo, hi);
    double Q = 0.0;
    for (int i = 0; i < ni; i++) {
        const int n = sd_npanel(hi[i] - lo[i], T.w);
        double a = lo[i];
        for (int k = 1; k <= n; k++) {
            const double b = sd_edge(lo[i], hi[i], k, n);
            Q = Q + sd_panel(a, b, d2, T.A, T.c);
            a = b;
        }
    }
    return Q;
}

// the s at which the integral from the support start reaches target
// (0 <= target < the full integral): panel by the running sum, then 60
// bisections of the panel's partial integral
__device__ double sd_invert(double d2, double sA, double sB, const KmcType &T, double target) {
    double lo[2], hi[2];
    const int ni = sd_support(d2, sA, sB, T, lo, hi);
    double cum = 0.0, last = sA;
    for (int i = 0; i < ni; i++) {
        const int n = sd_npanel(hi[i] - lo[i], T.w);
        double a = lo[i];
        for (int k = 1; k <= n; k++) {
            const double b = sd_edge(lo[i], hi[i], k, n);
            const double P = sd_panel(a, b, d2, T.A, T.c);
            if (target < cum + P) {
                const double t = target - cum;
                double x0 = a, x1 = b;
                for (int it = 0; it < 60; it++) {
                    const double xm = 0.5 * (x0 + x1);
                    if (sd_panel(a, xm, d2, T.A, T.c) < t)
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

// Philox block b of protein gid at step: counter (gid, step, 'kmc' + b)
__device__ __forceinline__ void kmc_words(unsigned long long seed, long long gid, long long step, uint32_t b,
                                          uint32_t w[4]) {
    w[0] = (uint32_t)(unsigned long long)gid;
    w[1] = (uint32_t)((unsigned long long)gid >> 32);
    w[2] = (uint32_t)(unsigned long long)step;
    w[3] = 0x6B6D6300u + b;
    philox4x32_10(w, (uint32_t)seed, (uint32_t)(seed >> 32));
}

// uniform in [0, 1) with 53 random bits
__device__ __forceinline__ double u53(uint32_t hi, uint32_t lo) {
    return ((double)(hi >> 5) * 67108864.0 + (double)(lo >> 6)) * (1.0 / 9007199254740992.0);
}

// one head (0 or 1) or none (-1) from two stacked probabilities; the roll
// is shifted to the chosen head's interval
__device__ __forceinline__ int kmc_choose(double p0, double p1, double *roll) {
    const double u = *roll;
    if (u < p0) return 0;
    if (u < p0 + p1) {
        *roll = u - p0;
        return 1;
    }
    return -1;
}

__device__ __forceinline__ int kmc_cell_coord(double v, double lo, double cs, int n) {
    const double f = floor((v - lo) / cs);
    return f < 0.0 ? 0 : (f > (double)(n - 1) ? n - 1 : (int)f);
}

__device__ __forceinline__ double kmc_wrap(double v, double lo, double hi, double L) {
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

__device__ __forceinline__ void kmc_wrap_point(const KmcRep &Q, double p[3]) {
    for (int d = 0; d < 3; d++)
        if (Q.pbc[d]) p[d] = kmc_wrap(p[d], Q.lo[d], Q.hi[d], Q.L[d]);
}

// x - c reduced to the minimum image
__device__ __forceinline__ void kmc_rel(const KmcRep &Q, const double x[3], const double4 &c, double u[3]) {
    u[0] = x[0] - c.x;
    u[1] = x[1] - c.y;
    u[2] = x[2] - c.z;
    for (int d = 0; d < 3; d++)
        if (Q.pbc[d]) u[d] = u[d] - Q.L[d] * floor(u[d] / Q.L[d] + 0.5);
}

// the distinct cells of the 3x3x3 stencil around cell c
template <class F>
__device__ void kmc_for_cells(const KmcRep &Q, const int c[3], F &&f) {
    int lo[3], hi[3];
    for (int d = 0; d < 3; d++) {
        const int n = Q.ncell[d];
        if (Q.pbc[d]) {
            lo[d] = n >= 3 ? -1 : 0;
            hi[d] = n >= 3 ? 1 : n - 1;
        } else {
            lo[d] = c[d] > 0 ? -1 : 0;
            hi[d] = c[d] < n - 1 ? 1 : 0;
        }
    }
    for (int dz = lo[2]; dz <= hi[2]; dz++)
        for (int dy = lo[1]; dy <= hi[1]; dy++)
            for (int dx = lo[0]; dx <= hi[0]; dx++) {
                int cc[3] = {c[0] + dx, c[1] + dy, c[2] + dz};
                for (int d = 0; d < 3; d++)
                    if (Q.pbc[d]) cc[d] = (cc[d] + Q.ncell[d]) % Q.ncell[d];
                f(Q.cellOffset + (cc[2] * Q.ncell[1] + cc[1]) * Q.ncell[0] + cc[0]);
            }
}

__device__ __forceinline__ double qnan() { return __longlong_as_double(0x7ff8000000000000LL); }

// rod view and cell counts
__global__ void k_kmc_bin(KmcDev K, DevState S) {
    ALENS_PDL_PROLOGUE();
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < S.nRods; r += gridDim.x * blockDim.x) {
        const KmcRep &Q = K.rep[S.rodRep[r]];
        double p[3] = {S.px[r], S.py[r], S.pz[r]};
        kmc_wrap_point(Q, p);
        double a[3];
        quat_axis(S.qx[r], S.qy[r], S.qz[r], S.qw[r], a);
        const double L = S.len[r];
        const bool sphere = L < 2.0 * S.rad[r];
        K.rodC[r] = make_double4(p[0], p[1], p[2], 0.5 * L);
        K.rodA[r] = make_double4(a[0], a[1], a[2], sphere ? 1.0 : 0.0);
        int c[3];
        for (int d = 0; d < 3; d++) c[d] = kmc_cell_coord(p[d], Q.lo[d], Q.cellsz[d], Q.ncell[d]);
        atomicAdd(&K.cellCount[Q.cellOffset + (c[2] * Q.ncell[1] + c[1]) * Q.ncell[0] + c[0]], 1);
    }
}

__global__ void k_kmc_scatter(KmcDev K, DevState S) {
    ALENS_PDL_PROLOGUE();
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < S.nRods; r += gridDim.x * blockDim.x) {
        const KmcRep &Q = K.rep[S.rodRep[r]];
        const double4 C = K.rodC[r];
        const double p[3] = {C.x, C.y, C.z};
        int c[3];
        for (int d = 0; d < 3; d++) c[d] = kmc_cell_coord(p[d], Q.lo[d], Q.cellsz[d], Q.ncell[d]);
        const int cid = Q.cellOffset + (c[2] * Q.ncell[1] + c[1]) * Q.ncell[0] + c[0];
        K.cellRod[K.cellStart[cid] + atomicAdd(&K.cellCursor[cid], 1)] = r;
    }
}

// candidate list of one protein, ascending local rod index
struct KmcCands {
    int n;
    bool overflow;
    int li[kKmcMaxCand];
    double v0[kKmcMaxCand], v1[kKmcMaxCand], v2[kKmcMaxCand], v3[kKmcMaxCand];

    __device__ void insert(int l, double a, double b, double c, double d) {
        if (n == kKmcMaxCand) {
            overflow = true;
            return;
        }
        int k = n;
        while (k > 0 && li[k - 1] > l) {
            li[k] = li[k - 1];
            v0[k] = v0[k - 1];
            v1[k] = v1[k - 1];
            v2[k] = v2[k - 1];
            v3[k] = v3[k - 1];
            k--;
        }
        li[k] = l;
        v0[k] = a;
        v1[k] = b;
        v2[k] = c;
        v3[k] = d;
        n++;
    }
};

// the candidate j whose slice of the stacked probabilities p[] (times
// scale) holds roll, and the roll's fraction within that slice
__device__ int kmc_pick(const KmcCands &C, const double *p, double scale, double roll, double *frac) {
    double cum = 0.0;
    for (int j = 0; j < C.n; j++) {
        const double pj = p[j] * scale;
        const double nc = cum + pj;
        if (roll < nc || j == C.n - 1) {
            double f = pj > 0.0 ? (roll - cum) / pj : 0.0;
            *frac = f < 0.0 ? 0.0 : (f > 1.0 ? 1.0 : f);
            return j;
        }
        cum = nc;
    }
    *frac = 0.0;
    return -1;
}

// code per protein: final stage (bits 0-1), transition + 1 (bits 2-4:
// 1 U->S, 2 S->U, 3 S->D, 4 D->S), candidates (bits 8-)
__global__ void __launch_bounds__(128) k_kmc_bind(KmcDev K, int *code) {
    ALENS_PDL_PROLOGUE();
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < K.nProt; p += gridDim.x * blockDim.x) {
        AlensProtein pr = K.prot[p];
        const KmcRep &Q = K.rep[K.protRep[p]];
        const KmcType &T = K.types[K.protRep[p] * K.nTypes + pr.type];
        // an end bound to a rod the replica no longer holds is released
        // (the reference releases an end whose rod it cannot find)
        for (int e = 0; e < 2; e++)
            if (pr.idBind[e] < 0 || pr.idBind[e] >= Q.nRods) pr.idBind[e] = -1;
        double4 Cb[2], Ab[2];
        double P[2][3];
        for (int e = 0; e < 2; e++) {
            if (pr.idBind[e] < 0) continue;
            const int r = Q.rodOffset + pr.idBind[e];
            Cb[e] = K.rodC[r];
            Ab[e] = K.rodA[r];
            P[e][0] = Cb[e].x + pr.distBind[e] * Ab[e].x;
            P[e][1] = Cb[e].y + pr.distBind[e] * Ab[e].y;
            P[e][2] = Cb[e].z + pr.distBind[e] * Ab[e].z;
        }
        const int nb = (pr.idBind[0] >= 0 ? 1 : 0) + (pr.idBind[1] >= 0 ? 1 : 0);
        uint32_t w[4];
        kmc_words(Q.seed, pr.gid, K.step, 0, w);
        double roll = u53(w[0], w[1]);
        int trans = 0, ncand = 0;
        bool overflow = false;
        KmcCands C;
        C.n = 0;
        C.overflow = false;
        if (nb == 0) {
            double X[3] = {pr.pos[0], pr.pos[1], pr.pos[2]};
            kmc_wrap_point(Q, X);
            pr.pos[0] = X[0];
            pr.pos[1] = X[1];
            pr.pos[2] = X[2];
            const double r2 = T.rcap * T.rcap;
            int c[3];
            for (int d = 0; d < 3; d++) c[d] = kmc_cell_coord(X[d], Q.lo[d], Q.cellsz[d], Q.ncell[d]);
            kmc_for_cells(Q, c, [&](int cid) {
                for (int s = K.cellStart[cid]; s < K.cellStart[cid + 1]; s++) {
                    const int r = K.cellRod[s];
                    const double4 Cr = K.rodC[r], Ar = K.rodA[r];
                    if (Ar.w != 0.0) continue;
                    double u[3];
                    kmc_rel(Q, X, Cr, u);
                    const double t0 = u[0] * Ar.x + u[1] * Ar.y + u[2] * Ar.z;
                    const double q0 = u[0] - t0 * Ar.x, q1 = u[1] - t0 * Ar.y, q2 = u[2] - t0 * Ar.z;
                    const double d2 = q0 * q0 + q1 * q1 + q2 * q2;
                    if (!(d2 < r2)) continue;
                    const double hc = sqrt(r2 - d2);
                    const double lo = dmax(-Cr.w, t0 - hc), hi = dmin(Cr.w, t0 + hc);
                    const double Lc = hi - lo;
                    if (!(Lc > 0.0)) continue;
                    C.insert(r - Q.rodOffset, Lc, lo, Cr.w, 0.0);
                }
            });
            ncand = C.n;
            overflow = C.overflow;
            if (!overflow) {
                double P0 = 0.0, P1 = 0.0;
                for (int j = 0; j < C.n; j++) P0 = P0 + C.v0[j] * T.usCoef[0];
                for (int j = 0; j < C.n; j++) P1 = P1 + C.v0[j] * T.usCoef[1];
                const int e = kmc_choose(P0, P1, &roll);
                if (e >= 0) {
                    double frac;
                    const int j = kmc_pick(C, C.v0, T.usCoef[e], roll, &frac);
                    double s = C.v1[j] + frac * C.v0[j];
                    s = dmax(-C.v2[j], dmin(C.v2[j], s));
                    pr.idBind[e] = C.li[j];
                    pr.distBind[e] = s;
                    trans = 1;
                }
            }
        } else if (nb == 1) {
            const int b = pr.idBind[0] >= 0 ? 0 : 1, f = 1 - b;
            double X[3] = {P[b][0], P[b][1], P[b][2]};
            kmc_wrap_point(Q, X);
            const double ro2 = T.rOuter * T.rOuter;
            const double4 Abb = Ab[b];
            int c[3];
            for (int d = 0; d < 3; d++) c[d] = kmc_cell_coord(X[d], Q.lo[d], Q.cellsz[d], Q.ncell[d]);
            kmc_for_cells(Q, c, [&](int cid) {
                for (int s = K.cellStart[cid]; s < K.cellStart[cid + 1]; s++) {
                    const int r = K.cellRod[s];
                    if (r - Q.rodOffset == pr.idBind[b]) continue;
                    const double4 Cr = K.rodC[r], Ar = K.rodA[r];
                    if (Ar.w != 0.0) continue;
                    double u[3];
                    kmc_rel(Q, X, Cr, u);
                    const double t0 = u[0] * Ar.x + u[1] * Ar.y + u[2] * Ar.z;
                    const double q0 = u[0] - t0 * Ar.x, q1 = u[1] - t0 * Ar.y, q2 = u[2] - t0 * Ar.z;
                    const double d2 = q0 * q0 + q1 * q1 + q2 * q2;
                    if (!(d2 < ro2)) continue;
                    const double I = sd_integral(d2, -Cr.w - t0, Cr.w - t0, T);
                    if (!(I > 0.0)) continue;
                    const bool par = Ar.x * Abb.x + Ar.y * Abb.y + Ar.z * Abb.z > 0.0;
                    double pref = 1.0;
                    if (par && T.PtoAP < 1.0)
                        pref = T.PtoAP;
                    else if (!par && T.PtoAP > 1.0)
                        pref = 1.0 / T.PtoAP;
                    C.insert(r - Q.rodOffset, (pref * T.sdCoef[f]) * I, t0, d2, I);
                }
            });
            ncand = C.n;
            overflow = C.overflow;
            if (!overflow) {
                double Pb = 0.0;
                for (int j = 0; j < C.n; j++) Pb = Pb + C.v0[j];
                const double pU = T.suProb[b];
                const int e = kmc_choose(b == 0 ? pU : Pb, b == 0 ? Pb : pU, &roll);
                if (e == b) {
                    // released uniformly in the capture sphere around the head
                    double off[3] = {0.0, 0.0, 0.0};
                    for (uint32_t k = 0; k < 32; k++) {
                        uint32_t v[4];
                        kmc_words(Q.seed, pr.gid, K.step, 2 + k, v);
                        const double x = 2.0 * (((double)v[0] + 0.5) * 2.3283064365386963e-10) - 1.0;
                        const double y = 2.0 * (((double)v[1] + 0.5) * 2.3283064365386963e-10) - 1.0;
                        const double z = 2.0 * (((double)v[2] + 0.5) * 2.3283064365386963e-10) - 1.0;
                        if ((x * x + y * y) + z * z <= 1.0) {
                            off[0] = x;
                            off[1] = y;
                            off[2] = z;
                            break;
                        }
                    }
                    pr.pos[0] = P[b][0] + T.rcap * off[0];
                    pr.pos[1] = P[b][1] + T.rcap * off[1];
                    pr.pos[2] = P[b][2] + T.rcap * off[2];
                    pr.idBind[b] = -1;
                    trans = 2;
                } else if (e == f) {
                    double frac;
                    const int j = kmc_pick(C, C.v0, 1.0, roll, &frac);
                    const int r = Q.rodOffset + C.li[j];
                    const double hl = K.rodC[r].w;
                    const double t0 = C.v1[j];
                    const double sStar = sd_invert(C.v2[j], -hl - t0, hl - t0, T, frac * C.v3[j]);
                    pr.idBind[f] = C.li[j];
                    pr.distBind[f] = dmax(-hl, dmin(hl, t0 + sStar));
                    trans = 3;
                }
            }
        } else {
            double dv[3] = {P[1][0] - P[0][0], P[1][1] - P[0][1], P[1][2] - P[0][2]};
            for (int d = 0; d < 3; d++)
                if (Q.pbc[d]) dv[d] = dv[d] - Q.L[d] * floor(dv[d] / Q.L[d] + 0.5);
            const double ell = sqrt(dv[0] * dv[0] + dv[1] * dv[1] + dv[2] * dv[2]);
            const double x = (ell - K.D) - T.ell0;
            const double M = T.Ads * (x * x);
            const double g = kmc_exp(M);
            const double p0 = (T.koD[0] * g) * T.dt, p1 = (T.koD[1] * g) * T.dt;
            const int e = kmc_choose(p0, p1, &roll);
            if (e >= 0) {
                pr.idBind[e] = -1;
                trans = 4;
            }
        }
        if (overflow) atomicOr(K.err, kKmcErrCand);
        // the new geometry
        for (int e = 0; e < 2; e++) {
            if (pr.idBind[e] < 0) {
                pr.distBind[e] = qnan();
                pr.posEnd[e][0] = pr.posEnd[e][1] = pr.posEnd[e][2] = qnan();
                continue;
            }
            const int r = Q.rodOffset + pr.idBind[e];
            const double4 Cr = K.rodC[r], Ar = K.rodA[r];
            pr.posEnd[e][0] = Cr.x + pr.distBind[e] * Ar.x;
            pr.posEnd[e][1] = Cr.y + pr.distBind[e] * Ar.y;
            pr.posEnd[e][2] = Cr.z + pr.distBind[e] * Ar.z;
        }
        const int nb2 = (pr.idBind[0] >= 0 ? 1 : 0) + (pr.idBind[1] >= 0 ? 1 : 0);
        if (nb2 == 1) {
            const int b = pr.idBind[0] >= 0 ? 0 : 1;
            pr.pos[0] = pr.posEnd[b][0];
            pr.pos[1] = pr.posEnd[b][1];
            pr.pos[2] = pr.posEnd[b][2];
        } else if (nb2 == 2) {
            double dv[3];
            for (int d = 0; d < 3; d++) {
                dv[d] = pr.posEnd[1][d] - pr.posEnd[0][d];
                if (Q.pbc[d]) dv[d] = dv[d] - Q.L[d] * floor(dv[d] / Q.L[d] + 0.5);
                pr.pos[d] = pr.posEnd[0][d] + 0.5 * dv[d];
            }
        }
        double X[3] = {pr.pos[0], pr.pos[1], pr.pos[2]};
        kmc_wrap_point(Q, X);
        pr.pos[0] = X[0];
        pr.pos[1] = X[1];
        pr.pos[2] = X[2];
        K.prot[p] = pr;
        code[p] = nb2 | (trans << 2) | (ncand << 8);
    }
}

// per replica: stage counts, transitions and the most candidates
__global__ void __launch_bounds__(256) k_kmc_stats(KmcDev K, const int *code) {
    ALENS_PDL_PROLOGUE();
    __shared__ int cnt[8];
    if (threadIdx.x < 8) cnt[threadIdx.x] = 0;
    __syncthreads();
    const KmcRep &Q = K.rep[blockIdx.x];
    int loc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int i = threadIdx.x; i < Q.nProt; i += blockDim.x) {
        const int c = code[Q.protOffset + i];
        loc[c & 3]++;
        const int t = (c >> 2) & 7;
        if (t > 0) loc[2 + t]++;
        loc[7] = max(loc[7], c >> 8);
    }
    for (int k = 0; k < 7; k++)
        if (loc[k]) atomicAdd(&cnt[k], loc[k]);
    atomicMax(&cnt[7], loc[7]);
    __syncthreads();
    if (threadIdx.x < 8) K.stats[8 * blockIdx.x + threadIdx.x] = cnt[threadIdx.x];
}

__global__ void k_kmc_dflag(KmcDev K) {
    ALENS_PDL_PROLOGUE();
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p <= K.nProt; p += gridDim.x * blockDim.x) {
        if (p == K.nProt) {
            K.dFlag[p] = 0;
            continue;
        }
        const AlensProtein &pr = K.prot[p];
        const KmcRep &Q = K.rep[K.protRep[p]];
        const bool d = pr.idBind[0] >= 0 && pr.idBind[0] < Q.nRods && pr.idBind[1] >= 0 && pr.idBind[1] < Q.nRods;
        K.dFlag[p] = d ? 1 : 0;
    }
}

// the doubly bound proteins as link rows (after the alens_set_links rows):
// anchors at distBind on the two rods, rest length ell0 + D, stiffness
// kappa; the link-block kernel turns them into bilateral blocks each step
// (the ConstraintBlock of SRC/TubuleSystem.cpp:706-736)
__global__ void k_kmc_springs(KmcDev K, DevState S, int userTotal, int linkCap) {
    ALENS_PDL_PROLOGUE();
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < K.nProt; p += gridDim.x * blockDim.x) {
        if (!K.dFlag[p]) continue;
        const int rep = K.protRep[p];
        const KmcRep &Q = K.rep[rep];
        const AlensProtein &pr = K.prot[p];
        const KmcType &T = K.types[rep * K.nTypes + pr.type];
        const int L = userTotal + K.dScan[p];
        if (L >= linkCap) {
            atomicOr(K.err, kKmcErrSpring);
            continue;
        }
        S.linkI[L] = Q.rodOffset + pr.idBind[0];
        S.linkJ[L] = Q.rodOffset + pr.idBind[1];
        S.linkRep[L] = rep;
        S.linkLocal[L] = Q.userLinks + (K.dScan[p] - K.dScan[Q.protOffset]);
        S.linkSI[L] = pr.distBind[0];
        S.linkSJ[L] = pr.distBind[1];
        S.linkRest[L] = T.c;
        S.linkKappa[L] = T.kappa;
    }
}

__global__ void k_kmc_dcount(KmcDev K) {
    ALENS_PDL_PROLOGUE();
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < K.R; r += gridDim.x * blockDim.x) {
        const KmcRep &Q = K.rep[r];
        K.dCount[r] = K.dScan[Q.protOffset + Q.nProt] - K.dScan[Q.protOffset];
    }
}

int grid_kmc(int n, int threads) {
    static int sms = 0;
    if (sms == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
    }
    const long long b = ((long long)n + threads - 1) / threads;
    const long long cap = 32LL * sms;
    return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

}  // namespace

void launch_kmc_bin(const KmcDev &K, const DevState &S, cudaStream_t st) {
    launch_pdl(k_kmc_bin, dim3(grid_kmc(S.nRods, 256)), dim3(256), 0, st, K, S);
}

void launch_kmc_scatter(const KmcDev &K, const DevState &S, cudaStream_t st) {
    launch_pdl(k_kmc_scatter, dim3(grid_kmc(S.nRods, 256)), dim3(256), 0, st, K, S);
}

// code[] reuses the doubly bound flags' buffer, which the springs pass
// rewrites afterwards
void launch_kmc_bind(const KmcDev &K, cudaStream_t st) {
    if (K.nProt <= 0) return;
    launch_pdl(k_kmc_bind, dim3(grid_kmc(K.nProt, 128)), dim3(128), 0, st, K, K.dScan);
    launch_pdl(k_kmc_stats, dim3(K.R), dim3(256), 0, st, K, (const int *)K.dScan);
}

int launch_kmc_springs(const KmcDev &K, const DevState &S, int userTotal, int linkCap, cudaStream_t st) {
    int n = 0;
    launch_pdl(k_kmc_dflag, dim3(grid_kmc(K.nProt + 1, 256)), dim3(256), 0, st, K);
    n += 1 + launch_scan(K.dFlag, K.dScan, K.nProt + 1, S.scanTmp, st);
    if (K.nProt > 0) {
        launch_pdl(k_kmc_springs, dim3(grid_kmc(K.nProt, 256)), dim3(256), 0, st, K, S, userTotal, linkCap);
        n++;
    }
    launch_pdl(k_kmc_dcount, dim3(1), dim3(64), 0, st, K);
    return n + 1;
}

}  // namespace alens
