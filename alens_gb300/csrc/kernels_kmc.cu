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
// below e^-36), split into at most two arcs and into panels of w/4; the
// integrand in FP32 (relative error of the integral ~1e-6, against ~1e-3
// for a 256 x 256 table), edges, sums and probabilities in FP64.
//
// Arithmetic: IEEE +,-,*,/,sqrt only (no FMA contraction: this file is
// compiled with --fmad=false) and the project's own exp in FP64 and FP32
// (Cody-Waite reduction by ln 2, Taylor polynomials to r^13 / r^8),
// Philox4x32-10 rolls keyed by (seed, protein gid, step).  The CPU oracle states the same operations,
// so both produce the same protein states bit for bit.
#include "kmc.cuh"

namespace alens {
namespace {

// Gauss-Legendre on [-1, 1], 8 points: roots of P_8 and their weights,
// rounded to FP32
__constant__ float kGLx[8] = {
    -0.9602898359298706f, -0.7966665029525757f, -0.5255324244499207f, -0.1834346354007721f,
    0.1834346354007721f,  0.5255324244499207f,  0.7966665029525757f,  0.9602898359298706f};
__constant__ float kGLw[8] = {
    0.10122853517532349f, 0.22238104045391083f, 0.313706636428833f, 0.3626837730407715f,
    0.3626837730407715f,  0.313706636428833f,   0.22238104045391083f, 0.10122853517532349f};

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

// FP32 e^x for the S->D integrand: the same reduction with ln2 split into
// 0.693145751953125 (15 significant bits, k ln2_hi exact for |k| < 2^9) and
// its tail, Taylor polynomial to r^8 (remainder below 3e-10); results below
// e^-87 flush to zero
__device__ float kmc_expf(float x) {
    if (!(x == x)) return x;
    if (x < -87.0f) return 0.0f;
    if (x > 88.0f) return __uint_as_float(0x7f800000u);
    const float k = floorf(x * 1.4426950216293335f + 0.5f);
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
    return p * __uint_as_float((unsigned)((int)k + 127) << 23);
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

__device__ __forceinline__ double qnan() { return __longlong_as_double(0x7ff8000000000000LL); }

// rod view and cell counts
__global__ void k_kmc_bin(KmcDev K, DevState S, int count) {
    ALENS_PDL_PROLOGUE();
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < S.nRods; r += gridDim.x * blockDim.x) {
        const KmcRep &Q = K.rep[S.rodRep[r]];
        double p[3] = {S.px[r], S.py[r], S.pz[r]};
        kmc_wrap_point(Q, p);
        double a[3];
        quat_axis(S.qx[r], S.qy[r], S.qz[r], S.qw[r], a);
        const double L = S.len[r];
        const bool sphere = L < 2.0 * S.rad[r];
        K.rodC[r] = make_kd4(p[0], p[1], p[2], 0.5 * L);
        K.rodA[r] = make_kd4(a[0], a[1], a[2], sphere ? 1.0 : 0.0);
        if (!count) continue;
        int c[3];
        for (int d = 0; d < 3; d++) c[d] = kmc_cell_coord(p[d], Q.lo[d], Q.cellsz[d], Q.ncell[d]);
        atomicAdd(&K.cellCount[Q.cellOffset + (c[2] * Q.ncell[1] + c[1]) * Q.ncell[0] + c[0]], 1);
    }
}

__global__ void k_kmc_scatter(KmcDev K, DevState S) {
    ALENS_PDL_PROLOGUE();
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < S.nRods; r += gridDim.x * blockDim.x) {
        const KmcRep &Q = K.rep[S.rodRep[r]];
        const KDouble4 C = K.rodC[r];
        const double p[3] = {C.x, C.y, C.z};
        int c[3];
        for (int d = 0; d < 3; d++) c[d] = kmc_cell_coord(p[d], Q.lo[d], Q.cellsz[d], Q.ncell[d]);
        const int cid = Q.cellOffset + (c[2] * Q.ncell[1] + c[1]) * Q.ncell[0] + c[0];
        const int slot = K.cellStart[cid] + atomicAdd(&K.cellCursor[cid], 1);
        // FP32 screening geometry: centre relative to its cell's origin
        float rel[3];
        for (int d = 0; d < 3; d++) rel[d] = (float)(p[d] - (Q.lo[d] + (double)c[d] * Q.cellsz[d]));
        const KDouble4 A = K.rodA[r];
        K.cellRod[slot] = r;
        K.cellRel[slot] = make_float4(rel[0], rel[1], rel[2], (float)C.w);
        K.cellAx[slot] = make_float4((float)A.x, (float)A.y, (float)A.z, (float)A.w);
    }
}

// ---- S->D integral, FP32 (the FP64 pipe of GB300 issues a warp
// instruction in 64 cycles, the FP32 pipe in one; a rate needs no more)
__device__ __forceinline__ float fmaxf_(float a, float b) { return a > b ? a : b; }
__device__ __forceinline__ float fminf_(float a, float b) { return a < b ? a : b; }

// one Gauss-Legendre panel of the integrand over s in [a, b]
__device__ float sd_panel(float a, float b, float d2, float A, float c, float sc) {
    const float h = 0.5f * (b - a), m = 0.5f * (a + b);
    float acc = 0.0f;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        const float s = m + h * kGLx[k];
        const float x = sc * sqrtf(d2 + s * s) - c;
        acc = acc + kGLw[k] * kmc_expf(-(A * (x * x)));
    }
    return h * acc;
}

// per-candidate constants of the integral
struct SdGeom {
    float d2, A, c, k;   // exponent -A (k r - c)^2, r = sqrt(d2 + s^2)
    float lo[2], hi[2], step[2];
    int n[2];
};

// the integrand's support within [sA, sB]: head distances within w of c,
// |s| in [sl, sh]; at most two arcs, each cut into panels of at most w/4
// lookupType 1: the stretch is (1 - D/d) r, d the distance from the axis;
// head distances up to ell0 + D + w as for lookupType 0, none when d <= D
__device__ __forceinline__ void sd_geom(float d2, float sA, float sB, const KmcType &T, SdGeom &G) {
    const float rO = T.rOuterf, w = T.wf;
    G.d2 = d2;
    G.A = T.Af;
    G.c = T.cf;
    G.k = 1.0f;
    G.n[0] = G.n[1] = 0;
    float ro2 = rO * rO;
    if (!(d2 < ro2)) return;
    float ri = G.c - w;
    if (T.lookup == 1) {
        G.k = 1.0f - T.Df / sqrtf(d2);
        if (!(G.k > 0.0f)) return;
        const float rh = (G.c + w) / G.k;
        if (rh < rO) ro2 = rh * rh;
        if (!(d2 < ro2)) return;
        ri = (G.c - w) / G.k;
    }
    const float sh = sqrtf(ro2 - d2);
    const float sl = (ri > 0.0f && ri * ri > d2) ? sqrtf(ri * ri - d2) : 0.0f;
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
        const float q = ceilf((G.hi[i] - G.lo[i]) / (0.25f * w));
        G.n[i] = q < 1.0f ? 1 : (q > 64.0f ? 64 : (int)q);
        G.step[i] = (G.hi[i] - G.lo[i]) / (float)G.n[i];
    }
}

// edges of panel j (arc 0 first, then arc 1)
__device__ __forceinline__ void sd_edges(const SdGeom &G, int j, float *a, float *b) {
    const int i = j < G.n[0] ? 0 : 1;
    const int k = i == 0 ? j : j - G.n[0];
    *a = G.lo[i] + G.step[i] * (float)k;
    *b = k == G.n[i] - 1 ? G.hi[i] : G.lo[i] + G.step[i] * (float)(k + 1);
}

// the integral of one candidate: panel k on lane k mod 32, each lane's
// panels summed in order, then the lanes by a fixed tree (16, 8, 4, 2, 1);
// the result on every lane
__device__ float sd_integral_warp(const SdGeom &G, int lane) {
    const int m = G.n[0] + G.n[1];
    float s = 0.0f;
    for (int k = lane; k < m; k += 32) {
        float a, b;
        sd_edges(G, k, &a, &b);
        s = s + sd_panel(a, b, G.d2, G.A, G.c, G.k);
    }
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) s = s + __shfl_down_sync(0xffffffffu, s, off);
    return __shfl_sync(0xffffffffu, s, 0);
}

// ---- warp-per-protein binding step
constexpr int kKmcWarps = 4;        // warps per block
constexpr int kKmcPanels = 128;     // panels of one integral (2 arcs x 64)

struct KmcWarpBuf {
    int idx[kKmcMaxCand], sidx[kKmcMaxCand];
    float4 v[kKmcMaxCand], sv[kKmcMaxCand];  // per candidate (gather order / ascending rod)
    unsigned long long F[kKmcMaxCand];       // per sorted candidate: fixed-point probability
    float I[kKmcMaxCand];                    // S: integral per sorted candidate
    float panel[kKmcPanels];
};

// the 27 stencil cells of cell c, with the offset of each; periodic sides
// wrap (two cells per side at least: every offset names one image)
__device__ __forceinline__ void kmc_stencil(const KmcRep &Q, const int c[3], int lo[3], int hi[3]) {
    for (int d = 0; d < 3; d++) {
        if (Q.pbc[d]) {
            lo[d] = -1;
            hi[d] = 1;
        } else {
            lo[d] = c[d] > 0 ? -1 : 0;
            hi[d] = c[d] < Q.ncell[d] - 1 ? 1 : 0;
        }
    }
}

// Decisions of the U and S stages in fixed point: a probability p (FP32)
// becomes floor(p 2^53) (2^53 for p >= 1), the roll is the 53-bit integer
// of the first two Philox words, and an event happens when the roll lies
// below the stacked integers.  Integer sums are exact; no FP64 issue.
__device__ __forceinline__ unsigned long long kmc_fix53(float p) {
    if (!(p > 0.0f)) return 0ull;
    if (p >= 1.0f) return 1ull << 53;
    const unsigned bits = __float_as_uint(p);
    const int ex = (int)((bits >> 23) & 0xffu);
    if (ex == 0) return 0ull;
    const unsigned long long man = (unsigned long long)((bits & 0x7fffffu) | 0x800000u);
    const int sh = ex - 97;  // p = man 2^(ex - 150); p 2^53 = man 2^(ex - 97)
    return sh >= 0 ? man << sh : (-sh >= 64 ? 0ull : man >> (-sh));
}

__device__ __forceinline__ unsigned long long kmc_roll53(const uint32_t w[4]) {
    return ((unsigned long long)(w[0] >> 5) << 26) | (unsigned long long)(w[1] >> 6);
}

__device__ __forceinline__ int kmc_choose_fix(unsigned long long F0, unsigned long long F1, unsigned long long *roll) {
    const unsigned long long u = *roll;
    if (u < F0) return 0;
    if (u < F0 + F1) {
        *roll = u - F0;
        return 1;
    }
    return -1;
}

// the sorted candidate whose slice of the stacked integers holds roll, and
// the roll's fraction of that slice (FP32)
__device__ int kmc_pick_fix(const KmcWarpBuf &B, int n, unsigned long long roll, float *frac) {
    unsigned long long cum = 0ull;
    int last = -1;
    for (int j = 0; j < n; j++) {
        const unsigned long long Fj = B.F[j];
        if (Fj == 0ull) continue;
        last = j;
        if (roll < cum + Fj) {
            *frac = (float)(roll - cum) / (float)Fj;
            return j;
        }
        cum = cum + Fj;
    }
    *frac = 1.0f;
    return last;
}

// Distance from point P to the axis segment of rod r (minimum image).
__device__ __forceinline__ double kmc_dist_point_seg(const KmcDev &K, const KmcRep &Q, const double P[3], int r) {
    const KDouble4 C = K.rodC[r], A = K.rodA[r];
    double u[3] = {P[0] - C.x, P[1] - C.y, P[2] - C.z};
    for (int d = 0; d < 3; d++)
        if (Q.pbc[d]) u[d] = u[d] - Q.L[d] * floor(u[d] / Q.L[d] + 0.5);
    double t = u[0] * A.x + u[1] * A.y + u[2] * A.z;
    t = t > C.w ? C.w : (t < -C.w ? -C.w : t);
    const double q0 = u[0] - t * A.x, q1 = u[1] - t * A.y, q2 = u[2] - t * A.z;
    return sqrt(q0 * q0 + q1 * q1 + q2 * q2);
}

// ProteinData::getProteinForceLength (Protein/ProteinData.hpp:171-195): the
// heads' distance ell less the rod diameter (lookupType 0), or scaled by
// 1 - D/d, d the distance of head 0 from the segment of head 1's rod (1)
__device__ __forceinline__ double kmc_force_length(const KmcDev &K, const KmcRep &Q, const KmcType &T,
                                                   const double P0[3], int r1, double ell) {
    if (T.lookup == 0) return ell - K.D;
    const double d = kmc_dist_point_seg(K, Q, P0, r1);
    return (1.0 - K.D / d) * ell;
}

// prepared per unbound / singly bound protein for the warp kernel: the
// stencil centre cell, the search point relative to it (FP32), the bound
// head's rod axis (FP32), the stage
struct KmcTask {
    int4 cell;      // c[0..2], nb | (b << 2)
    float4 rel;     // point relative to the cell origin, w: bound rod (bits)
    float4 ab;      // bound rod axis
    int4 roll;      // the 53-bit roll (low, high words)
};

// code per protein: final stage (bits 0-1), transition (bits 2-4: 1 U->S,
// 2 S->U, 3 S->D, 4 D->S), candidates (bits 8-); -1: for k_kmc_bind
//
// One thread per protein: ends on rods the replica no longer holds are
// released (the reference releases an end whose rod it cannot find);
// doubly bound proteins take their D -> S step here (FP64, one exp); the
// others get their task.
__global__ void __launch_bounds__(256) k_kmc_prep(KmcDev K, int *code, KmcTask *task) {
    ALENS_PDL_PROLOGUE();
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < K.nProt; p += gridDim.x * blockDim.x) {
        const int rep = K.protRep[p];
        const KmcRep &Q = K.rep[rep];
        AlensProtein &pp = K.prot[p];
        int id[2] = {pp.idBind[0], pp.idBind[1]};
        for (int e = 0; e < 2; e++)
            if (id[e] < 0 || id[e] >= Q.nRods) id[e] = -1;
        double P[2][3];
        for (int e = 0; e < 2; e++) {
            if (id[e] < 0) continue;
            const int r = Q.rodOffset + id[e];
            const KDouble4 C = K.rodC[r], A = K.rodA[r];
            const double dist = pp.distBind[e];
            P[e][0] = C.x + dist * A.x;
            P[e][1] = C.y + dist * A.y;
            P[e][2] = C.z + dist * A.z;
        }
        const int nb = (id[0] >= 0 ? 1 : 0) + (id[1] >= 0 ? 1 : 0);
        if (nb == 2) {
            const KmcType &T = K.types[rep * K.nTypes + pp.type];
            uint32_t w[4];
            kmc_words(Q.seed, pp.gid, K.step, 0, w);
            double roll = u53(w[0], w[1]);
            double dv[3] = {P[1][0] - P[0][0], P[1][1] - P[0][1], P[1][2] - P[0][2]};
            for (int k = 0; k < 3; k++)
                if (Q.pbc[k]) dv[k] = dv[k] - Q.L[k] * floor(dv[k] / Q.L[k] + 0.5);
            const double ell = sqrt(dv[0] * dv[0] + dv[1] * dv[1] + dv[2] * dv[2]);
            const double x = kmc_force_length(K, Q, T, P[0], Q.rodOffset + id[1], ell) - T.ell0;
            const double M = T.Ads * (x * x);
            const double g = kmc_exp(M);
            const double p0 = (T.koD[0] * g) * T.dt, p1 = (T.koD[1] * g) * T.dt;
            const int e = kmc_choose(p0, p1, &roll);
            int trans = 0;
            if (e >= 0) {
                pp.idBind[e] = -1;
                trans = 4;
            }
            code[p] = (e >= 0 ? 1 : 2) | (trans << 2);
            continue;
        }
        pp.idBind[0] = id[0];
        pp.idBind[1] = id[1];
        const int b = id[0] >= 0 ? 0 : 1;
        double X[3];
        for (int d = 0; d < 3; d++) X[d] = nb == 0 ? pp.pos[d] : P[b][d];
        kmc_wrap_point(Q, X);
        if (nb == 0)
            for (int d = 0; d < 3; d++) pp.pos[d] = X[d];
        KmcTask t;
        int c[3];
        float r[3];
        for (int d = 0; d < 3; d++) {
            c[d] = kmc_cell_coord(X[d], Q.lo[d], Q.cellsz[d], Q.ncell[d]);
            r[d] = (float)(X[d] - (Q.lo[d] + (double)c[d] * Q.cellsz[d]));
        }
        float ab[3] = {0.0f, 0.0f, 0.0f};
        if (nb == 1) {
            const KDouble4 A = K.rodA[Q.rodOffset + id[b]];
            ab[0] = (float)A.x;
            ab[1] = (float)A.y;
            ab[2] = (float)A.z;
        }
        t.cell = make_int4(c[0], c[1], c[2], nb | (b << 2));
        t.rel = make_float4(r[0], r[1], r[2], __int_as_float(nb == 1 ? id[b] : -1));
        t.ab = make_float4(ab[0], ab[1], ab[2], 0.0f);
        uint32_t w[4];
        kmc_words(Q.seed, pp.gid, K.step, 0, w);
        const unsigned long long roll = kmc_roll53(w);
        t.roll = make_int4((int)(unsigned)roll, (int)(unsigned)(roll >> 32), 0, 0);
        task[p] = t;
        code[p] = -1;
    }
}

// One warp per unbound or singly bound protein: the candidate rods of the
// 27 cells around the protein (all cell ranges in one load, the rods spread
// over the lanes, FP32 geometry), ascending rod index, the S->D integrals
// (one panel per lane), then the event (fixed-point decisions on lane 0).
__global__ void __launch_bounds__(32 * kKmcWarps) k_kmc_bind(KmcDev K, int *code, const KmcTask *task) {
    ALENS_PDL_PROLOGUE();
    __shared__ KmcWarpBuf bufs[kKmcWarps];
    KmcWarpBuf &B = bufs[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    for (int p = blockIdx.x * kKmcWarps + (threadIdx.x >> 5); p < K.nProt; p += gridDim.x * kKmcWarps) {
        if (code[p] >= 0) continue;   // doubly bound: done in k_kmc_prep
        const KmcTask tk = task[p];
        const int rep = K.protRep[p];
        const KmcRep &Q = K.rep[rep];
        const long long gid = K.prot[p].gid;
        const KmcType &T = K.types[rep * K.nTypes + K.prot[p].type];
        const int nb = tk.cell.w & 3, b = (tk.cell.w >> 2) & 1, f = 1 - b;
        const int idb = __float_as_int(tk.rel.w);
        const int c[3] = {tk.cell.x, tk.cell.y, tk.cell.z};
        const float rx[3] = {tk.rel.x, tk.rel.y, tk.rel.z};
        int lo[3], hi[3];
        kmc_stencil(Q, c, lo, hi);
        // stencil cell k = lane (k < 27; offsets -1..1 per side; clipped
        // cells empty): its rod range
        const int ox = lane % 3 - 1, oy = (lane / 3) % 3 - 1, oz = lane / 9 - 1;
        int cs0 = 0, cn = 0;
        if (lane < 27 && ox >= lo[0] && ox <= hi[0] && oy >= lo[1] && oy <= hi[1] && oz >= lo[2] && oz <= hi[2]) {
            int cc[3] = {c[0] + ox, c[1] + oy, c[2] + oz};
            for (int d = 0; d < 3; d++)
                if (Q.pbc[d]) cc[d] = cc[d] < 0 ? cc[d] + Q.ncell[d] : (cc[d] >= Q.ncell[d] ? cc[d] - Q.ncell[d] : cc[d]);
            const int cid = Q.cellOffset + (cc[2] * Q.ncell[1] + cc[1]) * Q.ncell[0] + cc[0];
            cs0 = K.cellStart[cid];
            cn = K.cellStart[cid + 1] - cs0;
        }
        int incl = cn;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, incl, off);
            if (lane >= off) incl += v;
        }
        const int total = __shfl_sync(0xffffffffu, incl, 31);
        const int excl = incl - cn;
        const float csf[3] = {Q.cellszf[0], Q.cellszf[1], Q.cellszf[2]};
        const float r2 = T.rcapf * T.rcapf;
        const float ro2 = T.rOuterf * T.rOuterf;
        int n = 0;
        for (int base = 0; base < total; base += 32) {
            const int i = base + lane;
            bool cand = false;
            float4 rec = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            int li = 0;
            // the last stencil cell whose first flattened rod is <= i
            // (prefixes ascend): five rounds of a binary search
            int k = 0, khi = 26;
#pragma unroll
            for (int it = 0; it < 5; it++) {
                const int mid = (k + khi + 1) >> 1;
                if (__shfl_sync(0xffffffffu, excl, mid) <= i)
                    k = mid;
                else
                    khi = mid - 1;
            }
            const int kstart = __shfl_sync(0xffffffffu, cs0, k);
            const int kex = __shfl_sync(0xffffffffu, excl, k);
            if (i < total) {
                const int s = kstart + (i - kex);
                const float4 R = K.cellRel[s], Ax = K.cellAx[s];
                li = K.cellRod[s] - Q.rodOffset;
                const float sh0 = (float)(k % 3 - 1) * csf[0];
                const float sh1 = (float)((k / 3) % 3 - 1) * csf[1];
                const float sh2 = (float)(k / 9 - 1) * csf[2];
                const float v0 = (rx[0] - R.x) - sh0;
                const float v1 = (rx[1] - R.y) - sh1;
                const float v2 = (rx[2] - R.z) - sh2;
                const float t0 = (v0 * Ax.x + v1 * Ax.y) + v2 * Ax.z;
                const float q0 = v0 - t0 * Ax.x, q1 = v1 - t0 * Ax.y, q2 = v2 - t0 * Ax.z;
                const float d2 = (q0 * q0 + q1 * q1) + q2 * q2;
                if (Ax.w == 0.0f) {
                    if (nb == 0) {
                        if (d2 < r2) {
                            const float hc = sqrtf(r2 - d2);
                            const float l = fmaxf_(-R.w, t0 - hc), h = fminf_(R.w, t0 + hc);
                            const float Lc = h - l;
                            if (Lc > 0.0f) {
                                cand = true;
                                rec = make_float4(Lc, l, R.w, 0.0f);
                            }
                        }
                    } else if (li != idb && d2 < ro2) {
                        cand = true;
                        rec = make_float4(t0, d2, R.w, (Ax.x * tk.ab.x + Ax.y * tk.ab.y) + Ax.z * tk.ab.z);
                    }
                }
            }
            const unsigned m = __ballot_sync(0xffffffffu, cand);
            if (cand) {
                const int slot = n + __popc(m & ((1u << lane) - 1u));
                if (slot < kKmcMaxCand) {
                    B.idx[slot] = li;
                    B.v[slot] = rec;
                }
            }
            n += __popc(m);
        }
        __syncwarp();
        const int nc = n < kKmcMaxCand ? n : kKmcMaxCand;
        // ascending rod index (a rod appears once: one image within reach)
        for (int k = lane; k < nc; k += 32) {
            const int me = B.idx[k];
            int rank = 0;
            for (int j = 0; j < nc; j++) rank += B.idx[j] < me ? 1 : 0;
            B.sidx[rank] = me;
            B.sv[rank] = B.v[k];
        }
        __syncwarp();
        unsigned long long roll =
            ((unsigned long long)(unsigned)tk.roll.y << 32) | (unsigned long long)(unsigned)tk.roll.x;
        int trans = 0;
        if (n > kKmcMaxCand) {
            if (lane == 0) atomicOr(K.err, kKmcErrCand);
        } else if (nb == 0) {
            if (lane == 0) {
                unsigned long long S0 = 0ull, S1 = 0ull;
                for (int j = 0; j < nc; j++) S0 = S0 + kmc_fix53(B.sv[j].x * T.usCoeff[0]);
                for (int j = 0; j < nc; j++) S1 = S1 + kmc_fix53(B.sv[j].x * T.usCoeff[1]);
                const int e = kmc_choose_fix(S0, S1, &roll);
                if (e >= 0) {
                    for (int j = 0; j < nc; j++) B.F[j] = kmc_fix53(B.sv[j].x * T.usCoeff[e]);
                    float frac;
                    const int j = kmc_pick_fix(B, nc, roll, &frac);
                    if (j >= 0) {
                        const float4 cv = B.sv[j];
                        const double hl = K.rodC[Q.rodOffset + B.sidx[j]].w;
                        const double s = (double)(cv.y + frac * cv.x);
                        AlensProtein &pp = K.prot[p];
                        pp.idBind[e] = B.sidx[j];
                        pp.distBind[e] = s > hl ? hl : (s < -hl ? -hl : s);
                        trans = 1;
                    }
                }
            }
        } else {
            // S->D integral of every candidate
            for (int j = 0; j < nc; j++) {
                const float4 cv = B.sv[j];
                SdGeom G;
                sd_geom(cv.y, -cv.z - cv.x, cv.z - cv.x, T, G);
                const float Iq = sd_integral_warp(G, lane);
                if (lane == 0) {
                    const float pref = cv.w > 0.0f ? T.prefPar : T.prefAnti;
                    B.I[j] = Iq;
                    B.F[j] = kmc_fix53((pref * T.sdCoeff[f]) * Iq);
                }
            }
            __syncwarp();
            int e = -2, j = -1;
            float frac = 0.0f;
            if (lane == 0) {
                unsigned long long Sb = 0ull;
                for (int k = 0; k < nc; k++) Sb = Sb + B.F[k];
                const unsigned long long FU = kmc_fix53(T.suProbf[b]);
                e = kmc_choose_fix(b == 0 ? FU : Sb, b == 0 ? Sb : FU, &roll);
                if (e == f) j = kmc_pick_fix(B, nc, roll, &frac);
            }
            e = __shfl_sync(0xffffffffu, e, 0);
            j = __shfl_sync(0xffffffffu, j, 0);
            frac = __shfl_sync(0xffffffffu, frac, 0);
            if (e == b) {
                if (lane == 0) {
                    // released uniformly in the capture sphere around the head
                    double off[3] = {0.0, 0.0, 0.0};
                    for (uint32_t k = 0; k < 32; k++) {
                        uint32_t v[4];
                        kmc_words(Q.seed, gid, K.step, 2 + k, v);
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
                    AlensProtein &pp = K.prot[p];
                    const int r = Q.rodOffset + pp.idBind[b];
                    const KDouble4 C = K.rodC[r], A = K.rodA[r];
                    const double dist = pp.distBind[b];
                    pp.pos[0] = (C.x + dist * A.x) + T.rcap * off[0];
                    pp.pos[1] = (C.y + dist * A.y) + T.rcap * off[1];
                    pp.pos[2] = (C.z + dist * A.z) + T.rcap * off[2];
                    pp.idBind[b] = -1;
                    trans = 2;
                }
            } else if (e == f && j >= 0) {
                // the binding point: the panel holding the target (running
                // sum in panel order), then four rounds of a 32-way search of
                // that panel's partial integral
                const float4 cv = B.sv[j];
                SdGeom G;
                sd_geom(cv.y, -cv.z - cv.x, cv.z - cv.x, T, G);
                const int m = G.n[0] + G.n[1];
                for (int k = lane; k < m; k += 32) {
                    float a, bb;
                    sd_edges(G, k, &a, &bb);
                    B.panel[k] = sd_panel(a, bb, G.d2, G.A, G.c, G.k);
                }
                __syncwarp();
                const float target = frac * B.I[j];
                int kp = m - 1;
                float t = -1.0f;
                if (lane == 0) {
                    float cum = 0.0f;
                    for (int k = 0; k < m; k++) {
                        const float Pk = B.panel[k];
                        if (target < cum + Pk) {
                            kp = k;
                            t = target - cum;
                            break;
                        }
                        cum = cum + Pk;
                    }
                }
                kp = __shfl_sync(0xffffffffu, kp, 0);
                t = __shfl_sync(0xffffffffu, t, 0);
                float a, bb;
                sd_edges(G, kp, &a, &bb);
                float sStar = bb;
                if (t >= 0.0f) {
                    float x0 = a, x1 = bb;
                    for (int round = 0; round < 4; round++) {
                        const float step = (x1 - x0) / 32.0f;
                        const float xk = lane == 31 ? x1 : x0 + step * (float)(lane + 1);
                        const bool ge = !(sd_panel(a, xk, G.d2, G.A, G.c, G.k) < t);
                        const unsigned gm = __ballot_sync(0xffffffffu, ge);
                        const int first = gm ? __ffs(gm) - 1 : 31;
                        const float nx1 = __shfl_sync(0xffffffffu, xk, first);
                        const float nx0 = __shfl_sync(0xffffffffu, xk, first > 0 ? first - 1 : 0);
                        x0 = first > 0 ? nx0 : x0;
                        x1 = nx1;
                    }
                    sStar = 0.5f * (x0 + x1);
                }
                if (lane == 0) {
                    const double hl = K.rodC[Q.rodOffset + B.sidx[j]].w;
                    const double s = (double)(cv.x + sStar);
                    AlensProtein &pp = K.prot[p];
                    pp.idBind[f] = B.sidx[j];
                    pp.distBind[f] = s > hl ? hl : (s < -hl ? -hl : s);
                    trans = 3;
                }
            }
        }
        if (lane == 0) {
            const int nb2 = nb + (trans == 1 || trans == 3 ? 1 : 0) - (trans == 2 ? 1 : 0);
            code[p] = nb2 | (trans << 2) | (n << 8);
        }
        __syncwarp();
    }
}

// ---- motion step (TubuleSystem::updateProteinMotion)

// Box-Muller pair from two Philox words (24-bit uniforms, FP32, the
// project's log and sincos, as the rods' noise)
__device__ __forceinline__ void kmc_normal_pair(uint32_t wa, uint32_t wb, double *z0, double *z1) {
    const float ua = ((float)(wa >> 8) + 0.5f) * 5.9604644775390625e-08f;
    const float ub = ((float)(wb >> 8) + 0.5f) * 5.9604644775390625e-08f;
    const float r = sqrtf(-2.0f * det_logf(ua));
    const float ang = ub * 6.28318531f - 3.14159265f;
    float sn, cs;
    det_sincosf(ang, &sn, &cs);
    *z0 = (double)(r * -cs);
    *z1 = (double)(r * -sn);
}

// a point outside a boundary is moved onto it (Boundary::project as
// SRC/TubuleSystem.cpp:285-305 uses it): wall, sphere (inside / outside),
// tube (inside)
__device__ __forceinline__ void kmc_project(const BoundaryDev &B, double x[3]) {
    const double v[3] = {x[0] - B.c[0], x[1] - B.c[1], x[2] - B.c[2]};
    if (B.type == 0) {
        const double s = v[0] * B.a[0] + v[1] * B.a[1] + v[2] * B.a[2];
        if (s < 0.0)
            for (int d = 0; d < 3; d++) x[d] = x[d] - s * B.a[d];
    } else if (B.type == 1) {
        const double r = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        const bool out = B.inside ? r > B.R : r < B.R;
        if (out && r > 0.0)
            for (int d = 0; d < 3; d++) x[d] = B.c[d] + (B.R / r) * v[d];
    } else {
        const double s = v[0] * B.a[0] + v[1] * B.a[1] + v[2] * B.a[2];
        const double q[3] = {v[0] - s * B.a[0], v[1] - s * B.a[1], v[2] - s * B.a[2]};
        const double r = sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2]);
        if (r > B.R)
            for (int d = 0; d < 3; d++) x[d] = (B.c[d] + s * B.a[d]) + (B.R / r) * q[d];
    }
}

// One thread per protein (ProteinData::updatePosWalk / updatePosDiffuse,
// Protein/ProteinData.hpp:318-406, walk velocity :459-478, drag :489-498):
// rolls from Philox (seed, gid, step, 'mot' + block): block 0 gives the
// uniform (53 bits) and normals z0, z1, block 1 gives z2.
__global__ void __launch_bounds__(256) k_kmc_motion(KmcDev K, DevState S, int *code) {
    ALENS_PDL_PROLOGUE();
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < K.nProt; p += gridDim.x * blockDim.x) {
        const int rep = K.protRep[p];
        const KmcRep &Q = K.rep[rep];
        AlensProtein &pr = K.prot[p];
        const KmcType &T = K.types[rep * K.nTypes + pr.type];
        int id[2] = {pr.idBind[0], pr.idBind[1]};
        for (int e = 0; e < 2; e++)
            if (id[e] < 0 || id[e] >= Q.nRods) id[e] = -1;
        const int nb = (id[0] >= 0 ? 1 : 0) + (id[1] >= 0 ? 1 : 0);
        uint32_t w[4], v[4];
        w[0] = (uint32_t)(unsigned long long)pr.gid;
        w[1] = (uint32_t)((unsigned long long)pr.gid >> 32);
        w[2] = (uint32_t)(unsigned long long)K.step;
        w[3] = 0x6D6F7400u;
        v[0] = w[0];
        v[1] = w[1];
        v[2] = w[2];
        v[3] = 0x6D6F7401u;
        philox4x32_10(w, (uint32_t)Q.seed, (uint32_t)(Q.seed >> 32));
        philox4x32_10(v, (uint32_t)Q.seed, (uint32_t)(Q.seed >> 32));
        const double u01 = u53(w[0], w[1]);
        double z0, z1, z2, z3;
        kmc_normal_pair(w[2], w[3], &z0, &z1);
        kmc_normal_pair(v[0], v[1], &z2, &z3);
        int trans = 0;
        if (nb == 0) {
            pr.idBind[0] = pr.idBind[1] = -1;
            pr.pos[0] = pr.pos[0] + T.diffU * z0;
            pr.pos[1] = pr.pos[1] + T.diffU * z1;
            pr.pos[2] = pr.pos[2] + T.diffU * z2;
        } else {
            double dist[2] = {pr.distBind[0], pr.distBind[1]};
            if (nb == 2) {
                // spring load on each head (ProteinData::updateForceTorqueBind)
                double P[2][3];
                KDouble4 Ax[2];
                for (int e = 0; e < 2; e++) {
                    const int r = Q.rodOffset + id[e];
                    const KDouble4 C = K.rodC[r];
                    Ax[e] = K.rodA[r];
                    P[e][0] = C.x + dist[e] * Ax[e].x;
                    P[e][1] = C.y + dist[e] * Ax[e].y;
                    P[e][2] = C.z + dist[e] * Ax[e].z;
                }
                double rv[3] = {P[0][0] - P[1][0], P[0][1] - P[1][1], P[0][2] - P[1][2]};
                for (int d = 0; d < 3; d++)
                    if (Q.pbc[d]) rv[d] = rv[d] - Q.L[d] * floor(rv[d] / Q.L[d] + 0.5);
                const double ell = sqrt(rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2]);
                const double force = (kmc_force_length(K, Q, T, P[0], Q.rodOffset + id[1], ell) - T.ell0) * T.kappa;
                const double f0[3] = {-force * (rv[0] / ell), -force * (rv[1] / ell), -force * (rv[2] / ell)};
                const double par = Ax[0].x * Ax[1].x + Ax[0].y * Ax[1].y + Ax[0].z * Ax[1].z;
                const double z[2] = {z0, z1};
                for (int e = 0; e < 2; e++) {
                    const double sg = e == 0 ? 1.0 : -1.0;  // f1 = -f0
                    const double fdir = sg * (f0[0] * Ax[e].x + f0[1] * Ax[e].y + f0[2] * Ax[e].z);
                    const double sgn = T.vmax[e] > 0.0 ? 1.0 : (T.vmax[e] < 0.0 ? -1.0 : 0.0);
                    const double fproj = (sgn * fdir) / fabs(T.fstall);
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
                half[e] = K.rodC[Q.rodOffset + id[e]].w;
                off[e] = dist[e] > half[e] || dist[e] < -half[e];
            }
            if (T.walkOff) {
                if (off[0] && off[1]) {
                    const int e = u01 < 0.5 ? 0 : 1;
                    id[e] = -1;
                    dist[1 - e] = dist[1 - e] > half[1 - e] ? half[1 - e] : (dist[1 - e] < -half[1 - e] ? -half[1 - e] : dist[1 - e]);
                } else if (off[0]) {
                    id[0] = -1;
                } else if (off[1]) {
                    id[1] = -1;
                }
            } else {
                for (int e = 0; e < 2; e++)
                    if (id[e] >= 0) dist[e] = dist[e] > half[e] ? half[e] : (dist[e] < -half[e] ? -half[e] : dist[e]);
            }
            const int nb2 = (id[0] >= 0 ? 1 : 0) + (id[1] >= 0 ? 1 : 0);
            if (nb2 < nb) trans = nb == 2 ? 4 : 2;
            // a protein that walked off its only rod keeps its centre (the
            // last head position): ProteinBindStatus::updatePosWithEndBind
            // leaves an unbound protein's position alone
            for (int e = 0; e < 2; e++) {
                pr.idBind[e] = id[e];
                pr.distBind[e] = dist[e];
            }
        }
        // unbound proteins outside a boundary are moved onto it
        // (SRC/TubuleSystem.cpp:285-305: after the motion, every protein
        // that is unbound then)
        if (pr.idBind[0] < 0 && pr.idBind[1] < 0) {
            double x[3] = {pr.pos[0], pr.pos[1], pr.pos[2]};
            for (int b = S.bndStart[rep]; b < S.bndStart[rep + 1]; b++) kmc_project(S.bnd[b], x);
            pr.pos[0] = x[0];
            pr.pos[1] = x[1];
            pr.pos[2] = x[2];
        }
        code[p] = ((pr.idBind[0] >= 0 ? 1 : 0) + (pr.idBind[1] >= 0 ? 1 : 0)) | (trans << 2);
    }
}

// One thread per protein: head positions and centre of the new state
// (bound head; midpoint of the heads, minimum image; the free point),
// wrapped into the box; unbound ends NaN.
__global__ void __launch_bounds__(256) k_kmc_geom(KmcDev K) {
    ALENS_PDL_PROLOGUE();
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < K.nProt; p += gridDim.x * blockDim.x) {
        const KmcRep &Q = K.rep[K.protRep[p]];
        AlensProtein &pr = K.prot[p];
        const int id[2] = {pr.idBind[0], pr.idBind[1]};
        double E[2][3];
        for (int e = 0; e < 2; e++) {
            if (id[e] < 0) {
                pr.distBind[e] = qnan();
                pr.posEnd[e][0] = pr.posEnd[e][1] = pr.posEnd[e][2] = qnan();
                continue;
            }
            const int r = Q.rodOffset + id[e];
            const KDouble4 Cr = K.rodC[r], Ar = K.rodA[r];
            const double dist = pr.distBind[e];
            E[e][0] = Cr.x + dist * Ar.x;
            E[e][1] = Cr.y + dist * Ar.y;
            E[e][2] = Cr.z + dist * Ar.z;
            pr.posEnd[e][0] = E[e][0];
            pr.posEnd[e][1] = E[e][1];
            pr.posEnd[e][2] = E[e][2];
        }
        const int nb = (id[0] >= 0 ? 1 : 0) + (id[1] >= 0 ? 1 : 0);
        double X[3] = {pr.pos[0], pr.pos[1], pr.pos[2]};
        if (nb == 1) {
            const int bb = id[0] >= 0 ? 0 : 1;
            X[0] = E[bb][0];
            X[1] = E[bb][1];
            X[2] = E[bb][2];
        } else if (nb == 2) {
            for (int d = 0; d < 3; d++) {
                double dv = E[1][d] - E[0][d];
                if (Q.pbc[d]) dv = dv - Q.L[d] * floor(dv / Q.L[d] + 0.5);
                X[d] = E[0][d] + 0.5 * dv;
            }
        }
        kmc_wrap_point(Q, X);
        pr.pos[0] = X[0];
        pr.pos[1] = X[1];
        pr.pos[2] = X[2];
    }
}

// per replica: stage counts, transitions and the most candidates; each
// warp adds its lanes' counts with one atomic per counter when all its
// proteins belong to one replica (replicas own contiguous protein ranges)
__global__ void __launch_bounds__(256) k_kmc_stats(KmcDev K, const int *code) {
    ALENS_PDL_PROLOGUE();
    const int lane = threadIdx.x & 31;
    for (int base = (blockIdx.x * blockDim.x + threadIdx.x) & ~31; base < K.nProt;
         base += gridDim.x * blockDim.x) {
        const int p = base + lane;
        const bool on = p < K.nProt;
        const int c = on ? code[p] : 0;
        const int rep = on ? K.protRep[p] : -1;
        int v[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        if (on) {
            v[c & 3] = 1;
            const int t = (c >> 2) & 7;
            if (t > 0) v[2 + t] = 1;
            v[7] = c >> 8;
        }
        const int rep0 = __shfl_sync(0xffffffffu, rep, 0);
        const bool uniform = __all_sync(0xffffffffu, !on || rep == rep0);
        if (uniform) {
            int s[8];
#pragma unroll
            for (int k = 0; k < 7; k++) s[k] = __reduce_add_sync(0xffffffffu, (unsigned)v[k]);
            s[7] = __reduce_max_sync(0xffffffffu, (unsigned)v[7]);
            if (lane == 0) {
#pragma unroll
                for (int k = 0; k < 7; k++)
                    if (s[k]) atomicAdd(&K.stats[8 * rep0 + k], s[k]);
                atomicMax(&K.stats[8 * rep0 + 7], s[7]);
            }
        } else if (on) {
            for (int k = 0; k < 7; k++)
                if (v[k]) atomicAdd(&K.stats[8 * rep + k], v[k]);
            atomicMax(&K.stats[8 * rep + 7], v[7]);
        }
    }
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
        double rest = T.c;
        if (T.lookup == 1) {
            // rest length so that the spring's separation (head distance -
            // rest) is the lookupType 1 stretch at the current geometry
            const int r0 = Q.rodOffset + pr.idBind[0], r1 = Q.rodOffset + pr.idBind[1];
            const KDouble4 C0 = K.rodC[r0], A0 = K.rodA[r0], C1 = K.rodC[r1], A1 = K.rodA[r1];
            const double P0[3] = {C0.x + pr.distBind[0] * A0.x, C0.y + pr.distBind[0] * A0.y,
                                  C0.z + pr.distBind[0] * A0.z};
            double dv[3] = {(C1.x + pr.distBind[1] * A1.x) - P0[0], (C1.y + pr.distBind[1] * A1.y) - P0[1],
                            (C1.z + pr.distBind[1] * A1.z) - P0[2]};
            for (int d = 0; d < 3; d++)
                if (Q.pbc[d]) dv[d] = dv[d] - Q.L[d] * floor(dv[d] / Q.L[d] + 0.5);
            const double ell = sqrt(dv[0] * dv[0] + dv[1] * dv[1] + dv[2] * dv[2]);
            rest = T.ell0 + (K.D * ell) / kmc_dist_point_seg(K, Q, P0, r1);
        }
        S.linkRest[L] = rest;
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
    launch_pdl(k_kmc_bin, dim3(grid_kmc(S.nRods, 256)), dim3(256), 0, st, K, S, 1);
}

void launch_kmc_view(const KmcDev &K, const DevState &S, cudaStream_t st) {
    launch_pdl(k_kmc_bin, dim3(grid_kmc(S.nRods, 256)), dim3(256), 0, st, K, S, 0);
}

void launch_kmc_scatter(const KmcDev &K, const DevState &S, cudaStream_t st) {
    launch_pdl(k_kmc_scatter, dim3(grid_kmc(S.nRods, 256)), dim3(256), 0, st, K, S);
}

// code[] reuses the doubly bound flags' buffer, which the springs pass
// rewrites afterwards
int launch_kmc_bind(const KmcDev &K, cudaStream_t st) {
    if (K.nProt <= 0) return 0;
    KmcTask *task = reinterpret_cast<KmcTask *>(K.task);
    launch_pdl(k_kmc_prep, dim3(grid_kmc(K.nProt, 256)), dim3(256), 0, st, K, K.dScan, task);
    launch_pdl(k_kmc_bind, dim3(grid_kmc(K.nProt, kKmcWarps)), dim3(32 * kKmcWarps), 0, st, K, K.dScan,
               (const KmcTask *)task);
    launch_pdl(k_kmc_geom, dim3(grid_kmc(K.nProt, 256)), dim3(256), 0, st, K);
    launch_pdl(k_kmc_stats, dim3(grid_kmc(K.nProt, 256)), dim3(256), 0, st, K, (const int *)K.dScan);
    return 4;
}

int launch_kmc_motion(const KmcDev &K, const DevState &S, cudaStream_t st) {
    if (K.nProt <= 0) return 0;
    launch_pdl(k_kmc_motion, dim3(grid_kmc(K.nProt, 256)), dim3(256), 0, st, K, S, K.dScan);
    launch_pdl(k_kmc_geom, dim3(grid_kmc(K.nProt, 256)), dim3(256), 0, st, K);
    launch_pdl(k_kmc_stats, dim3(grid_kmc(K.nProt, 256)), dim3(256), 0, st, K, (const int *)K.dScan);
    return 3;
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
