// solve_impl.cuh - persistent BBPGD kernel over the explicit Delassus
// operator (the role of SimToolbox BCQPSolver's BBPGD, conSolverChoice 0,
// docs/source/quickstart.md:356-358; method: Yan, Zhang, Shelley, J. Chem.
// Phys. 150:064109 (2019) with alternating Barzilai-Borwein steps, IMA J.
// Numer. Anal. 8:141 (1988)).
//
// Problem per replica: min 1/2 x^T A x + q^T x  s.t.  x_k >= lb_k
// (lb = -inf on bilateral rows), A = dt D^T M D + diag(cinv).
//
// One cooperative launch runs every iteration of every replica, one grid
// barrier per pass.  Pass p:
//   1. decision (every block, for the replicas of its tiles): canonical
//      reduction of the pass p-1 tile partials -> residual test, step size;
//      the block holding a replica's first tile records its state
//   2. rows (64-constraint tiles, contiguous per block): row k forms
//      x_l for its columns, (A x)_k, the update and the tile partials
//   3. grid barrier
// Passes: 0 = G0 (x = gamma0, g = A x + q, residual), 1 = AG (x = g: step
// g.g / g.Ag), 2.. = iterations x = P(gamma - alpha g).  gamma and g
// ping-pong between two buffers by pass parity; retired replicas copy their
// values forward and mark their partials, so the last buffer always holds
// every replica's final state.
//
// Real = double reproduces the oracle bit for bit (compiled without FMA
// contraction; the fused multiply-adds of the row product are explicit on
// both sides).
// Real = float: FP32 operator, gamma and g, products and per-warp sums;
// FP64 tile/chunk accumulation of the dot products and step sizes; the
// residual min(g, x - lb) is exact for lb = 0 and bilateral rows.
#pragma once

#include "engine.cuh"

namespace alens {

enum SolveMode { kModeCopy = 0, kModeG0 = 1, kModeAG = 2, kModeIter = 3 };
constexpr int kSolveThreads = 256;
constexpr int kRowTile = 64;         // level-1 reduction tile
constexpr int kWindow = 64;          // replicas decided per block window
constexpr int kRowPrefetch = 8;      // row entries loaded together

template <class Real>
struct SolveView {
    const int *aptr;
    const int *acol;
    const Real *aval;
    Real *gam[2];
    Real *g[2];
    const Real *q;
    const Real *lb;
    const Real *cinv;
    double *alphaBuf;   // 2 x R, by pass parity
    int fp64;           // 1: exact oracle arithmetic
};

__device__ __forceinline__ double ldcg(const double *p) { return __ldcg(p); }
__device__ __forceinline__ float ldcg(const float *p) { return __ldcg(p); }
__device__ __forceinline__ int ldcg(const int *p) { return __ldcg(p); }

template <class Real>
__device__ __forceinline__ Real projlb(Real v, Real lb) {
    return v < lb ? lb : v;
}

// Levels >= 2 of the canonical reduction, run by one warp: chunks of 1024
// partials, lane l adds partials l, l+32, ..., l+992 in order, then the warp
// tree; chunk sums are kept in shared memory (up to 64 chunks) and reduced
// the same way until one value remains.  Loads bypass L1 (the partials are
// written by other SMs).  The max over all partials of kind `maxKind`
// (-1: none) is returned in *mx (order-free).  Result valid in lane 0.
template <int NV>
__device__ void warp_chunk_reduce(const double *const (&src)[NV], int m, double (*chunk)[64],
                                  double (&out)[NV], const double *maxSrc, double *mx) {
    const int lane = threadIdx.x & 31;
    double lmax = -2.0;
    int mc = (m + kChunk - 1) / kChunk;
    for (int c = 0; c < mc; c++) {
        double acc[NV];
#pragma unroll
        for (int q = 0; q < NV; q++) acc[q] = 0.0;
#pragma unroll 4
        for (int j = 0; j < 32; j++) {
            const int i = c * kChunk + lane + 32 * j;
            if (i < m) {
#pragma unroll
                for (int q = 0; q < NV; q++) acc[q] = acc[q] + __ldcg(src[q] + i);
                if (maxSrc) {
                    const double v = __ldcg(maxSrc + i);
                    lmax = v > lmax ? v : lmax;
                }
            }
        }
#pragma unroll
        for (int q = 0; q < NV; q++) {
            acc[q] = warp_tree_sum_t<double>(acc[q]);
            if (lane == 0) chunk[q][c] = acc[q];
        }
    }
    __syncwarp();
    while (mc > 1) {
        const int m2 = mc;
        mc = (m2 + kChunk - 1) / kChunk;  // == 1 while m2 <= 1024
        for (int c = 0; c < mc; c++) {
            double acc[NV];
#pragma unroll
            for (int q = 0; q < NV; q++) acc[q] = 0.0;
            for (int j = 0; j < 32; j++) {
                const int i = c * kChunk + lane + 32 * j;
                if (i < m2) {
#pragma unroll
                    for (int q = 0; q < NV; q++) acc[q] = acc[q] + chunk[q][i];
                }
            }
            __syncwarp();
#pragma unroll
            for (int q = 0; q < NV; q++) {
                acc[q] = warp_tree_sum_t<double>(acc[q]);
                if (lane == 0) chunk[q][c] = acc[q];
            }
            __syncwarp();
        }
    }
#pragma unroll
    for (int q = 0; q < NV; q++) out[q] = m > 0 ? chunk[q][0] : 0.0;
    if (mx) *mx = warp_max(lmax);
}

struct SolveShared {
    double chunk[3][64];
    double alpha[kWindow];
    int mode[kWindow];
    double tileVal[4][2][4];  // [group][warp][kind]
};

// Decision of replica r at pass p from the pass p-1 partials; identical in
// every block that evaluates it.
template <class Real>
__device__ void decide(const DevState &S, const SolveView<Real> &V, int p, int r, int t0, int t1,
                       SolveShared &sh, int slot) {
    const RepDyn &d = S.dyn[r];
    const RepParams &P = S.par[r];
    if (p == 0) {
        if (threadIdx.x == 0) {
            sh.mode[slot] = kModeG0;
            sh.alpha[slot] = 0.0;
            if (d.nCon > 0 && d.tileStart >= t0 && d.tileStart < t1) atomicAdd(&S.ctl->activeCnt[0], 1);
        }
        __syncthreads();
        return;
    }
    const int par = (p - 1) & 1;
    const size_t tc = (size_t)S.tileCap;
    const double *base = S.part + (size_t)par * 4 * tc;
    if (threadIdx.x < 32) {
        const double *const src[3] = {base + d.tileStart, base + tc + d.tileStart, base + 2 * tc + d.tileStart};
        double sums[3], mx;
        warp_chunk_reduce<3>(src, d.nTiles, sh.chunk, sums, base + 3 * tc + d.tileStart, &mx);
        if (threadIdx.x == 0) {
        const bool owner = d.tileStart >= t0 && d.tileStart < t1;
        int mode = kModeCopy;
        double alpha = 0.0;
        int status = -1, iter = 0;
        if (mx < 0.0) {
            mode = kModeCopy;  // retired in an earlier pass
        } else if (p == 1) {
            if (isinf(mx))
                status = ALENS_NAN_DETECTED;
            else if (mx <= P.tol)
                status = ALENS_OK;
            else if (P.maxIte <= 0)
                status = ALENS_NOT_CONVERGED;
            else
                mode = kModeAG;
        } else if (p == 2) {
            const double gg = sums[0], gAg = sums[1];
            alpha = (gAg > 0.0) ? gg / gAg : 1.0;
            if (!(alpha > 0.0) || isinf(alpha)) alpha = 1.0;
            mode = kModeIter;
        } else {
            const int itp = p - 2;
            iter = itp;
            if (isinf(mx)) {
                status = ALENS_NAN_DETECTED;
            } else if (mx <= P.tol) {
                status = ALENS_OK;
            } else {
                alpha = __ldcg(V.alphaBuf + (size_t)((p - 1) & 1) * S.R + r);
                const double ss = sums[0], sy = sums[1], yy = sums[2];
                if (sy > 0.0) {
                    const double a = (itp & 1) ? ss / sy : sy / yy;
                    if (a > 0.0 && !isinf(a)) alpha = a;
                }
                if (itp >= P.maxIte)
                    status = ALENS_NOT_CONVERGED;
                else
                    mode = kModeIter;
            }
        }
        sh.mode[slot] = mode;
        sh.alpha[slot] = alpha;
        if (owner) {
            if (status >= 0) {
                RepDyn *dw = &S.dyn[r];
                dw->status = status;
                dw->converged = status == ALENS_OK ? 1 : 0;
                dw->iter = iter;
                dw->res = mx;
                dw->active = 0;
            }
            if (mode != kModeCopy) {
                atomicAdd(&S.ctl->activeCnt[p % 3], 1);
                __stcg(V.alphaBuf + (size_t)(p & 1) * S.R + r, alpha);
            }
        }
        }
    }
    __syncthreads();
}

// One 64-constraint tile processed by a 64-thread group (two warps).
template <class Real>
__device__ void process_tile(const DevState &S, const SolveView<Real> &V, int p, int T, int mode,
                             Real alpha, SolveShared &sh, int group) {
    const int lane64 = threadIdx.x & 63;
    const int warpInGroup = (threadIdx.x >> 5) & 1;
    const int r = __ldg(S.tileRep + T);
    const RepDyn &d = S.dyn[r];
    const int local = (T - d.tileStart) * kRowTile + lane64;
    const bool valid = local < d.nCon;
    const int k = d.conStart + local;
    const int inB = (p + 1) & 1, outB = p & 1;
    Real v0 = Real(0), v1 = Real(0), v2 = Real(0);
    double rmax = 0.0;
    if (mode == kModeCopy) {
        rmax = -1.0;
        if (valid) {
            V.gam[outB][k] = ldcg(V.gam[inB] + k);
            V.g[outB][k] = ldcg(V.g[inB] + k);
        }
    } else if (valid) {
        const Real gam = ldcg(V.gam[inB] + k);
        const Real gold = mode == kModeG0 ? Real(0) : ldcg(V.g[inB] + k);
        const Real lbk = __ldg(V.lb + k);
        Real xk;
        if (mode == kModeG0)
            xk = gam;
        else if (mode == kModeAG)
            xk = gold;
        else
            xk = projlb<Real>(fma(-alpha, gold, gam), lbk);
        // row k of A: columns and values first, then the column iterates,
        // so that each group of loads is independent
        Real acc = Real(0);
        const int e0 = __ldg(V.aptr + k), e1 = __ldg(V.aptr + k + 1);
        for (int eb = e0; eb < e1; eb += kRowPrefetch) {
            int cols[kRowPrefetch];
            Real vals[kRowPrefetch];
#pragma unroll
            for (int j = 0; j < kRowPrefetch; j++) {
                cols[j] = eb + j < e1 ? __ldg(V.acol + eb + j) : k;
                vals[j] = eb + j < e1 ? __ldg(V.aval + eb + j) : Real(0);
            }
            Real xa[kRowPrefetch], xb[kRowPrefetch], xc[kRowPrefetch];
#pragma unroll
            for (int j = 0; j < kRowPrefetch; j++) {
                if (eb + j < e1) {
                    const int l = cols[j];
                    if (mode == kModeG0) {
                        xa[j] = ldcg(V.gam[inB] + l);
                    } else if (mode == kModeAG) {
                        xa[j] = ldcg(V.g[inB] + l);
                    } else {
                        xa[j] = ldcg(V.gam[inB] + l);
                        xb[j] = ldcg(V.g[inB] + l);
                        xc[j] = __ldg(V.lb + l);
                    }
                }
            }
#pragma unroll
            for (int j = 0; j < kRowPrefetch; j++) {
                if (eb + j < e1) {
                    const Real xl = mode == kModeIter ? projlb<Real>(fma(-alpha, xb[j], xa[j]), xc[j]) : xa[j];
                    acc = fma(vals[j], xl, acc);
                }
            }
        }
        acc = fma(__ldg(V.cinv + k), xk, acc);
        if (mode == kModeAG) {
            v0 = gold * gold;
            v1 = gold * acc;
            V.gam[outB][k] = gam;
            V.g[outB][k] = gold;
        } else {
            const Real gn = acc + __ldg(V.q + k);
            if (V.fp64) {
                const double xd = (double)xk;
                const double gd = (double)gn;
                rmax = fabs(xd - projlb<double>(xd - gd, (double)lbk));
            } else {
                // x - P(x - g) = min(g, x - lb): exact for lb = 0 and lb = -inf
                const Real m = gn < xk - lbk ? gn : xk - lbk;
                rmax = fabs((double)m);
            }
            if (rmax != rmax) {
                atomicOr(&S.ctl->errFlags, kErrNaN);
                rmax = INFINITY;
            }
            if (mode == kModeIter) {
                const Real s = xk - gam;
                const Real y = gn - gold;
                v0 = s * s;
                v1 = s * y;
                v2 = y * y;
            }
            V.gam[outB][k] = xk;
            V.g[outB][k] = gn;
        }
    }
    // warp trees in Real, tile = warp0 + warp1 in FP64
    Real w0 = warp_tree_sum_t<Real>(v0);
    Real w1 = warp_tree_sum_t<Real>(v1);
    Real w2 = warp_tree_sum_t<Real>(v2);
    double wm = warp_max(rmax);
    if ((threadIdx.x & 31) == 0) {
        sh.tileVal[group][warpInGroup][0] = (double)w0;
        sh.tileVal[group][warpInGroup][1] = (double)w1;
        sh.tileVal[group][warpInGroup][2] = (double)w2;
        sh.tileVal[group][warpInGroup][3] = wm;
    }
}

template <class Real>
__global__ void __launch_bounds__(kSolveThreads) k_solve(DevState S, SolveView<Real> V,
                                                         unsigned long long timeout_ns) {
    __shared__ SolveShared sh;
    if (ld_volatile_i32(&S.ctl->errFlags) & (kErrOverflow | kErrNaN | kErrTimeout)) return;
    const unsigned int nb = gridDim.x;
    const int nTiles = S.ctl->nTiles;
    const int tpb = (nTiles + (int)nb - 1) / (int)nb;
    const int t0 = min((int)blockIdx.x * tpb, nTiles);
    const int t1 = min(t0 + tpb, nTiles);
    const int maxPass = S.ctl->maxIte + 3;
    const size_t tc = (size_t)S.tileCap;
    const int group = threadIdx.x >> 6;
    int lastPass = 0;
    for (int p = 0; p <= maxPass; p++) {
        if (blockIdx.x == 0 && threadIdx.x == 0) S.ctl->activeCnt[(p + 1) % 3] = 0;
        double *partBase = S.part + (size_t)(p & 1) * 4 * tc;
        // replica windows of this block's tile range
        int T = t0;
        while (T < t1) {
            const int rFirst = __ldg(S.tileRep + T);
            const int rLast = min(__ldg(S.tileRep + t1 - 1), rFirst + kWindow - 1);
            for (int r = rFirst; r <= rLast; r++) decide<Real>(S, V, p, r, t0, t1, sh, r - rFirst);
            // tiles of the window, four per round
            int Tend = T;
            while (Tend < t1 && __ldg(S.tileRep + Tend) <= rLast) Tend++;
            for (int base = T; base < Tend; base += 4) {
                const int Tg = base + group;
                if (Tg < Tend) {
                    const int slot = __ldg(S.tileRep + Tg) - rFirst;
                    process_tile<Real>(S, V, p, Tg, sh.mode[slot], (Real)sh.alpha[slot], sh, group);
                }
                __syncthreads();
                if (threadIdx.x < 4 && base + (int)threadIdx.x < Tend) {
                    const int g = threadIdx.x;
                    const int Tw = base + g;
#pragma unroll
                    for (int q = 0; q < 3; q++)
                        __stcg(partBase + q * tc + Tw, sh.tileVal[g][0][q] + sh.tileVal[g][1][q]);
                    const double a = sh.tileVal[g][0][3], b = sh.tileVal[g][1][3];
                    __stcg(partBase + 3 * tc + Tw, a > b ? a : b);
                }
                __syncthreads();
            }
            T = Tend;
        }
        lastPass = p;
        if (!grid_sync(&S.ctl->bar, nb, &S.ctl->errFlags, timeout_ns)) return;
        if (ldcg(&S.ctl->activeCnt[p % 3]) == 0) break;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) S.ctl->finalParity = lastPass & 1;
}

}  // namespace alens
