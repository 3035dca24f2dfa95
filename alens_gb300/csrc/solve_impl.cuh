// solve_impl.cuh - persistent BBPGD kernel (the role of SimToolbox
// BCQPSolver's BBPGD, conSolverChoice 0, docs/source/quickstart.md:356-358;
// method: Yan, Zhang, Shelley, J. Chem. Phys. 150:064109 (2019) with
// Barzilai-Borwein steps, IMA J. Numer. Anal. 8:141 (1988)).
//
// Problem per replica: min 1/2 g^T A g + q^T g  s.t.  gamma_k >= lb_k
// (lb = -inf for bilateral rows), A = dt D^T M D + diag(cinv).
//
// One cooperative launch runs every iteration of every replica.  Each pass is
//   phase A (per rod):        x = source vector, F = D x, U = M F
//   grid barrier
//   phase B (per 256-tile):   (A x)_k = dt (D_I.U_I + D_J.U_J) + cinv_k x_k,
//                             per-constraint update, tile partial sums
//   last block of a replica:  canonical reduction of its tiles -> step size,
//                             residual, convergence
//   grid barrier
// Passes: G0 (x = gamma0: g0 = A gamma0 + q, residual), AG (x = g0: initial
// step g.g / g.Ag), then iterations x = P(gamma - alpha g).
//
// Real = double: the oracle's arithmetic bit for bit (compiled without FMA).
// Real = float: FP32 Jacobian, velocities, gamma and g; FP64 dot products,
// residual and step sizes.
#pragma once

#include "engine.cuh"

namespace alens {

enum SolveMode { kModeG0 = 0, kModeAG = 1, kModeIter = 2 };

template <class Real>
struct SolveView {
    const Real *jac;
    Real *gamma;
    Real *g;
    const Real *q;
    const Real *lb;
    const Real *cinv;
    Real *U;
};

__device__ __forceinline__ double ldcg(const double *p) { return __ldcg(p); }
__device__ __forceinline__ float ldcg(const float *p) { return __ldcg(p); }
__device__ __forceinline__ int ldcg(const int *p) { return __ldcg(p); }

template <class Real>
__device__ __forceinline__ Real projlb(Real v, Real lb) {
    return v < lb ? lb : v;
}

template <class Real>
__device__ __forceinline__ Real dot6u(const Real *J, const Real *U, size_t st, int r) {
    return J[0] * ldcg(U + r) + J[1] * ldcg(U + st + r) + J[2] * ldcg(U + 2 * st + r) +
           J[3] * ldcg(U + 3 * st + r) + J[4] * ldcg(U + 4 * st + r) + J[5] * ldcg(U + 5 * st + r);
}

template <class Real>
__device__ __forceinline__ Real source_x(int mode, Real gam, Real gold, Real alpha, Real lb) {
    if (mode == kModeG0) return gam;
    if (mode == kModeAG) return gold;
    return projlb<Real>(gam - alpha * gold, lb);
}

template <class Real>
__device__ void phase_rods(const DevState &S, const SolveView<Real> &V, int mode) {
    const size_t st = (size_t)S.nRods;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < S.nRods; r += gridDim.x * blockDim.x) {
        const int rep = __ldg(S.rodRep + r);
        if (!ldcg(&S.dyn[rep].active)) continue;
        const Real alpha = (Real)ldcg(&S.dyn[rep].alpha);
        Real F[6] = {Real(0), Real(0), Real(0), Real(0), Real(0), Real(0)};
        const int e1 = __ldg(S.rowPtr + r + 1);
        for (int e = __ldg(S.rowPtr + r); e < e1; e++) {
            const int ent = __ldg(S.rowEnt + e);
            const int k = ent >> 1;
            const Real x = source_x<Real>(mode, ldcg(V.gamma + k), ldcg(V.g + k), alpha, __ldg(V.lb + k));
            const Real *J = V.jac + 12 * (size_t)k + 6 * (ent & 1);
#pragma unroll
            for (int c = 0; c < 6; c++) F[c] = F[c] + x * __ldg(J + c);
        }
        Real Uo[6] = {Real(0), Real(0), Real(0), Real(0), Real(0), Real(0)};
        if (!__ldg(S.imm + r)) {
            const Real a[3] = {(Real)__ldg(S.ax + r), (Real)__ldg(S.ay + r), (Real)__ldg(S.az + r)};
            const Real m[3] = {(Real)__ldg(S.m0 + r), (Real)__ldg(S.m1 + r), (Real)__ldg(S.m2 + r)};
            mobility_apply<Real>(a, m, __ldg(S.sph + r) != 0, S.par[rep].mono != 0, F, Uo);
        }
#pragma unroll
        for (int c = 0; c < 6; c++) V.U[c * st + r] = Uo[c];
    }
}

// chunk reduction of tile partials with L2-coherent loads
template <int NV>
__device__ void chunk_reduce_cg(const double *const (&src)[NV], int m, double *const (&work)[NV],
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
                    if (i < m) acc = acc + __ldcg(cur[q] + i);
                }
                v[q] = acc;
            }
            block_tree_sum256<NV>(v, scratch);
            if (threadIdx.x == 0) {
#pragma unroll
                for (int q = 0; q < NV; q++) __stcg(work[q] + c, v[q]);
            }
            __syncthreads();
        }
        if (mc == 1) {
#pragma unroll
            for (int q = 0; q < NV; q++) out[q] = __ldcg(work[q]);
            return;
        }
#pragma unroll
        for (int q = 0; q < NV; q++) cur[q] = work[q];
        m = mc;
    }
}

__device__ __forceinline__ void retire(DevCtl *ctl, RepDyn *d, int status, int converged) {
    d->status = status;
    d->converged = converged;
    d->active = 0;
    atomicSub(&ctl->activeCount, 1);
}

// Final reduction and state update of replica `rep`, run by its last block.
template <class Real>
__device__ void replica_update(const DevState &S, int rep, int mode, int it, double (*scr)[8],
                              double *scrmax) {
    RepDyn *d = &S.dyn[rep];
    const int t0 = d->tileStart, nt = d->nTiles;
    const size_t tc = (size_t)S.tileCap, wc = (size_t)S.workCap;
    const double *const src[3] = {S.part + t0, S.part + tc + t0, S.part + 2 * tc + t0};
    double *const work[3] = {S.work, S.work + wc, S.work + 2 * wc};
    double sums[3];
    chunk_reduce_cg<3>(src, nt, work, sums, scr);
    double mx = 0.0;
    for (int i = threadIdx.x; i < nt; i += blockDim.x) {
        const double v = __ldcg(S.part + 3 * tc + t0 + i);
        mx = v > mx ? v : mx;
    }
    mx = block_max256(mx, scrmax);
    if (threadIdx.x == 0) {
        const RepParams &P = S.par[rep];
        DevCtl *ctl = S.ctl;
        if (mode == kModeG0) {
            d->res = mx;
            if (isinf(mx))
                retire(ctl, d, ALENS_NAN_DETECTED, 0);
            else if (mx <= P.tol)
                retire(ctl, d, ALENS_OK, 1);
            else if (P.maxIte <= 0)
                retire(ctl, d, ALENS_NOT_CONVERGED, 0);
        } else if (mode == kModeAG) {
            const double gg = sums[0], gAg = sums[1];
            double alpha = (gAg > 0.0) ? gg / gAg : 1.0;
            if (!(alpha > 0.0) || isinf(alpha)) alpha = 1.0;
            d->alpha = alpha;
        } else {
            d->iter = it;
            d->res = mx;
            if (isinf(mx)) {
                retire(ctl, d, ALENS_NAN_DETECTED, 0);
            } else if (mx <= P.tol) {
                retire(ctl, d, ALENS_OK, 1);
            } else {
                const double ss = sums[0], sy = sums[1], yy = sums[2];
                if (sy > 0.0) {
                    const double a = (it & 1) ? ss / sy : sy / yy;
                    if (a > 0.0 && !isinf(a)) d->alpha = a;
                }
                if (it >= P.maxIte) retire(ctl, d, ALENS_NOT_CONVERGED, 0);
            }
        }
        d->counter = 0;
        __threadfence();
    }
    __syncthreads();
}

template <class Real>
__device__ void phase_tiles(const DevState &S, const SolveView<Real> &V, int mode, int it,
                            double (*scr)[8], double *scrmax, int *s_last) {
    const size_t st = (size_t)S.nRods;
    const size_t tc = (size_t)S.tileCap;
    const int nTiles = S.ctl->nTiles;
    for (int T = blockIdx.x; T < nTiles; T += gridDim.x) {
        const int rep = __ldg(S.tileRep + T);
        RepDyn *d = &S.dyn[rep];
        if (!ldcg(&d->active)) continue;
        const int local = (T - d->tileStart) * kTile + (int)threadIdx.x;
        const int k = d->conStart + local;
        double v[3] = {0.0, 0.0, 0.0};
        double r = 0.0;
        if (local < d->nCon) {
            const Real alpha = (Real)ldcg(&d->alpha);
            const Real *J = V.jac + 12 * (size_t)k;
            const int I = __ldg(S.conI + k), Jr = __ldg(S.conJ + k);
            const Real dI = dot6u<Real>(J, V.U, st, I);
            const Real dJ = Jr >= 0 ? dot6u<Real>(J + 6, V.U, st, Jr) : Real(0);
            const Real gam = ldcg(V.gamma + k), gold = ldcg(V.g + k);
            const Real lbk = __ldg(V.lb + k);
            const Real x = source_x<Real>(mode, gam, gold, alpha, lbk);
            Real Ax = (Real)S.par[rep].dt * (dI + dJ);
            Ax = Ax + __ldg(V.cinv + k) * x;
            if (mode == kModeAG) {
                const double gd = (double)gold;
                v[0] = gd * gd;
                v[1] = gd * (double)Ax;
            } else {
                const Real gn = Ax + __ldg(V.q + k);
                const double xd = (double)x, gnd = (double)gn, lbd = (double)lbk;
                r = fabs(xd - projlb<double>(xd - gnd, lbd));
                if (mode == kModeIter) {
                    const double s = xd - (double)gam;
                    const double y = gnd - (double)gold;
                    v[0] = s * s;
                    v[1] = s * y;
                    v[2] = y * y;
                    V.gamma[k] = x;
                }
                V.g[k] = gn;
                if (r != r) {
                    atomicOr(&S.ctl->errFlags, kErrNaN);
                    r = INFINITY;
                }
            }
        }
        block_tree_sum256<3>(v, scr);
        r = block_max256(r, scrmax);
        if (threadIdx.x == 0) {
            __stcg(S.part + T, v[0]);
            __stcg(S.part + tc + T, v[1]);
            __stcg(S.part + 2 * tc + T, v[2]);
            __stcg(S.part + 3 * tc + T, r);
            __threadfence();
            const int ticket = atomicAdd(&d->counter, 1);
            *s_last = (ticket == d->nTiles - 1);
        }
        __syncthreads();
        if (*s_last) {
            __threadfence();
            replica_update<Real>(S, rep, mode, it, scr, scrmax);
        }
        __syncthreads();
    }
}

template <class Real>
__global__ void __launch_bounds__(256) k_solve(DevState S, SolveView<Real> V,
                                               unsigned long long timeout_ns) {
    __shared__ double scr[3][8];
    __shared__ double scrmax[8];
    __shared__ int s_last;
    if (ld_volatile_i32(&S.ctl->errFlags) & (kErrOverflow | kErrNaN | kErrTimeout)) return;
    const unsigned int nb = gridDim.x;
    const int maxIte = S.ctl->maxIte;
    for (int pass = 0;; pass++) {
        const int mode = pass == 0 ? kModeG0 : (pass == 1 ? kModeAG : kModeIter);
        const int it = pass - 1;
        if (mode == kModeIter && it > maxIte) break;
        if (ldcg(&S.ctl->activeCount) <= 0) break;
        phase_rods<Real>(S, V, mode);
        if (!grid_sync(&S.ctl->bar, nb, &S.ctl->errFlags, timeout_ns)) return;
        phase_tiles<Real>(S, V, mode, it, scr, scrmax, &s_last);
        if (!grid_sync(&S.ctl->bar, nb, &S.ctl->errFlags, timeout_ns)) return;
    }
}

}  // namespace alens
