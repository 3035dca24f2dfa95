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
//      the block holding a replica's first tile records its state.  Under
//      it, the upper warps copy the previous iterates of the columns of the
//      block's cached operator rows into shared memory (cp.async)
//   2. rows (64-constraint tiles, contiguous per block): row k forms
//      x_l for its columns, (A x)_k, the update and the tile partials
//   3. grid barrier (per-pass counter polled by every block; the arrival
//      word also counts the replicas still iterating, which decides stop)
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
// FP64 tile/chunk accumulation of the dot products; the step-size quotient
// in FP32 (the step is used in FP32); the residual min(g, x - lb) is exact
// for lb = 0 and bilateral rows.
#pragma once

#include <cstdio>

#include "engine.cuh"

namespace alens {

enum SolveMode { kModeCopy = 0, kModeG0 = 1, kModeAG = 2, kModeIter = 3 };
constexpr int kSolveThreads = 256;
constexpr int kRowTile = 64;         // level-1 reduction tile
constexpr int kWindow = 64;          // replicas decided per block window
constexpr int kRowPrefetch = 8;      // row entries loaded together
#ifndef ALENS_ROW_PREFETCH_F32
#define ALENS_ROW_PREFETCH_F32 8
#endif
// entries per gather batch of the FP32 form (8: with 16 the kernel spills
// past its 128-register budget and runs ~5 % slower)
template <class Real>
struct RowBatch {
    static constexpr int value = kRowPrefetch;
};
template <>
struct RowBatch<float> {
    static constexpr int value = ALENS_ROW_PREFETCH_F32;
};

template <class Real>
struct Vec2;
template <>
struct Vec2<double> {
    using T = double2;
};
template <>
struct Vec2<float> {
    using T = float2;
};

// Packed solver data (one memory request per operator entry and per
// neighbour):
//  st[parity][k] = (gamma, g) of constraint k,
//  qc[k]         = (q, cinv),
//  aent[e]       = (column, lower-bound kind, value) of row entries:
//                  FP64 {col, kind, lo32(val), hi32(val)},
//                  FP32 {col, kind, bits(val), bits(lb)};
//  lower-bound kind 0: lb = 0 (collisions), 1: bilateral (no bound),
//  2: general (FP64 value in lbGeneral).
template <class Real>
struct SolveView {
    using V2 = typename Vec2<Real>::T;
    const int *aptr;
    const int4 *aent;
    V2 *st[2];
    const V2 *qc;
    const double *lbGeneral;
    double *alphaBuf;   // 2 x R, by pass parity
    int fp64;           // 1: exact oracle arithmetic
};

__device__ __forceinline__ double ldcg(const double *p) { return __ldcg(p); }
__device__ __forceinline__ float ldcg(const float *p) { return __ldcg(p); }
__device__ __forceinline__ int ldcg(const int *p) { return __ldcg(p); }
__device__ __forceinline__ double2 ldcg(const double2 *p) { return __ldcg(p); }
__device__ __forceinline__ float2 ldcg(const float2 *p) { return __ldcg(p); }

template <class Real>
__device__ __forceinline__ void decode_entry(const int4 &e, const double *lbGeneral, int &col, Real &val, Real &lb);

template <>
__device__ __forceinline__ void decode_entry<double>(const int4 &e, const double *lbGeneral, int &col, double &val,
                                                     double &lb) {
    col = e.x;
    val = __hiloint2double(e.w, e.z);
    lb = e.y == 0 ? 0.0 : (e.y == 1 ? -INFINITY : lbGeneral[e.x]);
}

template <>
__device__ __forceinline__ void decode_entry<float>(const int4 &e, const double *, int &col, float &val,
                                                    float &lb) {
    col = e.x;
    val = __int_as_float(e.z);
    lb = __int_as_float(e.w);
}

template <class Real>
__device__ __forceinline__ Real projlb(Real v, Real lb) {
    return v < lb ? lb : v;
}

// Levels >= 2 of the canonical reduction for one kind, run by one warp:
// chunks of 1024 partials, lane l adds partials l, l+32, ..., l+992 in
// order, then the warp tree; chunk sums are kept in shared memory (up to 64
// chunks) and reduced the same way until one value remains.  All loads of a
// chunk are issued before the adds; they bypass L1 (the partials are
// written by other SMs).  Result valid in lane 0.
__device__ inline double warp_chunk_sum(const double *src, int m, double *chunk) {
    const int lane = threadIdx.x & 31;
    int mc = (m + kChunk - 1) / kChunk;
    for (int c = 0; c < mc; c++) {
        double v[32];
#pragma unroll
        for (int j = 0; j < 32; j++) {
            const int i = c * kChunk + lane + 32 * j;
            v[j] = i < m ? __ldcg(src + i) : 0.0;
        }
        // only this lane's valid partials are added (same order as before):
        // each FP64 add of a full warp occupies the SM's FP64 pipe for 16
        // cycles on GB300
        double acc = 0.0;
#pragma unroll
        for (int j = 0; j < 32; j++) {
            if (c * kChunk + 32 * j >= m) break;  // uniform across the warp
            if (c * kChunk + lane + 32 * j < m) acc = acc + v[j];
        }
        acc = warp_tree_sum_t<double>(acc);
        if (lane == 0) chunk[c] = acc;
    }
    __syncwarp();
    while (mc > 1) {
        const int m2 = mc;
        mc = (m2 + kChunk - 1) / kChunk;
        for (int c = 0; c < mc; c++) {
            double acc = 0.0;
            for (int j = 0; j < 32; j++) {
                const int i = c * kChunk + lane + 32 * j;
                if (i < m2) acc = acc + chunk[i];
            }
            __syncwarp();
            acc = warp_tree_sum_t<double>(acc);
            if (lane == 0) chunk[c] = acc;
            __syncwarp();
        }
    }
    return m > 0 ? chunk[0] : 0.0;
}

// Max of m non-negative doubles (or all equal negative markers) through
// their bit patterns as signed 64-bit integers: no FP64 instructions.
__device__ __forceinline__ long long warp_max_bits(long long v) {
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) {
        const long long o = __shfl_down_sync(0xffffffffu, v, off);
        v = o > v ? o : v;
    }
    return v;
}

__device__ inline double warp_max_of(const double *src, int m) {
    const int lane = threadIdx.x & 31;
    long long mx = __double_as_longlong(-2.0);
    // all loads of a 1024-partial chunk are issued before the compares
    for (int c = 0; c < m; c += kChunk) {
        long long b[32];
#pragma unroll
        for (int j = 0; j < 32; j++) {
            const int i = c + lane + 32 * j;
            b[j] = i < m ? __double_as_longlong(__ldcg(src + i)) : mx;
        }
#pragma unroll
        for (int j = 0; j < 32; j++) mx = b[j] > mx ? b[j] : mx;
    }
    mx = warp_max_bits(mx);
    return __longlong_as_double(mx);
}

// Multi-kind form used by the stress sum (one warp does every kind).
template <int NV>
__device__ void warp_chunk_reduce(const double *const (&src)[NV], int m, double (*chunk)[64],
                                  double (&out)[NV], const double *, double *) {
#pragma unroll
    for (int q = 0; q < NV; q++) out[q] = warp_chunk_sum(src[q], m, chunk[q]);
}

struct SolveShared {
    double chunk[3][64];
    double red[4];
    double alpha[kWindow];
    int mode[kWindow];
    double tileVal[4][2][4];  // [group][warp][kind]
    int act;                  // replicas owned by this block iterating in this pass
#ifdef ALENS_TRACE
    long long trRed;
#endif
};

// Step-size quotient: the FP32 form uses its step in FP32, so its quotient
// is formed in FP32 (a few cycles instead of a dependent FP64 divide
// sequence on the 2-lane FP64 pipe); the FP64 form keeps the oracle's FP64
// divide.
template <class Real>
__device__ __forceinline__ double step_quot(double num, double den) {
    if constexpr (sizeof(Real) == 4)
        return (double)__fdiv_rn((float)num, (float)den);
    else
        return num / den;
}

// Decision of replica r at pass p from the pass p-1 partials; identical in
// every block that evaluates it.
template <class Real>
__device__ void decide(const DevState &S, const SolveView<Real> &V, int p, int r, int t0, int t1,
                       SolveShared &sh, int slot) {
    // fields that do not change while the solver runs go through the
    // read-only cache (hits after the first pass)
    const RepDyn *dr = S.dyn + r;
    const int dTileStart = __ldg(&dr->tileStart), dNTiles = __ldg(&dr->nTiles);
    const double Ptol = __ldg(&S.par[r].tol);
    const int PmaxIte = __ldg(&S.par[r].maxIte);
    if (p == 0) {
        if (threadIdx.x == 0) {
            const RepDyn &d = *dr;
            const bool done = d.refined != 0;
            sh.mode[slot] = done ? kModeCopy : kModeG0;
            sh.alpha[slot] = 0.0;
            if (!done && d.nCon > 0 && d.tileStart >= t0 && d.tileStart < t1) sh.act++;
        }
        __syncthreads();
        return;
    }
    const int par = (p - 1) & 1;
    const size_t tc = (size_t)S.tileCap;
    const double *base = S.part + (size_t)par * 4 * tc;
    // the previous step size (written before the last barrier), loaded
    // while the partials are reduced
    const double alphaPrev = (threadIdx.x == 0 && p > 2) ? __ldcg(V.alphaBuf + (size_t)((p - 1) & 1) * S.R + r) : 0.0;
    // warps 0-2: the three dot products, warp 3: the residual max
    const int warp = threadIdx.x >> 5;
    if (warp < 3) {
        const double v = warp_chunk_sum(base + (size_t)warp * tc + dTileStart, dNTiles, sh.chunk[warp]);
        if ((threadIdx.x & 31) == 0) sh.red[warp] = v;
    } else if (warp == 3) {
        const double v = warp_max_of(base + 3 * tc + dTileStart, dNTiles);
        if ((threadIdx.x & 31) == 0) sh.red[3] = v;
    }
    __syncthreads();
#ifdef ALENS_TRACE
    if (threadIdx.x == 0) sh.trRed = clock64();
#endif
    {
        const double sums[3] = {sh.red[0], sh.red[1], sh.red[2]};
        const double mx = sh.red[3];
        if (threadIdx.x == 0) {
        const struct {
            double tol;
            int maxIte;
        } P{Ptol, PmaxIte};
        const bool owner = dTileStart >= t0 && dTileStart < t1;
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
            alpha = (gAg > 0.0) ? step_quot<Real>(gg, gAg) : 1.0;
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
                alpha = alphaPrev;
                const double ss = sums[0], sy = sums[1], yy = sums[2];
                if (sy > 0.0) {
                    const double a = (itp & 1) ? step_quot<Real>(ss, sy) : step_quot<Real>(sy, yy);
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
                sh.act++;
                __stcg(V.alphaBuf + (size_t)(p & 1) * S.R + r, alpha);
            }
        }
        }
    }
    __syncthreads();
}

// Operator rows of one block cached in shared memory for the whole solve
// (the rows a block owns do not change between passes): entries
// [entBase, entBase + nEnt) and row pointers of rows [rowBase, rowBase +
// nRow].  Entries or rows outside are read from global memory.  gv holds,
// per cached entry, the previous iterate (gamma, g) of the entry's column,
// gathered at the start of each pass (see gather_columns).
struct RowCache {
    const int4 *ent;
    const int *rptr;
    const void *gv;
    int entBase, nEnt;
    int rowBase, nRow;
};

constexpr int kRowCacheRows = 1024;                  // row pointers cached per block
constexpr int kSolveDynSmem = 96 * 1024;             // dynamic shared memory of k_solve
// entries cached per block: an int4 entry plus its gathered column iterate
template <class Real>
__host__ __device__ constexpr int row_cache_ents() {
    return (kSolveDynSmem - 4 * (kRowCacheRows + 4)) / (16 + (int)sizeof(typename Vec2<Real>::T));
}
constexpr int kGatherWarp0 = 4;                      // warps kGatherWarp0.. gather
static_assert(kMaxSolverGrid < (1 << kBarActShift), "barrier arrival field too narrow");

// Start of a pass: the upper warps copy the previous iterate of every
// cached entry's column into shared memory (asynchronous copies, all in
// flight together, no registers held) while the lower warps reduce the
// previous pass's partials (decide); the row updates then read their
// neighbours from shared memory.  Each gathering thread waits for its own
// copies; the __syncthreads that follows publishes them to the block.
template <class Real>
__device__ __forceinline__ void gather_columns(const RowCache &C, const typename Vec2<Real>::T *stIn) {
    using V2 = typename Vec2<Real>::T;
    const int nt = (int)blockDim.x - 32 * kGatherWarp0;
    const int t = (int)threadIdx.x - 32 * kGatherWarp0;
    if (t < 0 || C.nEnt <= 0) return;
    const unsigned int gvBase = (unsigned int)__cvta_generic_to_shared(C.gv);
#pragma unroll 4
    for (int e = t; e < C.nEnt; e += nt) {
        const V2 *src = stIn + C.ent[e].x;  // L1-cacheable: written before the last barrier
        const unsigned int dst = gvBase + (unsigned int)(e * (int)sizeof(V2));
        if constexpr (sizeof(V2) == 16)
            asm volatile("cp.async.ca.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
        else
            asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(dst), "l"(src) : "memory");
    }
    asm volatile("cp.async.wait_all;" ::: "memory");
}

// Update of constraint k at pass p in `mode`: reads the previous iterates,
// forms x_k and (A x)_k, writes the new iterates, returns the dot-product
// terms (v0, v1, v2) and the residual term.  Row k always holds its own
// diagonal entry, which supplies gamma_k, g_k and the bound of k.
template <class Real>
__device__ __forceinline__ void row_update(const SolveView<Real> &V, int k, int mode, Real alpha,
                                           const typename Vec2<Real>::T *stIn, typename Vec2<Real>::T *stOut,
                                           Real &v0, Real &v1, Real &v2, Real &rmax, int *errFlags,
                                           const RowCache &C) {
    using V2 = typename Vec2<Real>::T;
    if (mode == kModeCopy) {
        stOut[k] = ldcg(stIn + k);
        return;
    }
    const V2 qc = __ldg(V.qc + k);
    Real acc = Real(0);
    Real gam = Real(0), gold = Real(0), lbk = Real(0), xk = Real(0);
    const int kr = k - C.rowBase;
    const bool rc = kr >= 0 && kr < C.nRow;
    const int e0 = rc ? C.rptr[kr] : __ldg(V.aptr + k), e1 = rc ? C.rptr[kr + 1] : __ldg(V.aptr + k + 1);
    constexpr int B = RowBatch<Real>::value;
    const int ce0 = e0 - C.entBase, ce1 = e1 - C.entBase;
    if (ce0 >= 0 && ce1 <= C.nEnt) {
        // whole row cached: entries and their column iterates from shared
        // memory, one at a time (same operations, same order)
        const V2 *gv = reinterpret_cast<const V2 *>(C.gv);
        for (int ce = ce0; ce < ce1; ce++) {
            const int4 en = C.ent[ce];
            const V2 sv = gv[ce];
            int l;
            Real val, lbl;
            decode_entry<Real>(en, V.lbGeneral, l, val, lbl);
            Real xl;
            if (mode == kModeG0)
                xl = sv.x;
            else if (mode == kModeAG)
                xl = sv.y;
            else
                xl = projlb<Real>(fma(-alpha, sv.y, sv.x), lbl);
            if (l == k) {
                gam = sv.x;
                gold = sv.y;
                lbk = lbl;
                xk = xl;
            }
            acc = fma(val, xl, acc);
        }
    } else {
        for (int eb = e0; eb < e1; eb += B) {
            // entries from the block's shared-memory copy when cached; all
            // neighbour iterates of the batch are requested before any is
            // used
            int4 ent[B];
#pragma unroll
            for (int j = 0; j < B; j++) {
                const int ce = eb + j - C.entBase;
                ent[j] = eb + j < e1 ? ((ce >= 0 && ce < C.nEnt) ? C.ent[ce] : __ldg(V.aent + eb + j))
                                     : make_int4(k, 1, 0, 0);
            }
            V2 sv[B];
#pragma unroll
            for (int j = 0; j < B; j++)
                if (eb + j < e1) sv[j] = stIn[ent[j].x];  // L1-cacheable: rows of a block share neighbours
#pragma unroll
            for (int j = 0; j < B; j++) {
                if (eb + j < e1) {
                    int l;
                    Real val, lbl;
                    decode_entry<Real>(ent[j], V.lbGeneral, l, val, lbl);
                    Real xl;
                    if (mode == kModeG0)
                        xl = sv[j].x;
                    else if (mode == kModeAG)
                        xl = sv[j].y;
                    else
                        xl = projlb<Real>(fma(-alpha, sv[j].y, sv[j].x), lbl);
                    if (l == k) {
                        gam = sv[j].x;
                        gold = sv[j].y;
                        lbk = lbl;
                        xk = xl;
                    }
                    acc = fma(val, xl, acc);
                }
            }
        }
    }
    acc = fma(qc.y, xk, acc);
    if (mode == kModeAG) {
        v0 = gold * gold;
        v1 = gold * acc;
        V2 o;
        o.x = gam;
        o.y = gold;
        stOut[k] = o;
        return;
    }
    const Real gn = acc + qc.x;
    if (V.fp64) {
        rmax = fabs(xk - projlb<Real>(xk - gn, lbk));
    } else {
        // x - P(x - g) = min(g, x - lb): exact for lb = 0 and lb = -inf
        const Real m = gn < xk - lbk ? gn : xk - lbk;
        rmax = fabs(m);
    }
    if (rmax != rmax) {
        atomicOr(errFlags, kErrNaN);
        rmax = Real(INFINITY);
    }
    if (mode == kModeIter) {
        const Real s = xk - gam;
        const Real y = gn - gold;
        v0 = s * s;
        v1 = s * y;
        v2 = y * y;
    }
    V2 o;
    o.x = xk;
    o.y = gn;
    stOut[k] = o;
}

// One 64-constraint tile processed by a 64-thread group (two warps).
template <class Real>
__device__ void process_tile(const DevState &S, const SolveView<Real> &V, int p, int T, int mode,
                             Real alpha, SolveShared &sh, int group, const RowCache &C) {
    const int lane64 = threadIdx.x & 63;
    const int warpInGroup = (threadIdx.x >> 5) & 1;
    const int r = __ldg(S.tileRep + T);
    // constraint range of the replica: fixed while the solver runs
    const RepDyn *d = S.dyn + r;
    const int local = (T - __ldg(&d->tileStart)) * kRowTile + lane64;
    const bool valid = local < __ldg(&d->nCon);
    const int k = __ldg(&d->conStart) + local;
    // select the ping-pong buffers without indexing the parameter arrays
    // (a runtime index would copy the view to local memory)
    const bool odd = (p & 1) != 0;
    using V2 = typename Vec2<Real>::T;
    const V2 *const stIn = odd ? V.st[0] : V.st[1];
    V2 *const stOut = odd ? V.st[1] : V.st[0];
    Real v0 = Real(0), v1 = Real(0), v2 = Real(0);
    Real rmax = mode == kModeCopy ? Real(-1) : Real(0);
    if (valid) row_update<Real>(V, k, mode, alpha, stIn, stOut, v0, v1, v2, rmax, &S.ctl->errFlags, C);
    // warp trees in Real (modes that need them), tile = warp0 + warp1 in
    // FP64; the max through integer bit patterns
    Real w0 = Real(0), w1 = Real(0), w2 = Real(0);
    if (mode == kModeAG || mode == kModeIter) {
        w0 = warp_tree_sum_t<Real>(v0);
        w1 = warp_tree_sum_t<Real>(v1);
    }
    if (mode == kModeIter) w2 = warp_tree_sum_t<Real>(v2);
    const double wm = __longlong_as_double(warp_max_bits(__double_as_longlong((double)rmax)));
    if ((threadIdx.x & 31) == 0) {
        sh.tileVal[group][warpInGroup][0] = (double)w0;
        sh.tileVal[group][warpInGroup][1] = (double)w1;
        sh.tileVal[group][warpInGroup][2] = (double)w2;
        sh.tileVal[group][warpInGroup][3] = wm;
    }
}

template <class Real>
__global__ void __launch_bounds__(kSolveThreads, 2) k_solve(DevState S, SolveView<Real> V,
                                                         unsigned long long timeout_ns) {
    __shared__ SolveShared sh;
    extern __shared__ int4 dynCache[];
    if (ld_volatile_i32(&S.ctl->errFlags) & kErrStepAbort) return;
    // FP64 refinement after an FP32 solve whose result already met the FP64
    // tolerance (checked by the refinement set-up, which left the promoted
    // solution in buffer 1): nothing to do
    if constexpr (sizeof(Real) == 8) {
        if (S.precision == ALENS_PREC_MIXED && ld_volatile_i32(&S.ctl->allRefined)) return;
    }
    const unsigned int nb = gridDim.x;
    const int nTiles = S.ctl->nTiles;
    const int tpb = max(S.solveMinTiles, (nTiles + (int)nb - 1) / (int)nb);
    const int t0 = min((int)blockIdx.x * tpb, nTiles);
    const int t1 = min(t0 + tpb, nTiles);
    // blocks without tiles leave at once; the barrier counts the others
    // (block 0 always stays: it arms the pass counters)
    const int nActive = nTiles > 0 ? (nTiles + tpb - 1) / tpb : 1;
    if ((int)blockIdx.x >= nActive) return;
    // this block's operator rows, cached for every pass: the rows of tiles
    // [t0, t1) are one contiguous range of constraints
    RowCache C{};
    constexpr int kEnts = row_cache_ents<Real>();
    {
        using V2 = typename Vec2<Real>::T;
        V2 *gv = reinterpret_cast<V2 *>(dynCache + kEnts);
        int *rptr = reinterpret_cast<int *>(gv + kEnts);
        C.ent = dynCache;
        C.rptr = rptr;
        C.gv = gv;
        if (t0 < t1) {
            const RepDyn &da = S.dyn[__ldg(S.tileRep + t0)];
            const RepDyn &db = S.dyn[__ldg(S.tileRep + t1 - 1)];
            const int rowBeg = da.conStart + (t0 - da.tileStart) * kRowTile;
            const int rowEnd = min(db.conStart + (t1 - db.tileStart) * kRowTile, db.conStart + db.nCon);
            const int eBeg = __ldg(V.aptr + rowBeg), eEnd = __ldg(V.aptr + rowEnd);
            C.entBase = eBeg;
            C.nEnt = min(eEnd - eBeg, kEnts);
            C.rowBase = rowBeg;
            C.nRow = rowEnd - rowBeg <= kRowCacheRows ? rowEnd - rowBeg : 0;
            for (int e = threadIdx.x; e < C.nEnt; e += blockDim.x) dynCache[e] = __ldg(V.aent + eBeg + e);
            if (C.nRow > 0)
                for (int i = threadIdx.x; i <= C.nRow; i += blockDim.x) rptr[i] = __ldg(V.aptr + rowBeg + i);
        }
        __syncthreads();
    }
    const int maxPass = S.ctl->maxIte + 3;
    const size_t tc = (size_t)S.tileCap;
    const int group = threadIdx.x >> 6;
    int lastPass = 0;
#ifdef ALENS_TRACE
    unsigned long long trDecide = 0, trTiles = 0, trBar = 0, trT0 = 0, trT1 = 0;
    long long cA = 0, cSum[6] = {0, 0, 0, 0, 0, 0};
#endif
    for (int p = 0; p <= maxPass; p++) {
#ifdef ALENS_TRACE
        trT0 = global_ns();
        trT1 = 0;
        cA = clock64();
        long long cDec = 0, cRow = 0, cStore = 0;
        sh.trRed = 0;
#endif
        if (threadIdx.x == 0) sh.act = 0;
        if (blockIdx.x == 0 && threadIdx.x == 0) st_relaxed_u32(&S.ctl->bar.pass[(p + 1) % 3][0], 0u);
        double *partBase = S.part + (size_t)(p & 1) * 4 * tc;
        // completes before the first decide()'s __syncthreads
        gather_columns<Real>(C, (p & 1) ? V.st[0] : V.st[1]);
        // replica windows of this block's tile range
        int T = t0;
        while (T < t1) {
            const int rFirst = __ldg(S.tileRep + T);
            const int rLast = min(__ldg(S.tileRep + t1 - 1), rFirst + kWindow - 1);
            for (int r = rFirst; r <= rLast; r++) decide<Real>(S, V, p, r, t0, t1, sh, r - rFirst);
#ifdef ALENS_TRACE
            if (trT1 == 0) trT1 = global_ns();
            if (cDec == 0) cDec = clock64();
#endif
            // tiles of the window, four per round
            int Tend = T;
            while (Tend < t1 && __ldg(S.tileRep + Tend) <= rLast) Tend++;
            for (int base = T; base < Tend; base += 4) {
                const int Tg = base + group;
                if (Tg < Tend) {
                    const int slot = __ldg(S.tileRep + Tg) - rFirst;
                    process_tile<Real>(S, V, p, Tg, sh.mode[slot], (Real)sh.alpha[slot], sh, group, C);
                }
#ifdef ALENS_TRACE
                if (cRow == 0) cRow = clock64();
#endif
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
#ifdef ALENS_TRACE
        const unsigned long long trT2 = global_ns();
        if (trT1 == 0) trT1 = trT2;
        cStore = clock64();
#endif
        int stop = 0;
        if (!grid_sync_pass(&S.ctl->bar, (unsigned int)(nActive + S.barrierExtra), &S.ctl->errFlags, timeout_ns,
                            p, sh.act, stop))
            return;
#ifdef ALENS_TRACE
        const unsigned long long trT3 = global_ns();
        trDecide += trT1 - trT0;
        trTiles += trT2 - trT1;
        trBar += trT3 - trT2;
        {
            const long long cE = clock64();
            const long long red = sh.trRed ? sh.trRed : cA;
            if (cDec && cRow && p > 2) {
                cSum[0] += red - cA;        // partial reductions
                cSum[1] += cDec - red;      // decision
                cSum[2] += cRow - cDec;     // row updates
                cSum[3] += cStore - cRow;   // tile partial stores + syncs
                cSum[4] += cE - cStore;     // barrier
                cSum[5] += 1;
            }
        }
#endif
        if (stop) break;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        S.ctl->finalParity = lastPass & 1;
        for (int r = 0; r < S.R; r++) S.dyn[r].finalPar = lastPass & 1;
    }
#ifdef ALENS_TRACE
    if (threadIdx.x == 0 && (blockIdx.x == 0 || blockIdx.x == gridDim.x / 2 || blockIdx.x == gridDim.x - 1))
        printf("trace block %d passes %d: decide %.2f us, tiles %.2f us, barrier %.2f us per pass (tiles %d) | "
               "cycles/pass: reduce %lld decide %lld rows %lld store %lld barrier %lld\n",
               blockIdx.x, lastPass + 1, 1e-3 * trDecide / (lastPass + 1), 1e-3 * trTiles / (lastPass + 1),
               1e-3 * trBar / (lastPass + 1), t1 - t0, cSum[5] ? cSum[0] / cSum[5] : 0LL,
               cSum[5] ? cSum[1] / cSum[5] : 0LL, cSum[5] ? cSum[2] / cSum[5] : 0LL,
               cSum[5] ? cSum[3] / cSum[5] : 0LL, cSum[5] ? cSum[4] / cSum[5] : 0LL);
#endif
}

}  // namespace alens
