// kernels_assemble.cu - explicit Delassus operator A = dt D^T M D of a step.
//
// SimToolbox applies D^T M D matrix-free inside every BBPGD iteration
// (ConstraintOperator, CMakeLists.txt:111).  On GB300 the FP64 pipe issues
// 2 lanes per cycle per SM and every grid-wide synchronisation costs
// microseconds, so the operator is assembled once per step and each BBPGD
// pass is a single sparse product (one grid barrier, ~5x fewer FP64
// operations than the two-phase form).
//
// Row k holds every constraint l that shares a rod with k, ascending in l;
// A_kl = dt * sum of J_k,sk . W_l,sl over the shared rods, where
// W_l,s = M_rod J_l,s, contributions ordered by k's side (rod I first) and
// then by the rod row (entry 2l+s ascending).  The oracle assembles the
// same rows with the same arithmetic.
//
// Compiled with --fmad=false.
#include "engine.cuh"

namespace alens {

namespace {

__device__ __forceinline__ int flags(const DevState &S) { return ld_volatile_i32(&S.ctl->errFlags); }

__device__ __forceinline__ double dot6d(const double *a, const double *b) {
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2] + a[3] * b[3] + a[4] * b[4] + a[5] * b[5];
}

// W = M J for both sides of every constraint.
__global__ void k_weights(DevState S) {
    if (flags(S) & (kErrNaN | kErrOverflow)) return;
    const int nc = S.ctl->totalCon;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nc; k += gridDim.x * blockDim.x) {
#pragma unroll
        for (int side = 0; side < 2; side++) {
            const int r = side == 0 ? S.conI[k] : S.conJ[k];
            double U[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
            if (r >= 0 && !S.imm[r]) {
                const double a[3] = {S.ax[r], S.ay[r], S.az[r]};
                const double m[3] = {S.m0[r], S.m1[r], S.m2[r]};
                double F[6];
#pragma unroll
                for (int c = 0; c < 6; c++) F[c] = S.jac[12 * (size_t)k + 6 * side + c];
                mobility_apply<double>(a, m, S.sph[r] != 0, S.par[S.rodRep[r]].mono != 0, F, U);
            }
#pragma unroll
            for (int c = 0; c < 6; c++) S.W[12 * (size_t)k + 6 * side + c] = U[c];
        }
    }
}

// Merge of the rod rows of k's two rods; with fill == false only counts.
template <bool fill>
__device__ int merge_row(const DevState &S, int k, int out0) {
    const int rI = S.conI[k], rJ = S.conJ[k];
    const int aI0 = S.rowPtr[rI], nI = S.rowPtr[rI + 1] - aI0;
    const int aJ0 = rJ >= 0 ? S.rowPtr[rJ] : 0;
    const int nJ = rJ >= 0 ? S.rowPtr[rJ + 1] - aJ0 : 0;
    const double *JkI = S.jac + 12 * (size_t)k;
    const double *JkJ = JkI + 6;
    const double dt = S.par[S.rodRep[rI]].dt;
    int a = 0, b = 0, cnt = 0;
    while (a < nI || b < nJ) {
        const int la = a < nI ? (S.rowEnt[aI0 + a] >> 1) : 0x7fffffff;
        const int lb = b < nJ ? (S.rowEnt[aJ0 + b] >> 1) : 0x7fffffff;
        const int l = la < lb ? la : lb;
        double acc = 0.0;
        while (a < nI && (S.rowEnt[aI0 + a] >> 1) == l) {
            if (fill) acc = acc + dot6d(JkI, S.W + 12 * (size_t)l + 6 * (S.rowEnt[aI0 + a] & 1));
            a++;
        }
        while (b < nJ && (S.rowEnt[aJ0 + b] >> 1) == l) {
            if (fill) acc = acc + dot6d(JkJ, S.W + 12 * (size_t)l + 6 * (S.rowEnt[aJ0 + b] & 1));
            b++;
        }
        if (fill) {
            const int o = out0 + cnt;
            const double v = dt * acc;
            const int kind = S.lbKind[l];
            S.aent[o] = make_int4(l, kind, __double2loint(v), __double2hiint(v));
            if (S.precision == ALENS_PREC_MIXED)
                S.aent32[o] = make_int4(l, kind, __float_as_int((float)v), __float_as_int((float)S.lb[l]));
        }
        cnt++;
    }
    return cnt;
}

__global__ void k_arow_count(DevState S) {
    if (flags(S) & (kErrNaN | kErrOverflow)) return;
    const int nc = S.ctl->totalCon;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < S.cap; k += gridDim.x * blockDim.x)
        S.annz[k] = k < nc ? merge_row<false>(S, k, 0) : 0;
}

__global__ void k_arow_fill(DevState S) {
    if (flags(S) & (kErrNaN | kErrOverflow)) return;
    const int nc = S.ctl->totalCon;
    const int nnz = S.aptr[nc];
    if (blockIdx.x == 0 && threadIdx.x == 0) S.ctl->totalNnz = nnz;
    if (nnz > S.nnzCap) {
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(&S.ctl->errFlags, kErrOverflow);
        return;
    }
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nc; k += gridDim.x * blockDim.x)
        merge_row<true>(S, k, S.aptr[k]);
}

int grid_for(int n, int block) {
    int g = (n + block - 1) / block;
    return g < 1 ? 1 : (g > 4096 ? 4096 : g);
}

}  // namespace

int launch_assemble(const DevState &S, cudaStream_t st) {
    k_weights<<<grid_for(S.cap, 128), 128, 0, st>>>(S);
    k_arow_count<<<grid_for(S.cap, 128), 128, 0, st>>>(S);
    const int n = launch_scan(S.annz, S.aptr, S.cap, S.scanTmp, st);
    k_arow_fill<<<grid_for(S.cap, 128), 128, 0, st>>>(S);
    return n + 3;
}

}  // namespace alens
