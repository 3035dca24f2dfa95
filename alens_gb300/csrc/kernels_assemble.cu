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

// W = M J for both sides of every constraint, one thread per side
// (adjacent lanes: the two sides of a constraint).
__global__ void k_weights(DevState S) {
    ALENS_PDL_PROLOGUE();
    if (flags(S) & (kErrNaN | kErrOverflow)) return;
    const int nc = S.ctl->totalCon;
    for (int it = blockIdx.x * blockDim.x + threadIdx.x; it < 2 * nc; it += gridDim.x * blockDim.x) {
        const int k = it >> 1, side = it & 1;
        {
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

// Row k of A is the merge of the rod rows of k's two rods (entries 2l+s,
// ascending): one output per distinct l, in ascending l.  The structure
// (which entries of the two rod rows feed each output) is found by one
// thread per row with integer work only; the values are then formed by one
// thread per output (full warps for the FP64 pipe).
struct RowLists {
    int aI0, nI, aJ0, nJ;
};

__device__ __forceinline__ RowLists row_lists(const DevState &S, int k) {
    RowLists L;
    const int rI = S.conI[k], rJ = S.conJ[k];
    L.aI0 = S.rowPtr[rI];
    L.nI = S.rowPtr[rI + 1] - L.aI0;
    L.aJ0 = rJ >= 0 ? S.rowPtr[rJ] : 0;
    L.nJ = rJ >= 0 ? S.rowPtr[rJ + 1] - L.aJ0 : 0;
    return L;
}

// Merge of the two rod rows: the number of outputs, or (fill) the record
// (k, eI, eJ, l) of each output written to aent at out0 (eI/eJ: index into
// rowEnt of the first entry of l in rod I's / rod J's row, -1 when absent).
template <bool fill>
__device__ int merge_rows(const DevState &S, int k, const RowLists &L, int out0) {
    int a = 0, b = 0, cnt = 0;
    while (a < L.nI || b < L.nJ) {
        const int la = a < L.nI ? (S.rowEnt[L.aI0 + a] >> 1) : 0x7fffffff;
        const int lb = b < L.nJ ? (S.rowEnt[L.aJ0 + b] >> 1) : 0x7fffffff;
        const int l = la < lb ? la : lb;
        const int eI = la == l ? L.aI0 + a : -1, eJ = lb == l ? L.aJ0 + b : -1;
        while (a < L.nI && (S.rowEnt[L.aI0 + a] >> 1) == l) a++;
        while (b < L.nJ && (S.rowEnt[L.aJ0 + b] >> 1) == l) b++;
        if (fill) S.aent[out0 + cnt] = make_int4(k, eI, eJ, l);
        cnt++;
    }
    return cnt;
}

// The same merge for rod rows of at most kMergeStage entries, staged in
// shared memory: both rows are loaded with independent loads (one memory
// round trip instead of one per merge step), each thread's copy in the
// column of its lane ([entry][lane]: no bank conflicts whatever entry each
// lane reads).  One warp per block.  Outputs and (eI, eJ) as merge_rows.
constexpr int kMergeStage = 16;
constexpr int kMergeThreads = 32;
template <bool fill>
__device__ int merge_rows_staged(const DevState &S, int k, const RowLists &L, int out0, int *stA, int *stB) {
    const int lane = threadIdx.x;
#pragma unroll
    for (int q = 0; q < kMergeStage; q++) {
        if (q < L.nI) stA[q * kMergeThreads + lane] = __ldg(S.rowEnt + L.aI0 + q) >> 1;
        if (q < L.nJ) stB[q * kMergeThreads + lane] = __ldg(S.rowEnt + L.aJ0 + q) >> 1;
    }
    auto at = [&](const int *st, int q, int n) { return q < n ? st[q * kMergeThreads + lane] : 0x7fffffff; };
    int a = 0, b = 0, cnt = 0;
    int la = at(stA, 0, L.nI), lb = at(stB, 0, L.nJ);
    while (a < L.nI || b < L.nJ) {
        const int l = la < lb ? la : lb;
        const int eI = la == l ? L.aI0 + a : -1, eJ = lb == l ? L.aJ0 + b : -1;
        while (la == l) la = at(stA, ++a, L.nI);
        while (lb == l) lb = at(stB, ++b, L.nJ);
        if (fill) S.aent[out0 + cnt] = make_int4(k, eI, eJ, l);
        cnt++;
    }
    return cnt;
}

template <bool fill>
__device__ __forceinline__ int merge_any(const DevState &S, int k, int out0, int *stA, int *stB) {
    const RowLists L = row_lists(S, k);
    if (L.nI <= kMergeStage && L.nJ <= kMergeStage) return merge_rows_staged<fill>(S, k, L, out0, stA, stB);
    return merge_rows<fill>(S, k, L, out0);
}

__global__ void __launch_bounds__(kMergeThreads) k_arow_count(DevState S) {
    __shared__ int stA[kMergeStage * kMergeThreads], stB[kMergeStage * kMergeThreads];
    ALENS_PDL_PROLOGUE();
    if (flags(S) & (kErrNaN | kErrOverflow)) return;
    const int nc = S.ctl->totalCon;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < S.cap; k += gridDim.x * blockDim.x)
        S.annz[k] = k < nc ? merge_any<false>(S, k, 0, stA, stB) : 0;
}

__global__ void __launch_bounds__(kMergeThreads) k_arow_struct(DevState S) {
    __shared__ int stA[kMergeStage * kMergeThreads], stB[kMergeStage * kMergeThreads];
    ALENS_PDL_PROLOGUE();
    if (flags(S) & (kErrNaN | kErrOverflow)) return;
    const int nc = S.ctl->totalCon;
    const int nnz = S.aptr[nc];
    if (blockIdx.x == 0 && threadIdx.x == 0) S.ctl->totalNnz = nnz;
    if (nnz > S.nnzCap) {
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(&S.ctl->errFlags, kErrOverflow);
        return;
    }
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nc; k += gridDim.x * blockDim.x)
        merge_any<true>(S, k, S.aptr[k], stA, stB);
}

// A_kl = dt * (sum over l's entries in rod I's row of J_k,I . W_l,s, then
// over its entries in rod J's row of J_k,J . W_l,s), in entry order.
__global__ void k_arow_values(DevState S) {
    ALENS_PDL_PROLOGUE();
    if (flags(S) & (kErrNaN | kErrOverflow)) return;
    const int nc = S.ctl->totalCon;
    const int nnz = S.aptr[nc];
    if (nnz > S.nnzCap) return;
    for (int o = blockIdx.x * blockDim.x + threadIdx.x; o < nnz; o += gridDim.x * blockDim.x) {
        const int4 rec = S.aent[o];
        const int k = rec.x, l = rec.w;
        const int rI = S.conI[k], rJ = S.conJ[k];
        const double *JkI = S.jac + 12 * (size_t)k;
        const double *JkJ = JkI + 6;
        double acc = 0.0;
        if (rec.y >= 0) {
            const int end = S.rowPtr[rI + 1];
            for (int e = rec.y; e < end && (S.rowEnt[e] >> 1) == l; e++)
                acc = acc + dot6d(JkI, S.W + 12 * (size_t)l + 6 * (S.rowEnt[e] & 1));
        }
        if (rec.z >= 0) {
            const int end = S.rowPtr[rJ + 1];
            for (int e = rec.z; e < end && (S.rowEnt[e] >> 1) == l; e++)
                acc = acc + dot6d(JkJ, S.W + 12 * (size_t)l + 6 * (S.rowEnt[e] & 1));
        }
        const double v = S.par[S.rodRep[rI]].dt * acc;
        const int kind = S.lbKind[l];
        S.aent[o] = make_int4(l, kind, __double2loint(v), __double2hiint(v));
        if (S.precision == ALENS_PREC_MIXED)
            S.aent32[o] = make_int4(l, kind, __float_as_int((float)v), __float_as_int((float)S.lb[l]));
    }
}

int grid_for(int n, int block) {
    int g = (n + block - 1) / block;
    return g < 1 ? 1 : (g > 4096 ? 4096 : g);
}

}  // namespace

void launch_weights(const DevState &S, cudaStream_t st) { k_weights<<<grid_for(2 * S.cap, 32), 32, 0, st>>>(S); }

// Row structure on `st`; the values need the weights, which the caller
// launched on `side` (recorded in `join`) while the rows were sorted.
int launch_assemble(const DevState &S, cudaStream_t st, cudaStream_t side, cudaEvent_t join) {
    launch_pdl(k_arow_count, dim3(grid_for(S.cap, kMergeThreads)), dim3(kMergeThreads), 0, st, S);
    // row starts of the step's constraints (annz is zero past them)
    const int n = launch_scan_dev(S.annz, S.aptr, S.cap, &S.ctl->totalCon, S.scanTmp, st);
    launch_pdl(k_arow_struct, dim3(grid_for(S.cap, kMergeThreads)), dim3(kMergeThreads), 0, st, S);
    cudaEventRecord(join, side);
    cudaStreamWaitEvent(st, join, 0);
    k_arow_values<<<grid_for(S.nnzCap, 64), 64, 0, st>>>(S);
    return n + 3;
}

}  // namespace alens
