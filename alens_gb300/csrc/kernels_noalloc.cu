// kernels_noalloc.cu - BBPGD solve that allocates nothing.
//
// Some callers of this library cannot call cudaMalloc at the point where
// they solve.  Two kinds are common: a host code whose GPU memory is all
// owned by another allocator (a framework's caching pool that has reserved
// the device, or a fixed memory budget that must not be disturbed), and a
// time loop that must not stall the device, since cudaMalloc and cudaFree
// may synchronise it.  For them this file provides
// alens_bbpgd_solve_noalloc: the FP64 BBPGD of the library over an operator
// the caller already holds in device memory (CSR rows), with every scratch
// buffer in one file-scope __device__ array of fixed size.
//
// The arithmetic is the library's FP64 BBPGD: same projected step, same
// fused row product, same canonical reduction trees, so on the same operator
// it returns the same gamma as alens_solve.  The row entries are read from
// plain CSR arrays instead of the library's packed form.
//
// Limits and sharing:
//  * at most kNoAllocMaxConstraints rows (65,536); larger problems are
//    rejected with ALENS_INVALID_ARG;
//  * column indices must lie in [0, n) and rowPtr[0] must be 0; an entry
//    whose column lies outside is skipped and the call returns
//    ALENS_INVALID_ARG (the array holds the state of 65,536 rows, so an
//    unchecked column could read another call's leftovers or past its end);
//  * the scratch array (about 2.1 MB) lives on every GPU that loads the
//    library until the process exits;
//  * every call uses the same array and leaves its contents behind; each
//    call re-initialises what must start from zero, so two calls in a row
//    are independent, but calls that overlap on the GPU (other streams or
//    threads at the same time) race on it;
//  * the first call on a device resolves the array's device address
//    (cudaGetSymbolAddress) and the solver's launch size and keeps them for
//    the life of the process; cudaDeviceReset after that first call is not
//    supported;
//  * before returning, a call waits for its stream and copies the
//    iteration count, status, residual and error flags into host memory.
//
// Compiled with --fmad=false (the FP64 arithmetic matches the oracle).
#include <mutex>

#include "solve_impl.cuh"

namespace alens {

namespace {

constexpr int kNoAllocMaxConstraints = 65536;
constexpr int kNoAllocMaxTiles = kNoAllocMaxConstraints / kTile;
constexpr int kErrBadColumn = 1 << 8;  // a column index outside [0, n) was skipped

struct NoAllocScratch {
    double2 st[2][kNoAllocMaxConstraints];     // (gamma, g) by pass parity
    double part[8][kNoAllocMaxTiles];          // tile partials: parity x kind
    double alphaBuf[2];
    int tileRep[kNoAllocMaxTiles];
    DevCtl ctl;
    RepDyn dyn;
    RepParams par;
};

// The scratch itself: a fixed-size byte array viewed as NoAllocScratch.
static __device__ __align__(256) unsigned char g_noallocScratch[sizeof(NoAllocScratch)];

struct PlainOperator {
    const int *rowPtr;
    const int *cols;
    const double *vals;
    const double *q;
    const double *cinv;
    const double *lb;
};

// Clear the state a solve must start from and place the projected initial
// guess in the parity-1 buffer.
__global__ void k_noalloc_setup(NoAllocScratch *sc, PlainOperator op, const double *gamma0, int n, double tol,
                                int maxIte) {
    const int nTiles = (n + kTile - 1) / kTile;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const double g = gamma0[k];
        const double lb = op.lb[k];
        sc->st[1][k] = make_double2(g < lb ? lb : g, 0.0);
    }
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nTiles; t += gridDim.x * blockDim.x) sc->tileRep[t] = 0;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        DevCtl &c = sc->ctl;
        c.step = 0;
        c.rawCount = 0;
        c.errFlags = 0;
        c.totalColl = n;
        c.totalBil = 0;
        c.totalCon = n;
        c.nTiles = nTiles;
        c.totalNnz = 0;
        c.maxIte = maxIte;
        c.activeCnt[0] = c.activeCnt[1] = c.activeCnt[2] = 0;
        c.finalParity = 1;
        c.allRefined = 0;
        c.setupDone = 0u;
        c.bar.count = 0;
        c.bar.gen = 0;
        c.bar.pass[0][0] = c.bar.pass[1][0] = c.bar.pass[2][0] = 0u;
        RepDyn &d = sc->dyn;
        d.collStart = 0;
        d.collEnd = n;
        d.conStart = 0;
        d.nCon = n;
        d.tileStart = 0;
        d.nTiles = nTiles;
        d.iter = 0;
        d.active = n > 0 ? 1 : 0;
        d.converged = n > 0 ? 0 : 1;
        d.status = 0;
        d.counter = 0;
        d.refineIter = 0;
        d.finalPar = 1;
        d.refined = 0;
        d.res64bits = 0ULL;
        d.alpha = 0.0;
        d.res = 0.0;
        RepParams &P = sc->par;
        P.tol = tol;
        P.maxIte = maxIte;
        P.nRods = 0;
        sc->alphaBuf[0] = sc->alphaBuf[1] = 0.0;
    }
}

// Row update over plain CSR: the operations of row_update<double>.
__device__ __forceinline__ void row_update_plain(const PlainOperator &op, int n, int k, int mode, double alpha,
                                                 const double2 *stIn, double2 *stOut, double &v0, double &v1,
                                                 double &v2, double &rmax, int *errFlags) {
    if (mode == kModeCopy) {
        stOut[k] = ldcg(stIn + k);
        return;
    }
    const double2 own = ldcg(stIn + k);
    const double gam = own.x, gold = mode == kModeG0 ? 0.0 : own.y;
    const double lbk = __ldg(op.lb + k);
    double xk;
    if (mode == kModeG0)
        xk = gam;
    else if (mode == kModeAG)
        xk = gold;
    else
        xk = projlb<double>(fma(-alpha, gold, gam), lbk);
    double acc = 0.0;
    const int e0 = __ldg(op.rowPtr + k), e1 = __ldg(op.rowPtr + k + 1);
    for (int eb = e0; eb < e1; eb += kRowPrefetch) {
        int cols[kRowPrefetch];
        double vals[kRowPrefetch];
        bool use[kRowPrefetch];
#pragma unroll
        for (int j = 0; j < kRowPrefetch; j++) {
            cols[j] = eb + j < e1 ? __ldg(op.cols + eb + j) : k;
            vals[j] = eb + j < e1 ? __ldg(op.vals + eb + j) : 0.0;
            // a column outside [0, n) is flagged and skipped, never read
            const bool inRange = cols[j] >= 0 && cols[j] < n;
            if (eb + j < e1 && !inRange) atomicOr(errFlags, kErrBadColumn);
            use[j] = eb + j < e1 && inRange;
        }
        double2 sv[kRowPrefetch];
        double lbs[kRowPrefetch];
#pragma unroll
        for (int j = 0; j < kRowPrefetch; j++) {
            if (use[j]) {
                sv[j] = ldcg(stIn + cols[j]);
                lbs[j] = __ldg(op.lb + cols[j]);
            }
        }
#pragma unroll
        for (int j = 0; j < kRowPrefetch; j++) {
            if (use[j]) {
                double xl;
                if (mode == kModeG0)
                    xl = sv[j].x;
                else if (mode == kModeAG)
                    xl = sv[j].y;
                else
                    xl = projlb<double>(fma(-alpha, sv[j].y, sv[j].x), lbs[j]);
                acc = fma(vals[j], xl, acc);
            }
        }
    }
    acc = fma(__ldg(op.cinv + k), xk, acc);
    if (mode == kModeAG) {
        v0 = gold * gold;
        v1 = gold * acc;
        stOut[k] = make_double2(gam, gold);
        return;
    }
    const double gn = acc + __ldg(op.q + k);
    rmax = fabs(xk - projlb<double>(xk - gn, lbk));
    if (rmax != rmax) {
        atomicOr(errFlags, kErrNaN);
        rmax = INFINITY;
    }
    if (mode == kModeIter) {
        const double s = xk - gam;
        const double y = gn - gold;
        v0 = s * s;
        v1 = s * y;
        v2 = y * y;
    }
    stOut[k] = make_double2(xk, gn);
}

// Persistent cooperative BBPGD over the plain operator: the pass structure,
// decisions and reduction trees of k_solve<double> for one replica.
__global__ void __launch_bounds__(kSolveThreads) k_noalloc_solve(DevState S, SolveView<double> V, PlainOperator op,
                                                                 double2 *st0, double2 *st1,
                                                                 unsigned long long timeout_ns) {
    __shared__ SolveShared sh;
    const unsigned int nb = gridDim.x;
    const int nTiles = S.ctl->nTiles;
    const int tpb = (nTiles + (int)nb - 1) / (int)nb;
    const int t0 = min((int)blockIdx.x * tpb, nTiles);
    const int t1 = min(t0 + tpb, nTiles);
    const int maxPass = S.ctl->maxIte + 3;
    const size_t tc = (size_t)S.tileCap;
    const int group = threadIdx.x >> 6;
    const int lane64 = threadIdx.x & 63;
    const int warpInGroup = (threadIdx.x >> 5) & 1;
    const int nCon = S.dyn[0].nCon;
    int lastPass = 0;
    for (int p = 0; p <= maxPass; p++) {
        if (blockIdx.x == 0 && threadIdx.x == 0) S.ctl->activeCnt[(p + 1) % 3] = 0;
        if (threadIdx.x == 0) sh.act = 0;
        double *partBase = S.part + (size_t)(p & 1) * 4 * tc;
        if (t0 < t1) decide<double>(S, V, p, 0, t0, t1, sh, 0);
        // the block owning the replica counts it active for this pass
        if (threadIdx.x == 0 && sh.act) atomicAdd(&S.ctl->activeCnt[p % 3], sh.act);
        const int mode = sh.mode[0];
        const double alpha = sh.alpha[0];
        const bool odd = (p & 1) != 0;
        const double2 *stIn = odd ? st0 : st1;
        double2 *stOut = odd ? st1 : st0;
        for (int base = t0; base < t1; base += 4) {
            const int T = base + group;
            if (T < t1) {
                const int local = T * kTile + lane64;
                double v0 = 0.0, v1 = 0.0, v2 = 0.0;
                double rmax = mode == kModeCopy ? -1.0 : 0.0;
                if (local < nCon)
                    row_update_plain(op, nCon, local, mode, alpha, stIn, stOut, v0, v1, v2, rmax, &S.ctl->errFlags);
                double w0 = 0.0, w1 = 0.0, w2 = 0.0;
                if (mode == kModeAG || mode == kModeIter) {
                    w0 = warp_tree_sum_t<double>(v0);
                    w1 = warp_tree_sum_t<double>(v1);
                }
                if (mode == kModeIter) w2 = warp_tree_sum_t<double>(v2);
                const double wm = __longlong_as_double(warp_max_bits(__double_as_longlong(rmax)));
                if ((threadIdx.x & 31) == 0) {
                    sh.tileVal[group][warpInGroup][0] = w0;
                    sh.tileVal[group][warpInGroup][1] = w1;
                    sh.tileVal[group][warpInGroup][2] = w2;
                    sh.tileVal[group][warpInGroup][3] = wm;
                }
            }
            __syncthreads();
            if (threadIdx.x < 4 && base + (int)threadIdx.x < t1) {
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
        lastPass = p;
        if (!grid_sync(&S.ctl->bar, nb, &S.ctl->errFlags, timeout_ns)) return;
        if (ldcg(&S.ctl->activeCnt[p % 3]) == 0) break;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) S.ctl->finalParity = lastPass & 1;
}

__global__ void k_noalloc_finish(NoAllocScratch *sc, double *gamma, int n) {
    const double2 *src = sc->ctl.finalParity ? sc->st[1] : sc->st[0];
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) gamma[k] = src[k].x;
}

struct DeviceSetup {
    NoAllocScratch *scratch = nullptr;
    int grid = 0;
};

std::mutex g_setupMutex;
DeviceSetup g_setup[64];

// Once per device, with that device current: the scratch array's device
// address and the cooperative launch size.
int noalloc_setup(int dev, DeviceSetup *out) {
    std::lock_guard<std::mutex> lock(g_setupMutex);
    if (dev < 0 || dev >= 64) return ALENS_INVALID_ARG;
    DeviceSetup &s = g_setup[dev];
    if (!s.scratch) {
        void *ptr = nullptr;
        if (cudaGetSymbolAddress(&ptr, g_noallocScratch) != cudaSuccess || !ptr) {
            cudaGetLastError();
            return ALENS_CUDA_ERROR;
        }
        int nsm = 0, per = 0;
        if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_noalloc_solve, kSolveThreads, 0) != cudaSuccess ||
            per < 1) {
            cudaGetLastError();
            return ALENS_CUDA_ERROR;
        }
        s.grid = nsm;  // one block per SM, as the library's solver
        s.scratch = (NoAllocScratch *)ptr;
    }
    *out = s;
    return ALENS_OK;
}

}  // namespace

}  // namespace alens

extern "C" int alens_bbpgd_solve_noalloc(int n, const int32_t *rowPtr, const int32_t *cols, const double *vals,
                                         const double *q, const double *cinv, const double *lowerBound,
                                         const double *gamma0, double *gamma, double tol, int maxIte,
                                         void *stream, int *iterations, double *residual, int *solveStatus) {
    using namespace alens;
    if (n < 0 || n > kNoAllocMaxConstraints) return ALENS_INVALID_ARG;  // beyond the fixed scratch size
    if (!(tol > 0.0) || maxIte < 0) return ALENS_INVALID_ARG;
    if (n > 0 && (!rowPtr || !cols || !vals || !q || !cinv || !lowerBound || !gamma0 || !gamma))
        return ALENS_INVALID_ARG;
    if (n == 0) {
        if (iterations) *iterations = 0;
        if (residual) *residual = 0.0;
        if (solveStatus) *solveStatus = ALENS_OK;
        return ALENS_OK;
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return ALENS_NO_DEVICE;
    }
    DeviceSetup su;
    const int rc = noalloc_setup(dev, &su);
    if (rc != ALENS_OK) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    NoAllocScratch *sc = su.scratch;
    PlainOperator op{rowPtr, cols, vals, q, cinv, lowerBound};
    k_noalloc_setup<<<64, 256, 0, st>>>(sc, op, gamma0, n, tol, maxIte);
    if (cudaGetLastError() != cudaSuccess) return ALENS_CUDA_ERROR;
    DevState S{};
    S.R = 1;
    S.tileCap = kNoAllocMaxTiles;
    S.par = &sc->par;
    S.dyn = &sc->dyn;
    S.ctl = &sc->ctl;
    S.part = &sc->part[0][0];
    S.tileRep = sc->tileRep;
    SolveView<double> V{};
    V.alphaBuf = sc->alphaBuf;
    V.fp64 = 1;
    double2 *st0 = sc->st[0], *st1 = sc->st[1];
    unsigned long long timeout = 2000000000ULL;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(su.grid);
    cfg.blockDim = dim3(kSolveThreads);
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (cudaLaunchKernelEx(&cfg, k_noalloc_solve, S, V, op, st0, st1, timeout) != cudaSuccess) {
        cudaGetLastError();
        return ALENS_CUDA_ERROR;
    }
    k_noalloc_finish<<<64, 256, 0, st>>>(sc, gamma, n);
    int hostIter = 0, hostStatus = 0, hostErr = 0;
    double hostRes = 0.0;
    if (cudaMemcpyAsync(&hostIter, &sc->dyn.iter, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaMemcpyAsync(&hostStatus, &sc->dyn.status, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaMemcpyAsync(&hostRes, &sc->dyn.res, sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaMemcpyAsync(&hostErr, &sc->ctl.errFlags, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) {
        cudaGetLastError();
        return ALENS_CUDA_ERROR;
    }
    if (iterations) *iterations = hostIter;
    if (residual) *residual = hostRes;
    if (solveStatus) *solveStatus = hostStatus;
    if (hostErr & kErrTimeout) return ALENS_TIMEOUT;
    if (hostErr & kErrBadColumn) return ALENS_INVALID_ARG;
    if (hostErr & kErrNaN) return ALENS_NAN_DETECTED;
    return hostStatus;
}
