// kernels_mixed.cu - BBPGD with FP32 bulk arithmetic: FP32 Delassus
// operator, gamma, g and per-warp partial sums (half the bytes and 1/64 of
// the FP64 instruction cost on GB300); FP64 accumulation of the dot
// products and step sizes, FP64 refinement sweeps afterwards
// (kernels_solve.cu).
//
// Two launch forms:
//  * grid form (k_solve<float>, solve_impl.cuh): one cooperative launch over
//    all SMs with a software grid barrier per pass;
//  * cluster form (k_solve_cluster): each replica is solved by one
//    thread-block cluster; a pass ends with the hardware cluster barrier and
//    the CTAs exchange their partial sums through distributed shared memory.
//    No grid-wide synchronisation; replicas finish independently.
// This path is not bit-compared, so its reductions follow the launch shape.
//
// Compiled with FMA contraction.
#include <cooperative_groups.h>

#include "solve_impl.cuh"

namespace cg = cooperative_groups;

namespace alens {

int solver_max_grid_fp32() {
    int dev = 0, nsm = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    cudaFuncSetAttribute(k_solve<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSolveDynSmem);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_solve<float>, kSolveThreads, kSolveDynSmem);
    return nsm * (per > 0 ? per : 0);
}

cudaError_t launch_solve_fp32(const DevState &S, int grid, unsigned long long timeout_ns, cudaStream_t st) {
    SolveView<float> V{};
    V.aptr = S.aptr;
    V.aent = S.aent32;
    V.st[0] = S.st32[0];
    V.st[1] = S.st32[1];
    V.qc = S.qc32;
    V.lbGeneral = S.lb;
    V.alphaBuf = S.alphaBuf;
    V.fp64 = 0;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(kSolveThreads);
    cfg.dynamicSmemBytes = kSolveDynSmem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_solve<float>, S, V, timeout_ns);
}

// ------------------------------------------------------------ cluster form
constexpr int kClusterThreads = 512;
constexpr int kClusterWarps = kClusterThreads / 32;

struct ClusterShared {
    double part[2][4];              // this CTA's partials by pass parity
    double warpVal[kClusterWarps][4];
    double alphaPrev;
    float alpha;
    int mode;
};

__global__ void __launch_bounds__(kClusterThreads) k_solve_cluster(DevState S, SolveView<float> V) {
    cg::cluster_group cluster = cg::this_cluster();
    const int CS = (int)cluster.num_blocks();
    const int rank = (int)cluster.block_rank();
    const int cid = (int)blockIdx.x / CS;
    const int nClusters = (int)gridDim.x / CS;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __shared__ ClusterShared sh;
    const bool skip = (ld_volatile_i32(&S.ctl->errFlags) & kErrStepAbort) != 0;
    for (int r = cid; r < S.R && !skip; r += nClusters) {
        const RepDyn &d = S.dyn[r];
        const RepParams &P = S.par[r];
        const int nCon = d.nCon;
        if (nCon <= 0) continue;
        const int chunk = (nCon + CS - 1) / CS;
        const int lo = rank * chunk, hi = min(lo + chunk, nCon);
        if (threadIdx.x == 0) {
            sh.mode = kModeG0;
            sh.alpha = 0.0f;
            sh.alphaPrev = 0.0;
        }
        __syncthreads();
        for (int p = 0;; p++) {
            const int mode = sh.mode;
            const float alpha = sh.alpha;
            const bool odd = (p & 1) != 0;
            const float2 *const stIn = odd ? V.st[0] : V.st[1];
            float2 *const stOut = odd ? V.st[1] : V.st[0];
            float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f, am = 0.0f;
            for (int i = lo + (int)threadIdx.x; i < hi; i += kClusterThreads) {
                float v0 = 0.0f, v1 = 0.0f, v2 = 0.0f, rm = 0.0f;
                row_update<float>(V, d.conStart + i, mode, alpha, stIn, stOut, v0, v1, v2, rm, &S.ctl->errFlags,
                                  RowCache{});
                a0 += v0;
                a1 += v1;
                a2 += v2;
                am = rm > am ? rm : am;
            }
            a0 = warp_tree_sum_t<float>(a0);
            a1 = warp_tree_sum_t<float>(a1);
            a2 = warp_tree_sum_t<float>(a2);
#pragma unroll
            for (int off = 16; off >= 1; off >>= 1) am = fmaxf(am, __shfl_down_sync(0xffffffffu, am, off));
            if (lane == 0) {
                sh.warpVal[warp][0] = a0;
                sh.warpVal[warp][1] = a1;
                sh.warpVal[warp][2] = a2;
                sh.warpVal[warp][3] = am;
            }
            __syncthreads();
            if (warp == 0) {
                double b0 = lane < kClusterWarps ? sh.warpVal[lane][0] : 0.0;
                double b1 = lane < kClusterWarps ? sh.warpVal[lane][1] : 0.0;
                double b2 = lane < kClusterWarps ? sh.warpVal[lane][2] : 0.0;
                double bm = lane < kClusterWarps ? sh.warpVal[lane][3] : 0.0;
                b0 = warp_tree_sum_t<double>(b0);
                b1 = warp_tree_sum_t<double>(b1);
                b2 = warp_tree_sum_t<double>(b2);
                bm = __longlong_as_double(warp_max_bits(__double_as_longlong(bm)));
                if (lane == 0) {
                    sh.part[p & 1][0] = b0;
                    sh.part[p & 1][1] = b1;
                    sh.part[p & 1][2] = b2;
                    sh.part[p & 1][3] = bm;
                }
            }
            // every CTA's partials and iterates are complete and visible
            cluster.sync();
            if (threadIdx.x == 0) {
                double t0 = 0.0, t1 = 0.0, t2 = 0.0, mx = 0.0;
                for (int q = 0; q < CS; q++) {
                    const double *pp = cluster.map_shared_rank(&sh.part[p & 1][0], q);
                    t0 = t0 + pp[0];
                    t1 = t1 + pp[1];
                    t2 = t2 + pp[2];
                    mx = pp[3] > mx ? pp[3] : mx;
                }
                int next = kModeCopy, status = -1, iter = 0;
                double alphaNew = sh.alphaPrev;
                if (p == 0) {
                    if (isinf(mx))
                        status = ALENS_NAN_DETECTED;
                    else if (mx <= P.tol)
                        status = ALENS_OK;
                    else if (P.maxIte <= 0)
                        status = ALENS_NOT_CONVERGED;
                    else
                        next = kModeAG;
                } else if (p == 1) {
                    alphaNew = (t1 > 0.0) ? t0 / t1 : 1.0;
                    if (!(alphaNew > 0.0) || isinf(alphaNew)) alphaNew = 1.0;
                    next = kModeIter;
                } else {
                    const int it = p - 1;
                    iter = it;
                    if (isinf(mx)) {
                        status = ALENS_NAN_DETECTED;
                    } else if (mx <= P.tol) {
                        status = ALENS_OK;
                    } else {
                        if (t1 > 0.0) {
                            const double a = (it & 1) ? t0 / t1 : t1 / t2;
                            if (a > 0.0 && !isinf(a)) alphaNew = a;
                        }
                        if (it >= P.maxIte)
                            status = ALENS_NOT_CONVERGED;
                        else
                            next = kModeIter;
                    }
                }
                sh.alphaPrev = alphaNew;
                sh.alpha = (float)alphaNew;
                sh.mode = next;
                if (status >= 0 && rank == 0) {
                    RepDyn *dw = &S.dyn[r];
                    dw->status = status;
                    dw->converged = status == ALENS_OK ? 1 : 0;
                    dw->iter = iter;
                    dw->res = mx;
                    dw->active = 0;
                    dw->finalPar = p & 1;
                }
            }
            __syncthreads();
            if (sh.mode == kModeCopy) break;
            if (p > P.maxIte + 3) break;
        }
        // the next replica reuses the partial slots only after every CTA
        // has read them
        cluster.sync();
    }
    // no CTA leaves while a peer may still read its shared memory
    cluster.sync();
}

int cluster_max_size() {
    static int cached = -1;
    if (cached >= 0) return cached;
    cudaFuncSetAttribute(k_solve_cluster, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    cudaGetLastError();
    int best = 1;
    for (int cs : {16, 8, 4, 2}) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(cs);
        cfg.blockDim = dim3(kClusterThreads);
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = cs;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        int n = 0;
        if (cudaOccupancyMaxActiveClusters(&n, k_solve_cluster, &cfg) == cudaSuccess && n > 0) {
            best = cs;
            break;
        }
        cudaGetLastError();
    }
    cached = best;
    return best;
}

int cluster_max_active(int cs) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(cs);
    cfg.blockDim = dim3(kClusterThreads);
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = cs;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, k_solve_cluster, &cfg) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

cudaError_t launch_solve_fp32_cluster(const DevState &S, int clusterSize, int nClusters, cudaStream_t st) {
    SolveView<float> V{};
    V.aptr = S.aptr;
    V.aent = S.aent32;
    V.st[0] = S.st32[0];
    V.st[1] = S.st32[1];
    V.qc = S.qc32;
    V.lbGeneral = S.lb;
    V.alphaBuf = S.alphaBuf;
    V.fp64 = 0;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(clusterSize * nClusters);
    cfg.blockDim = dim3(kClusterThreads);
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = clusterSize;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_solve_cluster, S, V);
}

}  // namespace alens
