// kernels_mixed.cu - BBPGD with FP32 bulk arithmetic: FP32 Delassus
// operator, gamma, g and per-warp partial sums (half the bytes and 1/64 of
// the FP64 instruction cost on GB300); FP64 accumulation of the dot
// products, step sizes and the refinement sweeps that follow
// (kernels_solve.cu).
//
// Compiled with FMA contraction (this path is not bit-compared).
#include "solve_impl.cuh"

namespace alens {

int solver_max_grid_fp32() {
    int dev = 0, nsm = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_solve<float>, kSolveThreads, 0);
    return nsm * (per > 0 ? per : 0);
}

cudaError_t launch_solve_fp32(const DevState &S, int grid, unsigned long long timeout_ns, cudaStream_t st) {
    SolveView<float> V{};
    V.aptr = S.aptr;
    V.acol = S.acol;
    V.aval = S.aval32;
    V.gam[0] = S.sgam32[0];
    V.gam[1] = S.sgam32[1];
    V.g[0] = S.sg32[0];
    V.g[1] = S.sg32[1];
    V.q = S.q32;
    V.lb = S.lb32;
    V.cinv = S.cinv32;
    V.alphaBuf = S.alphaBuf;
    V.fp64 = 0;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(kSolveThreads);
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_solve<float>, S, V, timeout_ns);
}

}  // namespace alens
