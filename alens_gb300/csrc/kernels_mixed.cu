// kernels_mixed.cu - BBPGD with FP32 bulk arithmetic: FP32 Jacobian,
// velocities, gamma and g (half the bytes of the FP64 solve); FP64 dot
// products, residual and Barzilai-Borwein step sizes.  The FP64 solver then
// runs from the FP32 solution as the refinement sweeps (kernels_solve.cu).
//
// Compiled with FMA contraction (this path is not bit-compared).
#include "solve_impl.cuh"

namespace alens {

int solver_max_grid_fp32() {
    int dev = 0, nsm = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_solve<float>, 256, 0);
    return nsm * (per > 0 ? per : 0);
}

cudaError_t launch_solve_fp32(const DevState &S, int grid, unsigned long long timeout_ns, cudaStream_t st) {
    SolveView<float> V{S.jac32, S.gamma32, S.g32, S.q32, S.lb32, S.cinv32, S.U32};
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(256);
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_solve<float>, S, V, timeout_ns);
}

}  // namespace alens
