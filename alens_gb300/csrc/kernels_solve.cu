// kernels_solve.cu - FP64 BBPGD (bit-compatible with the oracle), solver
// state reset, velocity write-back + Euler update (SimToolbox
// SylinderSystem::stepEuler, SRC/TubuleSystem.cpp:55) and the constraint
// stress sum (calcConStress, SRC/TubuleSystem.cpp:224).
//
// Compiled with --fmad=false.
#include "solve_impl.cuh"

namespace alens {

namespace {

__device__ __forceinline__ int flags(const DevState &S) { return ld_volatile_i32(&S.ctl->errFlags); }

// Re-arm the solver state of every replica; with from32, gamma starts from
// the FP32 solution (refinement sweeps of the mixed solver).
__global__ void k_solver_reset(DevState S, int from32) {
    if (flags(S) & (kErrOverflow | kErrNaN | kErrTimeout)) return;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        int active = 0;
        for (int r = 0; r < S.R; r++) {
            RepDyn &d = S.dyn[r];
            d.refineIter = d.iter;  // iterations of the previous (FP32) solve
            d.iter = 0;
            d.active = d.nCon > 0 ? 1 : 0;
            d.converged = d.nCon > 0 ? 0 : 1;
            d.status = 0;
            d.counter = 0;
            d.alpha = 0.0;
            d.res = 0.0;
            active += d.active;
        }
        S.ctl->activeCount = active;
        S.ctl->bar.count = 0;
        S.ctl->bar.gen = 0;
    }
    if (from32) {
        const int nc = S.ctl->totalCon;
        for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nc; k += gridDim.x * blockDim.x) {
            const double g = (double)S.gamma32[k];
            const double lb = S.lb[k];
            S.gamma[k] = g < lb ? lb : g;
        }
    }
}

__global__ void k_advance(DevState S) {
    if (flags(S) & (kErrOverflow | kErrNaN | kErrTimeout)) return;
    const size_t st = (size_t)S.nRods;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < S.nRods; r += gridDim.x * blockDim.x) {
        const int rep = S.rodRep[r];
        const RepParams &P = S.par[rep];
        if (S.imm[r]) {
#pragma unroll
            for (int c = 0; c < 6; c++) S.vel[c * st + r] = 0.0;
            continue;
        }
        double F[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
        const int e1 = S.rowPtr[r + 1];
        for (int e = S.rowPtr[r]; e < e1; e++) {
            const int ent = S.rowEnt[e];
            const int k = ent >> 1;
            const double *J = S.jac + 12 * (size_t)k + 6 * (ent & 1);
            const double gk = S.gamma[k];
#pragma unroll
            for (int c = 0; c < 6; c++) F[c] = F[c] + gk * J[c];
        }
        const double a[3] = {S.ax[r], S.ay[r], S.az[r]};
        const double m[3] = {S.m0[r], S.m1[r], S.m2[r]};
        double Uc[6], U[6];
        mobility_apply<double>(a, m, S.sph[r] != 0, P.mono != 0, F, Uc);
#pragma unroll
        for (int c = 0; c < 6; c++) U[c] = Uc[c] + S.unc[c * st + r];
#pragma unroll
        for (int c = 0; c < 6; c++) S.vel[c * st + r] = U[c];
        const double dt = P.dt;
        double p[3];
        p[0] = S.px[r] + dt * U[0];
        p[1] = S.py[r] + dt * U[1];
        p[2] = S.pz[r] + dt * U[2];
        const double w0 = U[3], w1 = U[4], w2 = U[5];
        const double wn2 = w0 * w0 + w1 * w1 + w2 * w2;
        if (wn2 > 0.0) {
            const double wn = sqrt(wn2);
            const double half = 0.5 * dt * wn;
            double sh, ch;
            det_sincos(half, &sh, &ch);
            const double kk = sh / wn;
            const double v0 = kk * w0, v1 = kk * w1, v2 = kk * w2;
            const double qx = S.qx[r], qy = S.qy[r], qz = S.qz[r], qw = S.qw[r];
            const double nw = ch * qw - (v0 * qx + v1 * qy + v2 * qz);
            const double nx = (ch * qx + qw * v0) + (v1 * qz - v2 * qy);
            const double ny = (ch * qy + qw * v1) + (v2 * qx - v0 * qz);
            const double nz = (ch * qz + qw * v2) + (v0 * qy - v1 * qx);
            const double nn = sqrt(nx * nx + ny * ny + nz * nz + nw * nw);
            S.qx[r] = nx / nn;
            S.qy[r] = ny / nn;
            S.qz[r] = nz / nn;
            S.qw[r] = nw / nn;
        }
        for (int d = 0; d < 3; d++) {
            if (!P.pbc[d]) continue;
            const double lo = P.lo[d], hi = P.hi[d], Lb = P.L[d];
            double v = p[d];
            for (int k = 0; k < 64; k++) {
                if (v < lo)
                    v = v + Lb;
                else if (v >= hi)
                    v = v - Lb;
                else
                    break;
            }
            p[d] = v;
        }
        S.px[r] = p[0];
        S.py[r] = p[1];
        S.pz[r] = p[2];
    }
    // collision keys and gamma of this step for the next warm start
    const int totalColl = S.ctl->totalColl;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < totalColl; p += gridDim.x * blockDim.x) {
        const unsigned long long key = S.keys[p];
        const int rep = S.rodRep[(int)(key >> 32)];
        S.prevKeys[p] = key;
        S.prevGamma[p] = S.gamma[p + S.bilPrefix[rep]];
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        *S.prevCount = totalColl;
        S.ctl->step = S.ctl->step + 1;
    }
}

// Pair virial sum_k gamma_k (labI - labJ)_a n_b per replica, canonical tree.
__global__ void __launch_bounds__(256) k_stress_tiles(DevState S) {
    __shared__ double scr[9][8];
    const int nTiles = S.ctl->nTiles;
    const size_t tc = (size_t)S.tileCap;
    for (int T = blockIdx.x; T < nTiles; T += gridDim.x) {
        const int rep = S.tileRep[T];
        const RepDyn &d = S.dyn[rep];
        const int local = (T - d.tileStart) * kTile + (int)threadIdx.x;
        double v[9];
#pragma unroll
        for (int q = 0; q < 9; q++) v[q] = 0.0;
        if (local < d.nCon) {
            const int k = d.conStart + local;
            const double gk = S.gamma[k];
#pragma unroll
            for (int a = 0; a < 3; a++) {
                const double r = S.lab[6 * (size_t)k + a] - S.lab[6 * (size_t)k + 3 + a];
#pragma unroll
                for (int b = 0; b < 3; b++) v[3 * a + b] = gk * r * S.jac[12 * (size_t)k + b];
            }
        }
        block_tree_sum256<9>(v, scr);
        if (threadIdx.x == 0)
#pragma unroll
            for (int q = 0; q < 9; q++) S.part[q * tc + T] = v[q];
        __syncthreads();
    }
}

__global__ void __launch_bounds__(256) k_stress_final(DevState S) {
    __shared__ double scr[9][8];
    const size_t tc = (size_t)S.tileCap, wc = (size_t)S.workCap;
    // replicas one after another: they share the chunk work space
    for (int r = 0; r < S.R; r++) {
        const RepDyn &d = S.dyn[r];
        const double *src[9];
        double *work[9];
        for (int q = 0; q < 9; q++) {
            src[q] = S.part + q * tc + d.tileStart;
            work[q] = S.work + q * wc;
        }
        const double *const(&srcr)[9] = src;
        double *const(&workr)[9] = work;
        double out[9];
        chunk_reduce_cg<9>(srcr, d.nTiles, workr, out, scr);
        if (threadIdx.x == 0)
            for (int q = 0; q < 9; q++) S.stress[9 * r + q] = out[q];
        __syncthreads();
    }
}

template <class Real>
int max_grid_for(void (*kernel)(DevState, SolveView<Real>, unsigned long long)) {
    int dev = 0, nsm = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, 256, 0);
    return nsm * (per > 0 ? per : 0);
}

}  // namespace

// defined in kernels_mixed.cu
cudaError_t launch_solve_fp32(const DevState &S, int grid, unsigned long long timeout_ns, cudaStream_t st);
int solver_max_grid_fp32();

int solver_max_grid(int precision) {
    if (precision == ALENS_PREC_MIXED) {
        const int a = solver_max_grid_fp32();
        const int b = max_grid_for<double>(k_solve<double>);
        return a < b ? a : b;
    }
    return max_grid_for<double>(k_solve<double>);
}

static cudaError_t launch_coop_fp64(const DevState &S, int grid, unsigned long long timeout_ns,
                                    cudaStream_t st) {
    SolveView<double> V{S.jac, S.gamma, S.g, S.q, S.lb, S.cinv, S.U};
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(256);
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_solve<double>, S, V, timeout_ns);
}

cudaError_t launch_solve(const DevState &S, int grid, int precision, unsigned long long timeout_ns,
                         cudaStream_t st, cudaEvent_t *ev, int *launches) {
    int n = 0;
    cudaError_t e;
    if (ev) cudaEventRecord(ev[0], st);
    if (precision == ALENS_PREC_MIXED) {
        e = launch_solve_fp32(S, grid, timeout_ns, st);
        if (e != cudaSuccess) return e;
        if (ev) cudaEventRecord(ev[1], st);
        k_solver_reset<<<256, 256, 0, st>>>(S, 1);
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        if (ev) cudaEventRecord(ev[2], st);
        e = launch_coop_fp64(S, grid, timeout_ns, st);
        if (ev) cudaEventRecord(ev[3], st);
        n = 3;
    } else {
        e = launch_coop_fp64(S, grid, timeout_ns, st);
        if (ev) {
            cudaEventRecord(ev[1], st);
            cudaEventRecord(ev[2], st);
            cudaEventRecord(ev[3], st);
        }
        n = 1;
    }
    if (launches) *launches += n;
    return e;
}

void launch_advance(const DevState &S, cudaStream_t st) {
    int g = (S.nRods + 255) / 256;
    if (g < 1) g = 1;
    if (g > 4096) g = 4096;
    k_advance<<<g, 256, 0, st>>>(S);
}

void launch_stress(const DevState &S, cudaStream_t st) {
    k_stress_tiles<<<1024, 256, 0, st>>>(S);
    k_stress_final<<<1, 256, 0, st>>>(S);
}

}  // namespace alens
