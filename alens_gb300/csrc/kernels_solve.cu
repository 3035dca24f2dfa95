// kernels_solve.cu - FP64 BBPGD launch (bit-compatible with the oracle),
// the hand-over from the FP32 solver to the FP64 refinement sweeps, the
// final gamma gather, velocity write-back + Euler update (SimToolbox
// SylinderSystem::stepEuler, SRC/TubuleSystem.cpp:55) and the constraint
// stress sum (calcConStress, SRC/TubuleSystem.cpp:224).
//
// Compiled with --fmad=false.
#include "solve_impl.cuh"

namespace alens {

namespace {

__device__ __forceinline__ int flags(const DevState &S) { return ld_volatile_i32(&S.ctl->errFlags); }

// Start of the FP64 refinement: gamma0 = the FP32 solution promoted and
// projected, and the FP64 residual of that point computed as the FP64
// solver's first pass would (the same entries, order and operations), max
// per replica.  The last block to finish (ticket counter, no waiting)
// re-arms the replicas: those within tolerance are marked refined and keep
// the FP32 status; when all are, the FP64 launch returns at once.  The FP32
// iteration count is kept in refineIter.
__global__ void k_refine_setup(DevState S) {
    ALENS_PDL_PROLOGUE();
    __shared__ int s_last;
    if (flags(S) & kErrStepAbort) return;
    const int nIdx = S.ctl->nTiles * kRowTile;
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < nIdx; idx += gridDim.x * blockDim.x) {
        const int T = idx / kRowTile;
        const int rep = S.tileRep[T];
        RepDyn &d = S.dyn[rep];
        const int local = (T - d.tileStart) * kRowTile + idx % kRowTile;
        unsigned long long bits = 0ULL;  // residual of this row (0: not counted)
        if (local < d.nCon) {
            const int k = d.conStart + local;
            const float2 *src = d.finalPar ? S.st32[1] : S.st32[0];
            const double lbk = S.lb[k];
            double xk = (double)src[k].x;
            xk = xk < lbk ? lbk : xk;
            S.st[1][k] = make_double2(xk, 0.0);
            if (!d.refined && d.status == ALENS_OK) {
                double acc = 0.0;
                const int e0 = S.aptr[k], e1 = S.aptr[k + 1];
                for (int eb = e0; eb < e1; eb += kRowPrefetch) {
                    int4 en[kRowPrefetch];
                    float xs[kRowPrefetch];
#pragma unroll
                    for (int j = 0; j < kRowPrefetch; j++)
                        en[j] = eb + j < e1 ? __ldg(S.aent + eb + j) : make_int4(k, 1, 0, 0);
#pragma unroll
                    for (int j = 0; j < kRowPrefetch; j++) xs[j] = src[en[j].x].x;
#pragma unroll
                    for (int j = 0; j < kRowPrefetch; j++) {
                        if (eb + j < e1) {
                            const double lbl = en[j].y == 0 ? 0.0 : (en[j].y == 1 ? -INFINITY : S.lb[en[j].x]);
                            double xl = (double)xs[j];
                            xl = xl < lbl ? lbl : xl;
                            acc = fma(__hiloint2double(en[j].w, en[j].z), xl, acc);
                        }
                    }
                }
                acc = fma(S.qc[k].y, xk, acc);
                const double gn = acc + S.qc[k].x;
                const double pr = xk - gn < lbk ? lbk : xk - gn;
                const double rr = fabs(xk - pr);
                bits = (unsigned long long)__double_as_longlong(rr == rr ? rr : INFINITY);
            }
        }
        // max over the warp's lanes of the same replica (non-negative
        // doubles order like their bit patterns), one atomic per group: a
        // per-row atomic on the replica's word serialises at one L2 slice
        const unsigned int act = __activemask();
        const unsigned int grp = __match_any_sync(act, rep);
        const unsigned int hi = (unsigned int)(bits >> 32);
        const unsigned int hiMax = __reduce_max_sync(grp, hi);
        const unsigned int loMax = __reduce_max_sync(grp, hi == hiMax ? (unsigned int)bits : 0u);
        if ((threadIdx.x & 31) == __ffs(grp) - 1 && (hiMax | loMax) != 0u)
            atomicMax(&d.res64bits, ((unsigned long long)hiMax << 32) | loMax);
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) s_last = atomicAdd(&S.ctl->setupDone, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!s_last || threadIdx.x != 0) return;
    __threadfence();
    int all = 1;
    for (int r = 0; r < S.R; r++) {
        RepDyn &d = S.dyn[r];
        d.refineIter = d.iter;
        d.iter = 0;
        if (d.nCon <= 0) continue;
        if (!d.refined && d.status == ALENS_OK) {
            const double res = __longlong_as_double((long long)ld_acquire_u64(&d.res64bits));
            if (res <= S.par[r].tol) {
                d.refined = 1;
                d.res = res;
            }
        }
        if (d.refined) {
            // FP64 residual verified: the FP64 pass copies the replica's
            // values through (status, residual kept)
            d.active = 0;
            continue;
        }
        all = 0;
        d.active = 1;
        d.converged = 0;
        d.status = 0;
        d.res = 0.0;
    }
    S.ctl->allRefined = all;
    S.ctl->setupDone = 0u;
    // re-arm the barrier and pass counters for the FP64 launch that follows
    DevCtl *c = S.ctl;
    c->activeCnt[0] = c->activeCnt[1] = c->activeCnt[2] = 0;
    c->bar.count = 0;
    c->bar.gen = 0;
    c->bar.pass[0][0] = c->bar.pass[1][0] = c->bar.pass[2][0] = 0u;
    c->finalParity = 1;
}

// The solution into gamma (alens_solve reports it before the update; a
// full step leaves the copy to k_advance).
__global__ void k_solver_finish(DevState S) {
    ALENS_PDL_PROLOGUE();
    if (flags(S) & kErrStepAbort) return;
    const int nc = S.ctl->totalCon;
    const double2 *src = S.ctl->finalParity ? S.st[1] : S.st[0];
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nc; k += gridDim.x * blockDim.x)
        S.gamma[k] = src[k].x;
}

__global__ void k_advance(DevState S) {
    ALENS_PDL_PROLOGUE();
    if (flags(S) & kErrStepAbort) return;
    const size_t st = (size_t)S.nRods;
    // the solver's last iterate (the solution)
    const double2 *fin = S.ctl->finalParity ? S.st[1] : S.st[0];
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
        constexpr int kB = 8;
        for (int eb = S.rowPtr[r]; eb < e1; eb += kB) {
            // the batch's entries, then their multipliers and Jacobian rows,
            // are requested before any is used; the sums keep entry order
            int ent[kB];
#pragma unroll
            for (int j = 0; j < kB; j++) ent[j] = eb + j < e1 ? S.rowEnt[eb + j] : -1;
            double gk[kB];
#pragma unroll
            for (int j = 0; j < kB; j++) gk[j] = ent[j] >= 0 ? fin[ent[j] >> 1].x : 0.0;
#pragma unroll
            for (int j = 0; j < kB; j++) {
                if (ent[j] < 0) continue;
                const double *J = S.jac + 12 * (size_t)(ent[j] >> 1) + 6 * (ent[j] & 1);
#pragma unroll
                for (int c = 0; c < 6; c++) F[c] = F[c] + gk[j] * J[c];
            }
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
    // the solution into gamma, and the collision keys and multipliers of
    // this step for the next warm start
    const int nc = S.ctl->totalCon;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nc; k += gridDim.x * blockDim.x) S.gamma[k] = fin[k].x;
    const int totalColl = S.ctl->totalColl;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < totalColl; p += gridDim.x * blockDim.x) {
        const unsigned long long key = S.keys[p];
        const int rep = S.rodRep[(int)(key >> 32)];
        S.prevKeys[p] = key;
        S.prevGamma[p] = fin[p + S.bilPrefix[rep]].x;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        *S.prevCount = totalColl;
        S.ctl->step = S.ctl->step + 1;
    }
}

// Pair virial sum_k gamma_k (labI - labJ)_a n_b per replica with the
// canonical tree: 64-constraint tiles (two warp trees, then warp0 + warp1),
// then chunk reduction per replica.
__global__ void __launch_bounds__(256) k_stress_tiles(DevState S) {
    __shared__ double tv[4][2][9];
    const int nTiles = S.ctl->nTiles;
    const size_t tc = (size_t)S.tileCap;
    const int group = threadIdx.x >> 6, lane64 = threadIdx.x & 63, w = (threadIdx.x >> 5) & 1;
    for (int base = blockIdx.x * 4; base < nTiles; base += gridDim.x * 4) {
        const int T = base + group;
        double v[9];
#pragma unroll
        for (int q = 0; q < 9; q++) v[q] = 0.0;
        if (T < nTiles) {
            const RepDyn &d = S.dyn[S.tileRep[T]];
            const int local = (T - d.tileStart) * kTile + lane64;
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
        }
#pragma unroll
        for (int q = 0; q < 9; q++) v[q] = warp_tree_sum_t<double>(v[q]);
        if ((threadIdx.x & 31) == 0)
#pragma unroll
            for (int q = 0; q < 9; q++) tv[group][w][q] = v[q];
        __syncthreads();
        if (threadIdx.x < 4 && base + (int)threadIdx.x < nTiles) {
            const int g = threadIdx.x;
            for (int q = 0; q < 9; q++) S.part[q * tc + base + g] = tv[g][0][q] + tv[g][1][q];
        }
        __syncthreads();
    }
}

__global__ void k_stress_final(DevState S) {
    __shared__ double chunk[9][64];
    const size_t tc = (size_t)S.tileCap;
    for (int r = 0; r < S.R; r++) {
        const RepDyn &d = S.dyn[r];
        const double *src[9];
        for (int q = 0; q < 9; q++) src[q] = S.part + q * tc + d.tileStart;
        const double *const(&srcr)[9] = src;
        double out[9];
        warp_chunk_reduce<9>(srcr, d.nTiles, chunk, out, nullptr, nullptr);
        if (threadIdx.x == 0)
            for (int q = 0; q < 9; q++) S.stress[9 * r + q] = out[q];
        __syncwarp();
    }
}

int occupancy_grid(const void *kernel) {
    int dev = 0, nsm = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSolveDynSmem);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, kSolveThreads, kSolveDynSmem);
    return nsm * (per > 0 ? per : 0);
}

template <class Real>
cudaError_t launch_coop(const DevState &S, const SolveView<Real> &V, int grid,
                        unsigned long long timeout_ns, cudaStream_t st) {
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
    return cudaLaunchKernelEx(&cfg, k_solve<Real>, S, V, timeout_ns);
}

}  // namespace

// defined in kernels_mixed.cu
cudaError_t launch_solve_fp32(const DevState &S, int grid, unsigned long long timeout_ns, cudaStream_t st);
cudaError_t launch_solve_fp32_cluster(const DevState &S, int clusterSize, int nClusters, cudaStream_t st);
int solver_max_grid_fp32();
// defined in kernels_csm.cu
cudaError_t launch_solve_fp32_csm(const DevState &S, int clusterSize, int nClusters, cudaStream_t st);
// defined in kernels_fast.cu
cudaError_t launch_solve_fast(const DevState &S, int grid, unsigned long long timeout_ns, cudaStream_t st);

int solver_max_grid(int precision) {
    int g = occupancy_grid((const void *)k_solve<double>);
    if (precision == ALENS_PREC_MIXED) {
        const int a = solver_max_grid_fp32();
        g = a < g ? a : g;
    }
    return g < kMaxSolverGrid ? g : kMaxSolverGrid;
}

cudaError_t launch_solve(const DevState &S, int grid, int precision, unsigned long long timeout_ns,
                         cudaStream_t st, cudaEvent_t *ev, int *launches, int form, int clusterSize,
                         int nClusters, bool finish) {
    int n = 0;
    cudaError_t e;
    SolveView<double> V{};
    V.aptr = S.aptr;
    V.aent = S.aent;
    V.st[0] = S.st[0];
    V.st[1] = S.st[1];
    V.qc = S.qc;
    V.lbGeneral = S.lb;
    V.alphaBuf = S.alphaBuf;
    V.fp64 = 1;
    if (ev) cudaEventRecord(ev[0], st);
    if (precision == ALENS_PREC_MIXED && form == kFormFast) {
        // FP32 iterations, FP64 check and refinement in one launch
        e = launch_solve_fast(S, grid, timeout_ns, st);
        n++;
        if (ev) {
            cudaEventRecord(ev[1], st);
            cudaEventRecord(ev[2], st);
            cudaEventRecord(ev[3], st);
        }
    } else if (precision == ALENS_PREC_MIXED) {
        if (form == kFormResident)
            e = launch_solve_fp32_csm(S, clusterSize, nClusters, st);
        else if (form == kFormCluster)
            e = launch_solve_fp32_cluster(S, clusterSize, nClusters, st);
        else
            e = launch_solve_fp32(S, grid, timeout_ns, st);
        if (e != cudaSuccess) return e;
        if (ev) cudaEventRecord(ev[1], st);
        launch_pdl(k_refine_setup, dim3(8 * (grid > 0 ? grid : 1)), dim3(32), 0, st, S);
        n += 2;
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        if (ev) cudaEventRecord(ev[2], st);
        e = launch_coop<double>(S, V, grid, timeout_ns, st);
        n++;
        if (ev) cudaEventRecord(ev[3], st);
    } else {
        e = launch_coop<double>(S, V, grid, timeout_ns, st);
        n++;
        if (ev) {
            cudaEventRecord(ev[1], st);
            cudaEventRecord(ev[2], st);
            cudaEventRecord(ev[3], st);
        }
    }
    if (e != cudaSuccess) return e;
    if (finish) {
        launch_pdl(k_solver_finish, dim3(512), dim3(256), 0, st, S);
        n++;
    }
    if (launches) *launches += n;
    return cudaGetLastError();
}

void launch_advance(const DevState &S, cudaStream_t st) {
    // one-warp blocks: the update is FP64-pipe bound (2 lanes/clk/SM on
    // GB300), so the rods are spread evenly over every SM
    int g = (S.nRods + 31) / 32;
    if (g < 1) g = 1;
    if (g > 16384) g = 16384;
    launch_pdl(k_advance, dim3(g), dim3(32), 0, st, S);
}

void launch_stress(const DevState &S, cudaStream_t st) {
    k_stress_tiles<<<1024, 256, 0, st>>>(S);
    k_stress_final<<<1, 32, 0, st>>>(S);
}

}  // namespace alens
