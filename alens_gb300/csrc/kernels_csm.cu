// kernels_csm.cu - cluster-resident FP32 BBPGD ("csm" form).
//
// The role of SimToolbox BCQPSolver's BBPGD (conSolverChoice 0,
// docs/source/quickstart.md:356-358) in mixed precision, laid out for a
// thread-block cluster: one cluster of up to 16 CTAs solves one replica
// with the whole problem held in the CTAs' shared memory.
//
//  * rows of the replica's Delassus operator are split into CS contiguous
//    chunks; CTA rank q keeps its chunk's rows in shared memory: packed
//    entries (owner rank, local row, bound kind | FP32 value), (q, cinv),
//    bounds and the iterates (gamma, g) of both pass parities;
//  * a pass reads every neighbour iterate through distributed shared memory
//    (ld.shared::cluster), writes its own rows' iterates locally, reduces
//    its partial dot products (FP32 per thread and warp, FP64 across warps)
//    and ends with one hardware cluster barrier; every CTA then sums the CS
//    partials in rank order (FP64) and takes the same decision;
//  * after convergence the FP32 solution's residual is evaluated once in
//    FP64 (FP64 operator values and q from global memory); when it meets
//    the tolerance the replica needs no FP64 refinement sweep.
//
// No grid-wide synchronisation and no global-memory traffic inside the
// iteration: the operator is read from HBM once per step.  Problems whose
// rows do not fit the clusters' shared memory set kErrSolverFit and the
// host reruns the step with the grid form.
//
// Compiled with FMA contraction (not bit-compared).
#include <cooperative_groups.h>

#include "solve_impl.cuh"

namespace cg = cooperative_groups;

namespace alens {

namespace {

constexpr int kCsmRowCap = 2048;        // rows per CTA
constexpr int kCsmMaxThreads = 1024;
constexpr int kCsmBatch = 8;            // entries whose loads are issued together

struct CsmCtl {
    double part[2][4];   // this CTA's partials by pass parity
    double warpVal[kCsmMaxThreads / 32][4];
    double alphaPrev;
    double res64;        // FP64 residual max of this CTA's rows
    float alpha;
    int mode;
    int fit;
    int status;          // status decided in the last pass (-1: none yet)
};

// byte offsets inside the dynamic shared memory
struct CsmLayout {
    static constexpr size_t ctl = 0;
    static constexpr size_t st0 = 2048;
    static constexpr size_t parity = 8 * kCsmRowCap;      // st1 = st0 + parity
    static constexpr size_t qc = st0 + 2 * parity;
    static constexpr size_t lb = qc + 8 * kCsmRowCap;
    static constexpr size_t rp = lb + 4 * kCsmRowCap;
    static constexpr size_t rowStart = rp + 4 * (kCsmRowCap + 16);
    static constexpr size_t ent = rowStart + 4 * (kCsmMaxThreads + 16);
};
static_assert(sizeof(CsmCtl) <= CsmLayout::st0, "csm control block");

__device__ __forceinline__ uint32_t cluster_addr(const void *p, int rank) {
    uint32_t a = (uint32_t)__cvta_generic_to_shared(p), r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
    return r;
}

__device__ __forceinline__ float2 ld_cluster_f2(uint32_t addr) {
    float2 v;
    asm volatile("ld.shared::cluster.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(addr));
    return v;
}

__device__ __forceinline__ double ld_cluster_d(uint32_t addr) {
    double v;
    asm volatile("ld.shared::cluster.f64 %0, [%1];" : "=d"(v) : "r"(addr));
    return v;
}

__device__ __forceinline__ int ld_cluster_i(uint32_t addr) {
    int v;
    asm volatile("ld.shared::cluster.s32 %0, [%1];" : "=r"(v) : "r"(addr));
    return v;
}

__device__ __forceinline__ void cluster_barrier() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// Shared-memory views of one CTA.
struct CsmView {
    CsmCtl *c;
    float2 *st0;      // st[parity] = st0 + parity * kCsmRowCap
    float2 *qc;
    float *lb;
    int *rp;
    int *rowStart;
    uint2 *ent;       // {cluster address of the neighbour's parity-0 slot | bound kind, FP32 value}
};

// Neighbour value x_l of one operator entry in a pass of mode MODE.
template <int MODE>
__device__ __forceinline__ float entry_x(float2 sv, uint32_t kind, float alpha) {
    if (MODE == kModeG0) return sv.x;
    if (MODE == kModeAG) return sv.y;
    const float x = fmaf(-alpha, sv.y, sv.x);
    return kind == 0 ? (x < 0.0f ? 0.0f : x) : x;  // kind 0: bound 0, kind 1: none
}

// Completion of row i: own value, step, residual and dot-product terms.
template <int MODE>
__device__ __forceinline__ void finish_row(const CsmView &v, int i, int pin, float acc, float alpha, float &a0,
                                           float &a1, float &a2, float &am, int *errFlags) {
    const float2 own = v.st0[pin * kCsmRowCap + i];
    const float lbk = v.lb[i];
    const float2 qc = v.qc[i];
    float xk;
    if (MODE == kModeG0)
        xk = own.x;
    else if (MODE == kModeAG)
        xk = own.y;
    else {
        xk = fmaf(-alpha, own.y, own.x);
        xk = xk < lbk ? lbk : xk;
    }
    acc = fmaf(qc.y, xk, acc);
    float2 *out = v.st0 + (pin ^ 1) * kCsmRowCap;
    if (MODE == kModeAG) {
        a0 = fmaf(own.y, own.y, a0);
        a1 = fmaf(own.y, acc, a1);
        out[i] = own;
        return;
    }
    const float gn = acc + qc.x;
    const float m = gn < xk - lbk ? gn : xk - lbk;
    float rm = fabsf(m);
    if (rm != rm) {
        atomicOr(errFlags, kErrNaN);
        rm = INFINITY;
    }
    am = rm > am ? rm : am;
    if (MODE == kModeIter) {
        const float s = xk - own.x, y = gn - own.y;
        a0 = fmaf(s, s, a0);
        a1 = fmaf(s, y, a1);
        a2 = fmaf(y, y, a2);
    }
    out[i] = make_float2(xk, gn);
}

// This thread's rows (contiguous, balanced by entry count) in one pass.
template <int MODE>
__device__ __forceinline__ void csm_rows(const CsmView &v, int pin, float alpha, float &a0, float &a1, float &a2,
                                         float &am, int *errFlags) {
    const int r0 = v.rowStart[threadIdx.x], r1 = v.rowStart[threadIdx.x + 1];
    if (r0 >= r1) return;
    const uint32_t pinOff = (uint32_t)(pin * CsmLayout::parity);
    int r = r0;
    int rowEnd = v.rp[r0 + 1];
    const int eEnd = v.rp[r1];
    float acc = 0.0f;
    for (int eb = v.rp[r0]; eb < eEnd; eb += kCsmBatch) {
        uint2 en[kCsmBatch];
        float2 sv[kCsmBatch];
#pragma unroll
        for (int j = 0; j < kCsmBatch; j++)
            if (eb + j < eEnd) en[j] = v.ent[eb + j];
#pragma unroll
        for (int j = 0; j < kCsmBatch; j++)
            if (eb + j < eEnd) sv[j] = ld_cluster_f2((en[j].x & ~7u) + pinOff);
#pragma unroll
        for (int j = 0; j < kCsmBatch; j++) {
            if (eb + j < eEnd) {
                acc = fmaf(__uint_as_float(en[j].y), entry_x<MODE>(sv[j], en[j].x & 3u, alpha), acc);
                if (eb + j + 1 == rowEnd) {
                    finish_row<MODE>(v, r, pin, acc, alpha, a0, a1, a2, am, errFlags);
                    acc = 0.0f;
                    r++;
                    rowEnd = r < r1 ? v.rp[r + 1] : 0x7fffffff;
                }
            }
        }
    }
}

// Block reduction of four per-thread values (three sums, one max) into
// ctl.part[par] (FP64 across warps).
template <int NT>
__device__ __forceinline__ void block_partials(CsmCtl &c, int par, float a0, float a1, float a2, float am) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    a0 = warp_tree_sum_t<float>(a0);
    a1 = warp_tree_sum_t<float>(a1);
    a2 = warp_tree_sum_t<float>(a2);
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) am = fmaxf(am, __shfl_down_sync(0xffffffffu, am, off));
    if (lane == 0) {
        c.warpVal[warp][0] = a0;
        c.warpVal[warp][1] = a1;
        c.warpVal[warp][2] = a2;
        c.warpVal[warp][3] = am;
    }
    __syncthreads();
    if (warp == 0) {
        constexpr int NW = NT / 32;
        double b0 = lane < NW ? c.warpVal[lane][0] : 0.0, b1 = lane < NW ? c.warpVal[lane][1] : 0.0;
        double b2 = lane < NW ? c.warpVal[lane][2] : 0.0, bm = lane < NW ? c.warpVal[lane][3] : 0.0;
        b0 = warp_tree_sum_t<double>(b0);
        b1 = warp_tree_sum_t<double>(b1);
        b2 = warp_tree_sum_t<double>(b2);
        bm = __longlong_as_double(warp_max_bits(__double_as_longlong(bm)));
        if (lane == 0) {
            c.part[par][0] = b0;
            c.part[par][1] = b1;
            c.part[par][2] = b2;
            c.part[par][3] = bm;
        }
    }
}

template <int NT>
__global__ void __launch_bounds__(NT, 1) k_solve_csm(DevState S, SolveView<float> V, int entCap) {
    extern __shared__ __align__(16) uint8_t sm[];
    cg::cluster_group cluster = cg::this_cluster();
    const int CS = (int)cluster.num_blocks();
    const int me = (int)cluster.block_rank();
    const int cid = (int)blockIdx.x / CS;
    const int nClusters = (int)gridDim.x / CS;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    CsmView v;
    v.c = reinterpret_cast<CsmCtl *>(sm + CsmLayout::ctl);
    v.st0 = reinterpret_cast<float2 *>(sm + CsmLayout::st0);
    v.qc = reinterpret_cast<float2 *>(sm + CsmLayout::qc);
    v.lb = reinterpret_cast<float *>(sm + CsmLayout::lb);
    v.rp = reinterpret_cast<int *>(sm + CsmLayout::rp);
    v.rowStart = reinterpret_cast<int *>(sm + CsmLayout::rowStart);
    v.ent = reinterpret_cast<uint2 *>(sm + CsmLayout::ent);
    CsmCtl &c = *v.c;
    // every CTA reads the same flags (nothing writes them while this runs)
    const bool skip = (ld_volatile_i32(&S.ctl->errFlags) & kErrStepAbort) != 0;
    for (int r = cid; r < S.R && !skip; r += nClusters) {
        const RepDyn &d = S.dyn[r];
        const RepParams &P = S.par[r];
        const int nCon = d.nCon;
        if (nCon <= 0) continue;
        const int k0 = d.conStart;
        const int chunk = (nCon + CS - 1) / CS;
        const int lo = min(me * chunk, nCon), hi = min(lo + chunk, nCon);
        const int nrow = hi - lo;
        const int eBeg = __ldg(V.aptr + k0 + lo), eEnd = __ldg(V.aptr + k0 + hi);
        const int nEnt = eEnd - eBeg;
        // ---- load this CTA's rows; general lower bounds are left to the grid form
        int fit = (chunk <= kCsmRowCap && nEnt <= entCap) ? 1 : 0;
        if (fit) {
            for (int i = tid; i < nrow; i += NT) {
                const int k = k0 + lo + i;
                v.qc[i] = __ldg(V.qc + k);
                v.st0[kCsmRowCap + i] = V.st[1][k];  // the solve starts from parity 1
                v.rp[i] = __ldg(V.aptr + k) - eBeg;
                v.lb[i] = (float)S.lb[k];
                if (S.lbKind[k] == 2) fit = 0;
            }
            if (tid == 0) v.rp[nrow] = nEnt;
            for (int e = tid; e < nEnt; e += NT) {
                const int4 en = __ldg(V.aent + eBeg + e);
                const int col = en.x - k0;
                const int owner = col / chunk;
                const uint32_t a = cluster_addr(v.st0 + (col - owner * chunk), owner);
                v.ent[e] = make_uint2(a | (uint32_t)(en.y & 3), (uint32_t)en.z);
            }
        }
        fit = __syncthreads_and(fit);
        if (fit && tid <= NT) {
            // rows of thread t: those whose first entry lies in [t E / NT, (t+1) E / NT)
            for (int t = tid; t <= NT; t += NT) {
                const long long target = (long long)nEnt * t / NT;
                int a = 0, b = nrow;
                while (a < b) {
                    const int m = (a + b) >> 1;
                    if (v.rp[m] < target)
                        a = m + 1;
                    else
                        b = m;
                }
                v.rowStart[t] = t == NT ? nrow : a;
            }
        }
        if (tid == 0) {
            c.fit = fit;
            c.mode = kModeG0;
            c.alpha = 0.0f;
            c.alphaPrev = 0.0;
            c.status = -1;
        }
        cluster_barrier();  // every CTA's rows are loaded and its fit flag set
        int allFit = 1;
        for (int q = 0; q < CS; q++) allFit &= ld_cluster_i(cluster_addr(&c.fit, q));
        if (!allFit) {
            if (me == 0 && tid == 0) atomicOr(&S.ctl->errFlags, kErrSolverFit);
            break;  // uniform: every CTA computed the same allFit
        }
        int p = 0;
        for (;; p++) {
            const int mode = c.mode;
            const float alpha = c.alpha;
            const int pin = (p & 1) ? 0 : 1;
            float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f, am = 0.0f;
            if (mode == kModeG0)
                csm_rows<kModeG0>(v, pin, alpha, a0, a1, a2, am, &S.ctl->errFlags);
            else if (mode == kModeAG)
                csm_rows<kModeAG>(v, pin, alpha, a0, a1, a2, am, &S.ctl->errFlags);
            else
                csm_rows<kModeIter>(v, pin, alpha, a0, a1, a2, am, &S.ctl->errFlags);
            block_partials<NT>(c, p & 1, a0, a1, a2, am);
            cluster_barrier();  // iterates and partials of pass p complete cluster-wide
            if (warp == 0) {
                double t0 = 0.0, t1 = 0.0, t2 = 0.0, mx = 0.0;
                if (lane < CS) {
                    const uint32_t pa = cluster_addr(&c.part[p & 1][0], lane);
                    t0 = ld_cluster_d(pa);
                    t1 = ld_cluster_d(pa + 8);
                    t2 = ld_cluster_d(pa + 16);
                    mx = ld_cluster_d(pa + 24);
                }
                t0 = warp_tree_sum_t<double>(t0);
                t1 = warp_tree_sum_t<double>(t1);
                t2 = warp_tree_sum_t<double>(t2);
                mx = __longlong_as_double(warp_max_bits(__double_as_longlong(mx)));
                if (lane == 0) {
                    int next = kModeCopy, status = -1, iter = 0;
                    double alphaNew = c.alphaPrev;
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
                    c.alphaPrev = alphaNew;
                    c.alpha = (float)alphaNew;
                    c.mode = next;
                    c.status = status;
                    if (status >= 0 && me == 0) {
                        RepDyn *dw = &S.dyn[r];
                        dw->status = status;
                        dw->converged = status == ALENS_OK ? 1 : 0;
                        dw->iter = iter;
                        dw->res = mx;
                        dw->active = 0;
                        dw->finalPar = p & 1;
                    }
                }
            }
            __syncthreads();
            if (c.mode == kModeCopy || p > P.maxIte + 3) break;
        }
        // ---- final iterate to global memory; FP64 residual of the FP32 solution
        const int fin = p & 1;  // parity written by the last pass
        const bool conv = c.status == ALENS_OK;
        const float2 *res = v.st0 + fin * kCsmRowCap;
        float2 *const gout = V.st[fin];
        const uint32_t finOff = (uint32_t)(fin * CsmLayout::parity);
        double rloc = 0.0;
        for (int i = tid; i < nrow; i += NT) {
            const int k = k0 + lo + i;
            gout[k] = res[i];
            // FP64: g = A x + cinv x + q with x the FP32 solution
            const double2 qc = S.qc[k];
            const int e0 = v.rp[i], e1 = v.rp[i + 1];
            double acc = 0.0;
            const double xk = (double)res[i].x, lbk = S.lb[k];
            for (int e = e0; e < e1; e++) {
                const int4 en = __ldg(S.aent + eBeg + e);
                const double xl = (double)ld_cluster_f2((v.ent[e].x & ~7u) + finOff).x;
                acc = fma(__hiloint2double(en.w, en.z), xl, acc);
            }
            acc = fma(qc.y, xk, acc);
            const double gn = acc + qc.x;
            const double pr = xk - gn < lbk ? lbk : xk - gn;
            const double rr = fabs(xk - pr);
            rloc = rr > rloc ? rr : rloc;
        }
        {
            long long b = warp_max_bits(__double_as_longlong(rloc));
            if (lane == 0) c.warpVal[warp][0] = __longlong_as_double(b);
            __syncthreads();
            if (warp == 0) {
                long long x = lane < NT / 32 ? __double_as_longlong(c.warpVal[lane][0]) : 0LL;
                x = warp_max_bits(x);
                if (lane == 0) c.res64 = __longlong_as_double(x);
            }
        }
        cluster_barrier();  // FP64 residuals ready; no remote reads of iterates after this
        if (tid == 0 && me == 0) {
            double mx = 0.0;
            for (int q = 0; q < CS; q++) {
                const double x = ld_cluster_d(cluster_addr(&c.res64, q));
                mx = x > mx ? x : mx;
            }
            RepDyn *dw = &S.dyn[r];
            if (conv && mx <= P.tol) {
                dw->refined = 1;
                dw->res = mx;
            } else {
                dw->refined = 0;
            }
        }
        cluster_barrier();  // rank 0 read the residuals before they are reused
    }
    // no CTA leaves while a peer may still read its shared memory
    cluster_barrier();
}

using CsmKernel = void (*)(DevState, SolveView<float>, int);

CsmKernel csm_kernel(int threads) {
    switch (threads) {
        case 256: return k_solve_csm<256>;
        case 1024: return k_solve_csm<1024>;
        default: return k_solve_csm<512>;
    }
}

int g_csm_threads = 512;

}  // namespace

size_t csm_smem_bytes() {
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    return (size_t)optin;
}

int csm_entry_capacity(size_t smem) {
    return smem > CsmLayout::ent ? (int)((smem - CsmLayout::ent) / 8) : 0;
}

// Threads per CTA of the cluster-resident solver (256, 512 or 1024).
void csm_set_threads(int threads) {
    g_csm_threads = (threads == 256 || threads == 1024) ? threads : 512;
}
int csm_threads() { return g_csm_threads; }

// Largest cluster size (16, 8, 4, 2) the device can co-schedule with the
// full shared memory; 0 if none.
int csm_cluster_size(int *maxActive) {
    static int cached = -1, active = 0;
    if (cached < 0) {
        const size_t smem = csm_smem_bytes();
        for (int t : {256, 512, 1024}) {
            cudaFuncSetAttribute(csm_kernel(t), cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            cudaFuncSetAttribute(csm_kernel(t), cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        }
        cudaGetLastError();
        cached = 0;
        for (int cs : {16, 8, 4, 2}) {
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3(cs);
            cfg.blockDim = dim3(1024);
            cfg.dynamicSmemBytes = smem;
            cudaLaunchAttribute attr[1];
            attr[0].id = cudaLaunchAttributeClusterDimension;
            attr[0].val.clusterDim.x = cs;
            attr[0].val.clusterDim.y = 1;
            attr[0].val.clusterDim.z = 1;
            cfg.attrs = attr;
            cfg.numAttrs = 1;
            int n = 0;
            if (cudaOccupancyMaxActiveClusters(&n, csm_kernel(1024), &cfg) == cudaSuccess && n > 0) {
                cached = cs;
                active = n;
                break;
            }
            cudaGetLastError();
        }
    }
    if (maxActive) *maxActive = active;
    return cached;
}

cudaError_t launch_solve_fp32_csm(const DevState &S, int clusterSize, int nClusters, cudaStream_t st) {
    SolveView<float> V{};
    V.aptr = S.aptr;
    V.aent = S.aent32;
    V.st[0] = S.st32[0];
    V.st[1] = S.st32[1];
    V.qc = S.qc32;
    V.lbGeneral = S.lb;
    V.alphaBuf = S.alphaBuf;
    V.fp64 = 0;
    const size_t smem = csm_smem_bytes();
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(clusterSize * nClusters);
    cfg.blockDim = dim3(g_csm_threads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = clusterSize;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, csm_kernel(g_csm_threads), S, V, csm_entry_capacity(smem));
}

}  // namespace alens
