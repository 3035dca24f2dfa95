// kernels_mlp.cu - learned warm start on the tensor cores.
//
// A 12 -> 64 -> 64 -> 1 SiLU network predicts each collision constraint's
// multiplier gamma from local pair geometry and the previous step's
// multiplier; the prediction only seeds BBPGD (SimToolbox BCQPSolver's
// iteration starts from the constraint's initial gamma, the `gamma` field
// of the ConstraintBlock built at SRC/TubuleSystem.cpp:727-736), so the
// solve still has to reach conResTol from it.
//
// Units: the network works in "overlap units" u = gamma * A_kk / d_k, where
// A_kk is the diagonal of the Delassus operator and d_k the sum of the two
// collision radii; for an isolated contact the converged multiplier is
// u = max(0, -q_k) / d_k exactly.
//
// Features of constraint k (all FP32, built from FP64 state):
//   0 phi0 / d          current separation
//   1 max(0, -q) / d    predicted overlap at the end of the step without
//                       constraint forces (q = phi0 + dt D^T U_known)
//   2 q / d             predicted signed separation
//   3 |a_I . a_J|       cosine of the rod axes
//   4, 5                rod lengths L_I, L_J (um)
//   6, 7                contact parameters s / h_I, t / h_J in [-1, 1]
//   8, 9                constraints on rod I and on rod J, divided by 8
//   10 gamma_prev A_kk / d   previous step's multiplier of the same pair
//                            and periodic image (0 for a new pair)
//   11 sum_{l != k, collision} A_kl max(0, -q_l) / (A_kk d)
//                       coupling-weighted predicted overlap of neighbours
//
// Kernels: one CTA of 128 threads owns one 128-row tile at a time (thread
// = row = TMEM lane).  Features and activations are written as BF16 into
// shared memory in the canonical K-major layout (tc.cuh), one elected
// thread issues tcgen05.mma into tensor memory, completion is signalled
// through an mbarrier, and every warp reads its 32 lanes back with
// tcgen05.ld for the bias + SiLU epilogue.  Training runs forward,
// backward and the weight gradients of a tile on the tensor cores too:
//   dH1 = dA2 W2             (A = dA2, B = W2^T)
//   [dW2 | . ; . | dW1] and the bias gradients in one M=128, N=96 product
//   of the stacked transposes [dA2^T; dA1^T] and [H1^T; X^T; 1],
//   accumulated in tensor memory over all tiles of the CTA.
#include "engine.cuh"
#include "mlp.h"
#include "tc.cuh"

namespace alens {

namespace {

constexpr unsigned long long kMmaTimeoutNs = 1000000000ULL;  // 1 s

// fast exponential and divide (a few instructions each): the activations
// are rounded to BF16 before the next layer, far coarser than their error
__device__ __forceinline__ float sigmoidf_(float a) { return __fdividef(1.0f, 1.0f + __expf(-a)); }
__device__ __forceinline__ float siluf_(float a) { return a * sigmoidf_(a); }
__device__ __forceinline__ float dsiluf_(float a) {
    const float s = sigmoidf_(a);
    return s * (1.0f + a * (1.0f - s));
}

// --------------------------------------------------------------- features
// FP64 six-term dot product without contraction (the operator assembly's
// arithmetic)
__device__ __forceinline__ double dot6_rn(const double *a, const double *b) {
    double s = __dmul_rn(a[0], b[0]);
#pragma unroll
    for (int c = 1; c < 6; c++) s = __dadd_rn(s, __dmul_rn(a[c], b[c]));
    return s;
}

// Features of constraint k; false when k is not a collision constraint or
// its operator diagonal is not positive (immovable rods).
__device__ bool mlp_features(const DevState &S, int k, float (&f)[kMlpInPad], float &scale) {
    // FP32 arithmetic on the FP64 state (the FP64 pipe of GB300 issues two
    // lanes per cycle per SM; the features only need FP32)
#pragma unroll
    for (int c = 0; c < kMlpInPad; c++) f[c] = 0.0f;
    scale = 0.0f;
    if (S.conImg[k] < 0 || S.conImg[k] >= kImageBoundary) return false;  // blocks, boundary contacts
    const int I = S.conI[k], J = S.conJ[k];
    const float q = (float)S.q[k];
    const float d = (float)S.rcol[I] + (float)S.rcol[J];
    // A_kk as the operator assembly forms it (FP64: dt times rod I's side
    // J_kI . W_kI plus rod J's side), and the coupling to the compressed
    // neighbours sum_l A_kl (-q_l) over collisions l != k with q_l < 0,
    // taken over the rod rows of I and J (A_kl = dt sum over the shared
    // rods of J_k,side . W_l,s), so no assembled operator is needed
    const double dt = S.par[S.rodRep[I]].dt;
    const double *Jk = S.jac + 12 * (size_t)k;
    const double *Wk = S.W + 12 * (size_t)k;
    double a = 0.0;
    a = __dadd_rn(a, dot6_rn(Jk, Wk));
    a = __dadd_rn(a, dot6_rn(Jk + 6, Wk + 6));
    const float akk = (float)__dmul_rn(dt, a);
    // sum_l A_kl (-q_l) over all compressed collisions l sharing a rod with
    // k (k included), from the per-rod sums, less k's own term (-q_k) A_kk
    const float dtf = (float)dt;
    float vI = 0.0f, vJ = 0.0f;
#pragma unroll
    for (int c = 0; c < 6; c++) {
        vI = fmaf((float)Jk[c], S.rodV[(size_t)c * S.nRods + I], vI);
        vJ = fmaf((float)Jk[6 + c], S.rodV[(size_t)c * S.nRods + J], vJ);
    }
    float nb = dtf * (vI + vJ);
    if (q < 0.0f) nb = fmaf(-q, -akk, nb);
    if (!(akk > 0.0f) || !(d > 0.0f)) return false;
    // the previous step's multiplier of this key: the constraint build
    // looked it up in the previous-gamma mode (gamma0 = max(0, prev)); with
    // the network running it is looked up here, on the warm-start branch
    float gprev = 0.0f;
    const int prevN = *S.prevCount;
    if (S.warm == ALENS_WARM_PREV || (S.warm == ALENS_WARM_MLP && !S.warmNet)) {
        gprev = (float)S.gamma[k];
    } else if (prevN > 0) {
        const int rep = S.rodRep[I];
        const unsigned long long key = S.keys[k - S.bilPrefix[rep]];
        int lo = 0, hi = prevN;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (S.prevKeys[mid] < key)
                lo = mid + 1;
            else
                hi = mid;
        }
        if (lo < prevN && S.prevKeys[lo] == key) gprev = (float)S.prevGamma[lo];
    }
    const float cosab = (float)S.ax[I] * (float)S.ax[J] + (float)S.ay[I] * (float)S.ay[J] +
                        (float)S.az[I] * (float)S.az[J];
    const float2 st = S.conST[k];
    const float invd = 1.0f / d;
    f[0] = (float)S.phi0[k] * invd;
    f[1] = (q < 0.0f ? -q : 0.0f) * invd;
    f[2] = q * invd;
    f[3] = fabsf(cosab);
    f[4] = (float)S.len[I];
    f[5] = (float)S.len[J];
    f[6] = st.x;
    f[7] = st.y;
    f[8] = (float)(S.rowPtr[I + 1] - S.rowPtr[I]) * 0.125f;
    f[9] = (float)(S.rowPtr[J + 1] - S.rowPtr[J]) * 0.125f;
    f[10] = gprev * akk * invd;
    f[11] = nb / akk * invd;
    scale = akk * invd;
    return true;
}

// ------------------------------------------------------- inference tile
struct InferSmem {
    alignas(1024) uint8_t x[kMlpTile * kMlpInPad * 2];   // 4 KB
    alignas(1024) uint8_t h1[kMlpTile * kMlpHid * 2];    // 16 KB
    alignas(1024) uint8_t w1[kW1Bytes];                  // 2 KB
    alignas(1024) uint8_t w2[kW2Bytes];                  // 8 KB
    float b1[kMlpHid], b2[kMlpHid], w3[kMlpHid];
    float b3;
    float ypart[kMlpTile];  // output-layer partial sums of the upper column half
    alignas(8) unsigned long long mbar;
    uint32_t tmem;
};

// Inference CTAs have 256 threads: thread t serves row t & 127 (its TMEM
// lane, 32 x32b lanes per warp quadrant) and column half t >> 7 of each
// hidden layer, so every epilogue is split over two threads per row.
constexpr int kInferThreads = 2 * kMlpTile;

__device__ void copy16(uint8_t *dst, const uint8_t *src, int bytes) {
    for (int o = (int)threadIdx.x * 16; o < bytes; o += (int)blockDim.x * 16)
        *reinterpret_cast<uint4 *>(dst + o) = __ldg(reinterpret_cast<const uint4 *>(src + o));
}

// Loads weights, allocates `ncols` TMEM columns and initialises the
// mbarrier.  Returns the TMEM base address (all threads).
template <class Sm>
__device__ uint32_t infer_setup(Sm &sh, const MlpView &V, uint32_t ncols) {
    copy16(sh.w1, V.w1c, kW1Bytes);
    copy16(sh.w2, V.w2c, kW2Bytes);
    for (int i = threadIdx.x; i < kMlpHid; i += blockDim.x) {
        sh.b1[i] = V.p[kOffB1 + i];
        sh.b2[i] = V.p[kOffB2 + i];
        sh.w3[i] = V.w3r[i];
    }
    if (threadIdx.x == 0) {
        sh.b3 = V.p[kOffB3];
        tc::mbar_init(tc::smem_addr(&sh.mbar), 1);
        tc::mbar_fence_init();
    }
    if ((threadIdx.x >> 5) == 0) {
        tc::tmem_alloc(tc::smem_addr(&sh.tmem), ncols);
        tc::tmem_relinquish();
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    return sh.tmem;
}

__device__ void tmem_release(uint32_t tbase, uint32_t ncols) {
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    if ((threadIdx.x >> 5) == 0) tc::tmem_dealloc(tbase, ncols);
}

// generic smem writes done -> MMA issue by thread 0
__device__ __forceinline__ void handoff_to_mma() {
    tc::fence_smem_async();
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
}

// Waits for the MMA batch just committed; false (in every thread) on timeout.
__device__ __forceinline__ bool wait_mma(uint32_t mbar, uint32_t &phase, int *err) {
    const bool ok = tc::mbar_wait(mbar, phase, kMmaTimeoutNs);
    phase ^= 1u;
    const int bad = __syncthreads_or(ok ? 0 : 1);
    if (bad) {
        if (threadIdx.x == 0 && err) atomicOr(err, kErrTimeout);
        return false;
    }
    tc::fence_after();
    return true;
}

// Forward pass of one tile whose features are already in sh.x; returns the
// network output of this thread's row in the threads of column half 0.
// False on timeout.
template <class Sm>
__device__ bool infer_tile(Sm &sh, uint32_t tbase, uint32_t &phase, int *err, float &y) {
    constexpr uint32_t idesc = tc::idesc_bf16(kMlpTile, kMlpHid);
    const uint32_t mbar = tc::smem_addr(&sh.mbar);
    const int tid = threadIdx.x;
    const int row = tid & (kMlpTile - 1), c0 = 32 * (tid >> 7);
    const uint32_t lane_base = tbase + ((uint32_t)(((tid >> 5) & 3) * 32) << 16);
    handoff_to_mma();
    if (tid == 0) {
        const uint64_t a = tc::smem_desc(tc::smem_addr(sh.x), 128, 256);
        const uint64_t b = tc::smem_desc(tc::smem_addr(sh.w1), 128, 256);
        tc::mma_bf16(tbase, a, b, idesc, 0);
        tc::commit(mbar);
    }
    if (!wait_mma(mbar, phase, err)) return false;
    {
        float v[32];
        tc::tmem_ld32(lane_base + c0, v);
#pragma unroll
        for (int g = 0; g < 32; g += 8) {
            float h[8];
#pragma unroll
            for (int e = 0; e < 8; e++) h[e] = siluf_(v[g + e] + sh.b1[c0 + g + e]);
            tc::st_bf16x8(sh.h1, tc::core_off(row, c0 + g, kMlpHid), h);
        }
    }
    handoff_to_mma();
    if (tid == 0) {
#pragma unroll
        for (int s = 0; s < kMlpHid / 16; s++) {
            const uint64_t a = tc::smem_desc(tc::smem_addr(sh.h1) + 256u * s, 128, 1024);
            const uint64_t b = tc::smem_desc(tc::smem_addr(sh.w2) + 256u * s, 128, 1024);
            tc::mma_bf16(tbase + kMlpHid, a, b, idesc, s > 0 ? 1u : 0u);
        }
        tc::commit(mbar);
    }
    if (!wait_mma(mbar, phase, err)) return false;
    float acc = 0.0f;
    {
        float v[32];
        tc::tmem_ld32(lane_base + kMlpHid + c0, v);
#pragma unroll
        for (int e = 0; e < 32; e++) acc = fmaf(siluf_(v[e] + sh.b2[c0 + e]), sh.w3[c0 + e], acc);
    }
    if (c0 != 0) sh.ypart[row] = acc;
    // the partial sums are in place and every lane's TMEM reads are
    // complete before the next tile's MMA
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    if (c0 == 0) y = (sh.b3 + acc) + sh.ypart[row];
    return true;
}

__device__ __forceinline__ void store_features(uint8_t *x, int row, const float (&f)[kMlpInPad]) {
    tc::st_bf16x8(x, tc::core_off(row, 0, kMlpInPad), f);
    tc::st_bf16x8(x, tc::core_off(row, 8, kMlpInPad), f + 8);
}

// Warm start of every collision constraint of the step (after the rod rows
// and the weights, beside the operator assembly, before the solve).
// Optionally records the features.
__global__ void __launch_bounds__(kInferThreads) k_mlp_warm(DevState S, MlpView V) {
    ALENS_PDL_PROLOGUE();
    __shared__ InferSmem sh;
    if (ld_volatile_i32(&S.ctl->errFlags) & (kErrNaN | kErrOverflow)) return;
    const int nc = S.ctl->totalCon;
    const int nTiles = (nc + kMlpTile - 1) / kMlpTile;
    if ((int)blockIdx.x >= nTiles) return;
    const uint32_t tbase = infer_setup(sh, V, 128);
    uint32_t phase = 0;
    const bool lead = threadIdx.x < kMlpTile;  // the row's features and output
    for (int t = blockIdx.x; t < nTiles; t += gridDim.x) {
        const int k = t * kMlpTile + (int)threadIdx.x;
        float scale = 0.0f;
        bool ok = false;
        if (lead) {
            float f[kMlpInPad];
            ok = k < nc && mlp_features(S, k, f, scale);
            if (S.feat && k < nc) {
#pragma unroll
                for (int c = 0; c < kMlpIn; c++) S.feat[(size_t)k * kMlpIn + c] = f[c];
                S.fscale[k] = scale;
            }
            store_features(sh.x, threadIdx.x, f);
        }
        float y = 0.0f;
        if (!infer_tile(sh, tbase, phase, &S.ctl->errFlags, y)) break;
        if (lead && ok) {
            const double g0 = y > 0.0f ? (double)(y / scale) : 0.0;
            S.gamma[k] = g0;
            S.st[1][k] = make_double2(g0, 0.0);
            if (S.precision == ALENS_PREC_MIXED) S.st32[1][k] = make_float2((float)g0, 0.0f);
        }
    }
    tmem_release(tbase, 128);
}

// Features only (recording without the learned warm start).
__global__ void k_mlp_features(DevState S) {
    ALENS_PDL_PROLOGUE();
    if (ld_volatile_i32(&S.ctl->errFlags) & (kErrNaN | kErrOverflow)) return;
    const int nc = S.ctl->totalCon;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nc; k += gridDim.x * blockDim.x) {
        float f[kMlpInPad];
        float scale = 0.0f;
        mlp_features(S, k, f, scale);
#pragma unroll
        for (int c = 0; c < kMlpIn; c++) S.feat[(size_t)k * kMlpIn + c] = f[c];
        S.fscale[k] = scale;
    }
}

// Dataset rows: features and label u = gamma * scale of constraints k0..k0+n.
__global__ void k_mlp_append(DevState S, int k0, int n, float *dsFeat, float *dsLabel) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int k = k0 + i;
#pragma unroll
        for (int c = 0; c < kMlpIn; c++) dsFeat[(size_t)i * kMlpIn + c] = S.feat[(size_t)k * kMlpIn + c];
        dsLabel[i] = (float)(S.gamma[k] * (double)S.fscale[k]);
    }
}

// Network output for rows of a feature matrix (n x 12, FP32).
__global__ void __launch_bounds__(kInferThreads) k_mlp_predict(MlpView V, const float *feat, int n, float *out) {
    __shared__ InferSmem sh;
    const int nTiles = (n + kMlpTile - 1) / kMlpTile;
    if ((int)blockIdx.x >= nTiles) return;
    const uint32_t tbase = infer_setup(sh, V, 128);
    uint32_t phase = 0;
    const bool lead = threadIdx.x < kMlpTile;
    for (int t = blockIdx.x; t < nTiles; t += gridDim.x) {
        const int r = t * kMlpTile + (int)threadIdx.x;
        if (lead) {
            float f[kMlpInPad];
#pragma unroll
            for (int c = 0; c < kMlpInPad; c++) f[c] = (r < n && c < kMlpIn) ? feat[(size_t)r * kMlpIn + c] : 0.0f;
            store_features(sh.x, threadIdx.x, f);
        }
        float y = 0.0f;
        if (!infer_tile(sh, tbase, phase, V.err, y)) break;
        if (lead && r < n) out[r] = y;
    }
    tmem_release(tbase, 128);
}

// ------------------------------------------------------------- training
// Tensor memory columns of the training CTA (512 allocated)
constexpr uint32_t kColZ1 = 0, kColZ2 = 64, kColDH1 = 128, kColAcc = 256;
constexpr int kAccN = 96;        // [H1^T (64); X^T (16); ones (1); zero (15)]
constexpr int kBatchK = kMlpTile;  // batch rows per tile = K of the weight-gradient product

struct TrainSmem {
    alignas(1024) uint8_t x[kMlpTile * kMlpInPad * 2];      // X   [b][k]      4 KB
    alignas(1024) uint8_t h1[kMlpTile * kMlpHid * 2];       // H1  [b][i]     16 KB
    alignas(1024) uint8_t da2[kMlpTile * kMlpHid * 2];      // dA2 [b][j]     16 KB
    alignas(1024) uint8_t sa[kMlpTile * kBatchK * 2];       // [dA2^T; dA1^T] [m][b] 32 KB
    alignas(1024) uint8_t sb[kAccN * kBatchK * 2];          // [H1^T; X^T; 1] [n][b] 24 KB
    alignas(1024) uint8_t w1[kW1Bytes];                     // 2 KB
    alignas(1024) uint8_t w2[kW2Bytes];                     // 8 KB
    alignas(1024) uint8_t w2t[kW2Bytes];                    // 8 KB
    float b1[kMlpHid], b2[kMlpHid], w3[kMlpHid];
    float gw3[kMlpHid];
    float b3, gb3;
    float lossPart[kMlpTile / 32];
    alignas(8) unsigned long long mbar;
    uint32_t tmem;
};
constexpr int kTrainSmemBytes = 120 * 1024;  // > half an SM: one CTA (512 TMEM columns) per SM
static_assert(sizeof(TrainSmem) + 1024 <= kTrainSmemBytes, "training shared memory");

__device__ __forceinline__ float warp_sum_f(float v) {
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// One batch (rows start..start+count of the permutation i -> (a i + b) mod
// nData) of the mean squared error 1/count sum (y - label)^2: gradients are
// accumulated into `grad` (zeroed by the caller), the loss sum into lossAcc.
__global__ void __launch_bounds__(kMlpTile) k_mlp_train(MlpView V, const float *feat, const float *label,
                                                        long long nData, long long permA, long long permB,
                                                        long long start, int count, float *grad,
                                                        double *lossAcc) {
    extern __shared__ uint8_t dyn_smem[];
    TrainSmem &sh = *reinterpret_cast<TrainSmem *>((reinterpret_cast<uintptr_t>(dyn_smem) + 1023) &
                                                   ~(uintptr_t)1023);
    const int nTiles = (count + kMlpTile - 1) / kMlpTile;
    if ((int)blockIdx.x >= nTiles) return;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    copy16(sh.w1, V.w1c, kW1Bytes);
    copy16(sh.w2, V.w2c, kW2Bytes);
    copy16(sh.w2t, V.w2tc, kW2Bytes);
    for (int i = tid; i < kMlpHid; i += blockDim.x) {
        sh.b1[i] = V.p[kOffB1 + i];
        sh.b2[i] = V.p[kOffB2 + i];
        sh.w3[i] = V.w3r[i];
        sh.gw3[i] = 0.0f;
    }
    // rows 81..95 of the stacked B stay zero; row 80 is all ones
    for (int o = tid * 16; o < (int)sizeof(sh.sb); o += blockDim.x * 16)
        *reinterpret_cast<uint4 *>(sh.sb + o) = make_uint4(0, 0, 0, 0);
    __syncthreads();
    for (int b = tid; b < kBatchK; b += blockDim.x) tc::st_bf16(sh.sb, tc::core_off(80, b, kBatchK), 1.0f);
    if (tid == 0) {
        sh.b3 = V.p[kOffB3];
        sh.gb3 = 0.0f;
        tc::mbar_init(tc::smem_addr(&sh.mbar), 1);
        tc::mbar_fence_init();
    }
    if (warp == 0) {
        tc::tmem_alloc(tc::smem_addr(&sh.tmem), 512);
        tc::tmem_relinquish();
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tbase = sh.tmem;
    const uint32_t lane_base = tbase + ((uint32_t)(warp * 32) << 16);
    const uint32_t mbar = tc::smem_addr(&sh.mbar);
    constexpr uint32_t idH = tc::idesc_bf16(kMlpTile, kMlpHid);
    constexpr uint32_t idAcc = tc::idesc_bf16(kMlpTile, kAccN);
    uint32_t phase = 0;
    float lossSum = 0.0f;
    bool failed = false;
    int tilesDone = 0;
    const float invCount = 1.0f / (float)count;
    for (int t = blockIdx.x; t < nTiles && !failed; t += gridDim.x) {
        const int r = t * kMlpTile + tid;
        const bool valid = r < count;
        float f[kMlpInPad];
        float tgt = 0.0f;
        if (valid) {
            const long long idx = (permA * (start + r) + permB) % nData;
#pragma unroll
            for (int c = 0; c < kMlpIn; c++) f[c] = feat[idx * kMlpIn + c];
            tgt = label[idx];
        } else {
#pragma unroll
            for (int c = 0; c < kMlpIn; c++) f[c] = 0.0f;
        }
#pragma unroll
        for (int c = kMlpIn; c < kMlpInPad; c++) f[c] = 0.0f;
        store_features(sh.x, tid, f);
#pragma unroll
        for (int c = 0; c < kMlpInPad; c++) tc::st_bf16(sh.sb, tc::core_off(64 + c, tid, kBatchK), f[c]);
        // ---- Z1 = X W1^T
        handoff_to_mma();
        if (tid == 0) {
            tc::mma_bf16(tbase + kColZ1, tc::smem_desc(tc::smem_addr(sh.x), 128, 256),
                         tc::smem_desc(tc::smem_addr(sh.w1), 128, 256), idH, 0);
            tc::commit(mbar);
        }
        if (!wait_mma(mbar, phase, V.err)) {
            failed = true;
            break;
        }
#pragma unroll
        for (int c = 0; c < kMlpHid; c += 32) {
            float v[32];
            tc::tmem_ld32(lane_base + kColZ1 + c, v);
#pragma unroll
            for (int g = 0; g < 32; g += 8) {
                float h[8];
#pragma unroll
                for (int e = 0; e < 8; e++) {
                    h[e] = siluf_(v[g + e] + sh.b1[c + g + e]);
                    tc::st_bf16(sh.sb, tc::core_off(c + g + e, tid, kBatchK), h[e]);
                }
                tc::st_bf16x8(sh.h1, tc::core_off(tid, c + g, kMlpHid), h);
            }
        }
        // ---- Z2 = H1 W2^T
        handoff_to_mma();
        if (tid == 0) {
#pragma unroll
            for (int s = 0; s < kMlpHid / 16; s++)
                tc::mma_bf16(tbase + kColZ2, tc::smem_desc(tc::smem_addr(sh.h1) + 256u * s, 128, 1024),
                             tc::smem_desc(tc::smem_addr(sh.w2) + 256u * s, 128, 1024), idH, s > 0 ? 1u : 0u);
            tc::commit(mbar);
        }
        if (!wait_mma(mbar, phase, V.err)) {
            failed = true;
            break;
        }
        float z2[kMlpHid];
        {
            float v[32];
            tc::tmem_ld32(lane_base + kColZ2, v);
#pragma unroll
            for (int e = 0; e < 32; e++) z2[e] = v[e] + sh.b2[e];
            tc::tmem_ld32(lane_base + kColZ2 + 32, v);
#pragma unroll
            for (int e = 0; e < 32; e++) z2[32 + e] = v[e] + sh.b2[32 + e];
        }
        float y = sh.b3;
#pragma unroll
        for (int e = 0; e < kMlpHid; e++) y = fmaf(siluf_(z2[e]), sh.w3[e], y);
        const float diff = valid ? y - tgt : 0.0f;
        lossSum += diff * diff;
        const float dy = 2.0f * diff * invCount;
        // w3 / b3 gradients: sum over the tile's rows (warp trees, then smem)
#pragma unroll
        for (int e = 0; e < kMlpHid; e++) {
            const float gsum = warp_sum_f(dy * siluf_(z2[e]));
            if (lane == 0) atomicAdd(&sh.gw3[e], gsum);
        }
        {
            const float gsum = warp_sum_f(dy);
            if (lane == 0) atomicAdd(&sh.gb3, gsum);
        }
        // dA2 = dy w3 * SiLU'(A2): row-major for dH1, transposed for dW2
#pragma unroll
        for (int g = 0; g < kMlpHid; g += 8) {
            float a[8];
#pragma unroll
            for (int e = 0; e < 8; e++) {
                a[e] = dy * sh.w3[g + e] * dsiluf_(z2[g + e]);
                tc::st_bf16(sh.sa, tc::core_off(g + e, tid, kBatchK), a[e]);
            }
            tc::st_bf16x8(sh.da2, tc::core_off(tid, g, kMlpHid), a);
        }
        // ---- dH1 = dA2 W2  (B operand = W2^T, K-major)
        handoff_to_mma();
        if (tid == 0) {
#pragma unroll
            for (int s = 0; s < kMlpHid / 16; s++)
                tc::mma_bf16(tbase + kColDH1, tc::smem_desc(tc::smem_addr(sh.da2) + 256u * s, 128, 1024),
                             tc::smem_desc(tc::smem_addr(sh.w2t) + 256u * s, 128, 1024), idH, s > 0 ? 1u : 0u);
            tc::commit(mbar);
        }
        if (!wait_mma(mbar, phase, V.err)) {
            failed = true;
            break;
        }
#pragma unroll
        for (int c = 0; c < kMlpHid; c += 32) {
            float dh[32], z1[32];
            tc::tmem_ld32(lane_base + kColDH1 + c, dh);
            tc::tmem_ld32(lane_base + kColZ1 + c, z1);
#pragma unroll
            for (int e = 0; e < 32; e++)
                tc::st_bf16(sh.sa, tc::core_off(64 + c + e, tid, kBatchK), dh[e] * dsiluf_(z1[e] + sh.b1[c + e]));
        }
        // ---- weight and bias gradients, accumulated over this CTA's tiles
        handoff_to_mma();
        if (tid == 0) {
#pragma unroll
            for (int s = 0; s < kBatchK / 16; s++)
                tc::mma_bf16(tbase + kColAcc, tc::smem_desc(tc::smem_addr(sh.sa) + 256u * s, 128, 2048),
                             tc::smem_desc(tc::smem_addr(sh.sb) + 256u * s, 128, 2048), idAcc,
                             (tilesDone > 0 || s > 0) ? 1u : 0u);
            tc::commit(mbar);
        }
        if (!wait_mma(mbar, phase, V.err)) {
            failed = true;
            break;
        }
        tilesDone++;
    }
    if (!failed && tilesDone > 0) {
        // row m of the accumulator: m < 64 -> dW2[m][:], db2[m];
        // m >= 64 -> dW1[m-64][:12], db1[m-64]
        const int m = tid;
        float v[32];
        if (m < kMlpHid) {
#pragma unroll
            for (int c = 0; c < kMlpHid; c += 32) {
                tc::tmem_ld32(lane_base + kColAcc + c, v);
#pragma unroll
                for (int e = 0; e < 32; e++) atomicAdd(grad + kOffW2 + m * kMlpHid + c + e, v[e]);
            }
            tc::tmem_ld32(lane_base + kColAcc + 64, v);
            atomicAdd(grad + kOffB2 + m, v[16]);
        } else {
            tc::tmem_ld32(lane_base + kColAcc + 64, v);
#pragma unroll
            for (int e = 0; e < kMlpIn; e++) atomicAdd(grad + kOffW1 + (m - kMlpHid) * kMlpIn + e, v[e]);
            atomicAdd(grad + kOffB1 + (m - kMlpHid), v[16]);
        }
        // (m is uniform per warp, so each warp takes one branch as a whole,
        // as the .sync.aligned loads require)
    }
    __syncthreads();
    if (!failed) {
        for (int i = tid; i < kMlpHid; i += blockDim.x) atomicAdd(grad + kOffW3 + i, sh.gw3[i]);
        if (tid == 0) atomicAdd(grad + kOffB3, sh.gb3);
        const float ls = warp_sum_f(lossSum);
        if (lane == 0) sh.lossPart[warp] = ls;
        __syncthreads();
        if (tid == 0) {
            double s = 0.0;
            for (int w = 0; w < kMlpTile / 32; w++) s += (double)sh.lossPart[w];
            atomicAdd(lossAcc, s);
        }
    }
    tmem_release(tbase, 512);
}

// Adam step of every parameter, then its BF16 packed copies.
__global__ void k_mlp_adam(float *p, const float *grad, float *m, float *v, uint8_t *w1c, uint8_t *w2c,
                           uint8_t *w2tc, float *w3r, float lr, float bc1, float bc2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kMlpParams) return;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const float g = grad[i];
    const float mi = b1 * m[i] + (1.0f - b1) * g;
    const float vi = b2 * v[i] + (1.0f - b2) * g * g;
    m[i] = mi;
    v[i] = vi;
    const float mh = mi / bc1, vh = vi / bc2;
    const float pi = p[i] - lr * mh / (sqrtf(vh) + eps);
    p[i] = pi;
    if (i < kOffB1) {
        const int o = i / kMlpIn, c = i % kMlpIn;
        tc::st_bf16(w1c, tc::core_off(o, c, kMlpInPad), pi);
    } else if (i >= kOffW2 && i < kOffB2) {
        const int o = (i - kOffW2) / kMlpHid, c = (i - kOffW2) % kMlpHid;
        tc::st_bf16(w2c, tc::core_off(o, c, kMlpHid), pi);
        tc::st_bf16(w2tc, tc::core_off(c, o, kMlpHid), pi);
    } else if (i >= kOffW3 && i < kOffB3) {
        w3r[i - kOffW3] = __bfloat162float(__float2bfloat16_rn(pi));
    }
}

// BF16 packed copies of the master weights (W1 padding is zeroed by the
// owner once).
__global__ void k_mlp_pack(const float *p, uint8_t *w1c, uint8_t *w2c, uint8_t *w2tc, float *w3r) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kMlpParams) return;
    const float pi = p[i];
    if (i < kOffB1) {
        const int o = i / kMlpIn, c = i % kMlpIn;
        tc::st_bf16(w1c, tc::core_off(o, c, kMlpInPad), pi);
    } else if (i >= kOffW2 && i < kOffB2) {
        const int o = (i - kOffW2) / kMlpHid, c = (i - kOffW2) % kMlpHid;
        tc::st_bf16(w2c, tc::core_off(o, c, kMlpHid), pi);
        tc::st_bf16(w2tc, tc::core_off(c, o, kMlpHid), pi);
    } else if (i >= kOffW3 && i < kOffB3) {
        w3r[i - kOffW3] = __bfloat162float(__float2bfloat16_rn(pi));
    }
}

int sm_count() {
    static int n = 0;
    if (n == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
    }
    return n;
}

}  // namespace

void launch_mlp_warm(const DevState &S, const MlpView &V, cudaStream_t st) {
    // tiles cover every constraint slot the step can hold; blocks without
    // a tile return at once
    const int tiles = (S.cap + kMlpTile - 1) / kMlpTile;
    const int grid = tiles < 2 * sm_count() ? tiles : 2 * sm_count();
    launch_pdl(k_mlp_warm, dim3(grid > 0 ? grid : 1), dim3(kInferThreads), 0, st, S, V);
}

void launch_mlp_features(const DevState &S, cudaStream_t st) {
    launch_pdl(k_mlp_features, dim3(2 * sm_count()), dim3(256), 0, st, S);
}

void launch_mlp_append(const DevState &S, int k0, int n, float *dsFeat, float *dsLabel, cudaStream_t st) {
    if (n <= 0) return;
    const int grid = (n + 255) / 256 < 4 * sm_count() ? (n + 255) / 256 : 4 * sm_count();
    k_mlp_append<<<grid, 256, 0, st>>>(S, k0, n, dsFeat, dsLabel);
}

void launch_mlp_predict(const MlpView &V, const float *feat, int n, float *out, cudaStream_t st) {
    if (n <= 0) return;
    const int tiles = (n + kMlpTile - 1) / kMlpTile;
    const int grid = tiles < 2 * sm_count() ? tiles : 2 * sm_count();
    k_mlp_predict<<<grid, kInferThreads, 0, st>>>(V, feat, n, out);
}

cudaError_t launch_mlp_train(const MlpView &V, const float *feat, const float *label, long long nData,
                             long long permA, long long permB, long long start, int count, float *grad,
                             double *lossAcc, cudaStream_t st) {
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             kTrainSmemBytes);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    const int tiles = (count + kMlpTile - 1) / kMlpTile;
    const int grid = tiles < sm_count() ? tiles : sm_count();
    if (grid <= 0) return cudaSuccess;
    k_mlp_train<<<grid, kMlpTile, kTrainSmemBytes, st>>>(V, feat, label, nData, permA, permB, start, count, grad,
                                                         lossAcc);
    return cudaGetLastError();
}

void launch_mlp_adam(float *p, const float *grad, float *m, float *v, uint8_t *w1c, uint8_t *w2c,
                     uint8_t *w2tc, float *w3r, float lr, float bc1, float bc2, cudaStream_t st) {
    k_mlp_adam<<<(kMlpParams + 255) / 256, 256, 0, st>>>(p, grad, m, v, w1c, w2c, w2tc, w3r, lr, bc1, bc2);
}

void launch_mlp_pack(const float *p, uint8_t *w1c, uint8_t *w2c, uint8_t *w2tc, float *w3r, cudaStream_t st) {
    k_mlp_pack<<<(kMlpParams + 255) / 256, 256, 0, st>>>(p, w1c, w2c, w2tc, w3r);
}

}  // namespace alens
