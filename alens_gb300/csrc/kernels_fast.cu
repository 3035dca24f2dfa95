// kernels_fast.cu - single-system BBPGD with FP32 bulk arithmetic, FP64
// residual check and FP64 refinement in one cooperative launch (the role of
// SimToolbox BCQPSolver's BBPGD, conSolverChoice 0,
// docs/source/quickstart.md:356-358; method: Yan, Zhang, Shelley, J. Chem.
// Phys. 150:064109 (2019), alternating Barzilai-Borwein steps, IMA J.
// Numer. Anal. 8:141 (1988)).
//
// The grid form of solve_impl.cuh serves any number of replicas in the
// oracle's canonical constraint order and canonical reduction tree.  A
// context holding one system is solved here in a form built around what a
// BBPGD pass costs on GB300 (measured on the 20,000-rod layer): the grid
// barrier (~1.3 us), scattered L2 gathers of neighbour iterates, and any
// FP64 instruction on the critical path (the FP64 pipe issues 2 lanes per
// cycle per SM, so a warp-wide FP64 instruction holds its SM sub-partition
// for ~64 cycles).
//
//   Ordering (per step, kernels k_order_count / k_order_place on a side
//     stream beside the operator assembly): constraints are permuted so
//     that each block owns a compact patch of space.  Cells are walked in
//     Morton order, the rods of a cell by index, and each rod's constraints
//     with the rod as I (collisions, then crosslinker and user blocks) in
//     ascending canonical order, read from the rod rows.  Deterministic.
//   Rows: block b owns permuted rows [r0, r1) and caches their operator rows
//     in shared memory (8 bytes per entry: column slot, FP32 value).  Each
//     entry's column is either one of the block's own rows (its iterate is
//     the block's own shared-memory copy) or a halo column, copied from
//     global memory at the start of each pass (~10 % of the entries on the
//     20,000-rod layer).  After the pass's decision every column's value
//     (iterate, gradient or projected step, by the pass's mode) is formed
//     once into a shared-memory slot.  When every row of the block has a
//     thread of its own, a row of up to kRegEnts entries is held in its
//     thread's registers for the whole solve, so a row entry costs one
//     4-byte shared-memory gather and one FMA per pass.
//   FP32 passes: the step size alternates BB1/BB2 as in the other forms.
//     Each block writes ONE record per pass: s.s, s.y, y.y (FP32 products
//     summed in FP32 over the block's rows) and the residual max, one
//     float4, the records of all blocks contiguous.  After the grid
//     barrier, warp 0 of every block reads all records (one coalesced load
//     per 32 blocks) and accumulates
//     them in block order in double-float arithmetic (each sum a pair of
//     FP32 numbers combined with the error-free TwoSum: 48 significand bits,
//     FP64-class accuracy on the FP32 pipe), then decides (converged, next
//     step size) at once.  Every block takes the same decision with no
//     further exchange; the sums depend on the launch shape, not on timing,
//     so results are reproducible on a given GPU.
//   FP64 check and refinement: when the FP32 iterate meets conResTol (or
//     the iteration cap), the next pass promotes it to FP64 (projected) and
//     computes its FP64 gradient and residual with the FP64 operator; if that
//     residual meets conResTol the solve ends, otherwise FP64 BBPGD passes
//     (canonical order, global memory, FP64 block sums and FP64 accumulation
//     of the records) continue from the promoted point in the same launch.
//     The solution is left in canonical order in the FP64 iterate buffer
//     that the rod update reads.
//
// Streaming blocks: a block whose rows hold more entries than its shared
// memory (the 50,000-rod bundle with 200,000 crosslinks: ~43,000 per block)
// sorts its rows by length (descending, ties by index) into slices of 32 and
// writes their entries column-major (entry j of the slice's 32 rows
// contiguous, short rows padded with zero entries) into its own region of a
// global buffer, once per solve.  Each pass a warp streams a slice's
// entries with coalesced loads; own columns come from shared memory, the
// others straight from the previous pass's global iterates (L1/L2).
//
// A block whose rows fit neither form (more than kFastRows rows, or a region
// too small) reports it in its first record; every block then stops after
// the first pass and the context falls back to the grid form (kErrSolverFit).
//
// Iterations are reported as in the other mixed-precision forms: FP32
// iterations in refineIter, FP64 refinement iterations in iter.
// Every wait is the bounded grid barrier of common.cuh (kErrTimeout).
// Compiled with FMA contraction.
#include "solve_impl.cuh"

namespace alens {

namespace {

constexpr int kFastThreads = 256;
constexpr int kFastWarps = kFastThreads / 32;
constexpr int kFastRows = 2048;          // own rows per block
constexpr int kFastEnts = 8000;          // operator entries per block held in shared memory
constexpr int kSlice = 32;               // rows per slice of the streaming layout
constexpr int kMaxSlices = kFastRows / kSlice;
constexpr int kFastHalo = 3000;          // halo columns per block
constexpr int kFastCellRods = 256;       // rods per cell staged in shared memory by the ordering
constexpr int kRowBatch = 8;             // row entries loaded together
constexpr int kRegEnts = 16;             // a thread's row entries held in registers for the whole solve
constexpr int kGatherWarp0 = 4;          // warps kGatherWarp0.. copy the halo

// streaming entry: x = source index | kind << 28 | own << 30, y = FP32 value bits
constexpr int kEntSrcMask = (1 << 28) - 1;
constexpr int kEntOwn = 1 << 30;

// One block's record of a pass.  FP32 passes: one float4 (s.s, s.y, y.y,
// residual max), the records of all blocks contiguous so that warp 0 of
// every block reads 32 of them per coalesced load; a block whose rows fit
// no layout writes kMisfitBits as its residual max (above every float's bit
// pattern, +inf included, under the integer max that combines them).
// FP64 passes: FP64 sums and max (32 bytes).
struct FastRecord {
    double d[4];
};
static_assert(sizeof(FastRecord) == 32, "record size");
constexpr int kMisfitBits = 0x7fffffff;
// the records region: FP64 records [2][kFastMaxGrid], then FP32 records
// [2][kFastMaxGrid] (fits the 2 x 8 x kFastMaxGrid doubles of DevState)
static_assert(2 * kFastMaxGrid * (sizeof(FastRecord) + sizeof(float4)) <= 2 * 8 * kFastMaxGrid * sizeof(double),
              "records region");

// dynamic shared memory layout (bytes)
constexpr int kOffOwnSt = 0;                                   // float2 [2][kFastRows]
constexpr int kOffOwnQc = kOffOwnSt + 2 * kFastRows * 8;        // float2 [kFastRows] (q, cinv)
constexpr int kOffOwnLb = kOffOwnQc + kFastRows * 8;            // float [kFastRows] lower bound
constexpr int kOffRowBeg = kOffOwnLb + kFastRows * 4;           // int [kFastRows + 4]
constexpr int kOffOwnK = kOffRowBeg + (kFastRows + 4) * 4;      // int [kFastRows] canonical row
constexpr int kOffOwnA = kOffOwnK + kFastRows * 4;              // int [kFastRows] first entry (aptr)
constexpr int kOffEnt = kOffOwnA + kFastRows * 4;               // int2 [kFastEnts] (column slot, value)
constexpr int kOffHaloPos = kOffEnt + kFastEnts * 8;            // int [kFastHalo] permuted column
constexpr int kOffHaloCol = kOffHaloPos + kFastHalo * 4;        // int [kFastHalo] canonical column
constexpr int kOffHaloLb = kOffHaloCol + kFastHalo * 4;         // float [kFastHalo] lower bound
constexpr int kOffGv = kOffHaloLb + kFastHalo * 4;              // float2 [kFastHalo] gathered iterates
constexpr int kOffXcol = kOffGv + kFastHalo * 8;                // float [kFastRows + kFastHalo] column values
constexpr int kFastSmem = kOffXcol + (kFastRows + kFastHalo) * 4;
static_assert(kOffEnt % 16 == 0 && kOffGv % 8 == 0, "shared-memory alignment");
static_assert(kFastSmem + 1024 <= 227 * 1024, "shared memory per block");
// the streaming layout's sort keys, slot order and slice table alias the
// shared-memory entry region (unused by a streaming block)
static_assert((2 * kFastRows + 2 * (kMaxSlices + 1)) * 4 <= kFastEnts * 8, "streaming scratch");

enum FastPhase { kPh32 = 0, kPhCheck = 1, kPh64 = 2 };
constexpr int kStatusMisfit = -1;

struct FastShared {
    double red[4];      // FP64 passes: s.s, s.y, y.y, residual max of the previous pass
    float red32[4];     // FP32 passes: the same
    float wsum[kFastWarps][4];
    double wsum64[kFastWarps][4];
    double alpha;       // FP64 phase step size
    float alpha32;      // FP32 phase step size
    float tol32;        // largest float not above conResTol
    double res;
    int mode;      // kModeG0 / kModeAG / kModeIter of the current pass
    int phase;     // FastPhase of the current pass
    int q;         // pass index within the phase: 0 = G0, 1 = AG, >= 2 iterations
    int stop;
    int status;
    int it32, it64;
    int haloCount;
    int misfit;
};

__device__ __forceinline__ int warp_sum_i(int v) { return __reduce_add_sync(0xffffffffu, v); }

// Inclusive warp scan of an int (Kogge-Stone).
__device__ __forceinline__ int warp_incl_scan_i(int v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const int o = __shfl_up_sync(0xffffffffu, v, off);
        if (lane >= off) v += o;
    }
    return v;
}

// Double-float addition (hi, lo) += (bh, bl): Knuth's TwoSum of the high
// parts, the low parts added to the error, renormalised with Dekker's
// FastTwoSum.  Only additions, so FMA contraction cannot change it.
__device__ __forceinline__ void df_add(float &hi, float &lo, float bh, float bl) {
    const float s = hi + bh;
    const float v = s - hi;
    float e = (hi - (s - v)) + (bh - v);
    e = e + (lo + bl);
    hi = s + e;
    lo = e - (hi - s);
}

// Grid barrier number bi (bounded wait).  Block 0 clears the counter of
// barrier bi + 1 before arriving (its last use, bi - 2, has been left by
// every block: each has arrived at bi - 1).
__device__ __forceinline__ bool fast_barrier(const DevState &S, int bi, int G, unsigned long long timeout_ns) {
    if (blockIdx.x == 0 && threadIdx.x == 0) st_relaxed_u32(&S.ctl->bar.pass[(bi + 1) % 3][0], 0u);
    int stopUnused = 0;
    return grid_sync_pass(&S.ctl->bar, (unsigned int)(G + S.barrierExtra), &S.ctl->errFlags, timeout_ns, bi, 1,
                          stopUnused);
}

// Block record: warp sums in Real, then warp 0 adds the eight warp values
// in Real (fixed xor tree; lane = 4 * warp + quantity); FP32 passes: lane 0
// stores the four values as one float4 (the misfit flag in the residual
// max), FP64 passes: lanes 0-3 store one value each.
template <class Real>
__device__ __forceinline__ void block_record(Real v0, Real v1, Real v2, Real vm, int misfit, FastShared &sh,
                                             FastRecord *rec, float4 *rec32) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    v0 = warp_tree_sum_t<Real>(v0);
    v1 = warp_tree_sum_t<Real>(v1);
    v2 = warp_tree_sum_t<Real>(v2);
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) {
        const Real o = __shfl_xor_sync(0xffffffffu, vm, off);
        vm = o > vm ? o : vm;
    }
    if (lane == 0) {
        if constexpr (sizeof(Real) == 4) {
            sh.wsum[warp][0] = v0;
            sh.wsum[warp][1] = v1;
            sh.wsum[warp][2] = v2;
            sh.wsum[warp][3] = vm;
        } else {
            sh.wsum64[warp][0] = v0;
            sh.wsum64[warp][1] = v1;
            sh.wsum64[warp][2] = v2;
            sh.wsum64[warp][3] = vm;
        }
    }
    __syncthreads();
    if (warp == 0) {
        const int w = lane >> 2, q = lane & 3;
        Real v;
        if constexpr (sizeof(Real) == 4)
            v = sh.wsum[w][q];
        else
            v = sh.wsum64[w][q];
#pragma unroll
        for (int off = 16; off >= 4; off >>= 1) {
            const Real o = __shfl_xor_sync(0xffffffffu, v, off);
            v = q == 3 ? (o > v ? o : v) : v + o;
        }
        if constexpr (sizeof(Real) == 4) {
            const float r1 = __shfl_sync(0xffffffffu, v, 1), r2 = __shfl_sync(0xffffffffu, v, 2);
            const float r3 = __shfl_sync(0xffffffffu, v, 3);
            if (lane == 0) __stcg(rec32, make_float4(v, r1, r2, misfit ? __int_as_float(kMisfitBits) : r3));
        } else {
            if (lane < 4) __stcg(&rec->d[lane], v);
        }
    }
}

// FP32 records of all G blocks, summed by warp 0 in double-float in block
// order (lane l adds blocks l, l+32, ..., then a fixed xor tree), residual
// max through the bit patterns of non-negative floats.  Results in lane 0.
__device__ __forceinline__ void grid_records32(const float4 *rec, int G, FastShared &sh) {
    const int lane = threadIdx.x & 31;
    constexpr int kMaxPer = (kFastMaxGrid + 31) / 32;
    float4 v[kMaxPer];
#pragma unroll
    for (int j = 0; j < kMaxPer; j++) {
        const int bb = lane + 32 * j;
        v[j] = bb < G ? __ldcg(rec + bb) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
    float h0 = 0.0f, l0 = 0.0f, h1 = 0.0f, l1 = 0.0f, h2 = 0.0f, l2 = 0.0f;
    int m = 0;
#pragma unroll
    for (int j = 0; j < kMaxPer; j++) {
        if (32 * j < G) {  // uniform; blocks beyond G add exact zeros
            df_add(h0, l0, v[j].x, 0.0f);
            df_add(h1, l1, v[j].y, 0.0f);
            df_add(h2, l2, v[j].z, 0.0f);
            m = max(m, __float_as_int(v[j].w));
        }
    }
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) {
        const float a0 = __shfl_xor_sync(0xffffffffu, h0, off), b0 = __shfl_xor_sync(0xffffffffu, l0, off);
        const float a1 = __shfl_xor_sync(0xffffffffu, h1, off), b1 = __shfl_xor_sync(0xffffffffu, l1, off);
        const float a2 = __shfl_xor_sync(0xffffffffu, h2, off), b2 = __shfl_xor_sync(0xffffffffu, l2, off);
        df_add(h0, l0, a0, b0);
        df_add(h1, l1, a1, b1);
        df_add(h2, l2, a2, b2);
        m = max(m, __shfl_xor_sync(0xffffffffu, m, off));
    }
    if (lane == 0) {
        // the double-float sums rounded to FP32 (the FP32 phase decides and
        // steps in FP32)
        sh.red32[0] = h0;
        sh.red32[1] = h1;
        sh.red32[2] = h2;
        sh.red32[3] = __int_as_float(m);
        sh.misfit = m == kMisfitBits ? 1 : 0;
    }
}

// FP64 records of all G blocks: warp q (0-2) accumulates quantity q in FP64
// in block order, warp 3 the max (the warps run on
// different SM sub-partitions).  Results after the next __syncthreads.
__device__ __forceinline__ void grid_records64(const FastRecord *rec, int G, FastShared &sh) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    constexpr int kMaxPer = (kFastMaxGrid + 31) / 32;
    if (warp < 3) {
        double v[kMaxPer];
#pragma unroll
        for (int j = 0; j < kMaxPer; j++) {
            const int bb = lane + 32 * j;
            v[j] = bb < G ? __ldcg(&rec[bb].d[warp]) : 0.0;
        }
        double a = 0.0;
#pragma unroll
        for (int j = 0; j < kMaxPer; j++)
            if (32 * j < G) a = a + v[j];
#pragma unroll
        for (int off = 16; off >= 1; off >>= 1) a = a + __shfl_xor_sync(0xffffffffu, a, off);
        if (lane == 0) sh.red[warp] = a;
    } else if (warp == 3) {
        long long m = 0;
#pragma unroll
        for (int j = 0; j < kMaxPer; j++) {
            const int bb = lane + 32 * j;
            if (bb < G) {
                const long long mb = __double_as_longlong(__ldcg(&rec[bb].d[3]));
                m = mb > m ? mb : m;
            }
        }
#pragma unroll
        for (int off = 16; off >= 1; off >>= 1) {
            const long long o = __shfl_xor_sync(0xffffffffu, m, off);
            m = o > m ? o : m;
        }
        if (lane == 0) {
            sh.red[3] = __longlong_as_double(m);
            sh.misfit = 0;  // reported by the first (FP32) pass's records
        }
    }
}

// Next pass from the records of the previous one (one thread; every block
// evaluates the same values in the same order).  The FP32 phase decides in
// FP32 (its residual and step size are FP32 quantities; conResTol enters as
// the largest float not above it), the FP64 phase in FP64.
__device__ void fast_decide(FastShared &sh, double tol, int maxIte) {
    if (sh.misfit) {  // a block's rows did not fit its shared memory
        sh.status = kStatusMisfit;
        sh.stop = 1;
        return;
    }
    const bool fp32 = sh.phase == kPh32;
    const int q = sh.q;
    bool conv, bad, pos1;
    if (fp32) {
        const float mx = sh.red32[3];
        conv = mx <= sh.tol32;
        bad = !(mx < INFINITY);  // inf or NaN
        pos1 = sh.red32[1] > 0.0f;
    } else {
        const double mx = sh.red[3];
        conv = mx <= tol;
        bad = !(mx < INFINITY);
        pos1 = sh.red[1] > 0.0;
    }
    // end of a phase: the FP32 phase hands over to the FP64 check, the
    // FP64 phase ends the solve
    auto phase_end = [&](int status) {
        if (fp32) {
            sh.phase = kPhCheck;
            sh.q = 0;
            sh.mode = kModeG0;
        } else {
            sh.status = status;
            sh.stop = 1;
            sh.res = sh.red[3];
        }
    };
    if (bad) {
        sh.status = ALENS_NAN_DETECTED;
        sh.stop = 1;
        return;
    }
    if (q == 0) {
        if (sh.phase == kPhCheck) sh.phase = kPh64;
        if (conv) {
            phase_end(ALENS_OK);
        } else if (maxIte <= 0) {
            phase_end(ALENS_NOT_CONVERGED);
        } else {
            sh.q = 1;
            sh.mode = kModeAG;
        }
        return;
    }
    if (q == 1) {
        if (fp32) {
            float a = pos1 ? __fdiv_rn(sh.red32[0], sh.red32[1]) : 1.0f;
            if (!(a > 0.0f) || !(a < INFINITY)) a = 1.0f;
            sh.alpha32 = a;
        } else {
            double a = pos1 ? sh.red[0] / sh.red[1] : 1.0;
            if (!(a > 0.0) || isinf(a)) a = 1.0;
            sh.alpha = a;
        }
        sh.q = 2;
        sh.mode = kModeIter;
        return;
    }
    const int it = q - 1;  // iterations completed in this phase
    if (fp32)
        sh.it32 = it;
    else
        sh.it64 = it;
    if (conv) {
        phase_end(ALENS_OK);
        return;
    }
    if (pos1) {
        if (fp32) {
            const float a = (it & 1) ? __fdiv_rn(sh.red32[0], sh.red32[1]) : __fdiv_rn(sh.red32[1], sh.red32[2]);
            if (a > 0.0f && a < INFINITY) sh.alpha32 = a;
        } else {
            const double a = (it & 1) ? sh.red[0] / sh.red[1] : sh.red[1] / sh.red[2];
            if (a > 0.0 && !isinf(a)) sh.alpha = a;
        }
    }
    if (it >= maxIte) {
        phase_end(ALENS_NOT_CONVERGED);
        return;
    }
    sh.q = q + 1;
}

__device__ __forceinline__ float lb32_of(int kind, int col, const double *lbGeneral) {
    return kind == 0 ? 0.0f : (kind == 1 ? -INFINITY : (float)lbGeneral[col]);
}
__device__ __forceinline__ double lb64_of(int kind, int col, const double *lbGeneral) {
    return kind == 0 ? 0.0 : (kind == 1 ? -INFINITY : lbGeneral[col]);
}

__global__ void __launch_bounds__(kFastThreads, 1) k_solve_fast(DevState S, FastRecord *recs, float4 *recs32,
                                                              const int *perm,
                                                              const int *inv, unsigned long long timeout_ns) {
    __shared__ FastShared sh;
    // NaNs met by this kernel's row updates are recorded here, not in the
    // context's flags: every block reads those flags at its start, and a
    // block starting late must not see a flag raised by another block's
    // first pass and leave while the others wait for it at a barrier.  A
    // NaN ends the solve through the (infinite) residual in every block at
    // the same pass; block 0 raises the context's flag at the end.
    __shared__ int nanSeen;
    extern __shared__ __align__(16) unsigned char smem[];
    float2 *ownSt = reinterpret_cast<float2 *>(smem + kOffOwnSt);
    float2 *ownQc = reinterpret_cast<float2 *>(smem + kOffOwnQc);
    float *ownLb = reinterpret_cast<float *>(smem + kOffOwnLb);
    int *rowBeg = reinterpret_cast<int *>(smem + kOffRowBeg);
    int *ownK = reinterpret_cast<int *>(smem + kOffOwnK);
    int *ownA = reinterpret_cast<int *>(smem + kOffOwnA);
    int2 *ent = reinterpret_cast<int2 *>(smem + kOffEnt);
    int *haloPos = reinterpret_cast<int *>(smem + kOffHaloPos);
    int *haloCol = reinterpret_cast<int *>(smem + kOffHaloCol);
    float *haloLb = reinterpret_cast<float *>(smem + kOffHaloLb);
    // this pass's value of every column the rows read: slots [0, nr) the
    // block's own rows, kFastRows + h halo column h
    float *xcol = reinterpret_cast<float *>(smem + kOffXcol);
    float2 *gv = reinterpret_cast<float2 *>(smem + kOffGv);
    // streaming layout (aliases the entry region)
    int *sortKey = reinterpret_cast<int *>(smem + kOffEnt);
    int *slotRow = sortKey + kFastRows;
    int *sliceBase = slotRow + kFastRows;
    int *sliceLen = sliceBase + kMaxSlices + 1;
    if (ld_volatile_i32(&S.ctl->errFlags) & kErrStepAbort) return;
    const int G = (int)gridDim.x, b = (int)blockIdx.x;
    const int tid = (int)threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int n = S.dyn[0].nCon;  // one system: constraints [0, n)
    const double tol = S.par[0].tol;
    const int maxIte = S.par[0].maxIte;
#ifdef ALENS_TRACE_FAST
    const long long tStart = clock64();
    long long tLoad = 0;
    long long trSum[6] = {0, 0, 0, 0, 0, 0}, trN = 0;
    __shared__ long long trWarp[kFastWarps];  // each warp's end of its rows
    long long trW[kFastWarps] = {0, 0, 0, 0, 0, 0, 0, 0};
#endif
    if (tid == 0) {
        nanSeen = 0;
        sh.haloCount = 0;
    }
    __syncthreads();

    // ---- this block's rows (permuted positions [r0, r1)) into shared memory
    const int rpb = (n + G - 1) / G;
    const int r0 = min(b * rpb, n), r1 = min(r0 + rpb, n), nr = r1 - r0;
    int fit = rpb <= kFastRows ? 1 : 0;
    int big = 0;  // 1: this block streams its entries from global memory
    if (fit) {
        for (int i = tid; i < nr; i += kFastThreads) {
            const int k = __ldcg(perm + r0 + i);
            const int a0 = __ldg(S.aptr + k);
            ownK[i] = k;
            ownA[i] = a0;
            rowBeg[i + 1] = __ldg(S.aptr + k + 1) - a0;
            ownQc[i] = __ldg(S.qc32 + k);
            ownLb[i] = lb32_of(__ldg(S.lbKind + k), k, S.lb);
            ownSt[i] = make_float2(__ldcg(S.st32[1] + k).x, 0.0f);  // gamma0 (pass 0 reads buffer 0)
        }
        __syncthreads();
        if (warp == 0) {  // inclusive scan of the row lengths
            int carry = 0;
            if (lane == 0) rowBeg[0] = 0;
            for (int c0 = 0; c0 < nr; c0 += 32) {
                const int i = c0 + lane;
                const int v = i < nr ? rowBeg[i + 1] : 0;
                const int incl = warp_incl_scan_i(v);
                if (i < nr) rowBeg[i + 1] = carry + incl;
                carry += __shfl_sync(0xffffffffu, incl, 31);
            }
        }
        __syncthreads();
        const int E = nr > 0 ? rowBeg[nr] : 0;
        if (E > kFastEnts) big = 1;
        if (!big) {
            // entry-parallel: entry e of row i (binary search in rowBeg)
            for (int e = tid; e < E; e += kFastThreads) {
                int lo = 0, hi = nr - 1;
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (rowBeg[mid] <= e)
                        lo = mid;
                    else
                        hi = mid - 1;
                }
                const int i = lo;
                const int4 en = __ldg(S.aent32 + ownA[i] + (e - rowBeg[i]));
                const int pc = __ldcg(inv + en.x);
                const bool own = (unsigned int)(pc - r0) < (unsigned int)nr;
                int slot;
                if (own) {
                    slot = pc - r0;
                } else {
                    const int h = atomicAdd(&sh.haloCount, 1);
                    if (h < kFastHalo) {
                        haloPos[h] = pc;
                        haloCol[h] = en.x;
                        haloLb[h] = lb32_of(en.y & 3, en.x, S.lb);
                    }
                    slot = kFastRows + h;  // unused when the halo overflows (the block streams)
                }
                ent[e] = make_int2(slot, en.z);
            }
        }
    }
    __syncthreads();
    if (fit && !big && sh.haloCount > kFastHalo) big = 1;  // too many halo columns: stream instead
    int2 *gEnt = S.fastEnt + (S.fastEntCap / G) * (long long)b;  // this block's streaming region
    int nSlices = 0;
    if (fit && big) {
        // rows sorted by length, descending (ties by index): keys in a
        // power-of-two bitonic network
        int P = 1;
        while (P < nr) P <<= 1;
        for (int i = tid; i < P; i += kFastThreads) {
            const int len = i < nr ? min(rowBeg[i + 1] - rowBeg[i], 1023) : 0;
            sortKey[i] = i < nr ? (((1023 - len) << 11) | i) : 0x7fffffff;
        }
        __syncthreads();
        for (int k = 2; k <= P; k <<= 1) {
            for (int j = k >> 1; j > 0; j >>= 1) {
                for (int i = tid; i < P; i += kFastThreads) {
                    const int ij = i ^ j;
                    if (ij > i) {
                        const int a = sortKey[i], c = sortKey[ij];
                        if (((i & k) == 0) == (a > c)) {
                            sortKey[i] = c;
                            sortKey[ij] = a;
                        }
                    }
                }
                __syncthreads();
            }
        }
        nSlices = (nr + kSlice - 1) / kSlice;
        for (int t = tid; t < nr; t += kFastThreads) slotRow[t] = sortKey[t] & 2047;
        __syncthreads();
        if (warp == 0) {  // slice lengths (first row of a slice is its longest) and bases
            int carry = 0;
            for (int c0 = 0; c0 < nSlices; c0 += 32) {
                const int sl = c0 + lane;
                int len = 0;
                if (sl < nSlices) {
                    const int i = slotRow[sl * kSlice];
                    len = rowBeg[i + 1] - rowBeg[i];
                    sliceLen[sl] = len;
                }
                const int v = kSlice * len;
                const int incl = warp_incl_scan_i(v);
                if (sl < nSlices) sliceBase[sl] = carry + incl - v;
                carry += __shfl_sync(0xffffffffu, incl, 31);
            }
            if (lane == 0) sliceBase[nSlices] = carry;
        }
        __syncthreads();
        const int total = sliceBase[nSlices];
        if ((long long)total > S.fastEntCap / G) {
            fit = 0;
        } else {
            // entries column-major per slice; padding: the row's own column,
            // value 0.  Eight entries per thread at a time: their operator
            // entries, then their columns' positions, are all requested
            // before any is used.
            constexpr int kFill = 8;
            for (int base = 0; base < total; base += kFill * kFastThreads) {
                int slot[kFill], rowI[kFill], jj[kFill];
                int4 en[kFill];
                int pc[kFill];
#pragma unroll
                for (int u = 0; u < kFill; u++) {
                    const int idx = base + u * kFastThreads + tid;
                    slot[u] = -1;
                    rowI[u] = 0;
                    jj[u] = 0;
                    if (idx < total) {
                        int lo = 0, hi = nSlices - 1;
                        while (lo < hi) {
                            const int mid = (lo + hi + 1) >> 1;
                            if (sliceBase[mid] <= idx)
                                lo = mid;
                            else
                                hi = mid - 1;
                        }
                        const int rel = idx - sliceBase[lo];
                        const int t = lo * kSlice + rel % kSlice;
                        jj[u] = rel / kSlice;
                        if (t < nr) {
                            rowI[u] = slotRow[t];
                            slot[u] = jj[u] < rowBeg[rowI[u] + 1] - rowBeg[rowI[u]] ? 1 : 0;
                        } else {
                            slot[u] = 0;
                        }
                    }
                }
#pragma unroll
                for (int u = 0; u < kFill; u++)
                    en[u] = slot[u] == 1 ? __ldg(S.aent32 + ownA[rowI[u]] + jj[u]) : make_int4(0, 0, 0, 0);
#pragma unroll
                for (int u = 0; u < kFill; u++) pc[u] = slot[u] == 1 ? __ldcg(inv + en[u].x) : 0;
#pragma unroll
                for (int u = 0; u < kFill; u++) {
                    const int idx = base + u * kFastThreads + tid;
                    if (slot[u] < 0) continue;
                    int2 out = make_int2(rowI[u] | kEntOwn, 0);
                    if (slot[u] == 1) {
                        const bool own = (unsigned int)(pc[u] - r0) < (unsigned int)nr;
                        out = make_int2(((own ? pc[u] - r0 : pc[u]) & kEntSrcMask) | ((en[u].y & 3) << 28) |
                                            (own ? kEntOwn : 0),
                                        en[u].z);
                    }
                    gEnt[idx] = out;
                }
            }
        }
    }
    __syncthreads();
    const int nHalo = (fit && !big) ? sh.haloCount : 0;
    // when every row of the block has its own thread, a row of at most
    // kRegEnts entries stays in its thread's registers for the whole solve
    // (column slot and value; entries past the row end: own column, 0)
    int regSlot[kRegEnts];
    float regVal[kRegEnts];
    bool inRegs = false;
    if (fit && !big && nr <= kFastThreads && tid < nr) {
        const int e0 = rowBeg[tid], len = rowBeg[tid + 1] - e0;
        inRegs = len <= kRegEnts;
#pragma unroll
        for (int j = 0; j < kRegEnts; j++) {
            const int2 en = (inRegs && j < len) ? ent[e0 + j] : make_int2(tid, 0);
            regSlot[j] = en.x;
            regVal[j] = __int_as_float(en.y);
        }
    }
#ifdef ALENS_TRACE_FAST
    tLoad = clock64();
#endif
    if (tid == 0) {
        float t32 = (float)tol;
        if ((double)t32 > tol) t32 = nextafterf(t32, 0.0f);
        sh.tol32 = t32;
        sh.alpha32 = 0.0f;
        sh.alpha = 0.0;
        sh.res = 0.0;
        sh.mode = kModeG0;
        sh.phase = kPh32;
        sh.q = 0;
        sh.stop = 0;
        sh.status = ALENS_OK;
        sh.it32 = sh.it64 = 0;
        sh.misfit = 0;
    }
    __syncthreads();

    SolveView<double> V64{};
    V64.aptr = S.aptr;
    V64.aent = S.aent;
    V64.st[0] = S.st[0];
    V64.st[1] = S.st[1];
    V64.qc = S.qc;
    V64.lbGeneral = S.lb;
    V64.fp64 = 1;
    // permuted FP32 iterates in global memory for the other blocks' halos:
    // pass p writes buffer p & 1; pass 0 reads the canonical initial guess
    // (buffer 1, canonical order), which pass 1 overwrites after every
    // block has gathered it
    float2 *const gst0 = S.st32[0], *const gst1 = S.st32[1];
    const unsigned int gvBase = (unsigned int)__cvta_generic_to_shared(gv);
    // FP32 phase: at most maxIte + 2 passes; FP64 phase (check included):
    // at most maxIte + 2 more
    const int maxPass = 2 * (maxIte + 2) + 2;
    int lastOut = 0;
    for (int p = 0; p < maxPass; p++) {
#ifdef ALENS_TRACE_FAST
        const long long tA = clock64();
        long long tB = 0, tE = 0, tF = 0;
#endif
        const bool odd = (p & 1) != 0;
        const FastRecord *recIn = recs + (size_t)((p - 1) & 1) * kFastMaxGrid;
        const float4 *rec32In = recs32 + (size_t)((p - 1) & 1) * kFastMaxGrid;
        if (sh.phase == kPh32) {
            // the previous pass ran in FP32: this pass (FP32 or the FP64
            // check) needs the halo columns' FP32 iterates; warp 0 reads the
            // FP32 records and decides
            if (warp >= kGatherWarp0 && nHalo > 0) {
                const float2 *src = p == 0 ? gst1 : (odd ? gst0 : gst1);
                const int *idx = p == 0 ? haloCol : haloPos;
                for (int h = tid - 32 * kGatherWarp0; h < nHalo; h += kFastThreads - 32 * kGatherWarp0)
                    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(gvBase + (unsigned int)(h * 8)),
                                 "l"(src + idx[h])
                                 : "memory");
                asm volatile("cp.async.wait_all;" ::: "memory");
            }
            if (p > 0 && warp == 0) {
                grid_records32(rec32In, G, sh);
                if (lane == 0) fast_decide(sh, tol, maxIte);
            }
        } else {
            if (warp < 4) grid_records64(recIn, G, sh);
            __syncthreads();
            if (tid == 0) fast_decide(sh, tol, maxIte);
        }
        __syncthreads();
#ifdef ALENS_TRACE_FAST
        tB = clock64();
#endif
        if (sh.stop) break;
        const int phase = sh.phase, mode = sh.mode;
        FastRecord *recOut = recs + (size_t)(p & 1) * kFastMaxGrid + b;
        float4 *rec32Out = recs32 + (size_t)(p & 1) * kFastMaxGrid + b;
        if (phase == kPh32) {
            const float alpha = sh.alpha32;
            const float2 *ownIn = ownSt + (odd ? kFastRows : 0);
            float2 *ownOut = ownSt + (odd ? 0 : kFastRows);
            float2 *gOut = odd ? gst1 : gst0;
            float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f, am = 0.0f;
            // iterates of the other blocks' columns (streaming blocks): the
            // previous pass's permuted buffer, or at pass 0 the canonical
            // initial guess
            const float2 *gIn = odd ? gst0 : gst1;
            // row tail shared by both layouts
            auto finish_row = [&](int i, float acc, float gam, float gold, float lbk, float xk) {
                const float2 qc = ownQc[i];
                acc = fmaf(qc.y, xk, acc);
                float2 o;
                if (mode == kModeAG) {
                    a0 += gold * gold;
                    a1 += gold * acc;
                    o = make_float2(gam, gold);
                } else {
                    const float gn = acc + qc.x;
                    // x - P(x - g) = min(g, x - lb)
                    const float mm = gn < xk - lbk ? gn : xk - lbk;
                    float rm = fabsf(mm);
                    if (rm != rm) {
                        atomicOr(&nanSeen, kErrNaN);
                        rm = INFINITY;
                    }
                    am = rm > am ? rm : am;
                    if (mode == kModeIter) {
                        const float s = xk - gam, y = gn - gold;
                        a0 += s * s;
                        a1 += s * y;
                        a2 += y * y;
                    }
                    o = make_float2(xk, gn);
                }
                ownOut[i] = o;
                gOut[r0 + i] = o;
            };
            if (fit && big) {
                // a warp per slice, a lane per row; entry j of the slice's rows
                // is one coalesced load
                for (int sl = warp; sl < nSlices; sl += kFastWarps) {
                    const int t = sl * kSlice + lane;
                    const int i = t < nr ? slotRow[t] : 0;
                    const float2 own = ownIn[i];
                    const float gam = own.x, gold = own.y, lbk = ownLb[i];
                    float xk;
                    if (mode == kModeG0)
                        xk = gam;
                    else if (mode == kModeAG)
                        xk = gold;
                    else
                        xk = projlb<float>(fmaf(-alpha, gold, gam), lbk);
                    float acc = 0.0f;
                    const int len = sliceLen[sl];
                    const int2 *se = gEnt + sliceBase[sl] + lane;
                    // software pipeline: the next batch's entries are requested
                    // before this batch's iterates
                    int2 nxt[kRowBatch];
#pragma unroll
                    for (int j = 0; j < kRowBatch; j++)
                        nxt[j] = j < len ? __ldg(se + j * kSlice) : make_int2(i | kEntOwn, 0);
                    for (int jb = 0; jb < len; jb += kRowBatch) {
                        int2 en[kRowBatch];
                        float2 sv[kRowBatch];
#pragma unroll
                        for (int j = 0; j < kRowBatch; j++) en[j] = nxt[j];
#pragma unroll
                        for (int j = 0; j < kRowBatch; j++)
                            nxt[j] = jb + kRowBatch + j < len ? __ldg(se + (jb + kRowBatch + j) * kSlice)
                                                              : make_int2(i | kEntOwn, 0);
#pragma unroll
                        for (int j = 0; j < kRowBatch; j++) {
                            const int src = en[j].x & kEntSrcMask;
                            if (en[j].x & kEntOwn)
                                sv[j] = ownIn[src];
                            else if (p == 0)
                                sv[j] = make_float2(__ldcg(gst1 + __ldcg(perm + src)).x, 0.0f);
                            else
                                sv[j] = gIn[src];
                        }
#pragma unroll
                        for (int j = 0; j < kRowBatch; j++) {
                            // lower bound of the column: 0 (collisions), none (crosslinks);
                            // only a general bound (kind 2) needs the column's value
                            const int kind = (en[j].x >> 28) & 3;
                            float lbl = kind == 0 ? 0.0f : -INFINITY;
                            if (kind == 2) {
                                const int src = en[j].x & kEntSrcMask;
                                lbl = (float)S.lb[(en[j].x & kEntOwn) ? ownK[src] : __ldcg(perm + src)];
                            }
                            float xl;
                            if (mode == kModeG0)
                                xl = sv[j].x;
                            else if (mode == kModeAG)
                                xl = sv[j].y;
                            else
                                xl = projlb<float>(fmaf(-alpha, sv[j].y, sv[j].x), lbl);
                            acc = fmaf(__int_as_float(en[j].y), xl, acc);
                        }
                    }
                    if (t < nr) finish_row(i, acc, gam, gold, lbk, xk);
                }
            }
            if (fit && !big) {
                // every column's value for this pass, once: the iterate
                // (G0), the gradient (AG) or the projected step (iterations)
                auto colval = [&](float2 v, float lb) {
                    if (mode == kModeG0) return v.x;
                    if (mode == kModeAG) return v.y;
                    return projlb<float>(fmaf(-alpha, v.y, v.x), lb);
                };
                const float2 *ownIn = ownSt + (odd ? kFastRows : 0);
                for (int i = tid; i < nr; i += kFastThreads) xcol[i] = colval(ownIn[i], ownLb[i]);
                for (int h = tid; h < nHalo; h += kFastThreads) xcol[kFastRows + h] = colval(gv[h], haloLb[h]);
                __syncthreads();
            }
            for (int i = tid; i < nr && fit && !big; i += kFastThreads) {
                const int e0 = rowBeg[i], e1 = rowBeg[i + 1];
                // the row's own iterate and its x (the diagonal entry's column)
                const float2 own = ownIn[i];
                const float gam = own.x, gold = own.y, lbk = ownLb[i];
                const float xk = xcol[i];
                float acc = 0.0f;
                if (inRegs) {
                    // the entries from registers: only the column values are
                    // read (padding entries add exact zeros)
                    float xl[kRegEnts];
#pragma unroll
                    for (int j = 0; j < kRegEnts; j++) xl[j] = regVal[j] != 0.0f ? xcol[regSlot[j]] : 0.0f;
#pragma unroll
                    for (int j = 0; j < kRegEnts; j++) acc = fmaf(regVal[j], xl[j], acc);
                }
                for (int eb = e0; eb < e1 && !inRegs; eb += kRowBatch) {
                    // all entries of the batch, then all their column values,
                    // are requested before any is used; entries past the row
                    // end read the row's own column with value 0
                    int2 en[kRowBatch];
                    float xl[kRowBatch];
#pragma unroll
                    for (int j = 0; j < kRowBatch; j++) en[j] = eb + j < e1 ? ent[eb + j] : make_int2(i, 0);
#pragma unroll
                    for (int j = 0; j < kRowBatch; j++) xl[j] = xcol[en[j].x];
#pragma unroll
                    for (int j = 0; j < kRowBatch; j++) acc = fmaf(__int_as_float(en[j].y), xl[j], acc);
                }
                finish_row(i, acc, gam, gold, lbk, xk);
            }
#ifdef ALENS_TRACE_FAST
            if (lane == 0) trWarp[warp] = clock64();
            __syncthreads();
            tE = clock64();
            if (tid == 0) {
                long long lo = trWarp[0], hi = trWarp[0];
                for (int w = 1; w < kFastWarps; w++) {
                    lo = trWarp[w] < lo ? trWarp[w] : lo;
                    hi = trWarp[w] > hi ? trWarp[w] : hi;
                }
                if (p > 2) {
                    trSum[4] += lo - tB;  // first warp done with its rows
                    trSum[5] += hi - tB;  // last warp done
                    for (int w = 0; w < kFastWarps; w++) trW[w] += trWarp[w] - tB;
                }
            }
#endif
            block_record<float>(a0, a1, a2, am, !fit, sh, recOut, rec32Out);
#ifdef ALENS_TRACE_FAST
            tF = clock64();
#endif
        } else if (phase == kPhCheck) {
            // FP64 residual of the promoted FP32 iterate (canonical FP64 buffer)
            const float2 *ownIn = ownSt + (odd ? kFastRows : 0);
            double2 *stOut = S.st[p & 1];
            double am = 0.0;
            const float2 *gIn = odd ? gst0 : gst1;  // the last FP32 pass's permuted iterates
            for (int i = tid; i < nr && fit; i += kFastThreads) {
                const int e0 = rowBeg[i], e1 = rowBeg[i + 1], k = ownK[i], a0 = ownA[i];
                const double lbk = lb64_of(__ldg(S.lbKind + k), k, S.lb);
                double xk = (double)ownIn[i].x;
                xk = xk < lbk ? lbk : xk;
                double acc = 0.0;
                for (int e = e0; e < e1; e++) {
                    const int4 e64 = __ldg(S.aent + a0 + (e - e0));
                    float xs;
                    double lbl;
                    if (big) {
                        const int pc = __ldcg(inv + e64.x);
                        xs = (unsigned int)(pc - r0) < (unsigned int)nr ? ownIn[pc - r0].x : gIn[pc].x;
                        lbl = lb64_of(e64.y & 3, e64.x, S.lb);
                    } else {
                        const int slot = ent[e].x;
                        xs = slot < kFastRows ? ownIn[slot].x : gv[slot - kFastRows].x;
                        lbl = lb64_of(e64.y & 3, e64.x, S.lb);
                    }
                    double xl = (double)xs;
                    xl = xl < lbl ? lbl : xl;
                    acc = fma(__hiloint2double(e64.w, e64.z), xl, acc);
                }
                const double2 qc = __ldg(S.qc + k);
                acc = fma(qc.y, xk, acc);
                const double gn = acc + qc.x;
                const double pr = xk - gn < lbk ? lbk : xk - gn;
                double rm = fabs(xk - pr);
                if (rm != rm) {
                    atomicOr(&nanSeen, kErrNaN);
                    rm = INFINITY;
                }
                am = rm > am ? rm : am;
                stOut[k] = make_double2(xk, gn);
            }
            block_record<double>(0.0, 0.0, 0.0, am, !fit, sh, recOut, rec32Out);
        } else {
            // FP64 refinement: canonical rows of this block, global memory
            const double alpha = sh.alpha;
            const double2 *stIn = S.st[odd ? 0 : 1];
            double2 *stOut = S.st[p & 1];
            double a0 = 0.0, a1 = 0.0, a2 = 0.0, am = 0.0;
            for (int i = tid; i < nr && fit; i += kFastThreads) {
                double v0 = 0.0, v1 = 0.0, v2 = 0.0, rm = 0.0;
                row_update<double>(V64, ownK[i], mode, alpha, stIn, stOut, v0, v1, v2, rm, &nanSeen, RowCache{});
                a0 = a0 + v0;
                a1 = a1 + v1;
                a2 = a2 + v2;
                am = rm > am ? rm : am;
            }
            block_record<double>(a0, a1, a2, am, !fit, sh, recOut, rec32Out);
        }
        lastOut = p;
        if (!fast_barrier(S, p, G, timeout_ns)) return;
#ifdef ALENS_TRACE_FAST
        if (tE != 0 && p > 2) {
            const long long tG = clock64();
            trSum[0] += tB - tA;  // halo copy, records, decision
            trSum[1] += tE - tB;  // rows
            trSum[2] += tF - tE;  // block record
            trSum[3] += tG - tF;  // barrier
            trN++;
        }
#endif
    }
#ifdef ALENS_TRACE_FAST
    if (tid == 0 && trN > 0 && b == 0)
        printf("fast trace block 0 warps: %lld %lld %lld %lld %lld %lld %lld %lld\n", trW[0] / trN, trW[1] / trN,
               trW[2] / trN, trW[3] / trN, trW[4] / trN, trW[5] / trN, trW[6] / trN, trW[7] / trN);
    if (tid == 0 && trN > 0 && (b == 0 || b == G / 2 || b == G - 1))
        printf("fast trace block %d: row loading %lld cycles; %d FP32 passes: halo+records+decision %lld, rows %lld, "
               "block record %lld, barrier %lld cycles per pass (warps done with rows after %lld..%lld); rows %d "
               "halo %d\n",
               b, tLoad - tStart, (int)trN, trSum[0] / trN, trSum[1] / trN, trSum[2] / trN, trSum[3] / trN,
               trSum[4] / trN, trSum[5] / trN, nr,
               nHalo);
#endif
    if (b == 0 && tid == 0) {
        RepDyn &d = S.dyn[0];
        if (sh.status == kStatusMisfit) {
            // rows too large for the blocks' shared memory: the step is rerun
            // with the grid form
            atomicOr(&S.ctl->errFlags, kErrSolverFit);
            return;
        }
        int status = sh.status;
        if (!sh.stop) status = ALENS_NOT_CONVERGED;  // pass bound reached (not expected)
        d.refineIter = sh.it32;
        d.iter = sh.it64;
        d.status = status;
        d.converged = status == ALENS_OK ? 1 : 0;
        d.res = sh.res;
        d.active = 0;
        d.refined = (status == ALENS_OK && sh.it64 == 0) ? 1 : 0;
        d.finalPar = lastOut & 1;
        S.ctl->finalParity = lastOut & 1;
        S.ctl->allRefined = 1;
        if (status == ALENS_NAN_DETECTED || nanSeen) atomicOr(&S.ctl->errFlags, kErrNaN);
    }
}

// ---------------------------------------------------------------- ordering
// Constraints whose rod I lies in the cell (a rod's side-I entries of the
// rod rows), one warp per cell in Morton rank order.
__global__ void k_order_count(DevState S) {
    if (ld_volatile_i32(&S.ctl->errFlags) & (kErrNaN | kErrOverflow)) return;
    const int w = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (w >= S.nCells) return;
    const int c = S.cellByRank[w];
    const int s0 = S.cellStart[c], s1 = S.cellStart[c + 1];
    int cnt = 0;
    for (int s = s0 + lane; s < s1; s += 32) {
        const int r = S.sidx[s];
        for (int e = S.rowPtr[r]; e < S.rowPtr[r + 1]; e++) cnt += (S.rowEnt[e] & 1) == 0 ? 1 : 0;
    }
    cnt = warp_sum_i(cnt);
    if (lane == 0) S.fastCellCnt[w] = cnt;
}

// Permutation and inverse, one warp per cell (rank order): a rod's
// constraints (those with the rod as I, ascending: its collisions, then its
// crosslinker and user blocks) start after those of the cell's rods with a
// smaller index (their counts summed, no sort needed), so the order within a
// cell is by rod index whatever order the cell list holds them in.
__global__ void __launch_bounds__(256) k_order_place(DevState S) {
    __shared__ int stage[8][2 * kFastCellRods];  // per warp: the cell's rods and their counts
    if (ld_volatile_i32(&S.ctl->errFlags) & (kErrNaN | kErrOverflow)) return;
    const int gw = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    if (gw >= S.nCells) return;
    const int c = S.cellByRank[gw];
    const int s0 = S.cellStart[c], m = S.cellStart[c + 1] - s0;
    const int base = S.fastCellBase[gw];
    int *rods = stage[warp], *cnts = stage[warp] + kFastCellRods;
    auto side_i_count = [&](int r) {
        int n = 0;
        for (int e = S.rowPtr[r]; e < S.rowPtr[r + 1]; e++) n += (S.rowEnt[e] & 1) == 0 ? 1 : 0;
        return n;
    };
    const bool staged = m <= kFastCellRods;
    if (staged) {
        for (int s = lane; s < m; s += 32) {
            const int r = S.sidx[s0 + s];
            rods[s] = r;
            cnts[s] = side_i_count(r);
        }
        __syncwarp();
    }
    for (int s = lane; s < m; s += 32) {
        const int r = staged ? rods[s] : S.sidx[s0 + s];
        int off = 0;
        for (int u = 0; u < m; u++) {
            const int ru = staged ? rods[u] : S.sidx[s0 + u];
            if (ru < r) off += staged ? cnts[u] : side_i_count(ru);
        }
        int pos = base + off;
        for (int e = S.rowPtr[r]; e < S.rowPtr[r + 1]; e++) {
            const int ent = S.rowEnt[e];
            if (ent & 1) continue;
            const int k = ent >> 1;
            S.fastPerm[pos] = k;
            S.fastInv[k] = pos;
            pos++;
        }
    }
}

}  // namespace

// The spatial row order of the single-system solver (count, scan, place);
// returns the kernels launched.
int launch_fast_order(const DevState &S, cudaStream_t st) {
    const int blocks = (S.nCells * 32 + 255) / 256;
    k_order_count<<<blocks > 0 ? blocks : 1, 256, 0, st>>>(S);
    int n = 1 + launch_scan(S.fastCellCnt, S.fastCellBase, S.nCells, S.fastScanTmp, st);
    k_order_place<<<blocks > 0 ? blocks : 1, 256, 0, st>>>(S);
    return n + 1;
}

// Blocks of the single-system form (one per SM), 0 if it cannot be resident.
int fast_solver_grid() {
    static int cached = -1;
    if (cached >= 0) return cached;
    int dev = 0, nsm = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (cudaFuncSetAttribute(k_solve_fast, cudaFuncAttributeMaxDynamicSharedMemorySize, kFastSmem) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_solve_fast, kFastThreads, kFastSmem) != cudaSuccess) {
        cudaGetLastError();
        per = 0;
    }
    cached = per > 0 ? (nsm < kFastMaxGrid ? nsm : kFastMaxGrid) : 0;
    return cached;
}

// Constraints the single-system form holds (rows per block x blocks).
long long fast_solver_capacity() { return (long long)kFastRows * fast_solver_grid(); }

cudaError_t launch_solve_fast(const DevState &S, int grid, unsigned long long timeout_ns, cudaStream_t st) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(kFastThreads);
    cfg.dynamicSmemBytes = kFastSmem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_solve_fast, S, reinterpret_cast<FastRecord *>(S.fastPart),
                              reinterpret_cast<float4 *>(S.fastPart + 2 * 4 * (size_t)kFastMaxGrid),
                              (const int *)S.fastPerm, (const int *)S.fastInv, timeout_ns);
}

}  // namespace alens
