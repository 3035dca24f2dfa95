// engine.cuh - device state of a context and the kernel launchers.
//
// Layout in HBM (all replicas of a context concatenated):
//   rods        SoA FP64: px py pz | qx qy qz qw | len rad (72 B/rod) + gid,
//               per-step axis, collision half-length/radius, mobilities,
//               known velocity (6 SoA) and solver velocity U (6 SoA)
//   cells       count/start/cursor per cell; cell-sorted copy of the search
//               geometry (centre, axis, half-length, radius, rod index)
//   pairs       raw 64-bit keys (i<<32 | j<<5 | image), per-rod counts and
//               offsets, canonical keys sorted by (i, j, image)
//   constraints AoS Jacobian 12 x FP64 (96 B), mobility-weighted Jacobian
//               W = M J (96 B), rod indices I/J, phi0, q, final gamma,
//               solver iterates gamma/g by pass parity, lower bound,
//               compliance, lab points (+ FP32 copies for the mixed solver)
//   rod rows    rod-major rows of D: entries 2k+side, ascending (CSR)
//   operator    Delassus rows A = dt D^T M D (CSR: aptr, acol, aval FP64
//               [+ aval32]); ~4-20 nonzeros per row
//   reduction   level-1 tile partials (64-constraint tiles) + per-block
//               chunk work space
#pragma once

#include <utility>

#include <cstdint>
#include <cuda_runtime.h>

#include "alens_gpu.h"
#include "common.cuh"

namespace alens {

struct RepParams {
    double lo[3], hi[3], L[3];
    double cellsz[3];
    double mu, kT, dt, colRatioD, colRatioL, colBuf, tol;
    unsigned long long seed;
    int pbc[3];
    int mono;
    int ncell[3];
    int cellOffset;
    int rodOffset;
    int nRods;
    int maxIte;
    int stencil;          // pair-search cells per dimension around a rod's cell (3 or 5)
    double halfReachMax;  // max over rods of collision half-length + radius
    double bcoef;         // sqrt(2 kT / dt), Brownian velocity scale (kT > 0)
    // FP32 copies for the pair screen (conversions from FP64 issue on the
    // FP64 pipe, 2 lanes/clk/SM on GB300)
    float cellsz32[3], colBuf32, halfReach32, pad32;
};

// per-replica state produced on the device
struct RepDyn {
    int collStart, collEnd;   // range in the canonical collision list
    int conStart, nCon;       // constraint range
    int tileStart, nTiles;    // level-1 tiles of the constraint range
    int iter, active, converged, status;
    int counter;              // last-arriver ticket of the current pass
    int refineIter;
    int finalPar;             // solver buffer holding this replica's result
    int refined;              // 1: the FP32 solution's FP64 residual is within
                              // tolerance (no FP64 refinement sweep needed)
    unsigned long long res64bits;  // FP64 residual of the FP32 solution (max, bits)
    double alpha, res;
};

struct DevCtl {
    long long step;
    int rawCount;     // collision pairs found (may exceed capacity)
    int errFlags;     // kErr* bits
    int borderCount;  // pair candidates left to the FP64 decision
    int totalColl, totalBil, totalCon, nTiles;
    int totalNnz;     // nonzeros of the Delassus operator
    int maxIte;       // max over replicas
    int activeCnt[3]; // replicas active per solver pass (mod 3)
    int finalParity;  // buffer holding the solver's last iterate
    int allRefined;   // every replica's FP32 solution met the FP64 tolerance
    unsigned int setupDone;  // blocks of the refinement set-up that finished
    GridBarrier bar;
};

// Programmatic dependent launch.  A kernel launched with launch_pdl may be
// scheduled while the previous kernel of its stream is still running: it
// first waits (griddepcontrol.wait) until that kernel has completed and its
// writes are visible, then lets its own dependents be scheduled.  Every
// kernel of the step starts with ALENS_PDL_PROLOGUE (a no-op when the
// kernel was launched normally).
#define ALENS_PDL_PROLOGUE()                                        \
    do {                                                            \
        asm volatile("griddepcontrol.wait;" ::: "memory");          \
        asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); \
    } while (0)

template <class... KArgs, class... Args>
inline void launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                       Args &&...args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

// Device pointers and sizes of one context; passed to kernels by value.
struct DevState {
    int R, nRods, cap, nCells, tileCap, workCap, blockCap, nnzCap;
    int warm, precision;
    int warmNet;               // 1: the learned warm start's network runs this step (ALENS_WARM_MLP with
                               // a model): its features look up the previous multipliers themselves
    int solveMinTiles;         // BBPGD: at least this many 64-row tiles per solver block
    int barrierExtra;          // solver grid barriers wait for this many blocks more than launched
                               // (0; 1 only to test the bounded-wait path: every wait runs out)
    int pairW[3];              // pair search: stencil width per dimension (max over replicas;
                               // 1 where every replica has one closed cell)
    RepParams *par;
    RepDyn *dyn;
    DevCtl *ctl;
    int *bilPrefix;  // [R+1] blocks per replica (prefix, host-written)
    // rods
    double *px, *py, *pz, *qx, *qy, *qz, *qw, *len, *rad;
    long long *gid;
    int *imm, *rodRep;
    double *ax, *ay, *az, *hcol, *rcol, *m0, *m1, *m2;
    double *sm0, *sm1, *sm2;   // square roots of the mobilities (Brownian noise)
    unsigned char *sph;
    double *unc, *vel;      // 6 x nRods SoA each
    double *stage;          // 7 x nRods host-transfer staging (interleaved)
    // cells
    int *cellOf, *cellCount, *cellStart, *cellCursor;
    float4 *sA, *sB;   // cell-sorted FP32 search geometry
    int *sidx;
    // pairs
    int *pairCount, *pairOff, *pairCursor;
    unsigned long long *rawKeys, *keys;
    int4 *border;              // pair candidates within the FP32 screen's margin: (i, j, image)
    // constraints
    int *conI, *conJ, *conImg;
    float2 *conST;             // contact parameters (s / h_I, t / h_J) of collisions
    float *rodV;               // learned warm start: per rod, sum over its compressed collisions l
                               // (q_l < 0) of (-q_l) W_l at the rod's side (6 x nRods, SoA;
                               // formed by k_rows_sort when features are wanted)
    float *feat, *fscale;      // learned warm start: 12 features and A_kk / d per
                               // constraint (allocated while features are recorded)
    double *jac;
    double *phi0, *q, *gamma, *lb, *cinv, *lab;
    int *lbKind;               // 0: lb = 0, 1: bilateral, 2: general lb
    double2 *qc;               // (q, cinv) FP64
    float2 *qc32;              // (q, cinv) FP32
    double2 *st[2];            // solver iterates (gamma, g) by pass parity
    float2 *st32[2];
    double *alphaBuf;          // 2 x R step sizes by pass parity
    // Delassus operator A = dt D^T M D (rows ascending in column)
    double *W;                 // 12 x cap: M J per constraint side
    int *annz, *aptr;
    int4 *aent;                // {col, kind, lo(val), hi(val)}
    int4 *aent32;              // {col, kind, bits(val32), bits(lb32)}
    int *rowCount, *rowPtr, *rowCursor, *rowEnt;
    unsigned long long *prevKeys;
    double *prevGamma;
    int *prevCount;
    AlensBlock *blocks;
    int *blockRep;
    // pre-bound crosslinkers (blocks built on the device every step)
    int nLinks;
    int *linkI, *linkJ, *linkRep, *linkLocal;  // global rod indices, replica, index in replica
    double *linkSI, *linkSJ, *linkRest, *linkKappa;
    int *linkSlot0;  // [R] block slot of each replica's first link (host-written)
    // confinement boundaries (unit axes), replica r owns [bndStart[r], bndStart[r+1])
    int nBnd;
    BoundaryDev *bnd;
    int *bndStart;
    // reductions
    double *part;   // 9 x tileCap (solver: 2 parities x 4 kinds; stress: 9)
    double *work;   // per block 9 x workCap
    int *tileRep;   // tileCap
    double *stress; // 9 x R outputs
    // single-system solver (kernels_fast.cu): per-block records (2 parities
    // x kFastMaxGrid blocks: 32-byte FP64 records, then 16-byte FP32
    // records), the spatial row permutation and its
    // inverse (constraint capacity), constraints per cell in Morton order and
    // their exclusive scan (nCells + 1 each), scan scratch, and the cells in
    // Morton order (fixed per context)
    double *fastPart;
    int *fastPerm, *fastInv, *fastCellCnt, *fastCellBase, *fastScanTmp, *cellByRank;
    int2 *fastEnt;             // streaming layout of the single-system solver (fastEntCap entries,
    long long fastEntCap;      // an equal region per block)
    // scan scratch
    int *scanTmp;
};

// ---- detect stage (kernels_detect.cu)
void launch_step_clear(const DevState &S, cudaStream_t st);
void launch_prep(const DevState &S, cudaStream_t st);
void launch_noise(const DevState &S, cudaStream_t st);
void launch_mobility(const DevState &S, cudaStream_t st);  // once per rod set
int launch_scan(const int *in, int *out, int n, int *tmp, cudaStream_t st);  // returns kernels launched
int launch_scan_dev(const int *in, int *out, int nMax, const int *nDev, int *tmp, cudaStream_t st);
void launch_scatter(const DevState &S, cudaStream_t st);
void launch_link_blocks(const DevState &S, cudaStream_t st);
void launch_pairs(const DevState &S, cudaStream_t st);
void launch_boundary_pairs(const DevState &S, cudaStream_t st);  // only when S.nBnd > 0
int launch_pair_sort(const DevState &S, cudaStream_t st);
void launch_ranges(const DevState &S, cudaStream_t st);
void launch_build(const DevState &S, cudaStream_t st);
// rod rows (scan, fill, sort); with `weights` (an event after the weights
// kernel) the sort also forms the learned warm start's per-rod sums
int launch_rows(const DevState &S, cudaStream_t st, cudaEvent_t weights);
// ---- Delassus operator (kernels_assemble.cu)
void launch_weights(const DevState &S, cudaStream_t st);
int launch_assemble(const DevState &S, cudaStream_t st, cudaStream_t side, cudaEvent_t join);
void launch_unpack_rods(const DevState &S, int rodOffset, int n, cudaStream_t st);
void launch_pack_rods(const DevState &S, int rodOffset, int n, int what, cudaStream_t st);

// ---- solve / advance (kernels_solve.cu)
constexpr int kMaxSolverGrid = 152 * 8;  // work space is sized for this
constexpr int kFastMaxGrid = 256;        // blocks of the single-system solver (one per SM)
int solver_max_grid(int precision);  // cooperative residency limit
// Forms of the FP32 (mixed-precision) solver
enum SolverForm {
    kFormGrid = 0,      // cooperative grid over all SMs, software grid barrier
    kFormCluster = 1,   // one cluster per replica, iterates in global memory
    kFormResident = 2,  // one cluster per replica, problem held in shared memory
    kFormFast = 3       // one system: spatial row order, per-block records, FP64 check and refinement
                        // in the same launch (kernels_fast.cu)
};
// precision == MIXED: FP32 kernel, state reset, FP64 refinement kernel
// (events ev[0..3] recorded around the two kernels when non-null).
cudaError_t launch_solve(const DevState &S, int grid, int precision, unsigned long long timeout_ns,
                         cudaStream_t st, cudaEvent_t *ev, int *launches, int form, int clusterSize,
                         int nClusters, bool finish);
int cluster_max_size();            // largest cluster the FP32 solver can use
int cluster_max_active(int cs);    // co-resident clusters of that size
int csm_cluster_size(int *maxActive);  // cluster-resident form: largest cluster, 0 if unusable
void csm_set_threads(int threads);     // cluster-resident form: threads per CTA (256/512/1024)
int csm_threads();
int fast_solver_grid();            // single-system form: blocks (one per SM), 0 if unusable
long long fast_solver_capacity();  // single-system form: constraints it holds
int launch_fast_order(const DevState &S, cudaStream_t st);  // its row order (side stream); kernels launched
void launch_advance(const DevState &S, cudaStream_t st);
void launch_stress(const DevState &S, cudaStream_t st);

}  // namespace alens
