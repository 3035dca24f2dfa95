/*
 * alens_gpu.h - C ABI of the GB300 rod collision-and-constraint step.
 *
 * One call of alens_step() performs what SimToolbox's
 * SylinderSystem::runStep() does for rigid spherocylinders ("sylinders") in
 * aLENS, on one GPU:
 *
 *   Brownian (known) velocity -> cell-list near-pair search -> segment-segment
 *   closest points -> constraint Jacobian D -> BBPGD solve of the bound
 *   constrained QP on  A = dt D^T M D (+ compliance)  -> velocity write-back
 *   -> Euler update of positions and orientations.
 *
 * The caller is aLENS's TubuleSystem (SRC/TubuleSystem.cpp:223 calls
 * rodSystem.runStep()); the entry points below are what a binding of that
 * call surface needs.  Each declaration cites the reference interface it
 * replaces.  The reference's SimToolbox submodule is not part of the
 * reference checkout, so those citations name the aLENS call site.
 *
 * Conventions
 *   - Every function returns an AlensStatus code; nothing throws or exits.
 *   - The library owns all device memory; the caller owns host buffers,
 *     which are only read or written during the call.
 *   - One context = one CUDA stream.  A context is not thread safe: call it
 *     from one host thread at a time (the reference calls runStep from the
 *     master thread, outside OpenMP regions, SRC/TubuleSystem.cpp:221-226).
 *   - A context may hold several independent systems ("replicas") that are
 *     stepped together in one launch sequence; a plain system is replica 0.
 *   - Units follow aLENS: um, pN, s (Protein/ProteinModel.md:14-19).
 *   - Orientation quaternions are stored (x, y, z, w), the storage order of
 *     Sylinder::orientation (an Eigen quaternion, SRC/TubuleBind.hpp:63); the
 *     rod axis is q * (0,0,1).
 */
#ifndef ALENS_GPU_H
#define ALENS_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  Replaces std::exit / assert error handling of the reference
 * (SRC/TubuleSystem.cpp:500,642). */
typedef enum AlensStatus {
    ALENS_OK = 0,
    ALENS_INVALID_ARG = 1,   /* bad argument, size or configuration          */
    ALENS_CUDA_ERROR = 2,    /* a CUDA runtime call failed                   */
    ALENS_NOT_CONVERGED = 3, /* BBPGD hit conMaxIte; the step still completed */
    ALENS_CAPACITY = 4,      /* fixed constraint capacity too small          */
    ALENS_TIMEOUT = 5,       /* a bounded device-side wait gave up           */
    ALENS_NAN_DETECTED = 6,  /* NaN/Inf in rod state or in the solve         */
    ALENS_NO_DEVICE = 7,     /* no usable CUDA device                        */
    ALENS_NOT_READY = 8      /* call order violated (e.g. no rods set)       */
} AlensStatus;

typedef enum AlensPrecision {
    ALENS_PREC_FP64 = 0,  /* everything FP64 (the oracle's arithmetic)        */
    ALENS_PREC_MIXED = 1  /* FP32 SpMV/projection, FP64 dots, residual and
                             final refinement sweeps                          */
} AlensPrecision;

typedef enum AlensWarmStart {
    ALENS_WARM_ZERO = 0,  /* gamma0 = 0 for collisions (block.gamma for
                             bilateral blocks)                                */
    ALENS_WARM_PREV = 1,  /* previous step's gamma for persisting pairs       */
    ALENS_WARM_MLP = 2    /* learned prediction (see alens_mlp_*), falling
                             back to the previous gamma when not loaded       */
} AlensWarmStart;

/* Hot-path subset of SimToolbox SylinderConfig (RunConfig.yaml keys,
 * docs/source/quickstart.md:316-358; example Examples/DenseMonoLayer/
 * RunConfig.yaml:1-36).  Field names keep the YAML key names. */
typedef struct AlensConfig {
    double simBoxLow[3];
    double simBoxHigh[3];
    int32_t simBoxPBC[3];
    int32_t monolayer;               /* motion restricted to the x-y plane    */
    double viscosity;                /* pN s / um^2                           */
    double KBT;                      /* pN um; <= 0 disables Brownian noise   */
    double dt;                       /* s                                     */
    double sylinderDiameterColRatio; /* collision diameter / diameter         */
    double sylinderLengthColRatio;   /* collision length / length             */
    double sylinderColBuf;           /* record pairs with separation < this   */
    double conResTol;                /* BBPGD residual tolerance (um)         */
    int32_t conMaxIte;               /* BBPGD iteration cap                   */
    int32_t conSolverChoice;         /* 0 = BBPGD (the only solver here)      */
    uint64_t rngSeed;
    /* GPU-specific knobs (no counterpart in SylinderConfig) */
    int32_t precision;               /* AlensPrecision                        */
    int32_t warmStart;               /* AlensWarmStart                        */
    int32_t maxConstraints;          /* 0 = grow automatically; >0 = fixed
                                        capacity, overflow -> ALENS_CAPACITY  */
    int32_t useGraph;                /* 1 = replay the step as a CUDA graph   */
    int32_t stageTiming;             /* 1 = time each stage with CUDA events
                                        (direct launches, no graph)           */
    void *stream;                    /* cudaStream_t to run on; NULL = own    */
} AlensConfig;

/* One constraint block as the reference builds it in
 * TubuleSystem::setProteinConstraints (SRC/TubuleSystem.cpp:727-736),
 * fields in the constructor's argument order, plus the 3x3 stress of
 * setStress (:742).  Column of D for this block: rod I gets force normI and
 * torque posI x normI; rod J gets normJ and posJ x normJ (absent when
 * oneSide).  Bilateral blocks with kappa > 0 carry compliance 1/kappa. */
typedef struct AlensBlock {
    double delta0;       /* current separation (unilateral) or extension  */
    double gamma;        /* initial guess of the constraint force         */
    int64_t gidI, gidJ;
    int32_t globalIndexI, globalIndexJ; /* rod indices within the replica */
    double normI[3], normJ[3];
    double posI[3], posJ[3]; /* lever arms relative to the rod centres    */
    double labI[3], labJ[3]; /* lab-frame contact points (stress only)    */
    int32_t oneSide;
    int32_t bilateral;
    double kappa;
    double gammaLB;      /* lower bound of gamma for unilateral blocks    */
    double stress[9];
} AlensBlock;

/* Per-step statistics (the reference prints them through Teuchos timers,
 * SRC/TubuleSystem.cpp:148-167, and spdlog). */
typedef struct AlensStepStats {
    int64_t step;            /* step index this call executed              */
    int32_t nRods;
    int32_t nCollision;      /* collision constraints found                */
    int32_t nBilateral;      /* bilateral/user blocks in the solve         */
    int32_t iterations;      /* BBPGD iterations (max over replicas)       */
    int32_t refineIterations;/* FP64 refinement iterations (mixed mode)    */
    int32_t converged;       /* 1 if every replica reached conResTol       */
    int32_t status;          /* AlensStatus of the step                    */
    double residual;         /* final residual (max over replicas)         */
    int64_t constraintsNeeded; /* on ALENS_CAPACITY: capacity to retry with */
} AlensStepStats;

typedef struct AlensCtx AlensCtx;

/* Fill *cfg with the defaults of SylinderConfig for the keys above. */
void alens_config_default(AlensConfig *cfg);

/* Text of a status code. */
const char *alens_status_str(int status);

/* Message of the last failed call on this context (the failing CUDA call
 * and its error string for ALENS_CUDA_ERROR); "" when none.  The reference
 * reports such failures through exceptions and spdlog
 * (SRC/TubuleSystem.cpp:500,642). */
const char *alens_get_last_error(AlensCtx *ctx);

/* Create a context for one system (replaces SylinderSystem::initialize's
 * configuration part, SRC/TubuleSystem.cpp:79).  Returns ALENS_NO_DEVICE
 * when no CUDA device is usable. */
int alens_create(const AlensConfig *cfg, AlensCtx **out);

/* Create a context holding nReplica independent systems with their own
 * configurations (box, seed, tolerances); all replicas share precision,
 * warmStart, maxConstraints, useGraph and stream of cfgs[0].  No
 * counterpart in the reference, which runs one system per process. */
int alens_create_ensemble(const AlensConfig *cfgs, int nReplica,
                          AlensCtx **out);

int alens_destroy(AlensCtx *ctx);

/* Set the rods of one replica (replaces reading TubuleInitial.dat inside
 * SylinderSystem::initialize / reinitialize, SRC/TubuleSystem.cpp:38,79).
 * pos[3n], orientation[4n] as (x,y,z,w), length[n], radius[n] (physical),
 * gid[n], immovable[n] (nullable; 1 = 'S' stationary rod). */
int alens_set_rods(AlensCtx *ctx, int replica, int n, const int64_t *gid,
                   const double *pos, const double *orientation,
                   const double *length, const double *radius,
                   const int32_t *immovable);

/* Overwrite the positions and orientations of one replica (same layout as
 * alens_set_rods; the rod set is unchanged). */
int alens_update_rods(AlensCtx *ctx, int replica, int n, const double *pos,
                      const double *orientation);

/* Copy rod state back (what SylinderSystem::getContainer() exposes). */
int alens_get_rods(AlensCtx *ctx, int replica, int n, double *pos,
                   double *orientation);

/* Velocity of the last step: vel[3n], omega[3n] (total = known +
 * constraint). */
int alens_get_velocity(AlensCtx *ctx, int replica, int n, double *vel,
                       double *omega);

/* Queue blocks for the next alens_step of one replica.  Replaces appending
 * to rodSystem.getConstraintPoolNonConst()[tid]
 * (SRC/TubuleSystem.cpp:697-743).  The blocks are copied; the queue is
 * consumed (emptied) by the next step. */
int alens_add_bilateral(AlensCtx *ctx, int replica, int n,
                        const AlensBlock *blocks);

/* Pre-bound two-headed crosslinkers of one replica (the doubly-bound
 * proteins whose blocks TubuleSystem::setProteinConstraints builds on the
 * host every step, SRC/TubuleSystem.cpp:694-745).  Link k joins rod
 * indexI[k] at arc position sI[k] (um from the centre along the axis) and
 * rod indexJ[k] at sJ[k] with a spring of rest length restLength[k] and
 * stiffness kappa[k].  Every step the library builds each link's bilateral
 * block on the device from the current rod state (minimum image across
 * periodic boundaries), after the blocks queued by alens_add_bilateral.
 * Replaces the replica's link set; n = 0 removes it. */
int alens_set_links(AlensCtx *ctx, int replica, int n, const int32_t *indexI, const int32_t *indexJ,
                    const double *sI, const double *sJ, const double *restLength, const double *kappa);

/* Confinement boundaries of one replica (the role of SimToolbox's Boundary
 * objects listed under `boundaries:` in RunConfig.yaml,
 * Examples/DenseStrainingMotion/RunConfig.yaml:36-41, and projected on by
 * Boundary::project, SRC/TubuleSystem.cpp:285-305).  Every step, each rod
 * contact point within sylinderColBuf of a boundary becomes a one-sided
 * unilateral constraint (force along the boundary normal into the allowed
 * region, gamma >= 0) in the same solve as the collisions:
 *   wall   : plane through center with unit normal axis; allowed side +axis;
 *            contact points: both rod ends
 *   sphere : center, radius; inside = 1 keeps rods inside (both rod ends),
 *            inside = 0 keeps them outside (the rod point nearest center)
 *   tube   : infinite cylinder (center, axis, radius), inside = 1 only
 *            (both rod ends)
 * Spheres (length < 2 radius) have one contact point, the centre.  These
 * constraints are reported by alens_get_constraints among the collisions
 * with indexJ = -1 and image 27 (first point) or 28 (second point).
 * Up to ALENS_MAX_BOUNDARIES per replica; n = 0 removes them. */
#define ALENS_MAX_BOUNDARIES 8
typedef enum AlensBoundaryType {
    ALENS_BOUNDARY_WALL = 0,
    ALENS_BOUNDARY_SPHERE = 1,
    ALENS_BOUNDARY_TUBE = 2
} AlensBoundaryType;

typedef struct AlensBoundary {
    int32_t type;       /* AlensBoundaryType                              */
    int32_t inside;     /* sphere/tube: 1 keep inside, 0 keep outside     */
    double center[3];   /* um                                             */
    double axis[3];     /* tube axis or wall normal (normalised here)     */
    double radius;      /* sphere/tube radius (um)                        */
} AlensBoundary;

int alens_set_boundaries(AlensCtx *ctx, int replica, int n, const AlensBoundary *boundaries);

/* One full step (replaces SylinderSystem::runStep, SRC/TubuleSystem.cpp:223).
 * Returns ALENS_OK, ALENS_NOT_CONVERGED (step completed with the last
 * iterate), or an error; *stats (nullable) receives the summary. */
int alens_step(AlensCtx *ctx, AlensStepStats *stats);

/* Step several contexts together (the batched call SURVEY's boundary names
 * for replicas kept in separate contexts; replicas in one context are
 * stepped together by alens_step already, see alens_create_ensemble).
 * Every context's step is enqueued on its own stream before any result is
 * read back, so steps on different streams run concurrently; a context
 * whose step must be repeated (buffer regrowth) repeats it alone.  stats
 * (nullable) receives n entries.  Returns the first status that is neither
 * ALENS_OK nor ALENS_NOT_CONVERGED, else ALENS_NOT_CONVERGED if any step
 * hit the cap, else ALENS_OK.  Replaces n calls of SylinderSystem::runStep
 * (SRC/TubuleSystem.cpp:223). */
int alens_step_batched(AlensCtx **ctxs, int n, AlensStepStats *stats);

/* The three parts of alens_step, for staged use and testing:
 * detect = known velocity + pair search + constraint assembly,
 * solve = BBPGD, advance = velocity write-back + Euler update
 * (SylinderSystem::stepEuler, SRC/TubuleSystem.cpp:55). */
int alens_detect(AlensCtx *ctx, AlensStepStats *stats);
int alens_solve(AlensCtx *ctx, AlensStepStats *stats);
int alens_advance(AlensCtx *ctx, AlensStepStats *stats);

/* Per-replica statistics of the last step. */
int alens_get_replica_stats(AlensCtx *ctx, int replica,
                            AlensStepStats *stats);

/* Constraint count of one replica after detect: collisions then blocks. */
int alens_get_num_constraints(AlensCtx *ctx, int replica, int *nCollision,
                              int *nBilateral);

/* Constraints of one replica in canonical order: collisions sorted by
 * (indexI, indexJ, image) with indexI <= indexJ, then queued blocks in
 * queue order.  Any pointer may be NULL.  image = (sx+1)*9+(sy+1)*3+(sz+1)
 * for the periodic shift applied to rod J (13 = none; -1 for blocks).
 * jac[12*k] = (normI, posI x normI, normJ, posJ x normJ). */
int alens_get_constraints(AlensCtx *ctx, int replica, int cap,
                          int32_t *indexI, int32_t *indexJ, int32_t *image,
                          double *delta0, double *gamma, double *jac);

/* The Delassus operator A = dt D^T M D of one replica after detect (the
 * operator SimToolbox's ConstraintOperator applies, CMakeLists.txt:111), in
 * CSR form over the replica's constraints (canonical order, local column
 * indices), with the vectors of the QP min 1/2 x^T (A + diag(cinv)) x + q^T x,
 * x >= lowerBound (-inf on bilateral rows).  gamma0 receives the current
 * gamma: the initial guess after alens_detect, the solution after
 * alens_solve.  Pass NULL for any output that is not wanted;
 * *nnz receives the number of nonzeros; ALENS_CAPACITY if capNnz is too
 * small for cols/vals. */
int alens_get_operator(AlensCtx *ctx, int replica, int capNnz, int *nnz, int32_t *rowPtr,
                       int32_t *cols, double *vals, double *q, double *cinv,
                       double *lowerBound, double *gamma0);

/* The multipliers of one replica's constraints after a solve, with the rod
 * pair of each (pairs[2k], pairs[2k+1] = indexI, indexJ), canonical order
 * as alens_get_constraints: the gamma a ConstraintBlock holds after
 * runStep (SRC/TubuleSystem.cpp:697-743 reads the pool).  *n receives the
 * count; ALENS_CAPACITY if cap < *n.  pairs and gamma may be NULL. */
int alens_get_gamma(AlensCtx *ctx, int replica, int cap, int *n, int32_t *pairs, double *gamma);

/* The collision constraints of one replica after detect (the near-pair
 * search's result: rod pairs with separation below sylinderColBuf, with the
 * periodic image of rod J, and boundary contacts with indexJ = -1), sorted by
 * (indexI, indexJ, image).  *n receives the count; ALENS_CAPACITY if
 * cap < *n.  Any array may be NULL.  The role of the pair list SimToolbox's
 * near-pair search hands to CalcSylinderNearForce (Protein/ProteinData.hpp:25). */
int alens_get_pairs(AlensCtx *ctx, int replica, int cap, int *n, int32_t *indexI, int32_t *indexJ,
                    int32_t *image);

/* Lab-frame contact points of one replica's constraints, canonical order:
 * lab[6k .. 6k+2] = point on rod I, lab[6k+3 .. 6k+5] = point on rod J (for
 * boundary contacts, the point on the boundary surface).  The labI / labJ
 * fields of the ConstraintBlocks (SRC/TubuleSystem.cpp:727-736) that the
 * ConBlock_<id>.pvtp snapshots draw (README.md:142).  ALENS_CAPACITY if
 * cap is below the constraint count. */
int alens_get_constraint_points(AlensCtx *ctx, int replica, int cap, double *lab);

/* Sum over the constraints of one replica of the pair virial
 * gamma * (lab_I - lab_J) (x) n  (3x3 row-major); the role of
 * SylinderSystem::calcConStress (SRC/TubuleSystem.cpp:224). */
int alens_get_con_stress(AlensCtx *ctx, int replica, double *stress9);

/* BBPGD solve that allocates no memory, for callers that cannot call
 * cudaMalloc where they solve: a host code whose GPU memory is all owned by
 * another allocator (a framework's caching pool, a fixed budget), or a time
 * loop that must not stall the device (cudaMalloc/cudaFree may synchronise
 * it).  No counterpart in the reference: SimToolbox's solver allocates its
 * Tpetra vectors per solve.
 * Solves min 1/2 x^T (A + diag(cinv)) x + q^T x, x >= lowerBound (-inf for
 * bilateral rows) with the library's FP64 BBPGD, starting from gamma0; all
 * array arguments are DEVICE pointers to the caller's memory: A as CSR
 * (rowPtr[n+1] with rowPtr[0] = 0, cols with every column in [0, n), vals;
 * the layout alens_get_operator returns), q, cinv, lowerBound, gamma0 and
 * the output gamma (n each).  An entry with a column outside [0, n) is
 * skipped and the call returns ALENS_INVALID_ARG.  iterations, residual and
 * solveStatus (nullable) are host pointers; before returning, the call
 * waits for `stream` (NULL: the default stream) and copies them there.
 * Scratch lives in one fixed __device__ array of about 2.1 MB per GPU that
 * loads the library: n is limited to 65,536 rows (larger: ALENS_INVALID_ARG).
 * The first call on a device looks up the array's address and keeps it for
 * the life of the process (cudaDeviceReset afterwards is not supported).
 * Calls share the array: calls that overlap on the GPU race.  Returns the
 * solve's status (ALENS_OK or ALENS_NOT_CONVERGED) or an error. */
int alens_bbpgd_solve_noalloc(int n, const int32_t *rowPtr, const int32_t *cols,
                              const double *vals, const double *q,
                              const double *cinv, const double *lowerBound,
                              const double *gamma0, double *gamma, double tol,
                              int maxIte, void *stream, int *iterations,
                              double *residual, int *solveStatus);

/* ---- Learned warm start ------------------------------------------------
 * A 12 -> 64 -> 64 -> 1 SiLU network (BF16 weights, FP32 accumulation on
 * the tensor cores) that predicts each collision constraint's initial
 * multiplier for BBPGD.  SimToolbox's solver starts from the gamma stored
 * in each ConstraintBlock (SRC/TubuleSystem.cpp:727-736, zero for
 * collisions); with warmStart = ALENS_WARM_MLP and a model attached, the
 * network supplies that start instead.  The solve still has to reach
 * conResTol, so the prediction changes iteration counts, never the
 * tolerance of the answer.  No counterpart in the reference.
 *
 * Features (per collision constraint, FP32): current separation, predicted
 * end-of-step overlap and signed separation (from q = phi0 + dt D^T U), the
 * cosine of the rod axes, both rod lengths, the contact parameters s/h_I
 * and t/h_J, the constraint counts of both rods, the previous step's
 * multiplier of the same pair and image, and the coupling-weighted
 * predicted overlap of the neighbouring constraints; lengths in units of
 * the pair's collision diameter, multipliers in "overlap units"
 * u = gamma * A_kk / d (A_kk = diagonal of the Delassus operator).
 * Parameters (ALENS_MLP_NUM_PARAMS floats): W1[64][12], b1[64],
 * W2[64][64], b2[64], w3[64], b3, weights stored [out][in]. */
#define ALENS_MLP_NUM_FEATURES 12
#define ALENS_MLP_NUM_PARAMS 5057

typedef struct AlensMlp AlensMlp;

/* Model with seeded initial weights and room for datasetCapacity
 * (feature, target) rows on the device. */
int alens_mlp_create(uint64_t seed, int64_t datasetCapacity, AlensMlp **out);
int alens_mlp_destroy(AlensMlp *mlp);
/* FP32 master parameters (host arrays of ALENS_MLP_NUM_PARAMS floats);
 * set also resets the Adam state. */
int alens_mlp_get_params(AlensMlp *mlp, float *params);
int alens_mlp_set_params(AlensMlp *mlp, const float *params);
/* Dataset: rows added from host arrays (features[n*12], targets[n] in
 * overlap units), current size, clear. */
int alens_mlp_add_samples(AlensMlp *mlp, int n, const float *features, const float *targets);
int alens_mlp_dataset_size(AlensMlp *mlp, int64_t *n);
int alens_mlp_clear_dataset(AlensMlp *mlp);
/* Adam (beta 0.9/0.999, eps 1e-8) on the mean squared error over the
 * dataset, `epochs` passes in a seeded random order, minibatches of
 * `batch` rows; lossPerEpoch[epochs] (nullable) receives each pass's mean
 * loss.  Forward, backward and the update run in the library's kernels. */
int alens_mlp_train(AlensMlp *mlp, int epochs, int batch, float lr, uint64_t seed, float *lossPerEpoch);
/* Network outputs for n feature rows (host arrays). */
int alens_mlp_predict(AlensMlp *mlp, int n, const float *features, float *out);
/* Gradient of the mean squared error over n rows with respect to every
 * parameter (grad[ALENS_MLP_NUM_PARAMS]) and the loss; no update. */
int alens_mlp_gradient(AlensMlp *mlp, int n, const float *features, const float *targets, float *grad,
                       float *loss);
/* Use `mlp` (NULL detaches) for the warm start of this context's steps when
 * warmStart = ALENS_WARM_MLP.  The model must outlive its attachment;
 * training it while attached is allowed between steps. */
int alens_attach_mlp(AlensCtx *ctx, AlensMlp *mlp);
/* Record the features of every constraint during each step (needed by
 * alens_mlp_collect and alens_get_features). */
int alens_set_feature_capture(AlensCtx *ctx, int enable);
/* Append the last step's collision constraints of every replica to the
 * model's dataset: features and the converged multiplier in overlap units
 * (stops at the dataset capacity); *added (nullable) receives the rows. */
int alens_mlp_collect(AlensCtx *ctx, AlensMlp *mlp, int64_t *added);
/* Features (features[12*n]) and overlap-unit scale A_kk/d (scale[n]) of the
 * last step's collision constraints of one replica, canonical order;
 * *n receives the count; ALENS_CAPACITY if cap < n. */
int alens_get_features(AlensCtx *ctx, int replica, int cap, float *features, float *scale, int *n);

/* Bounded device waits (no counterpart in the reference).  Every grid-wide
 * wait of the solver gives up after timeoutNs (0 = the default, 2 s), sets
 * ALENS_TIMEOUT and leaves the rods unmoved.  stallBarriers = 1 makes the
 * solver's grid barriers wait for one block more than the launch holds, so
 * that every such wait of the following steps runs out: a test of the
 * timeout path that faults nothing (the context stays usable); 0 restores
 * normal operation.  Not between alens_detect and alens_advance
 * (ALENS_NOT_READY). */
int alens_set_wait_limit(AlensCtx *ctx, uint64_t timeoutNs, int stallBarriers);

/* Steps executed so far (SylinderSystem::getStepCount). */
int alens_get_step_count(AlensCtx *ctx, int64_t *count);

/* Set the step count, i.e. the index of the next step, for a restart
 * (SylinderSystem::reinitialize from TimeStepInfo.txt, SRC/TubuleSystem.cpp:38).
 * The step index keys the Brownian noise, so a context restarted at step s
 * draws the noise an uninterrupted run draws from step s on.  count >= 0
 * (else ALENS_INVALID_ARG); not between alens_detect and alens_advance
 * (ALENS_NOT_READY). */
int alens_set_step_count(AlensCtx *ctx, int64_t count);

/* The CUDA stream of the context (cudaStream_t), for event timing. */
int alens_get_stream(AlensCtx *ctx, void **stream);

/* Kernels launched by this context so far (graph replays included).  The
 * role of the reference's per-phase Teuchos counters
 * (SRC/TubuleSystem.cpp:148-167) for device work. */
int alens_get_launch_count(AlensCtx *ctx, int64_t *count);

/* Project autotuner (no counterpart in the reference): detects the next
 * step's constraints, times every applicable configuration of the solver on
 * that problem (grid form with 1 or 2 blocks per SM and at least 1, 2, 4 or
 * 8 64-row tiles per block; for the mixed precision also the cluster forms
 * with 2-16 CTAs per cluster and 256 or 512 threads per CTA), each `reps`
 * times from the same initial iterate, and keeps the fastest for the
 * following steps.  The rods do not move.  report (nullable, reportCap
 * bytes) receives a JSON text with every candidate's median solve time and
 * the index of the chosen one.  The environment variables
 * ALENS_SOLVER_FORM (grid | cluster | resident), ALENS_SOLVER_BLOCKS_PER_SM,
 * ALENS_SOLVER_MIN_TILES, ALENS_CLUSTER_SIZE and ALENS_CSM_THREADS set the
 * same choices by hand when a context is created. */
int alens_autotune(AlensCtx *ctx, int reps, char *report, int reportCap);

/* ------------------------------------------------------------------------
 * Protein binding kinetics (the two-stage KMC model: unbound U, singly
 * bound S, doubly bound D; Protein/ProteinModel.md "The Binding/Unbinding
 * probabilities and rates in KMC").
 * ---------------------------------------------------------------------- */

/* One protein species.  Replaces ProteinType (Protein/ProteinType.hpp:24-76)
 * as read by ProteinType::readFromYaml (:81-129): the same YAML keys, in the
 * same units (um, pN, s; Ka in (uM)^-1; Ke in (uM)^-1 when useBindVol, else
 * a number per binding site).  The library applies readFromYaml's
 * conversion (Ka /= 602, Ke /= 602 when useBindVol) and, for fixedEnd0, the
 * rule of Protein/ProteinModel.md ("When fixedEnd0==true": ko_s[0] =
 * ko_d[0] = 0).  lookupType 0: stretch = head distance - rod diameter D;
 * lookupType 1: stretch = (1 - D/d) x head distance, d the distance of the
 * bound head from the other rod's axis (Protein/ProteinData.hpp:171-195);
 * other values are rejected.  The motion fields (walkOff, vdrag, fstall,
 * vmax, vmaxAP, diffBoundS, diffBoundD) are used by
 * alens_protein_motion_step; diffUnbound by both steps. */
typedef struct AlensProteinType {
    int32_t tag;
    int32_t fixedEnd0;
    int32_t useBindVol;
    int32_t lookupType;   /* 0 or 1 */
    double freeLength;    /* rest length ell0, um */
    double kappa;         /* spring constant, pN/um */
    double lambda;        /* unbinding load sensitivity */
    double PtoAPratio;    /* parallel / antiparallel S->D binding ratio */
    double diffUnbound;   /* um^2/s, sets the capture radius floor */
    double rc;            /* capture radius, um */
    double eps;           /* binding sites per um of rod */
    double ko_s[2], ko_d[2], Ka[2], Ke[2];
    /* motion (Protein/ProteinType.hpp:30-52) */
    int32_t walkOff;      /* 1: a head that walks past a rod end unbinds; 0: clamped */
    int32_t vdrag[2];     /* 1: a doubly bound head is also dragged by its load */
    int32_t pad2;
    double fstall;        /* stall force, pN */
    double vmax[2];       /* walking speed per head, um/s, + towards the plus end */
    double vmaxAP[2];     /* walking speed on antiparallel rods (doubly bound) */
    double diffBoundS[2]; /* head diffusivity when singly bound, um^2/s */
    double diffBoundD[2]; /* head diffusivity when doubly bound, um^2/s */
} AlensProteinType;

/* One protein (the binding part of ProteinData / ProteinBindStatus,
 * Protein/ProteinBindStatus.hpp:35-85).  idBind[e] is the index (within the
 * replica) of the rod head e is bound to, or -1 (ID_UB); distBind[e] is the
 * head's distance from that rod's centre along its axis, in
 * [-length/2, length/2].  pos is the protein centre: the free point of an
 * unbound protein (input and output), the bound head of a singly bound one
 * and the midpoint of the heads of a doubly bound one (output).  posEnd[e]
 * is head e's lab-frame position (output; NaN when unbound). */
typedef struct AlensProtein {
    int64_t gid;
    int32_t type;         /* index into the species table */
    int32_t idBind[2];
    int32_t pad;
    double distBind[2];
    double pos[3];
    double posEnd[2][3];
} AlensProtein;

/* Counts of one replica after a binding step: proteins per stage and the
 * transitions taken in the step. */
typedef struct AlensKmcStats {
    int32_t nU, nS, nD;
    int32_t nUS, nSU, nSD, nDS;
    int32_t maxCandidates;  /* most rods any protein could bind to this step */
} AlensKmcStats;

/* The species table of the context (all replicas) with the protein
 * temperature KBT (ProteinConfig KBT, pN um) and the rod diameter D
 * (RunConfig sylinderDiameter, um) that the binding rates use.  Replaces
 * ProteinConfig's type list (Protein/ProteinConfig.cpp:6-45) and
 * TubuleSystem::buildLookupTable (SRC/TubuleSystem.cpp:583-629): the S->D
 * binding integral is evaluated by quadrature, not tabulated.  Invalidates
 * no protein; proteins must refer to existing types at the next step. */
int alens_set_protein_types(AlensCtx *ctx, int n, const AlensProteinType *types, double KBT,
                            double rodDiameter);

/* The proteins of one replica (TubuleSystem::setInitialProteinFromFile /
 * readProteinVTK, SRC/TubuleSystem.cpp:761-872).  Bound heads must name a
 * rod of the replica (ALENS_INVALID_ARG otherwise); pos of a bound protein
 * is recomputed from its heads.  Doubly bound proteins are bilateral
 * springs of the next step (stiffness kappa; rest length freeLength +
 * rodDiameter, or for lookupType 1 the length whose difference from the
 * head distance is that type's stretch at the geometry when the springs are
 * built: by this call, alens_set_protein_types, alens_set_rods,
 * alens_set_links and each binding step), after the replica's
 * alens_set_links links.  n = 0 removes them. */
int alens_set_proteins(AlensCtx *ctx, int replica, int n, const AlensProtein *proteins);

/* The current proteins of one replica, in the order they were set.  cap too
 * small: ALENS_CAPACITY with *n set. */
int alens_get_proteins(AlensCtx *ctx, int replica, int cap, int *n, AlensProtein *proteins);

/* One KMC binding step of every protein of every replica on the current rod
 * state: U -> S, S -> U, S -> D and D -> S with the rates of
 * Protein/ProteinModel.md, one event at most per protein (the choice rule
 * of SRC/kmc_step_funcs.hpp:35-230), then the doubly bound proteins become
 * the replica's protein springs for the next alens_step.  Replaces
 * TubuleSystem::calcBindInteraction + setProteinConstraints
 * (SRC/TubuleSystem.cpp:232-259, 694-745) and CalcProteinBind::operator()
 * (SRC/CalcProteinBind.hpp:59-173).  The random numbers are Philox4x32-10
 * keyed by (rngSeed, protein gid, step count), so a step is reproducible
 * and independent of the device.  stats (nullable) receives one record per
 * replica.  Not between alens_detect and alens_advance (ALENS_NOT_READY). */
int alens_protein_bind_step(AlensCtx *ctx, AlensKmcStats *stats);

/* One motion step of every protein of every replica on the current rod
 * state (TubuleSystem::updateProteinMotion, SRC/TubuleSystem.cpp:261-306,
 * with ProteinData::updatePosWalk / updatePosDiffuse,
 * Protein/ProteinData.hpp:318-406): unbound proteins diffuse with
 * diffUnbound and are projected back onto the replica's boundaries when
 * outside; bound heads walk (vmax, or vmaxAP on antiparallel rods, slowed
 * linearly by the spring load towards fstall, Protein/ProteinData.hpp:459-478),
 * are dragged by the load when vdrag (:489-498) and diffuse along the rod;
 * a head past a rod end unbinds (walkOff; both past: one of them, chosen by
 * the roll) or is clamped to the end.  Philox rolls keyed by (rngSeed,
 * protein gid, step count), distinct from the binding step's.  stats
 * (nullable, one per replica): stages after the motion, nSU and nDS count
 * walk-offs.  The springs of doubly bound proteins are rebuilt.  aLENS calls
 * it before the binding step (SRC/TubuleSystem.cpp:185-189). */
int alens_protein_motion_step(AlensCtx *ctx, AlensKmcStats *stats);

/* CUDA-event times (ms) of the stages of the last step when stageTiming is
 * on: ms[0] detect, ms[1] main solve kernel (FP32 kernel in mixed mode),
 * ms[2] FP64 refinement (mixed mode; 0 otherwise), ms[3] advance,
 * ms[4] whole step.  The stage split of TubuleSystem's step timers
 * (SRC/TubuleSystem.cpp:148-167). */
int alens_get_stage_times(AlensCtx *ctx, double *ms5);

#ifdef __cplusplus
}
#endif

#endif /* ALENS_GPU_H */
