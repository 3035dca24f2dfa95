// engine.h - host-side context of the GPU rod step (one CUDA stream).
#pragma once

#include <cstdlib>
#include <string>
#include <vector>

#include "engine.cuh"
#include "kmc.cuh"
#include "mlp.h"

namespace alens {

// the three-pass scan covers up to 4096 x 1024 elements
constexpr int kMaxConstraints = 4096 * 1024;

struct ApiError {
    int status;
    explicit ApiError(int s) : status(s) {}
};

struct CudaFailure {
    cudaError_t err;
    const char *where;
    CudaFailure(cudaError_t e, const char *w) : err(e), where(w) {}
};

class Engine {
  public:
    Engine(const AlensConfig *cfgs, int nrep);
    ~Engine();
    Engine(const Engine &) = delete;
    Engine &operator=(const Engine &) = delete;

    void setRods(int rep, int n, const int64_t *gid, const double *pos, const double *quat,
                 const double *len, const double *rad, const int32_t *imm);
    void updateRods(int rep, int n, const double *pos, const double *quat);
    void getRods(int rep, int n, double *pos, double *quat);
    void getVelocity(int rep, int n, double *vel, double *omega);
    void addBilateral(int rep, int n, const AlensBlock *blocks);
    void setLinks(int rep, int n, const int32_t *idxI, const int32_t *idxJ, const double *sI, const double *sJ,
                  const double *rest, const double *kappa);
    void setBoundaries(int rep, int n, const AlensBoundary *b);
    int step(AlensStepStats *out);
    // the two halves of a step attempt, for stepping several contexts
    // together (alens_step_batched): stepLaunch enqueues, stepFinish reads
    // back and returns kStepRetry when the attempt must be repeated
    static constexpr int kStepRetry = -1000;
    bool stepLaunch();
    int stepFinish(AlensStepStats *out, bool direct);
    void finalizeForStep() { finalize(); }
    // bounded device waits: grid-barrier limit (0 = default) and the
    // barrier stall used to test the timeout path
    void setWaitLimit(unsigned long long timeoutNs, int stallBarriers);
    void getConstraintPoints(int rep, int cap, double *lab);
    // protein binding kinetics (engine_kmc.cu)
    void setProteinTypes(int n, const AlensProteinType *types, double KBT, double D);
    void setProteins(int rep, int n, const AlensProtein *p);
    void getProteins(int rep, int cap, int *n, AlensProtein *out);
    int proteinBindStep(AlensKmcStats *stats);
    int proteinMotionStep(AlensKmcStats *stats);
    int detect(AlensStepStats *out);
    int solve(AlensStepStats *out);
    int advance(AlensStepStats *out);
    void replicaStats(int rep, AlensStepStats *out) const;
    void numConstraints(int rep, int *nColl, int *nBil) const;
    void getConstraints(int rep, int cap, int32_t *ii, int32_t *jj, int32_t *img, double *d0,
                        double *gam, double *jac);
    void conStress(int rep, double *out9);
    void getOperator(int rep, int capNnz, int *nnz, int32_t *rowPtr, int32_t *cols, double *vals,
                     double *q, double *cinv, double *lowerBound, double *gamma0);
    // learned warm start (kernels_mlp.cu): the attached model seeds the
    // collision multipliers when warmStart == ALENS_WARM_MLP; with feature
    // capture on, every step records the features of its constraints
    void attachMlp(MlpModel *m);
    void setFeatureCapture(bool on);
    long long collect(MlpModel *m);
    int getFeatures(int rep, int cap, float *feat, float *scale);
    // Times the solver configurations on this step's detected problem and
    // keeps the fastest; returns a JSON report.  The rods do not move.
    std::string autotune(int reps);
    long long stepCount() const { return stepCount_; }
    // Index of the next step (it keys the Brownian noise); not while a
    // staged step is pending
    void setStepCount(long long s);
    cudaStream_t stream() const { return stream_; }
    long long lastNeeded() const { return lastNeeded_; }
    long long launches() const { return launches_; }
    const double *stageMs() const { return stageMs_; }
    const DevState &state() const { return S_; }
    int replicas() const { return R_; }

  private:
    struct HostRods {
        int n = 0;
        bool set = false;
        double hlMax = 0.0;  // largest half-length
        std::vector<long long> gid;
        std::vector<double> pos, quat, len, rad;
        std::vector<int> imm;
    };

    void makeParams(int rep, const HostRods &h, RepParams &P) const;
    void finalize();
    void allocConstraints(int cap, bool keepPrev);
    void allocOperator(long long nnz);
    void uploadBlocks();
    int enqueueDetect();
    // finish: copy the solution into gamma (a full step leaves it to the update)
    int enqueueSolve(cudaEvent_t *ev, bool finish = false);
    void ensureSolverGrid();
    int enqueueAdvance();
    void ensureEvents();
    void recordStageTimes();
    bool buildGraph();
    void invalidateGraph();
    void readBack();
    bool handleOverflow();
    bool handleSolverFit();
    void applySolverConfig(int form, int clusterSize, int threads, int blocksPerSM, int minTiles = 1);
    int collectStats(int stage);
    void freeGroup(std::vector<void *> &g);
    template <class T>
    T *alloc(std::vector<void *> &group, size_t n);

    std::vector<AlensConfig> cfg_;
    int R_ = 0;
    int device_ = 0, numSM_ = 0;
    cudaStream_t stream_ = nullptr;
    cudaStream_t side_ = nullptr;  // concurrent branch of the detect stage
    cudaStream_t side2_ = nullptr; // the single-system solver's row order, beside the assembly
    cudaStream_t side3_ = nullptr; // the learned warm start, beside the assembly
    cudaEvent_t orderJoin_ = nullptr, orderFork_ = nullptr;
    cudaEvent_t rowsDone_ = nullptr, weightsDone_ = nullptr, warmJoin_ = nullptr;
    cudaEvent_t forkEv_[3] = {nullptr, nullptr, nullptr}, joinEv_[3] = {nullptr, nullptr, nullptr};
    bool ownStream_ = false;
    int precision_ = 0, warm_ = 0;
    bool useGraph_ = true, graphFailed_ = false;
    int fixedCap_ = 0;
    int solverBlocksPerSM_ = 1;
    int solverMinTiles_ = 1;  // at least this many tiles per grid-form solver block
    int clusterSize_ = -1;   // FP32 solver: -1 automatic, 0 grid form, N cluster size
    int nClusters_ = 1;
    int solverForm_ = -1;    // SolverForm of the FP32 solver (-1: not chosen yet)
    int formRequest_ = -1;   // ALENS_SOLVER_FORM override (-1 automatic)
    bool residentFailed_ = false;  // a step did not fit the cluster-resident form
    bool fastFailed_ = false;      // a step did not fit the single-system form
    unsigned long long waitTimeoutNs_ = 2000000000ULL;  // grid-barrier wait limit (2 s)
    int stallBarriers_ = 0;                             // 1: barriers wait for one block more (tests)
    int prevCountHost_ = 0;  // valid warm-start keys on the device
    int solverGrid_ = 0;
    MlpModel *mlp_ = nullptr;
    bool capture_ = false;
    bool captured_ = false;  // the last completed step recorded its features
    std::vector<HostRods> rods_;
    std::vector<std::vector<AlensBlock>> queue_;
    struct HostLinks {
        std::vector<int> I, J;
        std::vector<double> sI, sJ, rest, kappa;
    };
    std::vector<HostLinks> links_;
    bool linksDirty_ = false;
    std::vector<std::vector<BoundaryDev>> bnd_;  // per replica, unit axes
    bool bndDirty_ = false;
    std::vector<void *> bndAllocs_;
    void uploadBoundaries();
    std::vector<void *> linkAllocs_;
    int *hLinkSlot0_ = nullptr;
    int userLinkTotal_ = 0;  // rows of alens_set_links links (all replicas)
    int linkCap_ = 0;        // link rows allocated: user links + one per protein
    void uploadLinks();
    // proteins: host copies per replica, the device state, and the springs
    // (doubly bound proteins) written after the user links
    std::vector<AlensProteinType> ptypes_;
    double kmcKBT_ = 0.0, kmcD_ = 0.0;
    std::vector<std::vector<AlensProtein>> prot_;
    bool protUpload_ = false;    // the host copies are newer than the device
    bool protDevNewer_ = false;  // bind steps advanced the device past the host copies
    bool springsDirty_ = false;  // the spring rows must be written again
    std::vector<int> springs_;   // spring rows per replica
    int nProt_ = 0;
    KmcDev K_{};
    std::vector<void *> protAllocs_, kmcAllocs_, kmcFixedAllocs_;
    int kmcCellCap_ = 0, kmcRodCap_ = 0, kmcTypeCap_ = 0;
    int *hKmc_ = nullptr;        // pinned: 8 x R stats, R spring counts, error flags
    std::vector<KmcType> kmcTypesUp_;  // the species and replica tables on the device
    std::vector<KmcRep> kmcRepsUp_;
    void uploadProteins();
    void syncProteinsToHost();
    void prepareKmc();
    void rebuildSprings();
    void readSprings(AlensKmcStats *stats);
    std::vector<RepParams> hostPar_;
    bool dirty_ = true;
    bool haveDetect_ = false, haveSolve_ = false;
    DevState S_{};
    std::vector<void *> rodAllocs_, conAllocs_, blockAllocs_, fixedAllocs_, opAllocs_;
    long long nnzCap_ = 0;
    int blockCap_ = 0;
    int nBilQueued_ = 0;
    AlensBlock *hBlocks_ = nullptr;
    int *hBlockRep_ = nullptr;
    DevCtl *hCtl_ = nullptr;
    RepDyn *hDyn_ = nullptr;
    int *hBilPrefix_ = nullptr;
    cudaGraphExec_t graphExec_ = nullptr;
    int graphLaunches_ = 0;
    long long launches_ = 0;
    bool stageTiming_ = false;
    cudaEvent_t events_[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    double stageMs_[5] = {0, 0, 0, 0, 0};
    long long stepCount_ = 0;
    long long lastNeeded_ = 0;
    AlensStepStats last_{};
    std::vector<AlensStepStats> repStats_;
};

}  // namespace alens
