// capi.cu - the C ABI of include/alens_gpu.h.  Every entry point converts
// exceptions into status codes; nothing crosses the ABI as a C++ exception.
#include <algorithm>
#include <cstring>
#include <new>
#include <vector>

#include "engine.h"

#include <string>

struct AlensCtx {
    alens::Engine *eng;
    std::string lastError;
};

struct AlensMlp {
    alens::MlpModel *model;
};

namespace {

template <class F>
int guarded_ctx(AlensCtx *ctx, F &&f) {
    try {
        const int rc = f();
        return rc;
    } catch (const alens::ApiError &e) {
        if (ctx) ctx->lastError = alens_status_str(e.status);
        return e.status;
    } catch (const alens::CudaFailure &e) {
        if (ctx) ctx->lastError = std::string(e.where) + ": " + cudaGetErrorString(e.err);
        cudaGetLastError();
        return ALENS_CUDA_ERROR;
    } catch (const std::bad_alloc &) {
        if (ctx) ctx->lastError = "host allocation failed";
        return ALENS_CUDA_ERROR;
    } catch (...) {
        if (ctx) ctx->lastError = "unknown exception";
        return ALENS_CUDA_ERROR;
    }
}

template <class F>
int guarded(F &&f) {
    return guarded_ctx(nullptr, f);
}

}  // namespace

extern "C" {

void alens_config_default(AlensConfig *c) {
    if (!c) return;
    std::memset(c, 0, sizeof(*c));
    for (int d = 0; d < 3; d++) {
        c->simBoxLow[d] = 0.0;
        c->simBoxHigh[d] = 1.0;
        c->simBoxPBC[d] = 0;
    }
    c->monolayer = 0;
    c->viscosity = 0.01;
    c->KBT = 0.00411;
    c->dt = 1e-4;
    c->sylinderDiameterColRatio = 1.0;
    c->sylinderLengthColRatio = 1.0;
    c->sylinderColBuf = 0.025;
    c->conResTol = 1e-5;
    c->conMaxIte = 2000;
    c->conSolverChoice = 0;
    c->rngSeed = 1234;
    c->precision = ALENS_PREC_FP64;
    c->warmStart = ALENS_WARM_ZERO;
    c->maxConstraints = 0;
    c->useGraph = 1;
    c->stageTiming = 0;
    c->stream = nullptr;
}

const char *alens_status_str(int s) {
    switch (s) {
        case ALENS_OK: return "ok";
        case ALENS_INVALID_ARG: return "invalid argument";
        case ALENS_CUDA_ERROR: return "CUDA error";
        case ALENS_NOT_CONVERGED: return "BBPGD did not converge";
        case ALENS_CAPACITY: return "constraint capacity exceeded";
        case ALENS_TIMEOUT: return "device wait timed out";
        case ALENS_NAN_DETECTED: return "NaN or Inf detected";
        case ALENS_NO_DEVICE: return "no CUDA device";
        case ALENS_NOT_READY: return "call order violated";
        default: return "unknown status";
    }
}

int alens_create(const AlensConfig *cfg, AlensCtx **out) { return alens_create_ensemble(cfg, 1, out); }

int alens_create_ensemble(const AlensConfig *cfgs, int nReplica, AlensCtx **out) {
    if (!cfgs || !out || nReplica < 1) return ALENS_INVALID_ARG;
    *out = nullptr;
    return guarded([&] {
        AlensCtx *c = new AlensCtx{new alens::Engine(cfgs, nReplica), std::string()};
        *out = c;
        return (int)ALENS_OK;
    });
}

int alens_destroy(AlensCtx *ctx) {
    if (!ctx) return ALENS_INVALID_ARG;
    return guarded([&] {
        delete ctx->eng;
        delete ctx;
        return (int)ALENS_OK;
    });
}

int alens_set_rods(AlensCtx *ctx, int replica, int n, const int64_t *gid, const double *pos,
                   const double *orientation, const double *length, const double *radius,
                   const int32_t *immovable) {
    if (!ctx) return ALENS_INVALID_ARG;
    return guarded_ctx(ctx, [&] {
        ctx->eng->setRods(replica, n, gid, pos, orientation, length, radius, immovable);
        return (int)ALENS_OK;
    });
}

int alens_update_rods(AlensCtx *ctx, int replica, int n, const double *pos, const double *orientation) {
    if (!ctx) return ALENS_INVALID_ARG;
    return guarded_ctx(ctx, [&] {
        ctx->eng->updateRods(replica, n, pos, orientation);
        return (int)ALENS_OK;
    });
}

int alens_get_rods(AlensCtx *ctx, int replica, int n, double *pos, double *orientation) {
    if (!ctx) return ALENS_INVALID_ARG;
    return guarded_ctx(ctx, [&] {
        ctx->eng->getRods(replica, n, pos, orientation);
        return (int)ALENS_OK;
    });
}

int alens_get_velocity(AlensCtx *ctx, int replica, int n, double *vel, double *omega) {
    if (!ctx) return ALENS_INVALID_ARG;
    return guarded_ctx(ctx, [&] {
        ctx->eng->getVelocity(replica, n, vel, omega);
        return (int)ALENS_OK;
    });
}

int alens_add_bilateral(AlensCtx *ctx, int replica, int n, const AlensBlock *blocks) {
    if (!ctx) return ALENS_INVALID_ARG;
    return guarded_ctx(ctx, [&] {
        ctx->eng->addBilateral(replica, n, blocks);
        return (int)ALENS_OK;
    });
}

int alens_set_links(AlensCtx *ctx, int replica, int n, const int32_t *indexI, const int32_t *indexJ,
                    const double *sI, const double *sJ, const double *restLength, const double *kappa) {
    if (!ctx) return ALENS_INVALID_ARG;
    return guarded_ctx(ctx, [&] {
        ctx->eng->setLinks(replica, n, indexI, indexJ, sI, sJ, restLength, kappa);
        return (int)ALENS_OK;
    });
}

int alens_set_boundaries(AlensCtx *ctx, int replica, int n, const AlensBoundary *boundaries) {
    if (!ctx) return ALENS_INVALID_ARG;
    return guarded_ctx(ctx, [&] {
        ctx->eng->setBoundaries(replica, n, boundaries);
        return (int)ALENS_OK;
    });
}

int alens_step(AlensCtx *ctx, AlensStepStats *stats) {
    if (!ctx) return ALENS_INVALID_ARG;
    return guarded_ctx(ctx, [&] { return ctx->eng->step(stats); });
}

int alens_detect(AlensCtx *ctx, AlensStepStats *stats) {
    if (!ctx) return ALENS_INVALID_ARG;
    return guarded_ctx(ctx, [&] { return ctx->eng->detect(stats); });
}

int alens_solve(AlensCtx *ctx, AlensStepStats *stats) {
    if (!ctx) return ALENS_INVALID_ARG;
    return guarded_ctx(ctx, [&] { return ctx->eng->solve(stats); });
}

int alens_advance(AlensCtx *ctx, AlensStepStats *stats) {
    if (!ctx) return ALENS_INVALID_ARG;
    return guarded_ctx(ctx, [&] { return ctx->eng->advance(stats); });
}

int alens_get_replica_stats(AlensCtx *ctx, int replica, AlensStepStats *stats) {
    if (!ctx) return ALENS_INVALID_ARG;
    return guarded_ctx(ctx, [&] {
        ctx->eng->replicaStats(replica, stats);
        return (int)ALENS_OK;
    });
}

int alens_get_num_constraints(AlensCtx *ctx, int replica, int *nCollision, int *nBilateral) {
    if (!ctx) return ALENS_INVALID_ARG;
    return guarded_ctx(ctx, [&] {
        ctx->eng->numConstraints(replica, nCollision, nBilateral);
        return (int)ALENS_OK;
    });
}

int alens_get_constraints(AlensCtx *ctx, int replica, int cap, int32_t *indexI, int32_t *indexJ,
                          int32_t *image, double *delta0, double *gamma, double *jac) {
    if (!ctx) return ALENS_INVALID_ARG;
    return guarded_ctx(ctx, [&] {
        ctx->eng->getConstraints(replica, cap, indexI, indexJ, image, delta0, gamma, jac);
        return (int)ALENS_OK;
    });
}

int alens_get_gamma(AlensCtx *ctx, int replica, int cap, int *n, int32_t *pairs, double *gamma) {
    if (!ctx || !n) return ALENS_INVALID_ARG;
    return guarded_ctx(ctx, [&] {
        int nc = 0, nb = 0;
        ctx->eng->numConstraints(replica, &nc, &nb);
        *n = nc + nb;
        if (cap < nc + nb) return (int)ALENS_CAPACITY;
        std::vector<int32_t> ii((size_t)(nc + nb)), jj((size_t)(nc + nb));
        ctx->eng->getConstraints(replica, nc + nb, ii.data(), jj.data(), nullptr, nullptr, gamma, nullptr);
        if (pairs)
            for (int k = 0; k < nc + nb; k++) {
                pairs[2 * k] = ii[(size_t)k];
                pairs[2 * k + 1] = jj[(size_t)k];
            }
        return (int)ALENS_OK;
    });
}

int alens_get_pairs(AlensCtx *ctx, int replica, int cap, int *n, int32_t *indexI, int32_t *indexJ,
                    int32_t *image) {
    if (!ctx || !n) return ALENS_INVALID_ARG;
    return guarded_ctx(ctx, [&] {
        int nc = 0, nb = 0;
        ctx->eng->numConstraints(replica, &nc, &nb);
        *n = nc;
        if (cap < nc) return (int)ALENS_CAPACITY;
        std::vector<int32_t> ii((size_t)(nc + nb)), jj((size_t)(nc + nb)), im((size_t)(nc + nb));
        ctx->eng->getConstraints(replica, nc + nb, ii.data(), jj.data(), im.data(), nullptr, nullptr, nullptr);
        for (int k = 0; k < nc; k++) {
            if (indexI) indexI[k] = ii[(size_t)k];
            if (indexJ) indexJ[k] = jj[(size_t)k];
            if (image) image[k] = im[(size_t)k];
        }
        return (int)ALENS_OK;
    });
}

int alens_get_constraint_points(AlensCtx *ctx, int replica, int cap, double *lab) {
    if (!ctx) return ALENS_INVALID_ARG;
    return guarded_ctx(ctx, [&] {
        ctx->eng->getConstraintPoints(replica, cap, lab);
        return (int)ALENS_OK;
    });
}

int alens_set_protein_types(AlensCtx *ctx, int n, const AlensProteinType *types, double KBT,
                            double rodDiameter) {
    if (!ctx) return ALENS_INVALID_ARG;
    return guarded_ctx(ctx, [&] {
        ctx->eng->setProteinTypes(n, types, KBT, rodDiameter);
        return (int)ALENS_OK;
    });
}

int alens_set_proteins(AlensCtx *ctx, int replica, int n, const AlensProtein *proteins) {
    if (!ctx) return ALENS_INVALID_ARG;
    return guarded_ctx(ctx, [&] {
        ctx->eng->setProteins(replica, n, proteins);
        return (int)ALENS_OK;
    });
}

int alens_get_proteins(AlensCtx *ctx, int replica, int cap, int *n, AlensProtein *proteins) {
    if (!ctx) return ALENS_INVALID_ARG;
    return guarded_ctx(ctx, [&] {
        ctx->eng->getProteins(replica, cap, n, proteins);
        return (int)ALENS_OK;
    });
}

int alens_protein_motion_step(AlensCtx *ctx, AlensKmcStats *stats) {
    if (!ctx) return ALENS_INVALID_ARG;
    return guarded_ctx(ctx, [&] { return ctx->eng->proteinMotionStep(stats); });
}

int alens_protein_bind_step(AlensCtx *ctx, AlensKmcStats *stats) {
    if (!ctx) return ALENS_INVALID_ARG;
    return guarded_ctx(ctx, [&] { return ctx->eng->proteinBindStep(stats); });
}

int alens_set_wait_limit(AlensCtx *ctx, uint64_t timeoutNs, int stallBarriers) {
    if (!ctx) return ALENS_INVALID_ARG;
    return guarded_ctx(ctx, [&] {
        ctx->eng->setWaitLimit((unsigned long long)timeoutNs, stallBarriers);
        return (int)ALENS_OK;
    });
}

int alens_step_batched(AlensCtx **ctxs, int n, AlensStepStats *stats) {
    if (n < 0 || (n > 0 && !ctxs)) return ALENS_INVALID_ARG;
    for (int i = 0; i < n; i++)
        if (!ctxs[i]) return ALENS_INVALID_ARG;
    std::vector<int> rc((size_t)n, ALENS_OK);
    std::vector<int> direct((size_t)n, 0), started((size_t)n, 0);
    // enqueue every context's step first ...
    for (int i = 0; i < n; i++) {
        AlensCtx *c = ctxs[i];
        rc[(size_t)i] = guarded_ctx(c, [&] {
            c->eng->finalizeForStep();
            direct[(size_t)i] = c->eng->stepLaunch() ? 1 : 0;
            started[(size_t)i] = 1;
            return (int)ALENS_OK;
        });
    }
    // ... then read them back; a step that must be repeated runs alone
    for (int i = 0; i < n; i++) {
        if (!started[(size_t)i]) continue;
        AlensCtx *c = ctxs[i];
        AlensStepStats *out = stats ? stats + i : nullptr;
        rc[(size_t)i] = guarded_ctx(c, [&] {
            const int r = c->eng->stepFinish(out, direct[(size_t)i] != 0);
            return r == alens::Engine::kStepRetry ? c->eng->step(out) : r;
        });
    }
    int worst = ALENS_OK;
    for (int i = 0; i < n; i++) {
        const int r = rc[(size_t)i];
        if (r != ALENS_OK && r != ALENS_NOT_CONVERGED) return r;
        if (r == ALENS_NOT_CONVERGED) worst = r;
    }
    return worst;
}

int alens_get_con_stress(AlensCtx *ctx, int replica, double *stress9) {
    if (!ctx) return ALENS_INVALID_ARG;
    return guarded_ctx(ctx, [&] {
        ctx->eng->conStress(replica, stress9);
        return (int)ALENS_OK;
    });
}

int alens_get_operator(AlensCtx *ctx, int replica, int capNnz, int *nnz, int32_t *rowPtr, int32_t *cols,
                       double *vals, double *q, double *cinv, double *lowerBound, double *gamma0) {
    if (!ctx) return ALENS_INVALID_ARG;
    return guarded_ctx(ctx, [&] {
        ctx->eng->getOperator(replica, capNnz, nnz, rowPtr, cols, vals, q, cinv, lowerBound, gamma0);
        return (int)ALENS_OK;
    });
}

// ------------------------------------------------------ learned warm start
static_assert(alens::kMlpParams == ALENS_MLP_NUM_PARAMS, "parameter count");
static_assert(alens::kMlpIn == ALENS_MLP_NUM_FEATURES, "feature count");

int alens_mlp_create(uint64_t seed, int64_t datasetCapacity, AlensMlp **out) {
    if (!out) return ALENS_INVALID_ARG;
    *out = nullptr;
    return guarded([&] {
        AlensMlp *m = new AlensMlp{nullptr};
        try {
            m->model = new alens::MlpModel(seed, datasetCapacity);
        } catch (...) {
            delete m;
            throw;
        }
        *out = m;
        return (int)ALENS_OK;
    });
}

int alens_mlp_destroy(AlensMlp *mlp) {
    if (!mlp) return ALENS_INVALID_ARG;
    return guarded([&] {
        delete mlp->model;
        delete mlp;
        return (int)ALENS_OK;
    });
}

int alens_mlp_get_params(AlensMlp *mlp, float *params) {
    if (!mlp || !params) return ALENS_INVALID_ARG;
    return guarded([&] {
        mlp->model->getParams(params);
        return (int)ALENS_OK;
    });
}

int alens_mlp_set_params(AlensMlp *mlp, const float *params) {
    if (!mlp || !params) return ALENS_INVALID_ARG;
    return guarded([&] {
        mlp->model->setParams(params);
        return (int)ALENS_OK;
    });
}

int alens_mlp_add_samples(AlensMlp *mlp, int n, const float *features, const float *targets) {
    if (!mlp) return ALENS_INVALID_ARG;
    return guarded([&] {
        mlp->model->uploadDataset(features, targets, n);
        return (int)ALENS_OK;
    });
}

int alens_mlp_dataset_size(AlensMlp *mlp, int64_t *n) {
    if (!mlp || !n) return ALENS_INVALID_ARG;
    *n = mlp->model->datasetSize();
    return ALENS_OK;
}

int alens_mlp_clear_dataset(AlensMlp *mlp) {
    if (!mlp) return ALENS_INVALID_ARG;
    mlp->model->clearDataset();
    return ALENS_OK;
}

int alens_mlp_train(AlensMlp *mlp, int epochs, int batch, float lr, uint64_t seed, float *lossPerEpoch) {
    if (!mlp) return ALENS_INVALID_ARG;
    return guarded([&] {
        mlp->model->train(epochs, batch, lr, seed, lossPerEpoch);
        return (int)ALENS_OK;
    });
}

int alens_mlp_predict(AlensMlp *mlp, int n, const float *features, float *out) {
    if (!mlp) return ALENS_INVALID_ARG;
    return guarded([&] {
        mlp->model->predict(n, features, out);
        return (int)ALENS_OK;
    });
}

int alens_mlp_gradient(AlensMlp *mlp, int n, const float *features, const float *targets, float *grad,
                       float *loss) {
    if (!mlp) return ALENS_INVALID_ARG;
    return guarded([&] {
        mlp->model->gradient(n, features, targets, grad, loss);
        return (int)ALENS_OK;
    });
}

int alens_attach_mlp(AlensCtx *ctx, AlensMlp *mlp) {
    if (!ctx) return ALENS_INVALID_ARG;
    return guarded_ctx(ctx, [&] {
        ctx->eng->attachMlp(mlp ? mlp->model : nullptr);
        return (int)ALENS_OK;
    });
}

int alens_set_feature_capture(AlensCtx *ctx, int enable) {
    if (!ctx) return ALENS_INVALID_ARG;
    return guarded_ctx(ctx, [&] {
        ctx->eng->setFeatureCapture(enable != 0);
        return (int)ALENS_OK;
    });
}

int alens_mlp_collect(AlensCtx *ctx, AlensMlp *mlp, int64_t *added) {
    if (!ctx || !mlp) return ALENS_INVALID_ARG;
    return guarded_ctx(ctx, [&] {
        const long long a = ctx->eng->collect(mlp->model);
        if (added) *added = a;
        return (int)ALENS_OK;
    });
}

int alens_get_features(AlensCtx *ctx, int replica, int cap, float *features, float *scale, int *n) {
    if (!ctx) return ALENS_INVALID_ARG;
    return guarded_ctx(ctx, [&] {
        const int m = ctx->eng->getFeatures(replica, cap, features, scale);
        if (n) *n = m;
        return (int)ALENS_OK;
    });
}

int alens_autotune(AlensCtx *ctx, int reps, char *report, int reportCap) {
    if (!ctx) return ALENS_INVALID_ARG;
    return guarded_ctx(ctx, [&] {
        const std::string js = ctx->eng->autotune(reps);
        if (report && reportCap > 0) {
            const size_t n = std::min<size_t>(js.size(), (size_t)reportCap - 1);
            std::memcpy(report, js.data(), n);
            report[n] = 0;
        }
        return (int)ALENS_OK;
    });
}

int alens_get_step_count(AlensCtx *ctx, int64_t *count) {
    if (!ctx || !count) return ALENS_INVALID_ARG;
    *count = ctx->eng->stepCount();
    return ALENS_OK;
}

int alens_set_step_count(AlensCtx *ctx, int64_t count) {
    if (!ctx) return ALENS_INVALID_ARG;
    return guarded_ctx(ctx, [&] {
        ctx->eng->setStepCount((long long)count);
        return (int)ALENS_OK;
    });
}

const char *alens_get_last_error(AlensCtx *ctx) {
    if (!ctx) return "";
    return ctx->lastError.c_str();
}

int alens_get_launch_count(AlensCtx *ctx, int64_t *count) {
    if (!ctx || !count) return ALENS_INVALID_ARG;
    *count = ctx->eng->launches();
    return ALENS_OK;
}

int alens_get_stage_times(AlensCtx *ctx, double *ms5) {
    if (!ctx || !ms5) return ALENS_INVALID_ARG;
    for (int i = 0; i < 5; i++) ms5[i] = ctx->eng->stageMs()[i];
    return ALENS_OK;
}

int alens_get_stream(AlensCtx *ctx, void **stream) {
    if (!ctx || !stream) return ALENS_INVALID_ARG;
    *stream = (void *)ctx->eng->stream();
    return ALENS_OK;
}

}  // extern "C"
