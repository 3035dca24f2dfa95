// engine.cu - host side of a context: device memory, the per-step launch
// sequence (optionally replayed as one CUDA graph), capacity growth and
// statistics.  Everything the reference's SylinderSystem keeps per rank
// (rod container, constraint pool, solver) lives here for one GPU.
#include "engine.h"

#include <algorithm>
#include <cstdio>
#include <cmath>
#include <cstring>
#include <stdexcept>
#include <string>
#include <type_traits>

namespace alens {

namespace {

constexpr unsigned long long kBarrierTimeoutNs = 2000000000ULL;  // 2 s

bool config_ok(const AlensConfig &c) {
    for (int d = 0; d < 3; d++)
        if (!(c.simBoxHigh[d] > c.simBoxLow[d]) || !std::isfinite(c.simBoxLow[d]) ||
            !std::isfinite(c.simBoxHigh[d]))
            return false;
    return c.dt > 0 && c.viscosity > 0 && c.sylinderColBuf >= 0 && c.sylinderDiameterColRatio > 0 &&
           c.sylinderLengthColRatio > 0 && c.conMaxIte >= 0 && c.conResTol > 0 &&
           c.conSolverChoice == 0 && (c.precision == ALENS_PREC_FP64 || c.precision == ALENS_PREC_MIXED) &&
           c.warmStart >= 0 && c.warmStart <= 2 && c.maxConstraints >= 0;
}

}  // namespace

#define CK(call)                                                   \
    do {                                                           \
        cudaError_t e_ = (call);                                   \
        if (e_ != cudaSuccess) throw CudaFailure(e_, #call);       \
    } while (0)

Engine::Engine(const AlensConfig *cfgs, int nrep) {
    if (nrep < 1) throw ApiError(ALENS_INVALID_ARG);
    for (int r = 0; r < nrep; r++)
        if (!config_ok(cfgs[r])) throw ApiError(ALENS_INVALID_ARG);
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
        cudaGetLastError();
        throw ApiError(ALENS_NO_DEVICE);
    }
    CK(cudaGetDevice(&device_));
    CK(cudaDeviceGetAttribute(&numSM_, cudaDevAttrMultiProcessorCount, device_));
    cfg_.assign(cfgs, cfgs + nrep);
    R_ = nrep;
    rods_.resize(R_);
    queue_.resize(R_);
    links_.resize(R_);
    prot_.resize(R_);
    springs_.assign(R_, 0);
    bnd_.resize(R_);
    repStats_.assign(R_, AlensStepStats{});
    if (cfg_[0].stream) {
        stream_ = (cudaStream_t)cfg_[0].stream;
        ownStream_ = false;
    } else {
        CK(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
        ownStream_ = true;
    }
    precision_ = cfg_[0].precision;
    warm_ = cfg_[0].warmStart;
    useGraph_ = cfg_[0].useGraph != 0;
    fixedCap_ = cfg_[0].maxConstraints;
    stageTiming_ = cfg_[0].stageTiming != 0;
    if (const char *e = std::getenv("ALENS_SOLVER_BLOCKS_PER_SM")) solverBlocksPerSM_ = std::max(1, atoi(e));
    if (const char *e = std::getenv("ALENS_SOLVER_MIN_TILES")) solverMinTiles_ = std::max(1, atoi(e));
    // FP32 solver form: -1 = automatic (grid form for one replica, where all
    // SMs share one system; cluster form for ensembles), 0 = grid form,
    // N = cluster form with clusters of N CTAs
    if (const char *e = std::getenv("ALENS_CLUSTER_SIZE")) clusterSize_ = atoi(e);
    if (const char *e = std::getenv("ALENS_CSM_THREADS")) csm_set_threads(atoi(e));
    if (const char *e = std::getenv("ALENS_SOLVER_FORM")) {
        const std::string f(e);
        formRequest_ = f == "grid"       ? kFormGrid
                       : f == "cluster"  ? kFormCluster
                       : f == "resident" ? kFormResident
                       : f == "fast"     ? kFormFast
                                         : -1;
    }
    CK(cudaStreamCreateWithFlags(&side_, cudaStreamNonBlocking));
    CK(cudaStreamCreateWithFlags(&side2_, cudaStreamNonBlocking));
    CK(cudaStreamCreateWithFlags(&side3_, cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&orderJoin_, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&orderFork_, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&rowsDone_, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&weightsDone_, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&warmJoin_, cudaEventDisableTiming));
    for (int i = 0; i < 3; i++) {
        CK(cudaEventCreateWithFlags(&forkEv_[i], cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&joinEv_[i], cudaEventDisableTiming));
    }
    CK(cudaMallocHost(&hCtl_, sizeof(DevCtl)));
    CK(cudaMallocHost(&hDyn_, sizeof(RepDyn) * R_));
    CK(cudaMallocHost(&hBilPrefix_, sizeof(int) * (R_ + 1)));
    CK(cudaMallocHost(&hLinkSlot0_, sizeof(int) * R_));
    CK(cudaMallocHost(&hKmc_, sizeof(int) * (9 * R_ + 1)));
    std::memset(hKmc_, 0, sizeof(int) * (9 * R_ + 1));
    std::memset(hCtl_, 0, sizeof(DevCtl));
    std::memset(hDyn_, 0, sizeof(RepDyn) * R_);
    std::memset(hBilPrefix_, 0, sizeof(int) * (R_ + 1));
}

Engine::~Engine() {
    if (graphExec_) cudaGraphExecDestroy(graphExec_);
    for (auto &e : events_)
        if (e) cudaEventDestroy(e);
    if (stream_) cudaStreamSynchronize(stream_);
    freeGroup(rodAllocs_);
    freeGroup(conAllocs_);
    freeGroup(blockAllocs_);
    freeGroup(fixedAllocs_);
    freeGroup(opAllocs_);
    if (hCtl_) cudaFreeHost(hCtl_);
    if (hDyn_) cudaFreeHost(hDyn_);
    if (hBilPrefix_) cudaFreeHost(hBilPrefix_);
    if (hBlocks_) cudaFreeHost(hBlocks_);
    if (hBlockRep_) cudaFreeHost(hBlockRep_);
    if (hLinkSlot0_) cudaFreeHost(hLinkSlot0_);
    if (hKmc_) cudaFreeHost(hKmc_);
    freeGroup(linkAllocs_);
    freeGroup(protAllocs_);
    freeGroup(kmcAllocs_);
    freeGroup(kmcFixedAllocs_);
    freeGroup(bndAllocs_);
    for (int i = 0; i < 3; i++) {
        if (forkEv_[i]) cudaEventDestroy(forkEv_[i]);
        if (joinEv_[i]) cudaEventDestroy(joinEv_[i]);
    }
    if (side_) cudaStreamDestroy(side_);
    if (side2_) cudaStreamDestroy(side2_);
    if (side3_) cudaStreamDestroy(side3_);
    if (orderJoin_) cudaEventDestroy(orderJoin_);
    if (orderFork_) cudaEventDestroy(orderFork_);
    for (cudaEvent_t e : {rowsDone_, weightsDone_, warmJoin_})
        if (e) cudaEventDestroy(e);
    if (ownStream_ && stream_) cudaStreamDestroy(stream_);
}

void Engine::freeGroup(std::vector<void *> &g) {
    for (void *p : g) cudaFree(p);
    g.clear();
}

template <class T>
T *Engine::alloc(std::vector<void *> &group, size_t n) {
    void *p = nullptr;
    const size_t bytes = std::max<size_t>(n, 1) * sizeof(T);
    CK(cudaMalloc(&p, bytes));
    group.push_back(p);
    return (T *)p;
}

// ------------------------------------------------------------------ rods
void Engine::setRods(int rep, int n, const int64_t *gid, const double *pos, const double *quat,
                     const double *len, const double *rad, const int32_t *imm) {
    if (rep < 0 || rep >= R_ || n < 0 || n > (4 << 20)) throw ApiError(ALENS_INVALID_ARG);
    if (n > 0 && (!gid || !pos || !quat || !len || !rad)) throw ApiError(ALENS_INVALID_ARG);
    for (int i = 0; i < n; i++)
        if (!(len[i] >= 0.0) || !(rad[i] > 0.0) || !std::isfinite(len[i]) || !std::isfinite(rad[i]))
            throw ApiError(ALENS_INVALID_ARG);
    HostRods h;
    h.n = n;
    h.gid.assign(gid, gid + n);
    h.pos.assign(pos, pos + 3 * (size_t)n);
    h.quat.assign(quat, quat + 4 * (size_t)n);
    h.len.assign(len, len + n);
    h.rad.assign(rad, rad + n);
    for (int i = 0; i < n; i++) h.hlMax = std::max(h.hlMax, 0.5 * len[i]);
    h.imm.assign(n, 0);
    if (imm)
        for (int i = 0; i < n; i++) h.imm[i] = imm[i] ? 1 : 0;
    h.set = true;
    // cell grid (validates the box against the search cutoff)
    RepParams P;
    makeParams(rep, h, P);
    rods_[rep] = std::move(h);
    dirty_ = true;
}

void Engine::makeParams(int rep, const HostRods &h, RepParams &P) const {
    const AlensConfig &c = cfg_[rep];
    std::memset(&P, 0, sizeof(P));
    double mx = 0.0;
    for (int i = 0; i < h.n; i++) {
        const bool sphere = h.len[i] < 2.0 * h.rad[i];
        const double hh = sphere ? 0.0 : 0.5 * (h.len[i] * c.sylinderLengthColRatio);
        const double rc = h.rad[i] * c.sylinderDiameterColRatio;
        mx = std::max(mx, 2.0 * hh + 2.0 * rc);
    }
    const double cutoff = mx + c.sylinderColBuf;
    for (int d = 0; d < 3; d++) {
        P.lo[d] = c.simBoxLow[d];
        P.hi[d] = c.simBoxHigh[d];
        P.L[d] = c.simBoxHigh[d] - c.simBoxLow[d];
        P.pbc[d] = c.simBoxPBC[d] ? 1 : 0;
        if (P.pbc[d] && P.L[d] < cutoff) throw ApiError(ALENS_INVALID_ARG);
        int nc = cutoff > 0 ? (int)std::floor(P.L[d] / cutoff) : 1;
        nc = std::max(1, std::min(nc, 1024));
        P.ncell[d] = nc;
    }
    // dense systems (many rods per cutoff-sized cell) use cells of half the
    // cutoff and a 5-cell stencil: the candidates then cover about a third
    // of the volume of the 27 full cells
    P.stencil = 3;
    {
        const long long cells = (long long)P.ncell[0] * P.ncell[1] * P.ncell[2];
        if (cutoff > 0 && (double)h.n > 24.0 * (double)cells) {
            P.stencil = 5;
            for (int d = 0; d < 3; d++) {
                int nc = (int)std::floor(P.L[d] / (0.5 * cutoff));
                P.ncell[d] = std::max(1, std::min(nc, 1024));
            }
        }
    }
    // keep the cell count proportional to the rod count (the grid only
    // affects the candidate enumeration, never the result)
    const long long limit = std::max<long long>(64, 2LL * h.n);
    while ((long long)P.ncell[0] * P.ncell[1] * P.ncell[2] > limit) {
        int d = 0;
        for (int e = 1; e < 3; e++)
            if (P.ncell[e] > P.ncell[d]) d = e;
        P.ncell[d] = std::max(1, P.ncell[d] / 2);
    }
    for (int d = 0; d < 3; d++) P.cellsz[d] = P.L[d] / P.ncell[d];
    P.mu = c.viscosity;
    P.kT = c.KBT;
    P.dt = c.dt;
    P.colRatioD = c.sylinderDiameterColRatio;
    P.colRatioL = c.sylinderLengthColRatio;
    P.colBuf = c.sylinderColBuf;
    P.tol = c.conResTol;
    P.seed = c.rngSeed;
    P.mono = c.monolayer ? 1 : 0;
    P.maxIte = c.conMaxIte;
    P.nRods = h.n;
    P.halfReachMax = 0.5 * mx;
    // the same IEEE operations as the per-rod expression it replaces
    P.bcoef = c.KBT > 0.0 ? std::sqrt(2.0 * c.KBT / c.dt) : 0.0;
    for (int d = 0; d < 3; d++) P.cellsz32[d] = (float)P.cellsz[d];
    P.colBuf32 = (float)P.colBuf;
    P.halfReach32 = (float)P.halfReachMax;
    P.pad32 = 0.0f;
}

void Engine::finalize() {
    if (!dirty_) return;
    for (int r = 0; r < R_; r++)
        if (!rods_[r].set) throw ApiError(ALENS_NOT_READY);
    CK(cudaStreamSynchronize(stream_));
    invalidateGraph();
    freeGroup(rodAllocs_);
    freeGroup(conAllocs_);
    freeGroup(fixedAllocs_);
    freeGroup(blockAllocs_);
    freeGroup(opAllocs_);
    blockCap_ = 0;
    freeGroup(linkAllocs_);
    S_.nLinks = 0;
    freeGroup(bndAllocs_);
    hostPar_.resize(R_);
    int rodOff = 0, cellOff = 0;
    for (int r = 0; r < R_; r++) {
        makeParams(r, rods_[r], hostPar_[r]);
        hostPar_[r].rodOffset = rodOff;
        hostPar_[r].cellOffset = cellOff;
        rodOff += rods_[r].n;
        cellOff += hostPar_[r].ncell[0] * hostPar_[r].ncell[1] * hostPar_[r].ncell[2];
    }
    const int N = rodOff;
    const int C = cellOff;
    // the three-pass scan handles up to 4096 x 1024 elements
    if (N > (4 << 20) || C > (4 << 20)) throw ApiError(ALENS_INVALID_ARG);
    DevState &S = S_;
    std::memset(&S, 0, sizeof(S));
    S.R = R_;
    for (int d = 0; d < 3; d++) {
        int rad = 0;
        for (int r = 0; r < R_; r++) {
            const RepParams &P = hostPar_[r];
            // one cell along a closed side: no neighbour cells that way
            if (!(P.ncell[d] == 1 && !P.pbc[d])) rad = std::max(rad, P.stencil >> 1);
        }
        S.pairW[d] = 2 * rad + 1;
    }
    S.nRods = N;
    S.nCells = C;
    S.warm = warm_;
    S.precision = precision_;
    S.solveMinTiles = solverMinTiles_;
    S.barrierExtra = stallBarriers_;
    // fixed-size control
    S.par = alloc<RepParams>(fixedAllocs_, R_);
    S.dyn = alloc<RepDyn>(fixedAllocs_, R_);
    S.ctl = alloc<DevCtl>(fixedAllocs_, 1);
    S.bilPrefix = alloc<int>(fixedAllocs_, R_ + 1);
    S.stress = alloc<double>(fixedAllocs_, 9 * (size_t)R_);
    S.scanTmp = alloc<int>(fixedAllocs_, 4096);
    S.prevCount = alloc<int>(fixedAllocs_, 1);
    S.linkSlot0 = alloc<int>(fixedAllocs_, R_);
    S.fastPart = alloc<double>(fixedAllocs_, 2 * 8 * (size_t)kFastMaxGrid);
    S.fastScanTmp = alloc<int>(fixedAllocs_, 4096);
    linksDirty_ = true;
    bndDirty_ = true;
    CK(cudaMemcpyAsync(S.par, hostPar_.data(), sizeof(RepParams) * R_, cudaMemcpyHostToDevice, stream_));
    CK(cudaMemsetAsync(S.dyn, 0, sizeof(RepDyn) * R_, stream_));
    CK(cudaMemsetAsync(S.bilPrefix, 0, sizeof(int) * (R_ + 1), stream_));
    CK(cudaMemsetAsync(S.prevCount, 0, sizeof(int), stream_));
    std::memset(hCtl_, 0, sizeof(DevCtl));
    hCtl_->step = stepCount_;
    CK(cudaMemcpyAsync(S.ctl, hCtl_, sizeof(DevCtl), cudaMemcpyHostToDevice, stream_));
    // rods
    auto &G = rodAllocs_;
    double **rodD[] = {&S.px, &S.py, &S.pz, &S.qx, &S.qy, &S.qz, &S.qw, &S.len, &S.rad,
                       &S.ax, &S.ay, &S.az, &S.hcol, &S.rcol, &S.m0, &S.m1, &S.m2,
                       &S.sm0, &S.sm1, &S.sm2};
    for (double **p : rodD) *p = alloc<double>(G, N);
    S.sA = alloc<float4>(G, N);
    S.sB = alloc<float4>(G, N);
    S.gid = alloc<long long>(G, N);
    S.imm = alloc<int>(G, N);
    S.rodRep = alloc<int>(G, N);
    S.sph = alloc<unsigned char>(G, N);
    S.unc = alloc<double>(G, 6 * (size_t)N);
    S.vel = alloc<double>(G, 6 * (size_t)N);
    S.rodV = alloc<float>(G, 6 * (size_t)N);
    S.alphaBuf = alloc<double>(G, 2 * (size_t)R_);
    S.stage = alloc<double>(G, 7 * (size_t)N);
    S.cellOf = alloc<int>(G, N);
    S.sidx = alloc<int>(G, N);
    S.pairCount = alloc<int>(G, N);
    S.pairOff = alloc<int>(G, N + 1);
    S.pairCursor = alloc<int>(G, N);
    S.rowCount = alloc<int>(G, N);
    S.rowPtr = alloc<int>(G, N + 1);
    S.rowCursor = alloc<int>(G, N);
    S.cellCount = alloc<int>(G, C);
    if (R_ == 1 && precision_ == ALENS_PREC_MIXED) {
        // cells in Morton (bit-interleaved) order of their grid coordinates,
        // for the single-system solver's spatial row order
        const RepParams &P0 = hostPar_[0];
        std::vector<std::pair<unsigned long long, int>> code((size_t)C);
        for (int c = 0; c < C; c++) {
            const int cx = c % P0.ncell[0], cy = (c / P0.ncell[0]) % P0.ncell[1], cz = c / (P0.ncell[0] * P0.ncell[1]);
            unsigned long long m = 0;
            for (int bit = 0; bit < 21; bit++) {
                m |= (unsigned long long)((cx >> bit) & 1) << (3 * bit);
                m |= (unsigned long long)((cy >> bit) & 1) << (3 * bit + 1);
                m |= (unsigned long long)((cz >> bit) & 1) << (3 * bit + 2);
            }
            code[(size_t)c] = {m, c};
        }
        std::sort(code.begin(), code.end());
        std::vector<int> byRank((size_t)C);
        for (int r = 0; r < C; r++) byRank[(size_t)r] = code[(size_t)r].second;
        S.cellByRank = alloc<int>(G, C);
        S.fastCellCnt = alloc<int>(G, C + 1);
        S.fastCellBase = alloc<int>(G, C + 1);
        CK(cudaMemcpy(S.cellByRank, byRank.data(), sizeof(int) * (size_t)C, cudaMemcpyHostToDevice));
    }
    S.cellStart = alloc<int>(G, C + 1);
    S.cellCursor = alloc<int>(G, C);
    CK(cudaMemsetAsync(S.vel, 0, sizeof(double) * 6 * (size_t)N, stream_));
    // upload SoA
    {
        std::vector<double> buf((size_t)N);
        std::vector<long long> gbuf((size_t)N);
        std::vector<int> ibuf((size_t)N), rbuf((size_t)N);
        auto up = [&](double *dst, auto getter) {
            size_t o = 0;
            for (int r = 0; r < R_; r++)
                for (int i = 0; i < rods_[r].n; i++) buf[o++] = getter(rods_[r], i);
            CK(cudaMemcpy(dst, buf.data(), sizeof(double) * N, cudaMemcpyHostToDevice));
        };
        up(S.px, [](const HostRods &h, int i) { return h.pos[3 * i]; });
        up(S.py, [](const HostRods &h, int i) { return h.pos[3 * i + 1]; });
        up(S.pz, [](const HostRods &h, int i) { return h.pos[3 * i + 2]; });
        up(S.qx, [](const HostRods &h, int i) { return h.quat[4 * i]; });
        up(S.qy, [](const HostRods &h, int i) { return h.quat[4 * i + 1]; });
        up(S.qz, [](const HostRods &h, int i) { return h.quat[4 * i + 2]; });
        up(S.qw, [](const HostRods &h, int i) { return h.quat[4 * i + 3]; });
        up(S.len, [](const HostRods &h, int i) { return h.len[i]; });
        up(S.rad, [](const HostRods &h, int i) { return h.rad[i]; });
        size_t o = 0;
        for (int r = 0; r < R_; r++)
            for (int i = 0; i < rods_[r].n; i++, o++) {
                gbuf[o] = rods_[r].gid[i];
                ibuf[o] = rods_[r].imm[i];
                rbuf[o] = r;
            }
        CK(cudaMemcpy(S.gid, gbuf.data(), sizeof(long long) * N, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(S.imm, ibuf.data(), sizeof(int) * N, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(S.rodRep, rbuf.data(), sizeof(int) * N, cudaMemcpyHostToDevice));
    }
    launch_mobility(S, stream_);
    CK(cudaGetLastError());
    // constraints
    int want = fixedCap_ > 0 ? fixedCap_ : std::max(4096, 4 * N + 1024);
    nnzCap_ = 0;
    allocConstraints(std::min(want, kMaxConstraints), false);
    solverGrid_ = 0;
    dirty_ = false;
    prevCountHost_ = 0;
    haveDetect_ = false;
    haveSolve_ = false;
    CK(cudaStreamSynchronize(stream_));
}

void Engine::allocConstraints(int cap, bool keepPrev) {
    DevState &S = S_;
    unsigned long long *oldKeys = S.prevKeys;
    double *oldGamma = S.prevGamma;
    std::vector<void *> old;
    old.swap(conAllocs_);
    const int prevN = keepPrev ? prevCountHost_ : 0;
    auto &G = conAllocs_;
    S.cap = cap;
    S.tileCap = cap / kTile + R_ + 2;
    S.workCap = S.tileCap / kChunk + R_ + 2;
    S.rawKeys = alloc<unsigned long long>(G, cap);
    S.keys = alloc<unsigned long long>(G, cap);
    S.border = alloc<int4>(G, cap);
    S.prevKeys = alloc<unsigned long long>(G, cap);
    S.prevGamma = alloc<double>(G, cap);
    S.conI = alloc<int>(G, cap);
    S.conJ = alloc<int>(G, cap);
    S.conImg = alloc<int>(G, cap);
    S.conST = alloc<float2>(G, cap);
    if (capture_) {
        S.feat = alloc<float>(G, (size_t)kMlpIn * cap);
        S.fscale = alloc<float>(G, cap);
    } else {
        S.feat = nullptr;
        S.fscale = nullptr;
    }
    S.jac = alloc<double>(G, 12 * (size_t)cap);
    S.W = alloc<double>(G, 12 * (size_t)cap);
    double **cd[] = {&S.phi0, &S.q, &S.gamma, &S.lb, &S.cinv};
    for (double **p : cd) *p = alloc<double>(G, cap);
    S.lbKind = alloc<int>(G, cap);
    S.qc = alloc<double2>(G, cap);
    S.st[0] = alloc<double2>(G, cap);
    S.st[1] = alloc<double2>(G, cap);
    S.lab = alloc<double>(G, 6 * (size_t)cap);
    S.rowEnt = alloc<int>(G, 2 * (size_t)cap);
    S.annz = alloc<int>(G, cap);
    S.aptr = alloc<int>(G, cap + 1);
    if (precision_ == ALENS_PREC_MIXED) {
        S.qc32 = alloc<float2>(G, cap);
        S.st32[0] = alloc<float2>(G, cap);
        S.st32[1] = alloc<float2>(G, cap);
        if (R_ == 1) {
            S.fastPerm = alloc<int>(G, cap);
            S.fastInv = alloc<int>(G, cap);
        }
    }
    S.part = alloc<double>(G, 9 * (size_t)S.tileCap);
    S.work = alloc<double>(G, (size_t)kMaxSolverGrid * 3 * S.workCap);
    S.tileRep = alloc<int>(G, S.tileCap);
    if (keepPrev && prevN > 0 && oldKeys) {
        const int n = std::min(prevN, cap);
        CK(cudaMemcpyAsync(S.prevKeys, oldKeys, sizeof(unsigned long long) * n, cudaMemcpyDeviceToDevice, stream_));
        CK(cudaMemcpyAsync(S.prevGamma, oldGamma, sizeof(double) * n, cudaMemcpyDeviceToDevice, stream_));
        CK(cudaStreamSynchronize(stream_));
    }
    freeGroup(old);
    allocOperator(std::max<long long>(nnzCap_, 10LL * cap));
}

void Engine::allocOperator(long long nnz) {
    if (nnz >= (1LL << 31) - 1) throw ApiError(ALENS_CAPACITY);
    freeGroup(opAllocs_);
    nnzCap_ = nnz;
    S_.nnzCap = (int)nnz;
    S_.aent = alloc<int4>(opAllocs_, (size_t)nnz);
    S_.aent32 = precision_ == ALENS_PREC_MIXED ? alloc<int4>(opAllocs_, (size_t)nnz) : nullptr;
    if (precision_ == ALENS_PREC_MIXED && R_ == 1) {
        // the streaming layout pads each 32-row slice to its longest row;
        // rows sorted by length bound the padding by 32 x the longest row
        // per block
        S_.fastEntCap = nnz + nnz / 2 + 32LL * 128 * kFastMaxGrid;
        S_.fastEnt = alloc<int2>(opAllocs_, (size_t)S_.fastEntCap);
    } else {
        S_.fastEnt = nullptr;
        S_.fastEntCap = 0;
    }
}

void Engine::updateRods(int rep, int n, const double *pos, const double *quat) {
    if (rep < 0 || rep >= R_ || !rods_[rep].set || n != rods_[rep].n || !pos || !quat)
        throw ApiError(ALENS_INVALID_ARG);
    if (dirty_) {
        std::copy(pos, pos + 3 * (size_t)n, rods_[rep].pos.begin());
        std::copy(quat, quat + 4 * (size_t)n, rods_[rep].quat.begin());
        return;
    }
    const int off = hostPar_[rep].rodOffset;
    CK(cudaMemcpyAsync(S_.stage, pos, sizeof(double) * 3 * (size_t)n, cudaMemcpyHostToDevice, stream_));
    CK(cudaMemcpyAsync(S_.stage + 3 * (size_t)n, quat, sizeof(double) * 4 * (size_t)n,
                       cudaMemcpyHostToDevice, stream_));
    launch_unpack_rods(S_, off, n, stream_);
    CK(cudaGetLastError());
    haveDetect_ = haveSolve_ = false;
}

void Engine::getRods(int rep, int n, double *pos, double *quat) {
    if (rep < 0 || rep >= R_ || !rods_[rep].set || n != rods_[rep].n) throw ApiError(ALENS_INVALID_ARG);
    if (dirty_) {
        if (pos) std::copy(rods_[rep].pos.begin(), rods_[rep].pos.end(), pos);
        if (quat) std::copy(rods_[rep].quat.begin(), rods_[rep].quat.end(), quat);
        return;
    }
    const int off = hostPar_[rep].rodOffset;
    launch_pack_rods(S_, off, n, 0, stream_);
    CK(cudaGetLastError());
    if (pos) CK(cudaMemcpyAsync(pos, S_.stage, sizeof(double) * 3 * (size_t)n, cudaMemcpyDeviceToHost, stream_));
    if (quat)
        CK(cudaMemcpyAsync(quat, S_.stage + 3 * (size_t)n, sizeof(double) * 4 * (size_t)n,
                           cudaMemcpyDeviceToHost, stream_));
    CK(cudaStreamSynchronize(stream_));
}

void Engine::getVelocity(int rep, int n, double *vel, double *omega) {
    if (rep < 0 || rep >= R_ || !rods_[rep].set || n != rods_[rep].n) throw ApiError(ALENS_INVALID_ARG);
    if (dirty_) throw ApiError(ALENS_NOT_READY);
    const int off = hostPar_[rep].rodOffset;
    launch_pack_rods(S_, off, n, 1, stream_);
    CK(cudaGetLastError());
    if (vel) CK(cudaMemcpyAsync(vel, S_.stage, sizeof(double) * 3 * (size_t)n, cudaMemcpyDeviceToHost, stream_));
    if (omega)
        CK(cudaMemcpyAsync(omega, S_.stage + 3 * (size_t)n, sizeof(double) * 3 * (size_t)n,
                           cudaMemcpyDeviceToHost, stream_));
    CK(cudaStreamSynchronize(stream_));
}

void Engine::addBilateral(int rep, int n, const AlensBlock *blocks) {
    if (rep < 0 || rep >= R_ || n < 0 || (n > 0 && !blocks)) throw ApiError(ALENS_INVALID_ARG);
    const int nr = rods_[rep].n;
    for (int b = 0; b < n; b++) {
        const AlensBlock &B = blocks[b];
        if (B.globalIndexI < 0 || B.globalIndexI >= nr) throw ApiError(ALENS_INVALID_ARG);
        if (!B.oneSide && (B.globalIndexJ < 0 || B.globalIndexJ >= nr)) throw ApiError(ALENS_INVALID_ARG);
    }
    queue_[rep].insert(queue_[rep].end(), blocks, blocks + n);
}

void Engine::setLinks(int rep, int n, const int32_t *idxI, const int32_t *idxJ, const double *sI,
                      const double *sJ, const double *rest, const double *kappa) {
    if (rep < 0 || rep >= R_ || n < 0) throw ApiError(ALENS_INVALID_ARG);
    if (n > 0 && (!idxI || !idxJ || !sI || !sJ || !rest || !kappa)) throw ApiError(ALENS_INVALID_ARG);
    const int nr = rods_[rep].n;
    for (int k = 0; k < n; k++) {
        if (idxI[k] < 0 || idxI[k] >= nr || idxJ[k] < 0 || idxJ[k] >= nr) throw ApiError(ALENS_INVALID_ARG);
        if (!(kappa[k] > 0.0) || !std::isfinite(sI[k]) || !std::isfinite(sJ[k]) || !std::isfinite(rest[k]))
            throw ApiError(ALENS_INVALID_ARG);
    }
    HostLinks &h = links_[rep];
    h.I.assign(idxI, idxI + n);
    h.J.assign(idxJ, idxJ + n);
    h.sI.assign(sI, sI + n);
    h.sJ.assign(sJ, sJ + n);
    h.rest.assign(rest, rest + n);
    h.kappa.assign(kappa, kappa + n);
    linksDirty_ = true;
}

void Engine::setBoundaries(int rep, int n, const AlensBoundary *b) {
    if (rep < 0 || rep >= R_ || n < 0 || n > ALENS_MAX_BOUNDARIES || (n > 0 && !b)) throw ApiError(ALENS_INVALID_ARG);
    std::vector<BoundaryDev> v;
    for (int k = 0; k < n; k++) {
        const AlensBoundary &B = b[k];
        BoundaryDev d{};
        d.type = B.type;
        d.inside = B.inside ? 1 : 0;
        if (B.type < ALENS_BOUNDARY_WALL || B.type > ALENS_BOUNDARY_TUBE) throw ApiError(ALENS_INVALID_ARG);
        if (B.type == ALENS_BOUNDARY_TUBE && !d.inside) throw ApiError(ALENS_INVALID_ARG);
        const double an = std::sqrt(B.axis[0] * B.axis[0] + B.axis[1] * B.axis[1] + B.axis[2] * B.axis[2]);
        if (B.type != ALENS_BOUNDARY_SPHERE && !(an > 0.0)) throw ApiError(ALENS_INVALID_ARG);
        if (B.type != ALENS_BOUNDARY_WALL && !(B.radius > 0.0)) throw ApiError(ALENS_INVALID_ARG);
        for (int c = 0; c < 3; c++) {
            if (!std::isfinite(B.center[c]) || !std::isfinite(B.axis[c])) throw ApiError(ALENS_INVALID_ARG);
            d.c[c] = B.center[c];
            d.a[c] = an > 0.0 ? B.axis[c] / an : 0.0;
        }
        d.R = B.radius;
        v.push_back(d);
    }
    bnd_[rep] = std::move(v);
    bndDirty_ = true;
}

// Device copy of every replica's boundaries.  Invalidates the captured
// graph: whether the boundary kernel runs is part of it.
void Engine::uploadBoundaries() {
    if (!bndDirty_) return;
    CK(cudaStreamSynchronize(stream_));
    invalidateGraph();
    freeGroup(bndAllocs_);
    std::vector<BoundaryDev> all;
    std::vector<int> start(R_ + 1, 0);
    for (int r = 0; r < R_; r++) {
        all.insert(all.end(), bnd_[r].begin(), bnd_[r].end());
        start[r + 1] = (int)all.size();
    }
    S_.nBnd = (int)all.size();
    S_.bnd = alloc<BoundaryDev>(bndAllocs_, all.size());
    S_.bndStart = alloc<int>(bndAllocs_, R_ + 1);
    if (!all.empty())
        CK(cudaMemcpy(S_.bnd, all.data(), sizeof(BoundaryDev) * all.size(), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(S_.bndStart, start.data(), sizeof(int) * (R_ + 1), cudaMemcpyHostToDevice));
    bndDirty_ = false;
}

// Concatenated device copy of every replica's links (rod indices made
// global).  Invalidates the captured graph: the link count is part of it.
void Engine::uploadLinks() {
    if (!linksDirty_) return;
    CK(cudaStreamSynchronize(stream_));
    invalidateGraph();
    freeGroup(linkAllocs_);
    int total = 0, nprot = 0;
    for (int r = 0; r < R_; r++) {
        total += (int)links_[r].I.size();
        nprot += (int)prot_[r].size();
        springs_[r] = 0;
    }
    userLinkTotal_ = total;
    // one row more per protein: the doubly bound ones become springs
    linkCap_ = total + nprot;
    S_.nLinks = total;
    if (linkCap_ > 0) {
        std::vector<int> I(total), J(total), rep(total), loc(total);
        std::vector<double> a(total), b(total), rest(total), kap(total);
        int o = 0;
        for (int r = 0; r < R_; r++) {
            const HostLinks &h = links_[r];
            const int off = hostPar_[r].rodOffset;
            for (size_t k = 0; k < h.I.size(); k++, o++) {
                I[o] = h.I[k] + off;
                J[o] = h.J[k] + off;
                rep[o] = r;
                loc[o] = (int)k;
                a[o] = h.sI[k];
                b[o] = h.sJ[k];
                rest[o] = h.rest[k];
                kap[o] = h.kappa[k];
            }
        }
        auto up = [&](auto *&dst, const auto &src) {
            using T = typename std::remove_reference<decltype(src[0])>::type;
            dst = alloc<typename std::remove_const<T>::type>(linkAllocs_, linkCap_);
            if (total > 0) CK(cudaMemcpy(dst, src.data(), sizeof(T) * total, cudaMemcpyHostToDevice));
        };
        up(S_.linkI, I);
        up(S_.linkJ, J);
        up(S_.linkRep, rep);
        up(S_.linkLocal, loc);
        up(S_.linkSI, a);
        up(S_.linkSJ, b);
        up(S_.linkRest, rest);
        up(S_.linkKappa, kap);
    }
    linksDirty_ = false;
    springsDirty_ = nprot > 0;
}

// --------------------------------------------------------------- blocks
// Per replica the blocks are [queued by alens_add_bilateral..., links...,
// protein springs...].
void Engine::uploadBlocks() {
    uploadLinks();
    if (springsDirty_) rebuildSprings();
    uploadBoundaries();
    int total = 0;
    hBilPrefix_[0] = 0;
    for (int r = 0; r < R_; r++) {
        hLinkSlot0_[r] = total + (int)queue_[r].size();
        total += (int)queue_[r].size() + (int)links_[r].I.size() + springs_[r];
        hBilPrefix_[r + 1] = total;
    }
    if (total > blockCap_) {
        CK(cudaStreamSynchronize(stream_));
        invalidateGraph();
        freeGroup(blockAllocs_);
        if (hBlocks_) cudaFreeHost(hBlocks_);
        if (hBlockRep_) cudaFreeHost(hBlockRep_);
        blockCap_ = std::max(total, blockCap_ * 3 / 2);
        S_.blocks = alloc<AlensBlock>(blockAllocs_, blockCap_);
        S_.blockRep = alloc<int>(blockAllocs_, blockCap_);
        CK(cudaMallocHost(&hBlocks_, sizeof(AlensBlock) * blockCap_));
        CK(cudaMallocHost(&hBlockRep_, sizeof(int) * blockCap_));
    }
    S_.blockCap = blockCap_;
    // the previous step's copies out of the pinned buffers are complete:
    // every step ends with a stream synchronisation
    for (int r = 0; r < R_; r++) {
        const int o = hBilPrefix_[r];
        const size_t nq = queue_[r].size();
        if (nq == 0) continue;
        std::memcpy(hBlocks_ + o, queue_[r].data(), sizeof(AlensBlock) * nq);
        for (size_t b = 0; b < nq; b++) hBlockRep_[o + b] = r;
        CK(cudaMemcpyAsync(S_.blocks + o, hBlocks_ + o, sizeof(AlensBlock) * nq, cudaMemcpyHostToDevice, stream_));
        CK(cudaMemcpyAsync(S_.blockRep + o, hBlockRep_ + o, sizeof(int) * nq, cudaMemcpyHostToDevice, stream_));
    }
    CK(cudaMemcpyAsync(S_.bilPrefix, hBilPrefix_, sizeof(int) * (R_ + 1), cudaMemcpyHostToDevice, stream_));
    CK(cudaMemcpyAsync(S_.linkSlot0, hLinkSlot0_, sizeof(int) * R_, cudaMemcpyHostToDevice, stream_));
    nBilQueued_ = total;
}

// ---------------------------------------------------------- launch paths
int Engine::enqueueDetect() {
    DevState &S = S_;
    int n = 0;
    S.warmNet = (warm_ == ALENS_WARM_MLP && mlp_) ? 1 : 0;
    ensureSolverGrid();
    launch_step_clear(S, stream_);  // rawCount, errFlags and the per-cell / per-rod counters
    launch_prep(S, stream_);
    // branch 0: the Brownian velocities beside the binning and pair search
    CK(cudaEventRecord(forkEv_[0], stream_));
    CK(cudaStreamWaitEvent(side_, forkEv_[0], 0));
    launch_noise(S, side_);
    n += 3;
    if (S.nLinks > 0) {
        launch_link_blocks(S, stream_);
        n += 1;
    }
    n += launch_scan(S.cellCount, S.cellStart, S.nCells, S.scanTmp, stream_);
    launch_scatter(S, stream_);
    launch_pairs(S, stream_);  // screen + FP64 decision of the borderline candidates
    n += 3;
    if (S.nBnd > 0) {
        launch_boundary_pairs(S, stream_);
        n += 1;
    }
    n += launch_scan(S.pairCount, S.pairOff, S.nRods, S.scanTmp, stream_);
    // the per-replica ranges (from the pair offsets) on the same branch,
    // beside the canonical sort of the keys
    CK(cudaEventRecord(forkEv_[2], stream_));
    CK(cudaStreamWaitEvent(side_, forkEv_[2], 0));
    launch_ranges(S, side_);

    CK(cudaEventRecord(joinEv_[0], side_));
    n += launch_pair_sort(S, stream_);
    CK(cudaStreamWaitEvent(stream_, joinEv_[0], 0));
    launch_build(S, stream_);
    // branch 1: the mobility-weighted Jacobian beside the rod rows and the
    // operator structure
    CK(cudaEventRecord(forkEv_[1], stream_));
    CK(cudaStreamWaitEvent(side_, forkEv_[1], 0));
    launch_weights(S, side_);
    CK(cudaEventRecord(weightsDone_, side_));
    n += 3;
    // the learned warm start reads the constraints, the rod rows, the
    // weights and the per-rod coupling sums (formed by the row sort when
    // features are wanted), not the assembled operator: a branch of its own
    // beside the assembly, joined before the solve
    const bool warmSide = warm_ == ALENS_WARM_MLP && mlp_;
    const bool coupling = warmSide || S.feat;
    n += launch_rows(S, stream_, coupling ? weightsDone_ : nullptr);
    if (warmSide) {
        CK(cudaEventRecord(rowsDone_, stream_));
        CK(cudaStreamWaitEvent(side3_, rowsDone_, 0));
        launch_mlp_warm(S, mlp_->view(), side3_);
        CK(cudaEventRecord(warmJoin_, side3_));
        n += 1;
    }
    // the single-system solver's spatial row order (from the cell list and
    // the rod rows) on a third branch, beside the operator assembly;
    // computed whenever that form may run, so that the autotuner can try it
    // on the detected problem
    const bool order = S.fastPerm && !fastFailed_;
    if (order) {
        CK(cudaEventRecord(orderFork_, stream_));
        CK(cudaStreamWaitEvent(side2_, orderFork_, 0));
        n += launch_fast_order(S, side2_);
        CK(cudaEventRecord(orderJoin_, side2_));
    }
    n += launch_assemble(S, stream_, side_, joinEv_[1]);
    if (!warmSide && S.feat) {
        launch_mlp_features(S, stream_);
        n += 1;
    }
    if (warmSide) CK(cudaStreamWaitEvent(stream_, warmJoin_, 0));
    if (order) CK(cudaStreamWaitEvent(stream_, orderJoin_, 0));
    CK(cudaGetLastError());
    return n;
}

// ------------------------------------------------------------- autotuner
void Engine::applySolverConfig(int form, int clusterSize, int threads, int blocksPerSM, int minTiles) {
    invalidateGraph();
    solverBlocksPerSM_ = std::max(1, blocksPerSM);
    solverMinTiles_ = std::max(1, minTiles);
    S_.solveMinTiles = solverMinTiles_;
    solverGrid_ = std::min(solver_max_grid(precision_), numSM_ * solverBlocksPerSM_);
    if (solverGrid_ < 1) throw CudaFailure(cudaErrorLaunchOutOfResources, "solver occupancy");
    solverForm_ = form;
    clusterSize_ = (form == kFormGrid || form == kFormFast) ? 0 : clusterSize;
    if (form == kFormFast) {
        solverGrid_ = fast_solver_grid();
        if (solverGrid_ < 1) throw CudaFailure(cudaErrorLaunchOutOfResources, "fast solver occupancy");
        nClusters_ = 1;
        return;
    }
    if (form == kFormResident) {
        csm_set_threads(threads);
        nClusters_ = R_;
    } else if (form == kFormCluster) {
        const int act = cluster_max_active(clusterSize);
        nClusters_ = std::max(1, std::min(R_, act > 0 ? act : 1));
    } else {
        nClusters_ = 1;
    }
}

std::string Engine::autotune(int reps) {
    if (reps < 1) throw ApiError(ALENS_INVALID_ARG);
    AlensStepStats st{};
    const int rc = detect(&st);
    if (rc != ALENS_OK) throw ApiError(rc);
    // snapshot of the detected problem: every trial starts from it
    const int nc = hCtl_->totalCon;
    std::vector<void *> tmp;
    auto snap = [&](const void *src, size_t bytes) {
        void *p = nullptr;
        CK(cudaMalloc(&p, std::max<size_t>(bytes, 1)));
        tmp.push_back(p);
        CK(cudaMemcpyAsync(p, src, bytes, cudaMemcpyDeviceToDevice, stream_));
        return p;
    };
    void *sDyn = snap(S_.dyn, sizeof(RepDyn) * R_);
    void *sCtl = snap(S_.ctl, sizeof(DevCtl));
    void *sSt = snap(S_.st[1], sizeof(double2) * (size_t)nc);
    void *sSt32 = precision_ == ALENS_PREC_MIXED ? snap(S_.st32[1], sizeof(float2) * (size_t)nc) : nullptr;
    auto restore = [&]() {
        CK(cudaMemcpyAsync(S_.dyn, sDyn, sizeof(RepDyn) * R_, cudaMemcpyDeviceToDevice, stream_));
        CK(cudaMemcpyAsync(S_.ctl, sCtl, sizeof(DevCtl), cudaMemcpyDeviceToDevice, stream_));
        CK(cudaMemcpyAsync(S_.st[1], sSt, sizeof(double2) * (size_t)nc, cudaMemcpyDeviceToDevice, stream_));
        if (sSt32)
            CK(cudaMemcpyAsync(S_.st32[1], sSt32, sizeof(float2) * (size_t)nc, cudaMemcpyDeviceToDevice, stream_));
    };
    struct Cand {
        int form, cs, threads, bps, mt;
        double ms;
        bool ok;
    };
    std::vector<Cand> cands;
    // grid form: blocks per SM x minimum tiles per block (fewer, fuller
    // blocks make the per-pass barrier and the redundant reductions cheaper)
    for (int bps : {1, 2})
        for (int mt : {1, 2, 4, 8}) cands.push_back({kFormGrid, 0, 256, bps, mt, 0.0, false});
    if (precision_ == ALENS_PREC_MIXED && R_ == 1 && S_.fastPerm && !fastFailed_ && fast_solver_grid() > 0 &&
        nc <= fast_solver_capacity())
        cands.push_back({kFormFast, 0, 256, 1, 1, 0.0, false});
    if (precision_ == ALENS_PREC_MIXED) {
        const int maxCs = cluster_max_size();
        for (int cs : {16, 8, 4, 2})
            if (cs <= maxCs) cands.push_back({kFormCluster, cs, 512, 1, 1, 0.0, false});
        const int csmMax = csm_cluster_size(nullptr);
        for (int cs : {16, 8, 4, 2})
            for (int th : {256, 512})
                if (cs <= csmMax) cands.push_back({kFormResident, cs, th, 1, 1, 0.0, false});
    }
    ensureEvents();
    const int saveForm = solverForm_, saveCs = clusterSize_, saveBps = solverBlocksPerSM_, saveTh = csm_threads();
    const int saveMt = solverMinTiles_;
    const int saveNcl = nClusters_, saveGrid = solverGrid_;
    for (Cand &c : cands) {
        applySolverConfig(c.form, c.cs, c.threads, c.bps, c.mt);
        std::vector<double> t;
        bool ok = true;
        for (int r = 0; r < reps + 1 && ok; r++) {
            restore();
            CK(cudaEventRecord(events_[0], stream_));
            enqueueSolve(nullptr);
            CK(cudaEventRecord(events_[1], stream_));
            readBack();
            if (hCtl_->errFlags & (kErrSolverFit | kErrTimeout | kErrNaN)) ok = false;
            float ms = 0.0f;
            CK(cudaEventElapsedTime(&ms, events_[0], events_[1]));
            if (r > 0) t.push_back(ms);  // first run warms up
        }
        c.ok = ok && !t.empty();
        if (c.ok) {
            std::sort(t.begin(), t.end());
            c.ms = t[t.size() / 2];
        }
    }
    int best = -1;
    for (size_t i = 0; i < cands.size(); i++)
        if (cands[i].ok && (best < 0 || cands[i].ms < cands[best].ms)) best = (int)i;
    if (best >= 0) {
        const Cand &b = cands[best];
        applySolverConfig(b.form, b.cs, b.threads, b.bps, b.mt);
    } else {
        solverForm_ = saveForm;
        clusterSize_ = saveCs;
        solverBlocksPerSM_ = saveBps;
        solverMinTiles_ = saveMt;
        S_.solveMinTiles = saveMt;
        csm_set_threads(saveTh);
        nClusters_ = saveNcl;
        solverGrid_ = saveGrid;
    }
    restore();
    CK(cudaStreamSynchronize(stream_));
    for (void *p : tmp) cudaFree(p);
    // the detected problem stands; the next step detects again (the step is
    // repeatable: noise is keyed by the step index)
    haveDetect_ = true;
    haveSolve_ = false;
    static const char *names[] = {"grid", "cluster", "resident", "fast"};
    std::string js = "{\"constraints\": " + std::to_string(nc) + ", \"candidates\": [";
    for (size_t i = 0; i < cands.size(); i++) {
        const Cand &c = cands[i];
        char buf[256];
        snprintf(buf, sizeof(buf),
                 "%s{\"form\": \"%s\", \"cluster\": %d, \"threads\": %d, \"blocks_per_sm\": %d, "
                 "\"min_tiles\": %d, \"ms\": %s}",
                 i ? ", " : "", names[c.form], c.cs, c.form == kFormResident ? c.threads : (c.form == kFormCluster ? 512 : 256),
                 c.bps, c.mt, c.ok ? std::to_string(c.ms).c_str() : "null");
        js += buf;
    }
    js += "], \"chosen\": " + std::to_string(best) + "}";
    return js;
}

// ------------------------------------------------------ learned warm start
void Engine::attachMlp(MlpModel *m) {
    CK(cudaStreamSynchronize(stream_));
    invalidateGraph();
    mlp_ = m;
}

void Engine::setFeatureCapture(bool on) {
    if (on == capture_) return;
    CK(cudaStreamSynchronize(stream_));
    invalidateGraph();
    capture_ = on;
    captured_ = false;
    if (!dirty_) {
        // the constraint buffers are reallocated with (or without) the
        // feature rows; warm-start keys of the last step are kept
        allocConstraints(S_.cap, true);
    }
}

// Appends the last completed step's collision constraints (features and
// converged multipliers in overlap units) to the model's dataset.
long long Engine::collect(MlpModel *m) {
    if (!m) throw ApiError(ALENS_INVALID_ARG);
    if (!captured_ || !S_.feat) throw ApiError(ALENS_NOT_READY);
    long long total = 0;
    for (int r = 0; r < R_; r++) {
        const RepDyn &d = hDyn_[r];
        const long long n = d.collEnd - d.collStart;
        const long long add = m->reserve(n);
        if (add <= 0) break;
        launch_mlp_append(S_, d.conStart, (int)add, m->dsFeatAt(m->datasetSize()), m->dsLabelAt(m->datasetSize()),
                          stream_);
        CK(cudaGetLastError());
        m->commitRows(add);
        total += add;
    }
    CK(cudaStreamSynchronize(stream_));
    return total;
}

int Engine::getFeatures(int rep, int cap, float *feat, float *scale) {
    if (rep < 0 || rep >= R_) throw ApiError(ALENS_INVALID_ARG);
    if (!captured_ || !S_.feat) throw ApiError(ALENS_NOT_READY);
    const RepDyn &d = hDyn_[rep];
    const int n = d.collEnd - d.collStart;
    if (cap < n) throw ApiError(ALENS_CAPACITY);
    if (n > 0) {
        if (feat)
            CK(cudaMemcpyAsync(feat, S_.feat + (size_t)kMlpIn * d.conStart, sizeof(float) * kMlpIn * n,
                               cudaMemcpyDeviceToHost, stream_));
        if (scale)
            CK(cudaMemcpyAsync(scale, S_.fscale + d.conStart, sizeof(float) * n, cudaMemcpyDeviceToHost, stream_));
        CK(cudaStreamSynchronize(stream_));
    }
    return n;
}

void Engine::ensureSolverGrid() {
    if (solverGrid_ > 0) return;
    const int maxg = solver_max_grid(precision_);
    solverGrid_ = std::min(maxg, numSM_ * solverBlocksPerSM_);
    if (solverGrid_ < 1) throw CudaFailure(cudaErrorLaunchOutOfResources, "solver occupancy");
    solverForm_ = kFormGrid;
    if (precision_ != ALENS_PREC_MIXED) return;
    // one system: the single-system form unless another form was requested
    if (R_ == 1 && (formRequest_ < 0 || formRequest_ == kFormFast) && clusterSize_ <= 0 && !fastFailed_ &&
        S_.fastPerm) {
        const int fg = fast_solver_grid();
        if (fg > 0) {
            solverForm_ = kFormFast;
            solverGrid_ = fg;
            clusterSize_ = 0;
            return;
        }
    }
    // FP32 solver form.  Measured on GB300 (20,000-rod layer, ~21,000
    // constraints): grid 9.6 us per pass, cluster-resident 14 us (random
    // 8-byte distributed-shared-memory gathers sustain ~0.4 loads per cycle
    // per SM), cluster with global iterates 16 us; so the grid form is the
    // default and the cluster forms are chosen on request (autotuner)
    const int csmCs = csm_cluster_size(nullptr);
    const bool residentOk = csmCs > 0 && !residentFailed_;
    if (formRequest_ == kFormResident && residentOk) {
        int cs = clusterSize_ > 0 ? std::min(clusterSize_, csmCs) : csmCs;
        // ensembles: clusters of 4 CTAs, as many as can be co-resident
        if (R_ > 1 && clusterSize_ <= 0) cs = std::min(cs, 4);
        // clusters never wait on one another: one per replica, the hardware
        // schedules them as SMs free up
        solverForm_ = kFormResident;
        clusterSize_ = cs;
        nClusters_ = R_;
        return;
    }
    if (formRequest_ == kFormGrid) {
        clusterSize_ = 0;
        return;
    }
    if (formRequest_ == kFormCluster && clusterSize_ == 0) clusterSize_ = -1;
    if (clusterSize_ < 0 && R_ == 1 && formRequest_ != kFormCluster) clusterSize_ = 0;
    if (clusterSize_ != 0) {
        solverForm_ = kFormCluster;
        const int maxCs = cluster_max_size();
        int cs = clusterSize_ > 0 ? std::min(clusterSize_, maxCs) : maxCs;
        // ensembles: one cluster per replica, at most the co-resident count
        if (R_ > 1) {
            while (cs > 1 && cluster_max_active(cs) < R_) cs /= 2;
        }
        const int act = cluster_max_active(cs);
        clusterSize_ = cs;
        nClusters_ = std::max(1, std::min(R_, act > 0 ? act : 1));
    }
}

int Engine::enqueueSolve(cudaEvent_t *ev, bool finish) {
    ensureSolverGrid();
    int n = 0;
    CK(launch_solve(S_, solverGrid_, precision_, waitTimeoutNs_, stream_, ev, &n, solverForm_,
                    clusterSize_ > 0 ? clusterSize_ : 0, nClusters_, finish));
    return n;
}

int Engine::enqueueAdvance() {
    launch_advance(S_, stream_);
    CK(cudaGetLastError());
    return 1;
}

void Engine::invalidateGraph() {
    if (graphExec_) {
        cudaGraphExecDestroy(graphExec_);
        graphExec_ = nullptr;
    }
}

bool Engine::buildGraph() {
    ensureSolverGrid();
    cudaGraph_t g = nullptr;
    if (cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    bool ok = true;
    int n = 0;
    try {
        n += enqueueDetect();
        n += enqueueSolve(nullptr);
        n += enqueueAdvance();
    } catch (...) {
        ok = false;
    }
    cudaError_t e = cudaStreamEndCapture(stream_, &g);
    if (!ok || e != cudaSuccess || !g) {
        cudaGetLastError();
        if (g) cudaGraphDestroy(g);
        return false;
    }
    e = cudaGraphInstantiate(&graphExec_, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        cudaGetLastError();
        graphExec_ = nullptr;
        return false;
    }
    graphLaunches_ = n;
    return true;
}

void Engine::readBack() {
    CK(cudaMemcpyAsync(hCtl_, S_.ctl, sizeof(DevCtl), cudaMemcpyDeviceToHost, stream_));
    CK(cudaMemcpyAsync(hDyn_, S_.dyn, sizeof(RepDyn) * R_, cudaMemcpyDeviceToHost, stream_));
    CK(cudaStreamSynchronize(stream_));
}

// Returns true if the constraint buffers were grown (the step must rerun).
bool Engine::handleOverflow() {
    if (!(hCtl_->errFlags & kErrOverflow)) return false;
    const long long needColl =
        std::max<long long>(std::max<long long>(hCtl_->rawCount, hCtl_->borderCount), hCtl_->totalColl);
    const long long need = needColl + nBilQueued_;
    lastNeeded_ = need;
    CK(cudaStreamSynchronize(stream_));
    if (need > S_.cap || hCtl_->nTiles > S_.tileCap) {
        if (fixedCap_ > 0 || need > kMaxConstraints) throw ApiError(ALENS_CAPACITY);
        invalidateGraph();
        allocConstraints((int)std::min<long long>(need + need / 2 + 1024, kMaxConstraints), true);
        return true;
    }
    if (hCtl_->totalNnz > S_.nnzCap) {
        invalidateGraph();
        allocOperator((long long)hCtl_->totalNnz * 3 / 2 + 4096);
        return true;
    }
    throw ApiError(ALENS_CAPACITY);
}

// A step that outgrew the cluster-resident solver: use the grid form from
// now on for this context.  Returns true if the step must be rerun.
bool Engine::handleSolverFit() {
    if (!(hCtl_->errFlags & kErrSolverFit)) return false;
    CK(cudaStreamSynchronize(stream_));
    invalidateGraph();
    if (solverForm_ == kFormFast)
        fastFailed_ = true;
    else
        residentFailed_ = true;
    solverGrid_ = 0;
    clusterSize_ = -1;
    return true;
}

int Engine::collectStats(int stage) {
    int status = ALENS_OK;
    const int fl = hCtl_->errFlags;
    if (fl & kErrNaN) status = ALENS_NAN_DETECTED;
    if (fl & kErrTimeout) status = ALENS_TIMEOUT;
    AlensStepStats tot{};
    tot.step = stepCount_;
    tot.converged = 1;
    for (int r = 0; r < R_; r++) {
        const RepDyn &d = hDyn_[r];
        AlensStepStats &s = repStats_[r];
        s = AlensStepStats{};
        s.step = stepCount_;
        s.nRods = rods_[r].n;
        s.nCollision = d.collEnd - d.collStart;
        s.nBilateral = hBilPrefix_[r + 1] - hBilPrefix_[r];
        if (stage >= 1) {
            if (precision_ == ALENS_PREC_MIXED) {
                s.iterations = d.refineIter;
                s.refineIterations = d.iter;
            } else {
                s.iterations = d.iter;
            }
            s.residual = d.res;
            s.converged = d.converged;
            s.status = d.status;
            if (d.status == ALENS_NOT_CONVERGED && status == ALENS_OK) status = ALENS_NOT_CONVERGED;
            if (d.status == ALENS_NAN_DETECTED) status = ALENS_NAN_DETECTED;
        }
        tot.nRods += s.nRods;
        tot.nCollision += s.nCollision;
        tot.nBilateral += s.nBilateral;
        tot.iterations = std::max(tot.iterations, s.iterations);
        tot.refineIterations = std::max(tot.refineIterations, s.refineIterations);
        tot.residual = std::max(tot.residual, s.residual);
        tot.converged = tot.converged && (stage < 1 || s.converged);
    }
    tot.status = status;
    last_ = tot;
    return status;
}

void Engine::ensureEvents() {
    if (events_[0]) return;
    for (auto &e : events_) CK(cudaEventCreate(&e));
}

void Engine::recordStageTimes() {
    float t[5] = {0, 0, 0, 0, 0};
    // events: 0 detect start, 1 detect end / solve start, 2 main end,
    // 3 refine start, 4 refine end, 5 advance end
    CK(cudaEventElapsedTime(&t[0], events_[0], events_[1]));
    CK(cudaEventElapsedTime(&t[1], events_[1], events_[2]));
    if (precision_ == ALENS_PREC_MIXED) CK(cudaEventElapsedTime(&t[2], events_[3], events_[4]));
    CK(cudaEventElapsedTime(&t[3], events_[4], events_[5]));
    CK(cudaEventElapsedTime(&t[4], events_[0], events_[5]));
    for (int i = 0; i < 5; i++) stageMs_[i] = t[i];
}

// Enqueues one attempt of a full step (graph replay or direct launches);
// returns whether the direct-launch path ran (stage timing).
bool Engine::stepLaunch() {
    uploadBlocks();
    bool launched = false;
    if (useGraph_ && !stageTiming_) {
        if (!graphExec_ && !graphFailed_) {
            if (!buildGraph()) graphFailed_ = true;
        }
        if (graphExec_) {
            CK(cudaGraphLaunch(graphExec_, stream_));
            launches_ += graphLaunches_;
            launched = true;
        }
    }
    if (!launched) {
        if (stageTiming_) {
            ensureEvents();
            CK(cudaEventRecord(events_[0], stream_));
            launches_ += enqueueDetect();
            // solve records events 1..4 (start, main end, refine start, refine end)
            launches_ += enqueueSolve(&events_[1]);
            launches_ += enqueueAdvance();
            CK(cudaEventRecord(events_[5], stream_));
        } else {
            launches_ += enqueueDetect();
            launches_ += enqueueSolve(nullptr);
            launches_ += enqueueAdvance();
        }
    }
    return !launched;
}

// Reads back the attempt's results.  Returns kStepRetry when the buffers
// were regrown or the solver form changed (the step is repeatable and must
// be run again), else the step's status.
int Engine::stepFinish(AlensStepStats *out, bool direct) {
    readBack();
    if (handleOverflow()) return kStepRetry;
    if (handleSolverFit()) return kStepRetry;
    if (stageTiming_ && direct) recordStageTimes();
    const int status = collectStats(2);
    if (status == ALENS_OK || status == ALENS_NOT_CONVERGED) {
        for (auto &q : queue_) q.clear();
        captured_ = S_.feat != nullptr;
        stepCount_++;
        last_.step = stepCount_ - 1;
        prevCountHost_ = hCtl_->totalColl;
    }
    haveDetect_ = haveSolve_ = false;
    if (out) *out = last_;
    return status;
}

int Engine::step(AlensStepStats *out) {
    finalize();
    for (int attempt = 0; attempt < 8; attempt++) {
        const bool direct = stepLaunch();
        const int rc = stepFinish(out, direct);
        if (rc != kStepRetry) return rc;
    }
    throw ApiError(ALENS_CAPACITY);
}

void Engine::setWaitLimit(unsigned long long timeoutNs, int stallBarriers) {
    if (stallBarriers != 0 && stallBarriers != 1) throw ApiError(ALENS_INVALID_ARG);
    if (haveDetect_ || haveSolve_) throw ApiError(ALENS_NOT_READY);
    CK(cudaStreamSynchronize(stream_));
    invalidateGraph();
    waitTimeoutNs_ = timeoutNs ? timeoutNs : kBarrierTimeoutNs;
    stallBarriers_ = stallBarriers;
    S_.barrierExtra = stallBarriers_;
}

int Engine::detect(AlensStepStats *out) {
    finalize();
    for (int attempt = 0; attempt < 8; attempt++) {
        uploadBlocks();
        launches_ += enqueueDetect();
        readBack();
        if (handleOverflow()) continue;
        const int status = collectStats(0);
        haveDetect_ = status == ALENS_OK;
        haveSolve_ = false;
        if (out) *out = last_;
        return status;
    }
    throw ApiError(ALENS_CAPACITY);
}

int Engine::solve(AlensStepStats *out) {
    if (!haveDetect_) throw ApiError(ALENS_NOT_READY);
    launches_ += enqueueSolve(nullptr, true);
    readBack();
    if (handleSolverFit()) {
        // the detect results are intact: clear the flag and solve in grid form
        CK(cudaMemsetAsync(&S_.ctl->errFlags, 0, sizeof(int), stream_));
        launches_ += enqueueSolve(nullptr, true);
        readBack();
    }
    const int status = collectStats(1);
    haveSolve_ = (status == ALENS_OK || status == ALENS_NOT_CONVERGED);
    if (out) *out = last_;
    return status;
}

void Engine::setStepCount(long long s) {
    if (s < 0) throw ApiError(ALENS_INVALID_ARG);
    if (haveDetect_ || haveSolve_) throw ApiError(ALENS_NOT_READY);
    stepCount_ = s;
    if (dirty_ || !S_.ctl) return;  // finalize() writes it with the device state
    CK(cudaStreamSynchronize(stream_));
    hCtl_->step = s;
    CK(cudaMemcpyAsync(&S_.ctl->step, &hCtl_->step, sizeof(long long), cudaMemcpyHostToDevice, stream_));
    CK(cudaStreamSynchronize(stream_));
}

int Engine::advance(AlensStepStats *out) {
    if (!haveSolve_) throw ApiError(ALENS_NOT_READY);
    launches_ += enqueueAdvance();
    readBack();
    for (auto &q : queue_) q.clear();
    captured_ = S_.feat != nullptr;
    stepCount_++;
    prevCountHost_ = hCtl_->totalColl;
    haveDetect_ = haveSolve_ = false;
    if (out) *out = last_;
    return ALENS_OK;
}

void Engine::replicaStats(int rep, AlensStepStats *out) const {
    if (rep < 0 || rep >= R_ || !out) throw ApiError(ALENS_INVALID_ARG);
    *out = repStats_[rep];
}

void Engine::numConstraints(int rep, int *nColl, int *nBil) const {
    if (rep < 0 || rep >= R_) throw ApiError(ALENS_INVALID_ARG);
    if (nColl) *nColl = hDyn_[rep].collEnd - hDyn_[rep].collStart;
    if (nBil) *nBil = hBilPrefix_[rep + 1] - hBilPrefix_[rep];
}

void Engine::getConstraints(int rep, int cap, int32_t *ii, int32_t *jj, int32_t *img, double *d0,
                            double *gam, double *jac) {
    if (rep < 0 || rep >= R_) throw ApiError(ALENS_INVALID_ARG);
    if (dirty_) throw ApiError(ALENS_NOT_READY);
    const RepDyn &d = hDyn_[rep];
    const int n = d.nCon;
    if (cap < n) throw ApiError(ALENS_CAPACITY);
    if (n == 0) return;
    const int k0 = d.conStart;
    auto cp = [&](void *dst, const void *src, size_t bytes) {
        CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, stream_));
    };
    if (ii) cp(ii, S_.conI + k0, sizeof(int) * n);
    if (jj) cp(jj, S_.conJ + k0, sizeof(int) * n);
    if (img) cp(img, S_.conImg + k0, sizeof(int) * n);
    if (d0) cp(d0, S_.phi0 + k0, sizeof(double) * n);
    if (gam) cp(gam, S_.gamma + k0, sizeof(double) * n);
    if (jac) cp(jac, S_.jac + 12 * (size_t)k0, sizeof(double) * 12 * n);
    CK(cudaStreamSynchronize(stream_));
    const int off = hostPar_[rep].rodOffset;
    for (int k = 0; k < n; k++) {
        if (ii) ii[k] -= off;
        if (jj && jj[k] >= 0) jj[k] -= off;
    }
}

void Engine::getConstraintPoints(int rep, int cap, double *lab) {
    if (rep < 0 || rep >= R_) throw ApiError(ALENS_INVALID_ARG);
    if (dirty_) throw ApiError(ALENS_NOT_READY);
    const RepDyn &d = hDyn_[rep];
    if (cap < d.nCon) throw ApiError(ALENS_CAPACITY);
    if (d.nCon == 0 || !lab) return;
    CK(cudaMemcpyAsync(lab, S_.lab + 6 * (size_t)d.conStart, sizeof(double) * 6 * (size_t)d.nCon,
                       cudaMemcpyDeviceToHost, stream_));
    CK(cudaStreamSynchronize(stream_));
}

void Engine::getOperator(int rep, int capNnz, int *nnz, int32_t *rowPtr, int32_t *cols, double *vals,
                         double *q, double *cinv, double *lowerBound, double *gamma0) {
    if (rep < 0 || rep >= R_) throw ApiError(ALENS_INVALID_ARG);
    if (dirty_) throw ApiError(ALENS_NOT_READY);
    const RepDyn &d = hDyn_[rep];
    const int n = d.nCon, k0 = d.conStart;
    std::vector<int> ptr(n + 1);
    if (n > 0) CK(cudaMemcpy(ptr.data(), S_.aptr + k0, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost));
    else ptr[0] = 0;
    const int e0 = ptr[0], total = ptr[n] - ptr[0];
    if (nnz) *nnz = total;
    if ((cols || vals) && capNnz < total) throw ApiError(ALENS_CAPACITY);
    if (rowPtr)
        for (int k = 0; k <= n; k++) rowPtr[k] = ptr[k] - e0;
    if ((cols || vals) && total > 0) {
        std::vector<int4> ent(total);
        CK(cudaMemcpy(ent.data(), S_.aent + e0, sizeof(int4) * total, cudaMemcpyDeviceToHost));
        for (int e = 0; e < total; e++) {
            if (cols) cols[e] = ent[e].x - k0;
            if (vals) {
                const unsigned long long bits =
                    ((unsigned long long)(unsigned)ent[e].w << 32) | (unsigned long long)(unsigned)ent[e].z;
                std::memcpy(&vals[e], &bits, 8);
            }
        }
    }
    if (n > 0) {
        if (q) CK(cudaMemcpy(q, S_.q + k0, sizeof(double) * n, cudaMemcpyDeviceToHost));
        if (cinv) CK(cudaMemcpy(cinv, S_.cinv + k0, sizeof(double) * n, cudaMemcpyDeviceToHost));
        if (lowerBound) CK(cudaMemcpy(lowerBound, S_.lb + k0, sizeof(double) * n, cudaMemcpyDeviceToHost));
        if (gamma0) CK(cudaMemcpy(gamma0, S_.gamma + k0, sizeof(double) * n, cudaMemcpyDeviceToHost));
    }
}

void Engine::conStress(int rep, double *out9) {
    if (rep < 0 || rep >= R_ || !out9) throw ApiError(ALENS_INVALID_ARG);
    if (dirty_) throw ApiError(ALENS_NOT_READY);
    launch_stress(S_, stream_);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(out9, S_.stress + 9 * (size_t)rep, sizeof(double) * 9, cudaMemcpyDeviceToHost, stream_));
    CK(cudaStreamSynchronize(stream_));
}

// ------------------------------------------------------ protein kinetics
namespace {

constexpr double kPiKmc = 3.141592653589793;

bool finite_nonneg(double v) { return std::isfinite(v) && v >= 0.0; }

// 4 pi int_0^inf r^2 exp(-a (r - c)^2) dr in closed form (lookupType 0:
// c = ell0 + D), the bind volume of Protein/ProteinModel.md
double bind_volume(double a, double c) {
    const double G = 0.5 * std::sqrt(kPiKmc / a) * (1.0 + std::erf(c * std::sqrt(a)));
    const double e = std::exp(-(a * (c * c)));
    return 4.0 * kPiKmc * ((c * e) / (2.0 * a) + G * (1.0 / (2.0 * a) + c * c));
}

// The species' rates with dt folded in (ProteinType::readFromYaml unit
// conversion, Protein/ProteinType.hpp:121-127; fixedEnd0 rule of
// Protein/ProteinModel.md; factors of Protein/ProteinData.hpp:90-140).
KmcType make_kmc_type(const AlensProteinType &in, double KBT, double D, double dt) {
    KmcType T;
    std::memset(&T, 0, sizeof(T));
    double koS[2] = {in.ko_s[0], in.ko_s[1]}, koD[2] = {in.ko_d[0], in.ko_d[1]};
    if (in.fixedEnd0) {
        koS[0] = 0.0;
        koD[0] = 0.0;
    }
    const double Ka[2] = {in.Ka[0] / 602.0, in.Ka[1] / 602.0};
    const double Ke[2] = {in.useBindVol ? in.Ke[0] / 602.0 : in.Ke[0], in.useBindVol ? in.Ke[1] / 602.0 : in.Ke[1]};
    T.ell0 = in.freeLength;
    T.lookup = in.lookupType;
    T.c = in.lookupType == 0 ? in.freeLength + D : in.freeLength;
    T.A = ((1.0 - in.lambda) * in.kappa) / (2.0 * KBT);
    T.w = 6.0 / std::sqrt(T.A);
    T.rOuter = (in.freeLength + D) + T.w;
    T.Ads = (in.lambda * in.kappa) / (2.0 * KBT);
    const double rd = std::sqrt((6.0 * in.diffUnbound) * dt);
    T.rcap = in.rc > rd ? in.rc : rd;
    T.PtoAP = in.PtoAPratio;
    const double vol = 3.0 / (4.0 * kPiKmc * ((T.rcap * T.rcap) * T.rcap));
    const double Vb = in.useBindVol ? bind_volume(T.A, T.c) : 1.0;
    for (int e = 0; e < 2; e++) {
        T.usCoef[e] = (((koS[e] * Ka[e]) * in.eps) * vol) * dt;
        T.suProb[e] = koS[e] * dt;
        T.sdCoef[e] = (((koD[e] * Ke[e]) * in.eps) * dt) / Vb;
        T.koD[e] = koD[e];
    }
    T.dt = dt;
    T.kappa = in.kappa;
    T.rcapf = (float)T.rcap;
    T.rOuterf = (float)T.rOuter;
    T.wf = (float)T.w;
    T.Af = (float)T.A;
    T.cf = (float)T.c;
    for (int e = 0; e < 2; e++) {
        T.usCoeff[e] = (float)T.usCoef[e];
        T.suProbf[e] = (float)T.suProb[e];
        T.sdCoeff[e] = (float)T.sdCoef[e];
    }
    const float r = (float)in.PtoAPratio;
    T.prefPar = r < 1.0f ? r : 1.0f;
    T.prefAnti = r > 1.0f ? 1.0f / r : 1.0f;
    T.Df = (float)D;
    T.walkOff = in.walkOff ? 1 : 0;
    T.fstall = in.fstall;
    for (int e = 0; e < 2; e++) {
        T.vdrag[e] = in.vdrag[e] ? 1 : 0;
        T.vmax[e] = in.vmax[e];
        T.vmaxAP[e] = in.vmaxAP[e];
        T.diffS[e] = std::sqrt((dt * in.diffBoundS[e]) * 2.0);
        T.diffD[e] = std::sqrt((dt * in.diffBoundD[e]) * 2.0);
        T.dragD[e] = in.diffBoundD[e];
    }
    T.diffU = std::sqrt((dt * in.diffUnbound) * 2.0);
    T.KBT = KBT;
    return T;
}

}  // namespace

void Engine::setProteinTypes(int n, const AlensProteinType *t, double KBT, double D) {
    if (n < 0 || (n > 0 && !t) || !(KBT > 0.0) || !std::isfinite(KBT) || !finite_nonneg(D))
        throw ApiError(ALENS_INVALID_ARG);
    for (int k = 0; k < n; k++) {
        const AlensProteinType &p = t[k];
        bool ok = (p.lookupType == 0 || p.lookupType == 1) && std::isfinite(p.kappa) && p.kappa > 0.0 && std::isfinite(p.lambda) &&
                  p.lambda >= 0.0 && p.lambda < 1.0 && finite_nonneg(p.freeLength) && std::isfinite(p.rc) &&
                  p.rc > 0.0 && finite_nonneg(p.eps) && finite_nonneg(p.diffUnbound) &&
                  std::isfinite(p.PtoAPratio) && p.PtoAPratio > 0.0;
        ok = ok && std::isfinite(p.fstall) && p.fstall != 0.0;
        for (int e = 0; e < 2; e++)
            ok = ok && finite_nonneg(p.ko_s[e]) && finite_nonneg(p.ko_d[e]) && finite_nonneg(p.Ka[e]) &&
                 finite_nonneg(p.Ke[e]) && std::isfinite(p.vmax[e]) && std::isfinite(p.vmaxAP[e]) &&
                 finite_nonneg(p.diffBoundS[e]) && finite_nonneg(p.diffBoundD[e]);
        if (!ok) throw ApiError(ALENS_INVALID_ARG);
    }
    syncProteinsToHost();
    for (const auto &v : prot_)
        for (const AlensProtein &p : v)
            if (p.type >= n) throw ApiError(ALENS_INVALID_ARG);
    ptypes_.assign(t, t + n);
    kmcKBT_ = KBT;
    kmcD_ = D;
    springsDirty_ = nProt_ > 0 || protUpload_;  // rest lengths and stiffness may change
}

void Engine::setProteins(int rep, int n, const AlensProtein *p) {
    if (rep < 0 || rep >= R_ || n < 0 || (n > 0 && !p)) throw ApiError(ALENS_INVALID_ARG);
    if (ptypes_.empty() && n > 0) throw ApiError(ALENS_NOT_READY);
    if (n > 0 && !rods_[rep].set) throw ApiError(ALENS_NOT_READY);
    if (haveDetect_ || haveSolve_) throw ApiError(ALENS_NOT_READY);
    const int nr = rods_[rep].n;
    for (int k = 0; k < n; k++) {
        const AlensProtein &q = p[k];
        if (q.type < 0 || q.type >= (int)ptypes_.size()) throw ApiError(ALENS_INVALID_ARG);
        int nb = 0;
        for (int e = 0; e < 2; e++) {
            if (q.idBind[e] == -1) continue;
            if (q.idBind[e] < 0 || q.idBind[e] >= nr || !std::isfinite(q.distBind[e])) throw ApiError(ALENS_INVALID_ARG);
            nb++;
        }
        if (nb == 0 && !(std::isfinite(q.pos[0]) && std::isfinite(q.pos[1]) && std::isfinite(q.pos[2])))
            throw ApiError(ALENS_INVALID_ARG);
    }
    int total = 0;
    for (int r = 0; r < R_; r++) total += r == rep ? n : (int)prot_[r].size();
    if (total > (4 << 20) - 1) throw ApiError(ALENS_INVALID_ARG);
    syncProteinsToHost();
    const size_t before = prot_[rep].size();
    prot_[rep].assign(p, p + n);
    protUpload_ = true;
    if ((size_t)n != before) linksDirty_ = true;  // one link row per protein
}

void Engine::getProteins(int rep, int cap, int *n, AlensProtein *out) {
    if (rep < 0 || rep >= R_ || !n || cap < 0) throw ApiError(ALENS_INVALID_ARG);
    syncProteinsToHost();
    const int m = (int)prot_[rep].size();
    *n = m;
    if (cap < m) throw ApiError(ALENS_CAPACITY);
    if (m > 0) {
        if (!out) throw ApiError(ALENS_INVALID_ARG);
        std::memcpy(out, prot_[rep].data(), sizeof(AlensProtein) * m);
    }
}

void Engine::syncProteinsToHost() {
    if (!protDevNewer_) return;
    CK(cudaStreamSynchronize(stream_));
    std::vector<AlensProtein> all(nProt_);
    if (nProt_ > 0) CK(cudaMemcpy(all.data(), K_.prot, sizeof(AlensProtein) * nProt_, cudaMemcpyDeviceToHost));
    int o = 0;
    for (int r = 0; r < R_; r++) {
        std::copy(all.begin() + o, all.begin() + o + prot_[r].size(), prot_[r].begin());
        o += (int)prot_[r].size();
    }
    protDevNewer_ = false;
}

void Engine::uploadProteins() {
    if (!protUpload_) return;
    CK(cudaStreamSynchronize(stream_));
    int total = 0;
    for (int r = 0; r < R_; r++) total += (int)prot_[r].size();
    freeGroup(protAllocs_);
    K_.prot = alloc<AlensProtein>(protAllocs_, total);
    K_.protRep = alloc<int>(protAllocs_, total);
    K_.dFlag = alloc<int>(protAllocs_, total + 1);
    K_.dScan = alloc<int>(protAllocs_, total + 1);
    K_.task = alloc<float4>(protAllocs_, 4 * (size_t)total);
    std::vector<AlensProtein> all;
    std::vector<int> rep;
    all.reserve(total);
    rep.reserve(total);
    for (int r = 0; r < R_; r++) {
        all.insert(all.end(), prot_[r].begin(), prot_[r].end());
        rep.insert(rep.end(), prot_[r].size(), r);
    }
    if (total > 0) {
        CK(cudaMemcpy(K_.prot, all.data(), sizeof(AlensProtein) * total, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(K_.protRep, rep.data(), sizeof(int) * total, cudaMemcpyHostToDevice));
    }
    nProt_ = total;
    K_.nProt = total;
    protUpload_ = false;
    protDevNewer_ = false;
    springsDirty_ = true;
}

// Species tables per replica, the binding grid of every replica (cell edge
// at least the largest rod half-length plus the largest capture distance)
// and the device buffers they size.  Needs the rods on the device.
void Engine::prepareKmc() {
    const int nt = (int)ptypes_.size();
    std::vector<KmcType> types((size_t)R_ * std::max(nt, 1));
    std::vector<KmcRep> reps(R_);
    int cells = 0, protOff = 0, userOff = 0;
    for (int r = 0; r < R_; r++) {
        const RepParams &P = hostPar_[r];
        double reachT = 0.0;
        for (int k = 0; k < nt; k++) {
            KmcType &T = types[(size_t)r * nt + k];
            T = make_kmc_type(ptypes_[k], kmcKBT_, kmcD_, cfg_[r].dt);
            reachT = std::max(reachT, std::max(T.rcap, T.rOuter));
        }
        const double reach = rods_[r].hlMax + reachT;
        KmcRep &Q = reps[r];
        std::memset(&Q, 0, sizeof(Q));
        for (int d = 0; d < 3; d++) {
            Q.lo[d] = P.lo[d];
            Q.hi[d] = P.hi[d];
            Q.L[d] = P.L[d];
            Q.pbc[d] = P.pbc[d];
            // one nearest periodic image within the reach
            if (P.pbc[d] && !prot_[r].empty() && !(P.L[d] >= 2.0 * reach)) throw ApiError(ALENS_INVALID_ARG);
            const double f = reach > 0.0 ? std::floor(P.L[d] / reach) : 1.0;
            Q.ncell[d] = f < 1.0 ? 1 : (f > 512.0 ? 512 : (int)f);
        }
        // at most max(64, 2 n) cells; a periodic side keeps two cells at
        // least (with one, an offset would not name one image)
        const long long limit = std::max<long long>(64, 2LL * rods_[r].n);
        while ((long long)Q.ncell[0] * Q.ncell[1] * Q.ncell[2] > limit) {
            int d = -1;
            for (int e = 0; e < 3; e++)
                if (Q.ncell[e] > (Q.pbc[e] ? 2 : 1) && (d < 0 || Q.ncell[e] > Q.ncell[d])) d = e;
            if (d < 0) break;
            Q.ncell[d] = std::max(Q.pbc[d] ? 2 : 1, Q.ncell[d] / 2);
        }
        for (int d = 0; d < 3; d++) {
            Q.cellsz[d] = Q.L[d] / Q.ncell[d];
            Q.cellszf[d] = (float)Q.cellsz[d];
        }
        Q.cellOffset = cells;
        cells += Q.ncell[0] * Q.ncell[1] * Q.ncell[2];
        Q.rodOffset = P.rodOffset;
        Q.nRods = rods_[r].n;
        Q.protOffset = protOff;
        Q.nProt = (int)prot_[r].size();
        protOff += Q.nProt;
        Q.userLinks = (int)links_[r].I.size();
        userOff += Q.userLinks;
        Q.seed = cfg_[r].rngSeed;
    }
    if (cells > (4 << 20) - 1) throw ApiError(ALENS_INVALID_ARG);
    const int nrod = S_.nRods;
    bool kmcAllocsFresh = false;
    if (kmcFixedAllocs_.empty() || kmcTypeCap_ < (int)types.size()) {
        kmcAllocsFresh = true;
        CK(cudaStreamSynchronize(stream_));
        freeGroup(kmcFixedAllocs_);
        kmcTypeCap_ = (int)types.size();
        K_.types = alloc<KmcType>(kmcFixedAllocs_, kmcTypeCap_);
        K_.rep = alloc<KmcRep>(kmcFixedAllocs_, R_);
        K_.stats = alloc<int>(kmcFixedAllocs_, 9 * (size_t)R_ + 1);
        K_.dCount = K_.stats + 8 * R_;
        K_.err = K_.stats + 9 * R_;
    }
    if (cells + 1 > kmcCellCap_ || nrod > kmcRodCap_) {
        CK(cudaStreamSynchronize(stream_));
        freeGroup(kmcAllocs_);
        kmcCellCap_ = std::max(cells + 1, kmcCellCap_);
        kmcRodCap_ = std::max(nrod, kmcRodCap_);
        K_.cellCount = alloc<int>(kmcAllocs_, kmcCellCap_);
        K_.cellStart = alloc<int>(kmcAllocs_, kmcCellCap_);
        K_.cellCursor = alloc<int>(kmcAllocs_, kmcCellCap_);
        K_.cellRod = alloc<int>(kmcAllocs_, kmcRodCap_);
        K_.rodC = alloc<KDouble4>(kmcAllocs_, kmcRodCap_);
        K_.rodA = alloc<KDouble4>(kmcAllocs_, kmcRodCap_);
        K_.cellRel = alloc<float4>(kmcAllocs_, kmcRodCap_);
        K_.cellAx = alloc<float4>(kmcAllocs_, kmcRodCap_);
    }
    // upload the tables when they changed (the host copies stay alive until
    // the next upload, which first waits for the stream)
    const bool sameT = kmcTypesUp_.size() == types.size() &&
                       std::memcmp(kmcTypesUp_.data(), types.data(), sizeof(KmcType) * types.size()) == 0;
    const bool sameR = kmcRepsUp_.size() == reps.size() &&
                       std::memcmp(kmcRepsUp_.data(), reps.data(), sizeof(KmcRep) * reps.size()) == 0;
    if (!sameT || !sameR || kmcAllocsFresh) {
        CK(cudaStreamSynchronize(stream_));
        kmcTypesUp_ = std::move(types);
        kmcRepsUp_ = std::move(reps);
        CK(cudaMemcpyAsync((void *)K_.types, kmcTypesUp_.data(), sizeof(KmcType) * kmcTypesUp_.size(),
                           cudaMemcpyHostToDevice, stream_));
        CK(cudaMemcpyAsync((void *)K_.rep, kmcRepsUp_.data(), sizeof(KmcRep) * R_, cudaMemcpyHostToDevice, stream_));
    }
    K_.R = R_;
    K_.nCells = cells;
    K_.nTypes = std::max(nt, 1);
    K_.nProt = nProt_;
    K_.step = stepCount_;
    K_.D = kmcD_;
}

// the springs' counts per replica (and the step's stats) back on the host
void Engine::readSprings(AlensKmcStats *stats) {
    CK(cudaMemcpyAsync(hKmc_, K_.stats, sizeof(int) * (9 * R_ + 1), cudaMemcpyDeviceToHost, stream_));
    CK(cudaStreamSynchronize(stream_));
    const int before = S_.nLinks;
    int total = userLinkTotal_;
    for (int r = 0; r < R_; r++) {
        springs_[r] = hKmc_[8 * R_ + r];
        total += springs_[r];
    }
    S_.nLinks = total;
    if (S_.nLinks != before) invalidateGraph();
    if (stats)
        for (int r = 0; r < R_; r++) {
            const int *c = hKmc_ + 8 * r;
            stats[r] = AlensKmcStats{c[0], c[1], c[2], c[3], c[4], c[5], c[6], c[7]};
        }
    springsDirty_ = false;
    if (hKmc_[9 * R_] & kKmcErrSpring) throw ApiError(ALENS_CAPACITY);
}

void Engine::rebuildSprings() {
    uploadProteins();
    if (nProt_ == 0) {
        for (int r = 0; r < R_; r++) springs_[r] = 0;
        if (S_.nLinks != userLinkTotal_) invalidateGraph();
        S_.nLinks = userLinkTotal_;
        springsDirty_ = false;
        return;
    }
    if (ptypes_.empty()) throw ApiError(ALENS_NOT_READY);
    prepareKmc();
    CK(cudaMemsetAsync(K_.stats, 0, sizeof(int) * (9 * R_ + 1), stream_));
    launch_kmc_view(K_, S_, stream_);  // lookupType 1 rest lengths read the rods
    launches_ += 1 + launch_kmc_springs(K_, S_, userLinkTotal_, linkCap_, stream_);
    CK(cudaGetLastError());
    readSprings(nullptr);
}

int Engine::proteinMotionStep(AlensKmcStats *stats) {
    if (haveDetect_ || haveSolve_) throw ApiError(ALENS_NOT_READY);
    finalize();
    uploadLinks();
    uploadBoundaries();
    uploadProteins();
    if (nProt_ == 0) {
        rebuildSprings();
        if (stats) std::memset(stats, 0, sizeof(AlensKmcStats) * R_);
        return ALENS_OK;
    }
    if (ptypes_.empty()) throw ApiError(ALENS_NOT_READY);
    prepareKmc();
    CK(cudaMemsetAsync(K_.stats, 0, sizeof(int) * (9 * R_ + 1), stream_));
    launch_kmc_view(K_, S_, stream_);
    int n = 1 + launch_kmc_motion(K_, S_, stream_);
    n += launch_kmc_springs(K_, S_, userLinkTotal_, linkCap_, stream_);
    CK(cudaGetLastError());
    launches_ += n;
    protDevNewer_ = true;
    readSprings(stats);
    return ALENS_OK;
}

int Engine::proteinBindStep(AlensKmcStats *stats) {
    if (haveDetect_ || haveSolve_) throw ApiError(ALENS_NOT_READY);
    finalize();
    uploadLinks();
    uploadProteins();
    if (nProt_ == 0) {
        rebuildSprings();
        if (stats) std::memset(stats, 0, sizeof(AlensKmcStats) * R_);
        return ALENS_OK;
    }
    if (ptypes_.empty()) throw ApiError(ALENS_NOT_READY);
    prepareKmc();
    CK(cudaMemsetAsync(K_.cellCount, 0, sizeof(int) * (K_.nCells + 1), stream_));
    CK(cudaMemsetAsync(K_.cellCursor, 0, sizeof(int) * (K_.nCells + 1), stream_));
    CK(cudaMemsetAsync(K_.stats, 0, sizeof(int) * (9 * R_ + 1), stream_));
    launch_kmc_bin(K_, S_, stream_);
    int n = 1 + launch_scan(K_.cellCount, K_.cellStart, K_.nCells + 1, S_.scanTmp, stream_);
    launch_kmc_scatter(K_, S_, stream_);
    n += 1 + launch_kmc_bind(K_, stream_);
    n += launch_kmc_springs(K_, S_, userLinkTotal_, linkCap_, stream_);
    CK(cudaGetLastError());
    launches_ += n;
    protDevNewer_ = true;
    readSprings(stats);
    return (hKmc_[9 * R_] & kKmcErrCand) ? ALENS_CAPACITY : ALENS_OK;
}

}  // namespace alens
