// SylinderSystem.hpp - C++ facade with the call surface aLENS's TubuleSystem
// uses on SimToolbox's SylinderSystem (SRC/TubuleSystem.cpp:38,55,79,100,105,
// 120,176,223,224,229,697), implemented over the C ABI of include/alens_gpu.h.
//
// One system on one GPU and one rank: the MPI/FDPS getters of the reference
// (getDomainInfo, getCommRcp, getRngPoolPtr) return single-rank values, and
// prepareStep() has no repartitioning to do.
#pragma once

#include <array>
#include <cstdint>
#include <memory>
#include <random>
#include <string>
#include <vector>

#include "alens_gpu.h"

namespace gpu {

// Hot-path subset of SylinderConfig (RunConfig.yaml keys,
// docs/source/quickstart.md:316-358) plus the keys TubuleSystem reads.
struct SylinderConfig {
    unsigned long long rngSeed = 1234;
    double simBoxLow[3] = {0, 0, 0};
    double simBoxHigh[3] = {1, 1, 1};
    bool simBoxPBC[3] = {false, false, false};
    bool monolayer = false;
    double viscosity = 0.01;
    double KBT = 0.00411;
    double linkKappa = 1000.0;
    double linkGap = 0.0;           // gap between the surfaces of linked rods (um)
    double sylinderDiameter = 0.025;
    double sylinderDiameterColRatio = 1.0;
    double sylinderLengthColRatio = 1.0;
    double sylinderColBuf = 0.025;
    double dt = 1e-4;
    double timeTotal = 1.0;
    double timeSnap = 1.0;
    double conResTol = 1e-5;
    int conMaxIte = 2000;
    int conSolverChoice = 0;

    // Reads the flat "key: value" / "key: [a, b, c]" lines of RunConfig.yaml;
    // unknown keys and nested blocks are ignored.
    // `boundaries:` list (type "wall" | "sphere" | "tube"; center, radius,
    // axis (or norm for walls), inside), as in
    // Examples/DenseStrainingMotion/RunConfig.yaml:36-41
    std::vector<AlensBoundary> boundaries;
    bool readYaml(const std::string &path, std::string *err = nullptr);
    AlensConfig toAlens() const;
};

// Host record of one rod (the fields of Sylinder that TubuleSystem reads,
// SRC/TubuleBind.hpp:54-67).
// One solved constraint block as the ConBlock snapshot draws it (the
// ConstraintBlock fields of SRC/TubuleSystem.cpp:727-736 that describe it):
// contact points labI (rod I) and labJ (rod J, or the boundary surface),
// normal on rod I, separation, multiplier, stiffness (0 for collisions).
struct ConBlockRecord {
    double gamma = 0.0, delta0 = 0.0, kappa = 0.0;
    int bilateral = 0, oneSide = 0;
    int64_t gidI = 0, gidJ = -1;
    int globalIndexI = 0, globalIndexJ = -1, image = 13;
    double normI[3] = {0, 0, 0};
    double labI[3] = {0, 0, 0};
    double labJ[3] = {0, 0, 0};
};

struct Sylinder {
    int64_t gid = 0;
    int globalIndex = 0;
    double radius = 0.0125;
    double length = 1.0;
    double pos[3] = {0, 0, 0};
    double orientation[4] = {0, 0, 0, 1};  // Eigen order (x, y, z, w)
    bool isImmovable = false;
    int group = -1;
};

// Constraint block with SimToolbox's ConstraintBlock constructor signature
// (SRC/TubuleSystem.cpp:727-736) and setStress (:742).
struct ConstraintBlock {
    AlensBlock blk;
    ConstraintBlock(double delta0, double gamma, int64_t gidI, int64_t gidJ, int globalIndexI, int globalIndexJ,
                    const double normI[3], const double normJ[3], const double posI[3], const double posJ[3],
                    const double labI[3], const double labJ[3], bool oneSide, bool bilateral, double kappa,
                    double gammaLB);
    void setStress(const double stress9[9]);
};

using ConstraintBlockQue = std::vector<ConstraintBlock>;
using ConstraintBlockPool = std::vector<ConstraintBlockQue>;

// Root domain of the single rank (the role of FDPS's DomainInfo that
// TubuleSystem hands to its protein container, SRC/TubuleSystem.cpp:121-125):
// the simulation box and its periodic axes.
struct DomainInfo {
    std::array<double, 3> low{{0, 0, 0}}, high{{1, 1, 1}};
    std::array<bool, 3> pbc{{false, false, false}};
    double getLen(int d) const { return high[d] - low[d]; }
    static DomainInfo fromConfig(const SylinderConfig &cfg);
};

// Communicator of the single rank (TubuleSystem asks getCommRcp()->getRank(),
// SRC/TubuleSystem.cpp:812-813).
struct Comm {
    int getRank() const { return 0; }
    int getSize() const { return 1; }
};

// Per-thread random streams for host-side callers (the role of the pool that
// TubuleSystem draws from with getU01(threadId) / getN01(threadId),
// SRC/TubuleSystem.cpp:273-279,381).  Stream t is a 64-bit Mersenne twister
// seeded with (seed, t); uniforms are (k + 1/2) 2^-53 for the top 53 bits k
// (open interval), normals come from the Box-Muller pair of two uniforms.
// A thread uses only its own stream.
class RngPool {
  public:
    RngPool(unsigned long long seed, int nThreads);
    double getU01(int threadId);
    double getN01(int threadId);
    int size() const { return (int)streams_.size(); }

  private:
    struct Stream {
        std::mt19937_64 eng;
        double spare = 0.0;
        bool hasSpare = false;
    };
    Stream &at(int threadId);
    std::vector<Stream> streams_;
};

class SylinderSystem {
  public:
    SylinderConfig runConfig;

    SylinderSystem() = default;
    ~SylinderSystem();
    SylinderSystem(const SylinderSystem &) = delete;
    SylinderSystem &operator=(const SylinderSystem &) = delete;

    // RunConfig.yaml + TubuleInitial.dat ("C|S gid radius mx my mz px py pz
    // [group]" lines, docs/source/quickstart.md:211-218); throws
    // std::runtime_error on failure.
    void initialize(const std::string &configFile, const std::string &posFile, int argc = 0,
                    char **argv = nullptr);
    // Restart from TimeStepInfo.txt written by writeResult() (the rods come
    // from that snapshot's SylinderAscii file, getSnapID() is its ID + 1, and
    // the step count, which keys the Brownian noise, continues from its
    // step), or directly from a SylinderAscii snapshot file.
    void reinitialize(const std::string &configFile, const std::string &restartFile, int argc = 0,
                      char **argv = nullptr, bool eulerStep = false);
    void initialize(const SylinderConfig &cfg, const std::vector<Sylinder> &rods);

    void prepareStep();           // nothing to repartition on one GPU
    void runStep();               // one full step (alens_step)
    void stepEuler();             // apply a solve prepared by detect/solve (restart path)
    void calcConStress();         // pair virial of the last step
    void calcOrderParameter();    // polar and nematic order of the rod axes
    void writeResult(const std::string &path) const;  // SylinderAscii text (rods, then link lines)
    // When a snapshot is due at the current step: SylinderAscii_<snapID>.dat,
    // Sylinder_<snapID>.pvtp (+ piece) and ConBlock_<snapID>.pvtp (+ piece,
    // the blocks of the last runStep) in the current result folder
    // (created) and ./TimeStepInfo.txt (step,
    // snapID and time, one per line; its presence is what makes aLENS
    // restart, SRC/main.cpp:28-37), then snapID + 1.  Called where the
    // reference calls writeResult() (SRC/TubuleSystem.cpp:100); its runStep
    // also writes before moving, which a caller does here with one more call.
    void writeResult();
    void setTimer(bool on) { timerOn_ = on; }
    void printTimingSummary() const;

    ConstraintBlockPool &getConstraintPoolNonConst() { return conPool_; }
    const std::vector<Sylinder> &getContainer();  // host copy, refreshed after steps
    long getStepCount() const;
    int getSnapID() const { return snapID_; }

    // single-rank getters (set up by initialize)
    const DomainInfo &getDomainInfo() const { return dinfo_; }
    DomainInfo &getDomainInfoNonConst() { return dinfo_; }
    const std::shared_ptr<const Comm> &getCommRcp() const { return comm_; }
    std::shared_ptr<RngPool> getRngPoolPtr() const { return rngPool_; }

    // Snapshot bookkeeping (SRC/TubuleSystem.cpp:50,309-310,321): a snapshot
    // every round(timeSnap / dt) steps; snapshots grouped 400 to a folder,
    // ./result/result0-399/, ./result/result400-799/, ... (the layout
    // docs/source/visualization.md:32 lists).
    bool getIfWriteResultCurrentStep() const { return snapshotDue(getStepCount(), runConfig.timeSnap, runConfig.dt); }
    std::string getCurrentResultFolder() const { return getResultFolderWithID(snapID_); }
    static std::string getResultFolderWithID(int snapID);
    static bool snapshotDue(long step, double timeSnap, double dt);
    // Sylinder_<snapID>.pvtp and its one piece Sylinder_r0_<snapID>.vtp in
    // `folder` (the aLENS snapshot pair, README.md:140-148): two points per
    // rod (minus end, plus end) joined by a line cell; cell data gid, radius,
    // length, group, isImmovable, direction; inline binary arrays (base64 of
    // a UInt64 byte count and the little-endian values).
    static void writeSylinderVTK(const std::string &folder, int snapID, const std::vector<Sylinder> &rods);
    // ConBlock_<snapID>.pvtp and its piece ConBlock_r0_<snapID>.vtp in
    // `folder` (the constraint-block snapshot of README.md:142): one line
    // cell per block from labI to labJ; cell data gamma, delta0, kappa,
    // bilateral, oneSide, gidI, gidJ, globalIndexI, globalIndexJ, image,
    // normI and the block's pair virial gamma (labI - labJ) (x) normI as
    // Stress (row-major 3x3).  Same bytes as alens_gb300.io.write_conblock_pvtp.
    static void writeConBlockVTK(const std::string &folder, int snapID, const std::vector<ConBlockRecord> &blocks);
    // The blocks of the last runStep (empty before the first one).
    std::vector<ConBlockRecord> getConBlocks();
    // TimeStepInfo.txt: exactly three numbers (step, snapID, time); false
    // for anything else (a SylinderAscii snapshot, say)
    static bool readTimeStepInfo(const std::string &path, long *step, int *snapID, double *time);
    // Protein binding kinetics on the device.  The species in
    // ProteinConfig.yaml units (the rod diameter is runConfig's
    // sylinderDiameter), the proteins with bound rods as container indices.
    void setProteinTypes(const std::vector<AlensProteinType> &types, double KBT);
    void setProteins(const std::vector<AlensProtein> &proteins);
    std::vector<AlensProtein> getProteins();
    // TubuleSystem::calcBindInteraction + setProteinConstraints
    // (SRC/TubuleSystem.cpp:232-259, 694-745): one binding step of every
    // protein; the doubly bound ones are springs of the next runStep()
    AlensKmcStats calcBindInteraction();
    // TubuleSystem::updateProteinMotion (SRC/TubuleSystem.cpp:261-306):
    // walking, drag and diffusion of the heads, diffusion of unbound
    // proteins, walk-off at rod ends, boundaries
    AlensKmcStats updateProteinMotion();
    // ProteinAscii_<snapID>.dat (Protein/ProteinData.hpp:545-564, 705-718):
    // header "count \n time", then "P gid tag end0 end1 gid0 gid1" per
    // protein (the heads when both are bound, the centre twice otherwise;
    // bound rods as gids).  Same bytes as alens_gb300.io.write_protein_ascii.
    static void writeProteinAscii(const std::string &path, const std::vector<AlensProtein> &proteins,
                                  const std::vector<int> &typeTag, const std::vector<int64_t> &rodGid, double time);
    // Protein_<snapID>.pvtp and its piece Protein_r0_<snapID>.vtp in
    // `folder` (ProteinData::writeVTP / writePVTP,
    // Protein/ProteinData.hpp:583-700): two points per protein (the heads
    // when both are bound, the centre twice otherwise) joined by a line
    // cell, point data idBind (rod gids), cell data gid and tag.  Same bytes
    // as alens_gb300.io.write_protein_pvtp.
    static void writeProteinVTK(const std::string &folder, int snapID, const std::vector<AlensProtein> &proteins,
                                const std::vector<int> &typeTag, const std::vector<int64_t> &rodGid);
    AlensCtx *context() const { return ctx_; }
    const AlensStepStats &lastStats() const { return stats_; }
    std::array<double, 9> conStress() const { return stress_; }
    std::array<double, 3> polarOrder() const { return polar_; }
    std::array<double, 9> nematicOrder() const { return nematic_; }

  private:
    void create();
    void flushPool();
    void check(int rc, const char *where) const;

    AlensCtx *ctx_ = nullptr;
    std::vector<int> proteinTags_;   // tag per species
    bool haveProteins_ = false;
    std::vector<Sylinder> rods_;
    std::vector<std::array<int64_t, 2>> links_;  // 'L a b' lines (gids): plus end of a to minus end of b
    void applyLinks();
    bool rodsStale_ = false;
    bool haveBlocks_ = false;  // a step has run on the current rods (its blocks are readable)
    ConstraintBlockPool conPool_;
    AlensStepStats stats_{};
    std::array<double, 9> stress_{};
    std::array<double, 3> polar_{};
    std::array<double, 9> nematic_{};
    int snapID_ = 0;
    bool timerOn_ = false;
    double lastStepMs_ = 0.0;
    DomainInfo dinfo_;
    std::shared_ptr<const Comm> comm_ = std::make_shared<const Comm>();
    std::shared_ptr<RngPool> rngPool_;
};

// Read TubuleInitial.dat / SylinderAscii lines; 'L' link lines are returned
// in links (pairs of gids).
std::vector<Sylinder> readSylinderAscii(const std::string &path, std::vector<std::array<int64_t, 2>> *links,
                                        std::string *err);

}  // namespace gpu
