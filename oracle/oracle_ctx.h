// oracle_ctx.h - the oracle's context (one system), shared by oracle.cpp
// (rods, constraints, solver) and oracle_kmc.cpp (protein binding).
// TEST INFRASTRUCTURE ONLY, like the rest of oracle/.
#pragma once

#include <cstdint>
#include <vector>

#include "oracle.h"

struct OrcCtx {
    AlensConfig cfg;
    int n = 0;
    std::vector<int64_t> gid;
    std::vector<double> pos, quat, len, rad;
    std::vector<int32_t> imm;
    double cutoff = 0.0;
    int ncell[3] = {1, 1, 1};
    double cellsz[3] = {1, 1, 1};
    // per-step rod data
    std::vector<double> axis, hcol, rcol, mob, unc, vel;
    std::vector<uint8_t> sph;
    // constraints
    int ncoll = 0, nbil = 0;
    std::vector<int32_t> ci, cj, cimg;
    std::vector<double> jac, phi0, q, gamma, cinv, lb, lab;
    std::vector<uint8_t> unil;
    std::vector<AlensBlock> queue, blocks;
    // confinement boundaries (unit axes)
    struct Bnd {
        int type, inside;
        double c[3], a[3], R;
    };
    std::vector<Bnd> bnd;
    // pre-bound crosslinkers: blocks built from the rod state every step
    std::vector<int> linkI, linkJ;
    std::vector<double> linkSI, linkSJ, linkRest, linkKappa;
    // proteins (oracle_kmc.cpp) and their springs, built after the links
    std::vector<AlensProteinType> ptypes;
    double kmcKBT = 0.0, kmcD = 0.0;
    std::vector<AlensProtein> prot;
    std::vector<int> springI, springJ;
    std::vector<double> springSI, springSJ, springRest, springKappa;
    // rod-major rows: entries 2k+side, ascending
    std::vector<int64_t> rowptr;
    std::vector<int64_t> rowent;
    // Delassus operator rows (ascending column)
    std::vector<int64_t> aptr;
    std::vector<int> acol;
    std::vector<double> aval;
    // warm start
    std::vector<uint64_t> prevKeys;
    std::vector<double> prevGamma;
    std::vector<double> initGammaOverride;
    int64_t step = 0;
    bool detected = false, solved = false;
    AlensStepStats last{};
};

// the springs (springI, ...) of the doubly bound proteins whose rods exist,
// in protein order: rest length freeLength + D, stiffness kappa
void kmc_springs(OrcCtx *x);
