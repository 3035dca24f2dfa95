// facade_driver.cpp - steps a system through gpu::SylinderSystem in the
// order aLENS's TubuleSystem::step() calls its rod system
// (SRC/TubuleSystem.cpp:144-230): prepareStep, calcOrderParameter, queue
// bilateral blocks in the per-thread pool (setProteinConstraints, :694-745),
// runStep, calcConStress, printTimingSummary.
//
// usage: facade_driver RunConfig.yaml TubuleInitial.dat steps [out.dat]
// The bilateral blocks are one spring (kappa = linkKappa) between the first
// two rods, rebuilt every step from their current geometry.  Prints one JSON
// line with the run summary.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>

#include "SylinderSystem.hpp"

int main(int argc, char **argv) {
    if (argc < 4) {
        std::fprintf(stderr, "usage: %s RunConfig.yaml TubuleInitial.dat steps [out.dat]\n", argv[0]);
        return 2;
    }
    const int steps = std::atoi(argv[3]);
    try {
        gpu::SylinderSystem rodSystem;
        rodSystem.initialize(argv[1], argv[2], argc, argv);
        rodSystem.setTimer(false);
        long iters = 0, coll = 0;
        double stressTrace = 0.0;
        for (int s = 0; s < steps; s++) {
            rodSystem.prepareStep();
            rodSystem.calcOrderParameter();
            const auto &rods = rodSystem.getContainer();
            if (rods.size() >= 2) {
                // one spring between rods 0 and 1, anchored at their centres
                const auto &a = rods[0], &b = rods[1];
                double d[3] = {a.pos[0] - b.pos[0], a.pos[1] - b.pos[1], a.pos[2] - b.pos[2]};
                const double len = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
                const double rest = 0.05, kappa = rodSystem.runConfig.linkKappa;
                const double nI[3] = {d[0] / len, d[1] / len, d[2] / len};
                const double nJ[3] = {-nI[0], -nI[1], -nI[2]};
                const double zero[3] = {0.0, 0.0, 0.0};
                auto &pool = rodSystem.getConstraintPoolNonConst();
                pool[0].emplace_back(len - rest, -(len - rest) * kappa, a.gid, b.gid, 0, 1, nI, nJ, zero, zero,
                                     a.pos, b.pos, false, true, kappa, 0.0);
                const double st[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
                pool[0].back().setStress(st);
            }
            rodSystem.runStep();
            rodSystem.calcConStress();
            rodSystem.printTimingSummary();
            iters += rodSystem.lastStats().iterations;
            coll += rodSystem.lastStats().nCollision;
            const auto s9 = rodSystem.conStress();
            stressTrace = s9[0] + s9[4] + s9[8];
        }
        if (argc > 4) rodSystem.writeResult(argv[4]);
        const auto &rods = rodSystem.getContainer();
        double sx = 0, sy = 0, sz = 0;
        for (const auto &r : rods) {
            sx += r.pos[0];
            sy += r.pos[1];
            sz += r.pos[2];
        }
        const auto P = rodSystem.polarOrder();
        std::printf("{\"rods\": %zu, \"steps\": %ld, \"iterations\": %ld, \"collisions\": %ld, "
                    "\"sum_pos\": [%.17g, %.17g, %.17g], \"stress_trace\": %.17g, \"polar\": [%.6g, %.6g, %.6g], "
                    "\"rod0\": [%.17g, %.17g, %.17g]}\n",
                    rods.size(), rodSystem.getStepCount(), iters, coll, sx, sy, sz, stressTrace, P[0], P[1], P[2],
                    rods[0].pos[0], rods[0].pos[1], rods[0].pos[2]);
    } catch (const std::exception &e) {
        std::fprintf(stderr, "facade_driver: %s\n", e.what());
        return 1;
    }
    return 0;
}
