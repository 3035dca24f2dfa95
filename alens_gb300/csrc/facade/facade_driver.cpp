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
//
// usage: facade_driver --host-checks RunConfig.yaml [restart files...]
// Prints one JSON line from the single-rank getters that need no device
// (result folders, snapshot schedule, domain, communicator, random pool)
// and, per restart file, [is TimeStepInfo, step, snapID, time].
//
// usage: facade_driver --write-vtk TubuleInitial.dat folder snapID
// Reads the rods and writes Sylinder_<snapID>.pvtp and its piece (no device).
//
// usage: facade_driver --write-protein-ascii records.txt out.dat time
// usage: facade_driver --write-protein-vtk records.txt folder snapID
// Writes a ProteinAscii file with SylinderSystem::writeProteinAscii, or
// Protein_<snapID>.pvtp and its piece with writeProteinVTK (no device).  records: "T tag..." (tag per species), "R gid..." (rod gids),
// then "gid type idBind0 idBind1 pos(3) posEnd0(3) posEnd1(3)" per protein.
//
// usage: facade_driver --proteins RunConfig.yaml TubuleInitial.dat setup.txt KBT steps out.txt
// Steps proteins and rods in TubuleSystem::step()'s order
// (SRC/TubuleSystem.cpp:185-224): updateProteinMotion(),
// calcBindInteraction(), then runStep().
// setup: "S tag fixedEnd0 useBindVol lookupType freeLength kappa lambda
// PtoAPratio diffUnbound rc eps ko_s(2) ko_d(2) Ka(2) Ke(2) walkOff vdrag(2)
// fstall vmax(2) vmaxAP(2) diffBoundS(2) diffBoundD(2)" per species and
// "P gid type idBind0 idBind1 distBind0 distBind1 x y z" per protein.  Writes
// the final proteins to out.txt ("gid type idBind0 idBind1 distBind(2)
// pos(3) posEnd(6)", %.17g) and prints one JSON line of per-step counts.
//
// usage: facade_driver --restart-check RunConfig.yaml TubuleInitial.dat steps
// Steps a system, calling writeResult() before each runStep (where the
// reference's runStep writes its snapshot), then restarts a second system
// from ./TimeStepInfo.txt and prints one JSON line: snapshot IDs and steps of
// both, and the largest centre and axis differences between the restarted
// rods and the first system's rods at its last snapshot.
#include <cmath>
#include <cstdio>
#include <fstream>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "SylinderSystem.hpp"

namespace {

int hostChecks(const char *yaml, int nFiles, char **files) {
    gpu::SylinderConfig cfg;
    std::string err;
    if (!cfg.readYaml(yaml, &err)) {
        std::fprintf(stderr, "facade_driver: %s\n", err.c_str());
        return 1;
    }
    const gpu::DomainInfo d = gpu::DomainInfo::fromConfig(cfg);
    const gpu::Comm comm;
    gpu::RngPool pool(cfg.rngSeed, 2), again(cfg.rngSeed, 2);
    const int n = 200000;
    double su = 0, suu = 0, sn = 0, snn = 0, umin = 1, umax = 0;
    for (int i = 0; i < n; i++) {
        const double u = pool.getU01(0), z = pool.getN01(0);
        su += u;
        suu += u * u;
        sn += z;
        snn += z * z;
        umin = u < umin ? u : umin;
        umax = u > umax ? u : umax;
    }
    const double first1 = pool.getU01(1), firstAgain0 = again.getU01(0), firstAgain1 = again.getU01(1);
    bool outOfRange = false;
    try {
        pool.getU01(2);
    } catch (const std::out_of_range &) {
        outOfRange = true;
    }
    std::string restart = "[";
    for (int f = 0; f < nFiles; f++) {
        long step = -1;
        int snap = -1;
        double time = -1.0;
        const bool info = gpu::SylinderSystem::readTimeStepInfo(files[f], &step, &snap, &time);
        char buf[160];
        std::snprintf(buf, sizeof(buf), "%s[%d, %ld, %d, %.17g]", f ? ", " : "", (int)info, step, snap, time);
        restart += buf;
    }
    restart += "]";
    const long every = std::lround(cfg.timeSnap / cfg.dt);
    std::printf("{\"folders\": [\"%s\", \"%s\", \"%s\", \"%s\"], \"snap_every\": %ld, "
                "\"due\": [%d, %d, %d, %d], \"low\": [%.17g, %.17g, %.17g], \"high\": [%.17g, %.17g, %.17g], "
                "\"pbc\": [%d, %d, %d], \"len0\": %.17g, \"rank\": %d, \"size\": %d, "
                "\"u_mean\": %.9g, \"u_var\": %.9g, \"u_min\": %.17g, \"u_max\": %.17g, "
                "\"n_mean\": %.9g, \"n_var\": %.9g, \"stream1_first\": %.17g, "
                "\"again0_first\": %.17g, \"again1_first\": %.17g, \"out_of_range\": %d, \"restart\": %s}\n",
                gpu::SylinderSystem::getResultFolderWithID(0).c_str(),
                gpu::SylinderSystem::getResultFolderWithID(399).c_str(),
                gpu::SylinderSystem::getResultFolderWithID(400).c_str(),
                gpu::SylinderSystem::getResultFolderWithID(1234).c_str(), every,
                (int)gpu::SylinderSystem::snapshotDue(0, cfg.timeSnap, cfg.dt),
                (int)gpu::SylinderSystem::snapshotDue(1, cfg.timeSnap, cfg.dt),
                (int)gpu::SylinderSystem::snapshotDue(every, cfg.timeSnap, cfg.dt),
                (int)gpu::SylinderSystem::snapshotDue(3 * every + 1, cfg.timeSnap, cfg.dt), d.low[0], d.low[1],
                d.low[2], d.high[0], d.high[1], d.high[2], (int)d.pbc[0], (int)d.pbc[1], (int)d.pbc[2], d.getLen(0),
                comm.getRank(), comm.getSize(), su / n, suu / n - (su / n) * (su / n), umin, umax, sn / n,
                snn / n - (sn / n) * (sn / n), first1, firstAgain0, firstAgain1, (int)outOfRange,
                restart.c_str());
    return 0;
}

void axisOf(const double q[4], double a[3]) {
    const double x = q[0], y = q[1], z = q[2], w = q[3];
    a[0] = 2.0 * (x * z + w * y);
    a[1] = 2.0 * (y * z - w * x);
    a[2] = 1.0 - 2.0 * (x * x + y * y);
}

int restartCheck(const char *yaml, const char *dat, int steps) {
    gpu::SylinderSystem first;
    first.initialize(yaml, dat);
    std::vector<gpu::Sylinder> snap;
    long snapStep = -1;
    int snapID = -1;
    for (int s = 0; s < steps; s++) {
        if (first.getIfWriteResultCurrentStep()) {
            snap = first.getContainer();
            snapStep = first.getStepCount();
            snapID = first.getSnapID();
        }
        first.writeResult();
        first.runStep();
    }
    gpu::SylinderSystem again;
    again.reinitialize(yaml, "TimeStepInfo.txt");
    const auto &rods = again.getContainer();
    double dpos = 0.0, daxis = 0.0;
    const bool same = rods.size() == snap.size();
    for (size_t i = 0; same && i < rods.size(); i++) {
        double a[3], b[3];
        axisOf(rods[i].orientation, a);
        axisOf(snap[i].orientation, b);
        for (int d = 0; d < 3; d++) {
            dpos = std::fmax(dpos, std::fabs(rods[i].pos[d] - snap[i].pos[d]));
            daxis = std::fmax(daxis, std::fabs(a[d] - b[d]));
        }
    }
    std::printf("{\"snap_id_after\": %d, \"last_snap_id\": %d, \"last_snap_step\": %ld, \"steps\": %ld, "
                "\"restart_snap_id\": %d, \"restart_step\": %ld, \"same_count\": %d, \"max_dpos\": %.3g, "
                "\"max_daxis\": %.3g, \"folder\": \"%s\"}\n",
                first.getSnapID(), snapID, snapStep, first.getStepCount(), again.getSnapID(), again.getStepCount(),
                (int)same, dpos, daxis, again.getResultFolderWithID(snapID).c_str());
    return 0;
}

}  // namespace

namespace {

std::vector<std::string> tokens(const std::string &line) {
    std::vector<std::string> t;
    std::string cur;
    for (char ch : line) {
        if (ch == ' ' || ch == '\t' || ch == '\r') {
            if (!cur.empty()) t.push_back(cur);
            cur.clear();
        } else {
            cur += ch;
        }
    }
    if (!cur.empty()) t.push_back(cur);
    return t;
}

double num(const std::string &s) { return std::strtod(s.c_str(), nullptr); }

int writeProteinAsciiMode(const char *records, const char *out, double time, int vtkSnap = -1) {
    std::ifstream in(records);
    std::string line;
    std::vector<int> tags;
    std::vector<int64_t> gids;
    std::vector<AlensProtein> prot;
    while (std::getline(in, line)) {
        const auto t = tokens(line);
        if (t.empty()) continue;
        if (t[0] == "T") {
            for (size_t k = 1; k < t.size(); k++) tags.push_back(std::atoi(t[k].c_str()));
        } else if (t[0] == "R") {
            for (size_t k = 1; k < t.size(); k++) gids.push_back(std::atoll(t[k].c_str()));
        } else if (t.size() >= 13) {
            AlensProtein p{};
            p.gid = std::atoll(t[0].c_str());
            p.type = std::atoi(t[1].c_str());
            p.idBind[0] = std::atoi(t[2].c_str());
            p.idBind[1] = std::atoi(t[3].c_str());
            for (int d = 0; d < 3; d++) {
                p.pos[d] = num(t[4 + d]);
                p.posEnd[0][d] = num(t[7 + d]);
                p.posEnd[1][d] = num(t[10 + d]);
            }
            prot.push_back(p);
        }
    }
    if (vtkSnap >= 0)
        gpu::SylinderSystem::writeProteinVTK(out, vtkSnap, prot, tags, gids);
    else
        gpu::SylinderSystem::writeProteinAscii(out, prot, tags, gids, time);
    return 0;
}

int proteinsMode(const char *runConfig, const char *tubules, const char *setup, double kbt, int steps,
                 const char *out) {
    gpu::SylinderSystem rodSystem;
    rodSystem.initialize(runConfig, tubules, 0, nullptr);
    rodSystem.setTimer(false);
    std::ifstream in(setup);
    std::string line;
    std::vector<AlensProteinType> types;
    std::vector<AlensProtein> prot;
    while (std::getline(in, line)) {
        const auto t = tokens(line);
        if (t.empty()) continue;
        if (t[0] == "S" && t.size() >= 32) {
            AlensProteinType y{};
            y.tag = std::atoi(t[1].c_str());
            y.fixedEnd0 = std::atoi(t[2].c_str());
            y.useBindVol = std::atoi(t[3].c_str());
            y.lookupType = std::atoi(t[4].c_str());
            y.freeLength = num(t[5]);
            y.kappa = num(t[6]);
            y.lambda = num(t[7]);
            y.PtoAPratio = num(t[8]);
            y.diffUnbound = num(t[9]);
            y.rc = num(t[10]);
            y.eps = num(t[11]);
            for (int e = 0; e < 2; e++) {
                y.ko_s[e] = num(t[12 + e]);
                y.ko_d[e] = num(t[14 + e]);
                y.Ka[e] = num(t[16 + e]);
                y.Ke[e] = num(t[18 + e]);
            }
            y.walkOff = std::atoi(t[20].c_str());
            y.vdrag[0] = std::atoi(t[21].c_str());
            y.vdrag[1] = std::atoi(t[22].c_str());
            y.fstall = num(t[23]);
            for (int e = 0; e < 2; e++) {
                y.vmax[e] = num(t[24 + e]);
                y.vmaxAP[e] = num(t[26 + e]);
                y.diffBoundS[e] = num(t[28 + e]);
                y.diffBoundD[e] = num(t[30 + e]);
            }
            types.push_back(y);
        } else if (t[0] == "P" && t.size() >= 10) {
            AlensProtein p{};
            p.gid = std::atoll(t[1].c_str());
            p.type = std::atoi(t[2].c_str());
            p.idBind[0] = std::atoi(t[3].c_str());
            p.idBind[1] = std::atoi(t[4].c_str());
            p.distBind[0] = num(t[5]);
            p.distBind[1] = num(t[6]);
            for (int d = 0; d < 3; d++) p.pos[d] = num(t[7 + d]);
            prot.push_back(p);
        }
    }
    if (types.empty()) throw std::runtime_error(std::string("no species in ") + setup);
    rodSystem.setProteinTypes(types, kbt);
    rodSystem.setProteins(prot);
    std::string counts;
    for (int s = 0; s < steps; s++) {
        rodSystem.prepareStep();
        rodSystem.updateProteinMotion();
        const AlensKmcStats st = rodSystem.calcBindInteraction();
        rodSystem.runStep();
        char buf[160];
        std::snprintf(buf, sizeof(buf), "%s[%d, %d, %d, %d, %d, %d, %d, %d]", s ? ", " : "", st.nU, st.nS, st.nD,
                      st.nUS, st.nSU, st.nSD, st.nDS, rodSystem.lastStats().nBilateral);
        counts += buf;
    }
    const auto res = rodSystem.getProteins();
    std::FILE *f = std::fopen(out, "w");
    if (!f) throw std::runtime_error(std::string("cannot write ") + out);
    for (const AlensProtein &p : res) {
        std::fprintf(f, "%lld %d %d %d %.17g %.17g", (long long)p.gid, p.type, p.idBind[0], p.idBind[1],
                     p.distBind[0], p.distBind[1]);
        for (int d = 0; d < 3; d++) std::fprintf(f, " %.17g", p.pos[d]);
        for (int e = 0; e < 2; e++)
            for (int d = 0; d < 3; d++) std::fprintf(f, " %.17g", p.posEnd[e][d]);
        std::fprintf(f, "\n");
    }
    std::fclose(f);
    std::printf("{\"steps\": %d, \"counts\": [%s], \"step_count\": %ld}\n", steps, counts.c_str(),
                rodSystem.getStepCount());
    return 0;
}

}  // namespace

int main(int argc, char **argv) {
    if (argc == 5 && std::strcmp(argv[1], "--write-protein-vtk") == 0) {
        try {
            return writeProteinAsciiMode(argv[2], argv[3], 0.0, std::atoi(argv[4]));
        } catch (const std::exception &e) {
            std::fprintf(stderr, "facade_driver: %s\n", e.what());
            return 1;
        }
    }
    if (argc == 5 && std::strcmp(argv[1], "--write-protein-ascii") == 0) {
        try {
            return writeProteinAsciiMode(argv[2], argv[3], std::strtod(argv[4], nullptr));
        } catch (const std::exception &e) {
            std::fprintf(stderr, "facade_driver: %s\n", e.what());
            return 1;
        }
    }
    if (argc == 8 && std::strcmp(argv[1], "--proteins") == 0) {
        try {
            return proteinsMode(argv[2], argv[3], argv[4], std::strtod(argv[5], nullptr), std::atoi(argv[6]),
                                argv[7]);
        } catch (const std::exception &e) {
            std::fprintf(stderr, "facade_driver: %s\n", e.what());
            return 1;
        }
    }
    if (argc >= 3 && std::strcmp(argv[1], "--host-checks") == 0) return hostChecks(argv[2], argc - 3, argv + 3);
    if (argc == 5 && std::strcmp(argv[1], "--write-vtk") == 0) {
        try {
            std::string err;
            const auto rods = gpu::readSylinderAscii(argv[2], nullptr, &err);
            if (rods.empty() && !err.empty()) throw std::runtime_error(err);
            gpu::SylinderSystem::writeSylinderVTK(argv[3], std::atoi(argv[4]), rods);
            return 0;
        } catch (const std::exception &e) {
            std::fprintf(stderr, "facade_driver: %s\n", e.what());
            return 1;
        }
    }
    if (argc == 5 && std::strcmp(argv[1], "--write-conblock") == 0) {
        // records: one block per line, "gamma delta0 kappa bilateral oneSide
        // gidI gidJ globalIndexI globalIndexJ image normI(3) labI(3) labJ(3)"
        std::ifstream in(argv[2]);
        std::vector<gpu::ConBlockRecord> blocks;
        gpu::ConBlockRecord b;
        long long gI = 0, gJ = 0;
        while (in >> b.gamma >> b.delta0 >> b.kappa >> b.bilateral >> b.oneSide >> gI >> gJ >> b.globalIndexI >>
               b.globalIndexJ >> b.image >> b.normI[0] >> b.normI[1] >> b.normI[2] >> b.labI[0] >> b.labI[1] >>
               b.labI[2] >> b.labJ[0] >> b.labJ[1] >> b.labJ[2]) {
            b.gidI = (int64_t)gI;
            b.gidJ = (int64_t)gJ;
            blocks.push_back(b);
        }
        try {
            gpu::SylinderSystem::writeConBlockVTK(argv[3], std::atoi(argv[4]), blocks);
        } catch (const std::exception &e) {
            std::fprintf(stderr, "%s\n", e.what());
            return 1;
        }
        return 0;
    }
    if (argc == 5 && std::strcmp(argv[1], "--restart-check") == 0) {
        try {
            return restartCheck(argv[2], argv[3], std::atoi(argv[4]));
        } catch (const std::exception &e) {
            std::fprintf(stderr, "facade_driver: %s\n", e.what());
            return 1;
        }
    }
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
