// SylinderSystem.cpp - facade over the C ABI (see SylinderSystem.hpp).
#include "SylinderSystem.hpp"

#include <omp.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <sstream>
#include <stdexcept>
#include <type_traits>
#include <unordered_map>

namespace gpu {

namespace {

std::string trim(const std::string &s) {
    const size_t a = s.find_first_not_of(" \t\r\n");
    if (a == std::string::npos) return "";
    const size_t b = s.find_last_not_of(" \t\r\n");
    return s.substr(a, b - a + 1);
}

bool parseBool(const std::string &v) {
    std::string t;
    for (char c : v) t += (char)std::tolower((unsigned char)c);
    return t == "true" || t == "1" || t == "yes";
}

std::vector<std::string> parseList(const std::string &v) {
    std::vector<std::string> out;
    const size_t a = v.find('['), b = v.find(']');
    if (a == std::string::npos || b == std::string::npos) return out;
    std::stringstream ss(v.substr(a + 1, b - a - 1));
    std::string item;
    while (std::getline(ss, item, ',')) out.push_back(trim(item));
    return out;
}

// rotation taking +z onto the unit vector d, as an (x,y,z,w) quaternion
void quatFromDirection(const double d[3], double q[4]) {
    double x = -d[1], y = d[0], z = 0.0, w = 1.0 + d[2];
    if (w < 1e-8) {
        x = 1.0;
        y = 0.0;
        z = 0.0;
        w = 0.0;
    }
    const double n = std::sqrt(x * x + y * y + z * z + w * w);
    q[0] = x / n;
    q[1] = y / n;
    q[2] = z / n;
    q[3] = w / n;
}

void directionFromQuat(const double q[4], double d[3]) {
    const double x = q[0], y = q[1], z = q[2], w = q[3];
    d[0] = 2.0 * (x * z + w * y);
    d[1] = 2.0 * (y * z - w * x);
    d[2] = 1.0 - 2.0 * (x * x + y * y);
}

}  // namespace

bool SylinderConfig::readYaml(const std::string &path, std::string *err) {
    std::ifstream f(path);
    if (!f) {
        if (err) *err = "cannot open " + path;
        return false;
    }
    std::string line;
    bool inBoundaries = false;
    boundaries.clear();
    while (std::getline(f, line)) {
        const size_t hash = line.find('#');
        if (hash != std::string::npos) line = line.substr(0, hash);
        if (trim(line).empty()) continue;
        const bool nested = line[0] == ' ' || line[0] == '\t' || line[0] == '-';
        if (inBoundaries && nested) {
            // "- type: ..." starts an entry; "key: value" lines fill the last one
            std::string t = trim(line);
            if (t[0] == '-') {
                AlensBoundary b;
                std::memset(&b, 0, sizeof(b));
                b.inside = 1;
                b.axis[2] = 1.0;
                boundaries.push_back(b);
                t = trim(t.substr(1));
            }
            const size_t c2 = t.find(':');
            if (c2 == std::string::npos || boundaries.empty()) continue;
            const std::string k = trim(t.substr(0, c2));
            std::string v = trim(t.substr(c2 + 1));
            AlensBoundary &b = boundaries.back();
            auto vec3b = [&](double *dst) {
                auto items = parseList(v);
                for (int d = 0; d < 3 && d < (int)items.size(); d++) dst[d] = std::stod(items[d]);
            };
            if (k == "type") {
                v.erase(std::remove(v.begin(), v.end(), '"'), v.end());
                v.erase(std::remove(v.begin(), v.end(), '\''), v.end());
                b.type = v == "sphere" ? ALENS_BOUNDARY_SPHERE : (v == "tube" ? ALENS_BOUNDARY_TUBE : ALENS_BOUNDARY_WALL);
            } else if (k == "center") {
                vec3b(b.center);
            } else if (k == "axis" || k == "norm") {
                vec3b(b.axis);
            } else if (k == "radius") {
                b.radius = std::stod(v);
            } else if (k == "inside") {
                b.inside = parseBool(v) ? 1 : 0;
            }
            continue;
        }
        if (nested) continue;  // other nested blocks
        inBoundaries = trim(line.substr(0, line.find(':'))) == "boundaries";
        if (inBoundaries) continue;
        const size_t colon = line.find(':');
        if (colon == std::string::npos) continue;
        const std::string key = trim(line.substr(0, colon));
        const std::string val = trim(line.substr(colon + 1));
        if (val.empty()) continue;
        auto vec3 = [&](double *dst) {
            auto items = parseList(val);
            for (int d = 0; d < 3 && d < (int)items.size(); d++) dst[d] = std::stod(items[d]);
        };
        if (key == "rngSeed") rngSeed = std::stoull(val);
        else if (key == "simBoxLow") vec3(simBoxLow);
        else if (key == "simBoxHigh") vec3(simBoxHigh);
        else if (key == "simBoxPBC") {
            auto items = parseList(val);
            for (int d = 0; d < 3 && d < (int)items.size(); d++) simBoxPBC[d] = parseBool(items[d]);
        } else if (key == "monolayer") monolayer = parseBool(val);
        else if (key == "viscosity") viscosity = std::stod(val);
        else if (key == "KBT") KBT = std::stod(val);
        else if (key == "linkKappa") linkKappa = std::stod(val);
        else if (key == "linkGap") linkGap = std::stod(val);
        else if (key == "sylinderDiameter") sylinderDiameter = std::stod(val);
        else if (key == "sylinderDiameterColRatio") sylinderDiameterColRatio = std::stod(val);
        else if (key == "sylinderLengthColRatio") sylinderLengthColRatio = std::stod(val);
        else if (key == "sylinderColBuf") sylinderColBuf = std::stod(val);
        else if (key == "dt") dt = std::stod(val);
        else if (key == "timeTotal") timeTotal = std::stod(val);
        else if (key == "timeSnap") timeSnap = std::stod(val);
        else if (key == "conResTol") conResTol = std::stod(val);
        else if (key == "conMaxIte") conMaxIte = (int)std::min(std::stod(val), 2.0e9);
        else if (key == "conSolverChoice") conSolverChoice = std::stoi(val);
    }
    return true;
}

AlensConfig SylinderConfig::toAlens() const {
    AlensConfig c;
    alens_config_default(&c);
    for (int d = 0; d < 3; d++) {
        c.simBoxLow[d] = simBoxLow[d];
        c.simBoxHigh[d] = simBoxHigh[d];
        c.simBoxPBC[d] = simBoxPBC[d] ? 1 : 0;
    }
    c.monolayer = monolayer ? 1 : 0;
    c.viscosity = viscosity;
    c.KBT = KBT;
    c.dt = dt;
    c.sylinderDiameterColRatio = sylinderDiameterColRatio;
    c.sylinderLengthColRatio = sylinderLengthColRatio;
    c.sylinderColBuf = sylinderColBuf;
    c.conResTol = conResTol;
    c.conMaxIte = conMaxIte;
    c.conSolverChoice = conSolverChoice;
    c.rngSeed = rngSeed;
    return c;
}

ConstraintBlock::ConstraintBlock(double delta0, double gamma, int64_t gidI, int64_t gidJ, int globalIndexI,
                                 int globalIndexJ, const double normI[3], const double normJ[3],
                                 const double posI[3], const double posJ[3], const double labI[3],
                                 const double labJ[3], bool oneSide, bool bilateral, double kappa,
                                 double gammaLB) {
    std::memset(&blk, 0, sizeof(blk));
    blk.delta0 = delta0;
    blk.gamma = gamma;
    blk.gidI = gidI;
    blk.gidJ = gidJ;
    blk.globalIndexI = globalIndexI;
    blk.globalIndexJ = globalIndexJ;
    for (int d = 0; d < 3; d++) {
        blk.normI[d] = normI[d];
        blk.normJ[d] = normJ[d];
        blk.posI[d] = posI[d];
        blk.posJ[d] = posJ[d];
        blk.labI[d] = labI[d];
        blk.labJ[d] = labJ[d];
    }
    blk.oneSide = oneSide ? 1 : 0;
    blk.bilateral = bilateral ? 1 : 0;
    blk.kappa = kappa;
    blk.gammaLB = gammaLB;
}

void ConstraintBlock::setStress(const double stress9[9]) {
    for (int i = 0; i < 9; i++) blk.stress[i] = stress9[i];
}

std::vector<Sylinder> readSylinderAscii(const std::string &path, std::vector<std::array<int64_t, 2>> *links,
                                        std::string *err) {
    std::vector<Sylinder> rods;
    std::ifstream f(path);
    if (!f) {
        if (err) *err = "cannot open " + path;
        return rods;
    }
    std::string line;
    while (std::getline(f, line)) {
        std::stringstream ss(line);
        std::string type;
        if (!(ss >> type)) continue;
        if (type == "L") {
            int64_t a, b;
            if ((ss >> a >> b) && links) links->push_back({a, b});
            continue;
        }
        if (type != "C" && type != "S") continue;
        Sylinder s;
        double m[3], p[3];
        if (!(ss >> s.gid >> s.radius >> m[0] >> m[1] >> m[2] >> p[0] >> p[1] >> p[2])) continue;
        if (!(ss >> s.group)) s.group = -1;
        s.isImmovable = type == "S";
        double d[3] = {p[0] - m[0], p[1] - m[1], p[2] - m[2]};
        s.length = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
        for (int k = 0; k < 3; k++) s.pos[k] = 0.5 * (m[k] + p[k]);
        if (s.length > 0) {
            for (int k = 0; k < 3; k++) d[k] /= s.length;
        } else {
            d[0] = 0;
            d[1] = 0;
            d[2] = 1;
        }
        quatFromDirection(d, s.orientation);
        s.globalIndex = (int)rods.size();
        rods.push_back(s);
    }
    return rods;
}

SylinderSystem::~SylinderSystem() {
    if (ctx_) alens_destroy(ctx_);
}

void SylinderSystem::check(int rc, const char *where) const {
    if (rc == ALENS_OK || rc == ALENS_NOT_CONVERGED) return;
    std::string msg = std::string(where) + ": " + alens_status_str(rc);
    if (ctx_) msg += std::string(" [") + alens_get_last_error(ctx_) + "]";
    throw std::runtime_error(msg);
}

void SylinderSystem::create() {
    if (ctx_) alens_destroy(ctx_);
    ctx_ = nullptr;
    const AlensConfig c = runConfig.toAlens();
    check(alens_create(&c, &ctx_), "alens_create");
    const int n = (int)rods_.size();
    std::vector<int64_t> gid(n);
    std::vector<double> pos(3 * (size_t)n), quat(4 * (size_t)n), len(n), rad(n);
    std::vector<int32_t> imm(n);
    for (int i = 0; i < n; i++) {
        gid[i] = rods_[i].gid;
        for (int d = 0; d < 3; d++) pos[3 * i + d] = rods_[i].pos[d];
        for (int d = 0; d < 4; d++) quat[4 * i + d] = rods_[i].orientation[d];
        len[i] = rods_[i].length;
        rad[i] = rods_[i].radius;
        imm[i] = rods_[i].isImmovable ? 1 : 0;
    }
    check(alens_set_rods(ctx_, 0, n, gid.data(), pos.data(), quat.data(), len.data(), rad.data(), imm.data()),
          "alens_set_rods");
    conPool_.assign(std::max(1, omp_get_max_threads()), ConstraintBlockQue());
    dinfo_ = DomainInfo::fromConfig(runConfig);
    rngPool_ = std::make_shared<RngPool>(runConfig.rngSeed, std::max(1, omp_get_max_threads()));
    snapID_ = 0;
    rodsStale_ = false;
    applyLinks();
    if (!runConfig.boundaries.empty())
        check(alens_set_boundaries(ctx_, 0, (int)runConfig.boundaries.size(), runConfig.boundaries.data()),
              "alens_set_boundaries");
}

// Links of a flexible filament ('L a b' lines of TubuleInitial.dat, as
// Utils/gen_flexible_init.py writes them; linkKappa / linkGap of
// RunConfig.yaml, Examples/FlexibleFilament/RunConfig.yaml:19-20): a spring
// of stiffness linkKappa from the plus end of rod a (centre + L/2 axis) to
// the minus end of rod b (centre - L/2 axis), rest length linkGap plus both
// radii (surfaces linkGap apart).  Built on the device every step
// (alens_set_links).
void SylinderSystem::applyLinks() {
    if (links_.empty()) return;
    std::unordered_map<int64_t, int> index;
    for (size_t i = 0; i < rods_.size(); i++) index[rods_[i].gid] = (int)i;
    std::vector<int32_t> I, J;
    std::vector<double> sI, sJ, rest, kap;
    for (const auto &l : links_) {
        auto a = index.find(l[0]), b = index.find(l[1]);
        if (a == index.end() || b == index.end()) throw std::runtime_error("link to an unknown rod gid");
        const Sylinder &ra = rods_[a->second];
        const Sylinder &rb = rods_[b->second];
        I.push_back(a->second);
        J.push_back(b->second);
        sI.push_back(0.5 * ra.length);
        sJ.push_back(-0.5 * rb.length);
        rest.push_back(runConfig.linkGap + ra.radius + rb.radius);
        kap.push_back(runConfig.linkKappa);
    }
    check(alens_set_links(ctx_, 0, (int)I.size(), I.data(), J.data(), sI.data(), sJ.data(), rest.data(), kap.data()),
          "alens_set_links");
}

void SylinderSystem::initialize(const std::string &configFile, const std::string &posFile, int, char **) {
    std::string err;
    if (!runConfig.readYaml(configFile, &err)) throw std::runtime_error(err);
    links_.clear();
    rods_ = readSylinderAscii(posFile, &links_, &err);
    if (rods_.empty() && !err.empty()) throw std::runtime_error(err);
    create();
}

void SylinderSystem::reinitialize(const std::string &configFile, const std::string &restartFile, int argc,
                                  char **argv, bool) {
    long step = 0;
    int snap = 0;
    double time = 0.0;
    {
        std::ifstream in(restartFile);
        if (!in) throw std::runtime_error("cannot read " + restartFile);
    }
    if (!readTimeStepInfo(restartFile, &step, &snap, &time)) {
        initialize(configFile, restartFile, argc, argv);
        return;
    }
    const std::string snapFile = getResultFolderWithID(snap) + "SylinderAscii_" + std::to_string(snap) + ".dat";
    initialize(configFile, snapFile, argc, argv);
    snapID_ = snap + 1;
    check(alens_set_step_count(ctx_, step), "alens_set_step_count");
}

void SylinderSystem::initialize(const SylinderConfig &cfg, const std::vector<Sylinder> &rods) {
    haveBlocks_ = false;
    runConfig = cfg;
    rods_ = rods;
    for (size_t i = 0; i < rods_.size(); i++) rods_[i].globalIndex = (int)i;
    create();
}

void SylinderSystem::prepareStep() {}

void SylinderSystem::flushPool() {
    std::vector<AlensBlock> all;
    for (auto &q : conPool_) {
        for (auto &b : q) all.push_back(b.blk);
        q.clear();
    }
    if (!all.empty()) check(alens_add_bilateral(ctx_, 0, (int)all.size(), all.data()), "alens_add_bilateral");
}

void SylinderSystem::runStep() {
    if (!ctx_) throw std::runtime_error("SylinderSystem::runStep before initialize");
    flushPool();
    const auto t0 = std::chrono::steady_clock::now();
    const int rc = alens_step(ctx_, &stats_);
    lastStepMs_ = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    check(rc, "alens_step");
    rodsStale_ = true;
    haveBlocks_ = true;
}

void SylinderSystem::stepEuler() {
    // a solve prepared through the staged C ABI (alens_detect/alens_solve)
    // is applied; without one there is nothing to move
    if (!ctx_) return;
    AlensStepStats st;
    const int rc = alens_advance(ctx_, &st);
    if (rc == ALENS_NOT_READY) return;
    check(rc, "alens_advance");
    rodsStale_ = true;
}

void SylinderSystem::calcConStress() {
    if (!ctx_) return;
    check(alens_get_con_stress(ctx_, 0, stress_.data()), "alens_get_con_stress");
}

void SylinderSystem::calcOrderParameter() {
    const auto &rods = getContainer();
    polar_ = {0, 0, 0};
    nematic_ = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    if (rods.empty()) return;
    for (const auto &r : rods) {
        double d[3];
        directionFromQuat(r.orientation, d);
        for (int a = 0; a < 3; a++) {
            polar_[a] += d[a];
            for (int b = 0; b < 3; b++) nematic_[3 * a + b] += d[a] * d[b] - (a == b ? 1.0 / 3.0 : 0.0);
        }
    }
    const double inv = 1.0 / (double)rods.size();
    for (auto &v : polar_) v *= inv;
    for (auto &v : nematic_) v *= inv;
}

const std::vector<Sylinder> &SylinderSystem::getContainer() {
    if (ctx_ && rodsStale_) {
        const int n = (int)rods_.size();
        std::vector<double> pos(3 * (size_t)n), quat(4 * (size_t)n);
        check(alens_get_rods(ctx_, 0, n, pos.data(), quat.data()), "alens_get_rods");
        for (int i = 0; i < n; i++) {
            for (int d = 0; d < 3; d++) rods_[i].pos[d] = pos[3 * i + d];
            for (int d = 0; d < 4; d++) rods_[i].orientation[d] = quat[4 * i + d];
        }
        rodsStale_ = false;
    }
    return rods_;
}

long SylinderSystem::getStepCount() const {
    int64_t c = 0;
    if (ctx_) alens_get_step_count(ctx_, &c);
    return (long)c;
}

bool SylinderSystem::readTimeStepInfo(const std::string &path, long *step, int *snapID, double *time) {
    std::ifstream in(path);
    std::string a, b, c, extra;
    if (!(in >> a >> b >> c) || (in >> extra)) return false;
    char *e1 = nullptr, *e2 = nullptr, *e3 = nullptr;
    const long st = std::strtol(a.c_str(), &e1, 10);
    const long sn = std::strtol(b.c_str(), &e2, 10);
    const double t = std::strtod(c.c_str(), &e3);
    if (*e1 != '\0' || *e2 != '\0' || *e3 != '\0' || st < 0 || sn < 0 || sn > 2147483647L) return false;
    *step = st;
    *snapID = (int)sn;
    *time = t;
    return true;
}

bool SylinderSystem::snapshotDue(long step, double timeSnap, double dt) {
    if (!(dt > 0.0) || !(timeSnap > 0.0)) return false;
    const long every = std::max(1L, (long)std::llround(timeSnap / dt));
    return step % every == 0;
}

std::string SylinderSystem::getResultFolderWithID(int snapID) {
    constexpr int kPerFolder = 400;
    const int lo = snapID / kPerFolder * kPerFolder;
    return "./result/result" + std::to_string(lo) + "-" + std::to_string(lo + kPerFolder - 1) + "/";
}

void SylinderSystem::writeResult() {
    if (!getIfWriteResultCurrentStep()) return;
    const std::string folder = getCurrentResultFolder();
    std::error_code ec;
    std::filesystem::create_directories(folder, ec);
    if (ec) throw std::runtime_error("cannot create " + folder + ": " + ec.message());
    writeResult(folder + "SylinderAscii_" + std::to_string(snapID_) + ".dat");
    writeSylinderVTK(folder, snapID_, getContainer());
    writeConBlockVTK(folder, snapID_, getConBlocks());
    if (haveProteins_) {
        std::vector<int64_t> gid;
        for (const Sylinder &r : getContainer()) gid.push_back(r.gid);
        const auto prot = getProteins();
        writeProteinAscii(folder + "ProteinAscii_" + std::to_string(snapID_) + ".dat", prot, proteinTags_, gid,
                          runConfig.dt * (double)getStepCount());
        writeProteinVTK(folder, snapID_, prot, proteinTags_, gid);
    }
    std::FILE *f = std::fopen("TimeStepInfo.txt", "w");
    if (!f) throw std::runtime_error("cannot write TimeStepInfo.txt");
    std::fprintf(f, "%ld\n%d\n%.17g\n", getStepCount(), snapID_, runConfig.dt * (double)getStepCount());
    std::fclose(f);
    snapID_++;
}

namespace {

// RFC 4648 base64 with padding
std::string base64(const std::vector<unsigned char> &in) {
    static const char kAlphabet[] = "ABCDEFGHIJKLMNOPQRSTUVWXYZabcdefghijklmnopqrstuvwxyz0123456789+/";
    std::string out;
    out.reserve((in.size() + 2) / 3 * 4);
    size_t i = 0;
    for (; i + 2 < in.size(); i += 3) {
        const unsigned v = (unsigned)in[i] << 16 | (unsigned)in[i + 1] << 8 | in[i + 2];
        out += kAlphabet[v >> 18 & 63];
        out += kAlphabet[v >> 12 & 63];
        out += kAlphabet[v >> 6 & 63];
        out += kAlphabet[v & 63];
    }
    if (i + 1 == in.size()) {
        const unsigned v = (unsigned)in[i] << 16;
        out += kAlphabet[v >> 18 & 63];
        out += kAlphabet[v >> 12 & 63];
        out += "==";
    } else if (i + 2 == in.size()) {
        const unsigned v = (unsigned)in[i] << 16 | (unsigned)in[i + 1] << 8;
        out += kAlphabet[v >> 18 & 63];
        out += kAlphabet[v >> 12 & 63];
        out += kAlphabet[v >> 6 & 63];
        out += '=';
    }
    return out;
}

// little-endian bytes of an integer or IEEE double, independent of the host order
template <class T>
void putLE(std::vector<unsigned char> &b, T v) {
    uint64_t u = 0;
    if constexpr (std::is_same<T, double>::value) {
        std::memcpy(&u, &v, 8);
    } else {
        u = (uint64_t)(int64_t)v;
    }
    for (size_t k = 0; k < sizeof(T); k++) b.push_back((unsigned char)(u >> (8 * k) & 0xff));
}

template <class T>
std::string dataArray(const char *name, const char *vtkType, int ncomp, const std::vector<T> &vals) {
    std::vector<unsigned char> bytes;
    bytes.reserve(8 + sizeof(T) * vals.size());
    putLE<uint64_t>(bytes, (uint64_t)(sizeof(T) * vals.size()));
    for (const T &v : vals) putLE<T>(bytes, v);
    return std::string("<DataArray type=\"") + vtkType + "\" Name=\"" + name + "\" NumberOfComponents=\"" +
           std::to_string(ncomp) + "\" format=\"binary\">" + base64(bytes) + "</DataArray>\n";
}

}  // namespace

void SylinderSystem::writeSylinderVTK(const std::string &folder, int snapID, const std::vector<Sylinder> &rods) {
    const size_t n = rods.size();
    std::vector<double> pts(6 * n), radius(n), length(n), dir(3 * n);
    std::vector<int64_t> gid(n);
    std::vector<int32_t> conn(2 * n), offs(n), group(n), imm(n);
    for (size_t i = 0; i < n; i++) {
        const Sylinder &r = rods[i];
        double d[3];
        directionFromQuat(r.orientation, d);
        const double h = 0.5 * r.length;
        for (int k = 0; k < 3; k++) {
            pts[6 * i + k] = r.pos[k] - h * d[k];
            pts[6 * i + 3 + k] = r.pos[k] + h * d[k];
            dir[3 * i + k] = d[k];
        }
        conn[2 * i] = (int32_t)(2 * i);
        conn[2 * i + 1] = (int32_t)(2 * i + 1);
        offs[i] = (int32_t)(2 * i + 2);
        gid[i] = r.gid;
        radius[i] = r.radius;
        length[i] = r.length;
        group[i] = r.group;
        imm[i] = r.isImmovable ? 1 : 0;
    }
    const std::string sep = (folder.empty() || folder.back() == '/') ? "" : "/";
    const std::string piece = "Sylinder_r0_" + std::to_string(snapID) + ".vtp";
    const char *head = "<?xml version=\"1.0\"?>\n";
    {
        std::ofstream f(folder + sep + piece, std::ios::binary);
        if (!f) throw std::runtime_error("cannot write " + folder + sep + piece);
        f << head << "<VTKFile type=\"PolyData\" version=\"1.0\" byte_order=\"LittleEndian\" header_type=\"UInt64\">\n"
          << "<PolyData>\n<Piece NumberOfPoints=\"" << 2 * n << "\" NumberOfVerts=\"0\" NumberOfLines=\"" << n
          << "\" NumberOfStrips=\"0\" NumberOfPolys=\"0\">\n"
          << "<Points>\n" << dataArray("position", "Float64", 3, pts) << "</Points>\n"
          << "<Lines>\n" << dataArray("connectivity", "Int32", 1, conn) << dataArray("offsets", "Int32", 1, offs)
          << "</Lines>\n<CellData Scalars=\"scalars\">\n"
          << dataArray("gid", "Int64", 1, gid) << dataArray("radius", "Float64", 1, radius)
          << dataArray("length", "Float64", 1, length) << dataArray("group", "Int32", 1, group)
          << dataArray("isImmovable", "Int32", 1, imm) << dataArray("direction", "Float64", 3, dir)
          << "</CellData>\n</Piece>\n</PolyData>\n</VTKFile>\n";
    }
    std::ofstream f(folder + sep + "Sylinder_" + std::to_string(snapID) + ".pvtp", std::ios::binary);
    if (!f) throw std::runtime_error("cannot write the index of " + piece);
    f << head << "<VTKFile type=\"PPolyData\" version=\"1.0\" byte_order=\"LittleEndian\" header_type=\"UInt64\">\n"
      << "<PPolyData GhostLevel=\"0\">\n<PPoints>\n"
      << "<PDataArray type=\"Float64\" Name=\"position\" NumberOfComponents=\"3\"/>\n</PPoints>\n"
      << "<PCellData Scalars=\"scalars\">\n"
      << "<PDataArray type=\"Int64\" Name=\"gid\" NumberOfComponents=\"1\"/>\n"
      << "<PDataArray type=\"Float64\" Name=\"radius\" NumberOfComponents=\"1\"/>\n"
      << "<PDataArray type=\"Float64\" Name=\"length\" NumberOfComponents=\"1\"/>\n"
      << "<PDataArray type=\"Int32\" Name=\"group\" NumberOfComponents=\"1\"/>\n"
      << "<PDataArray type=\"Int32\" Name=\"isImmovable\" NumberOfComponents=\"1\"/>\n"
      << "<PDataArray type=\"Float64\" Name=\"direction\" NumberOfComponents=\"3\"/>\n"
      << "</PCellData>\n<Piece Source=\"" << piece << "\"/>\n</PPolyData>\n</VTKFile>\n";
}

std::vector<ConBlockRecord> SylinderSystem::getConBlocks() {
    std::vector<ConBlockRecord> out;
    if (!ctx_ || !haveBlocks_) return out;
    int nc = 0, nb = 0;
    check(alens_get_num_constraints(ctx_, 0, &nc, &nb), "alens_get_num_constraints");
    const int n = nc + nb;
    if (n == 0) return out;
    std::vector<int32_t> ii(n), jj(n), img(n);
    std::vector<double> d0(n), gam(n), jac(12 * (size_t)n), lab(6 * (size_t)n), cinv(n), lb(n);
    check(alens_get_constraints(ctx_, 0, n, ii.data(), jj.data(), img.data(), d0.data(), gam.data(), jac.data()),
          "alens_get_constraints");
    check(alens_get_constraint_points(ctx_, 0, n, lab.data()), "alens_get_constraint_points");
    int nnz = 0;
    check(alens_get_operator(ctx_, 0, 0, &nnz, nullptr, nullptr, nullptr, nullptr, cinv.data(), lb.data(), nullptr),
          "alens_get_operator");
    const auto &rods = getContainer();
    out.resize((size_t)n);
    for (int k = 0; k < n; k++) {
        ConBlockRecord &r = out[(size_t)k];
        r.gamma = gam[k];
        r.delta0 = d0[k];
        r.kappa = cinv[k] > 0.0 ? 1.0 / cinv[k] : 0.0;
        r.bilateral = std::isinf(lb[k]) && lb[k] < 0.0 ? 1 : 0;
        r.oneSide = jj[k] < 0 ? 1 : 0;
        r.globalIndexI = ii[k];
        r.globalIndexJ = jj[k];
        r.gidI = rods[(size_t)ii[k]].gid;
        r.gidJ = jj[k] >= 0 ? rods[(size_t)jj[k]].gid : -1;
        r.image = img[k];
        for (int d = 0; d < 3; d++) {
            r.normI[d] = jac[12 * (size_t)k + d];
            r.labI[d] = lab[6 * (size_t)k + d];
            r.labJ[d] = lab[6 * (size_t)k + 3 + d];
        }
    }
    return out;
}

void SylinderSystem::writeConBlockVTK(const std::string &folder, int snapID, const std::vector<ConBlockRecord> &blocks) {
    const size_t n = blocks.size();
    std::vector<double> pts(6 * n), gamma(n), delta0(n), kappa(n), norm(3 * n), stress(9 * n);
    std::vector<int64_t> gidI(n), gidJ(n);
    std::vector<int32_t> conn(2 * n), offs(n), bil(n), one(n), gI(n), gJ(n), img(n);
    for (size_t k = 0; k < n; k++) {
        const ConBlockRecord &b = blocks[k];
        double r[3];
        for (int d = 0; d < 3; d++) {
            pts[6 * k + d] = b.labI[d];
            pts[6 * k + 3 + d] = b.labJ[d];
            norm[3 * k + d] = b.normI[d];
            r[d] = b.labI[d] - b.labJ[d];
        }
        for (int a = 0; a < 3; a++)
            for (int c = 0; c < 3; c++) stress[9 * k + 3 * a + c] = (b.gamma * r[a]) * b.normI[c];
        conn[2 * k] = (int32_t)(2 * k);
        conn[2 * k + 1] = (int32_t)(2 * k + 1);
        offs[k] = (int32_t)(2 * k + 2);
        gamma[k] = b.gamma;
        delta0[k] = b.delta0;
        kappa[k] = b.kappa;
        bil[k] = b.bilateral;
        one[k] = b.oneSide;
        gidI[k] = b.gidI;
        gidJ[k] = b.gidJ;
        gI[k] = b.globalIndexI;
        gJ[k] = b.globalIndexJ;
        img[k] = b.image;
    }
    const std::string sep = (folder.empty() || folder.back() == '/') ? "" : "/";
    const std::string piece = "ConBlock_r0_" + std::to_string(snapID) + ".vtp";
    const char *head = "<?xml version=\"1.0\"?>\n";
    {
        std::ofstream f(folder + sep + piece, std::ios::binary);
        if (!f) throw std::runtime_error("cannot write " + folder + sep + piece);
        f << head << "<VTKFile type=\"PolyData\" version=\"1.0\" byte_order=\"LittleEndian\" header_type=\"UInt64\">\n"
          << "<PolyData>\n<Piece NumberOfPoints=\"" << 2 * n << "\" NumberOfVerts=\"0\" NumberOfLines=\"" << n
          << "\" NumberOfStrips=\"0\" NumberOfPolys=\"0\">\n"
          << "<Points>\n" << dataArray("position", "Float64", 3, pts) << "</Points>\n"
          << "<Lines>\n" << dataArray("connectivity", "Int32", 1, conn) << dataArray("offsets", "Int32", 1, offs)
          << "</Lines>\n<CellData Scalars=\"scalars\">\n"
          << dataArray("gamma", "Float64", 1, gamma) << dataArray("delta0", "Float64", 1, delta0)
          << dataArray("kappa", "Float64", 1, kappa) << dataArray("bilateral", "Int32", 1, bil)
          << dataArray("oneSide", "Int32", 1, one) << dataArray("gidI", "Int64", 1, gidI)
          << dataArray("gidJ", "Int64", 1, gidJ) << dataArray("globalIndexI", "Int32", 1, gI)
          << dataArray("globalIndexJ", "Int32", 1, gJ) << dataArray("image", "Int32", 1, img)
          << dataArray("normI", "Float64", 3, norm) << dataArray("Stress", "Float64", 9, stress)
          << "</CellData>\n</Piece>\n</PolyData>\n</VTKFile>\n";
    }
    std::ofstream f(folder + sep + "ConBlock_" + std::to_string(snapID) + ".pvtp", std::ios::binary);
    if (!f) throw std::runtime_error("cannot write the index of " + piece);
    f << head << "<VTKFile type=\"PPolyData\" version=\"1.0\" byte_order=\"LittleEndian\" header_type=\"UInt64\">\n"
      << "<PPolyData GhostLevel=\"0\">\n<PPoints>\n"
      << "<PDataArray type=\"Float64\" Name=\"position\" NumberOfComponents=\"3\"/>\n</PPoints>\n"
      << "<PCellData Scalars=\"scalars\">\n";
    static const char *kFields[][3] = {{"Float64", "gamma", "1"},      {"Float64", "delta0", "1"},
                                       {"Float64", "kappa", "1"},      {"Int32", "bilateral", "1"},
                                       {"Int32", "oneSide", "1"},      {"Int64", "gidI", "1"},
                                       {"Int64", "gidJ", "1"},         {"Int32", "globalIndexI", "1"},
                                       {"Int32", "globalIndexJ", "1"}, {"Int32", "image", "1"},
                                       {"Float64", "normI", "3"},      {"Float64", "Stress", "9"}};
    for (const auto &fl : kFields)
        f << "<PDataArray type=\"" << fl[0] << "\" Name=\"" << fl[1] << "\" NumberOfComponents=\"" << fl[2] << "\"/>\n";
    f << "</PCellData>\n<Piece Source=\"" << piece << "\"/>\n</PPolyData>\n</VTKFile>\n";
}

DomainInfo DomainInfo::fromConfig(const SylinderConfig &cfg) {
    DomainInfo d;
    for (int k = 0; k < 3; k++) {
        d.low[k] = cfg.simBoxLow[k];
        d.high[k] = cfg.simBoxHigh[k];
        d.pbc[k] = cfg.simBoxPBC[k];
    }
    return d;
}

RngPool::RngPool(unsigned long long seed, int nThreads) {
    streams_.resize(std::max(1, nThreads));
    for (size_t t = 0; t < streams_.size(); t++) {
        std::seed_seq seq{(unsigned)(seed & 0xffffffffu), (unsigned)(seed >> 32), (unsigned)t};
        streams_[t].eng.seed(seq);
    }
}

RngPool::Stream &RngPool::at(int threadId) {
    if (threadId < 0 || threadId >= (int)streams_.size())
        throw std::out_of_range("RngPool: thread id " + std::to_string(threadId));
    return streams_[threadId];
}

double RngPool::getU01(int threadId) {
    Stream &s = at(threadId);
    return ((double)(s.eng() >> 11) + 0.5) * 0x1p-53;
}

double RngPool::getN01(int threadId) {
    Stream &s = at(threadId);
    if (s.hasSpare) {
        s.hasSpare = false;
        return s.spare;
    }
    const double u1 = ((double)(s.eng() >> 11) + 0.5) * 0x1p-53;
    const double u2 = ((double)(s.eng() >> 11) + 0.5) * 0x1p-53;
    const double r = std::sqrt(-2.0 * std::log(u1));
    const double th = 6.283185307179586 * u2;
    s.spare = r * std::sin(th);
    s.hasSpare = true;
    return r * std::cos(th);
}

void SylinderSystem::writeResult(const std::string &path) const {
    auto *self = const_cast<SylinderSystem *>(this);
    const auto &rods = self->getContainer();
    std::FILE *f = std::fopen(path.c_str(), "w");
    if (!f) throw std::runtime_error("cannot write " + path);
    std::fprintf(f, "%zu\n%.17g\n", rods.size(), runConfig.dt * (double)getStepCount());
    for (const auto &r : rods) {
        double d[3];
        directionFromQuat(r.orientation, d);
        const double h = 0.5 * r.length;
        std::fprintf(f, "%c %lld %.17g %.17g %.17g %.17g %.17g %.17g %.17g %d\n", r.isImmovable ? 'S' : 'C',
                     (long long)r.gid, r.radius, r.pos[0] - h * d[0], r.pos[1] - h * d[1], r.pos[2] - h * d[2],
                     r.pos[0] + h * d[0], r.pos[1] + h * d[1], r.pos[2] + h * d[2], r.group);
    }
    for (const auto &l : links_) std::fprintf(f, "L %lld %lld\n", (long long)l[0], (long long)l[1]);
    std::fclose(f);
}

void SylinderSystem::printTimingSummary() const {
    if (!timerOn_) return;
    std::printf("rodSystem step %ld: %d collisions, %d bilateral, %d BBPGD iterations, residual %.3e, %.3f ms\n",
                (long)stats_.step, stats_.nCollision, stats_.nBilateral, stats_.iterations, stats_.residual,
                lastStepMs_);
}


void SylinderSystem::setProteinTypes(const std::vector<AlensProteinType> &types, double KBT) {
    if (!ctx_) throw std::runtime_error("setProteinTypes: initialize() first");
    check(alens_set_protein_types(ctx_, (int)types.size(), types.data(), KBT, runConfig.sylinderDiameter),
          "alens_set_protein_types");
    proteinTags_.clear();
    for (const AlensProteinType &t : types) proteinTags_.push_back(t.tag);
}

void SylinderSystem::setProteins(const std::vector<AlensProtein> &proteins) {
    if (!ctx_) throw std::runtime_error("setProteins: initialize() first");
    check(alens_set_proteins(ctx_, 0, (int)proteins.size(), proteins.data()), "alens_set_proteins");
    haveProteins_ = !proteins.empty();
}

std::vector<AlensProtein> SylinderSystem::getProteins() {
    if (!ctx_) return {};
    int n = 0;
    const int rc = alens_get_proteins(ctx_, 0, 0, &n, nullptr);
    if (rc != ALENS_OK && rc != ALENS_CAPACITY) check(rc, "alens_get_proteins");
    std::vector<AlensProtein> out(n);
    if (n > 0) check(alens_get_proteins(ctx_, 0, n, &n, out.data()), "alens_get_proteins");
    return out;
}

AlensKmcStats SylinderSystem::updateProteinMotion() {
    if (!ctx_) throw std::runtime_error("updateProteinMotion: initialize() first");
    AlensKmcStats st{};
    check(alens_protein_motion_step(ctx_, &st), "alens_protein_motion_step");
    return st;
}

AlensKmcStats SylinderSystem::calcBindInteraction() {
    if (!ctx_) throw std::runtime_error("calcBindInteraction: initialize() first");
    AlensKmcStats st{};
    check(alens_protein_bind_step(ctx_, &st), "alens_protein_bind_step");
    return st;
}

void SylinderSystem::writeProteinVTK(const std::string &folder, int snapID, const std::vector<AlensProtein> &proteins,
                                     const std::vector<int> &typeTag, const std::vector<int64_t> &rodGid) {
    const size_t n = proteins.size();
    std::vector<double> pts(6 * n);
    std::vector<int32_t> conn(2 * n), offs(n), ids(2 * n), gid(n), tag(n);
    for (size_t k = 0; k < n; k++) {
        const AlensProtein &p = proteins[k];
        const bool both = p.idBind[0] >= 0 && p.idBind[1] >= 0;
        for (int d = 0; d < 3; d++) {
            pts[6 * k + d] = both ? p.posEnd[0][d] : p.pos[d];
            pts[6 * k + 3 + d] = both ? p.posEnd[1][d] : p.pos[d];
        }
        for (int e = 0; e < 2; e++) ids[2 * k + e] = p.idBind[e] >= 0 ? (int32_t)rodGid.at(p.idBind[e]) : -1;
        conn[2 * k] = (int32_t)(2 * k);
        conn[2 * k + 1] = (int32_t)(2 * k + 1);
        offs[k] = (int32_t)(2 * k + 2);
        gid[k] = (int32_t)p.gid;
        tag[k] = typeTag.at(p.type);
    }
    const std::string sep = (folder.empty() || folder.back() == '/') ? "" : "/";
    const std::string piece = "Protein_r0_" + std::to_string(snapID) + ".vtp";
    const char *head = "<?xml version=\"1.0\"?>\n";
    {
        std::ofstream f(folder + sep + piece, std::ios::binary);
        if (!f) throw std::runtime_error("cannot write " + folder + sep + piece);
        f << head << "<VTKFile type=\"PolyData\" version=\"1.0\" byte_order=\"LittleEndian\" header_type=\"UInt64\">\n"
          << "<PolyData>\n<Piece NumberOfPoints=\"" << 2 * n << "\" NumberOfVerts=\"0\" NumberOfLines=\"" << n
          << "\" NumberOfStrips=\"0\" NumberOfPolys=\"0\">\n"
          << "<Points>\n" << dataArray("position", "Float64", 3, pts) << "</Points>\n"
          << "<Lines>\n" << dataArray("connectivity", "Int32", 1, conn) << dataArray("offsets", "Int32", 1, offs)
          << "</Lines>\n<PointData Scalars=\"scalars\">\n" << dataArray("idBind", "Int32", 1, ids)
          << "</PointData>\n<CellData Scalars=\"scalars\">\n" << dataArray("gid", "Int32", 1, gid)
          << dataArray("tag", "Int32", 1, tag) << "</CellData>\n</Piece>\n</PolyData>\n</VTKFile>\n";
    }
    std::ofstream f(folder + sep + "Protein_" + std::to_string(snapID) + ".pvtp", std::ios::binary);
    if (!f) throw std::runtime_error("cannot write the index of " + piece);
    f << head << "<VTKFile type=\"PPolyData\" version=\"1.0\" byte_order=\"LittleEndian\" header_type=\"UInt64\">\n"
      << "<PPolyData GhostLevel=\"0\">\n<PPoints>\n"
      << "<PDataArray type=\"Float64\" Name=\"position\" NumberOfComponents=\"3\"/>\n</PPoints>\n"
      << "<PPointData Scalars=\"scalars\">\n<PDataArray type=\"Int32\" Name=\"idBind\" NumberOfComponents=\"1\"/>\n"
      << "</PPointData>\n<PCellData Scalars=\"scalars\">\n"
      << "<PDataArray type=\"Int32\" Name=\"gid\" NumberOfComponents=\"1\"/>\n"
      << "<PDataArray type=\"Int32\" Name=\"tag\" NumberOfComponents=\"1\"/>\n"
      << "</PCellData>\n<Piece Source=\"" << piece << "\"/>\n</PPolyData>\n</VTKFile>\n";
}

void SylinderSystem::writeProteinAscii(const std::string &path, const std::vector<AlensProtein> &proteins,
                                       const std::vector<int> &typeTag, const std::vector<int64_t> &rodGid,
                                       double time) {
    std::FILE *f = std::fopen(path.c_str(), "w");
    if (!f) throw std::runtime_error("cannot write " + path);
    std::fprintf(f, "%d \n %lf\n", (int)proteins.size(), time);
    for (const AlensProtein &p : proteins) {
        long long g[2];
        for (int e = 0; e < 2; e++) g[e] = p.idBind[e] >= 0 ? (long long)rodGid.at(p.idBind[e]) : -1LL;
        const double *a = p.pos, *b = p.pos;
        if (g[0] != -1 && g[1] != -1) {
            a = p.posEnd[0];
            b = p.posEnd[1];
        }
        std::fprintf(f, "P %lld %d %.6g %.6g %.6g %.6g %.6g %.6g %lld %lld\n", (long long)p.gid,
                     typeTag.at(p.type), a[0], a[1], a[2], b[0], b[1], b[2], g[0], g[1]);
    }
    std::fclose(f);
}

}  // namespace gpu
