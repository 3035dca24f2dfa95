// kmc.cuh - device state of the protein binding step (two-stage KMC model:
// unbound U, singly bound S, doubly bound D).
//
// Layout in HBM:
//   proteins   AoS AlensProtein (112 B) + replica index, all replicas
//              concatenated in the order they were set
//   species    KmcType per protein type (rates folded with dt, see below)
//   rod view   per rod (global index): wrapped centre + half-length, unit
//              axis + sphere flag (2 x 32 B, FP64), rebuilt each step
//   cells      uniform grid per replica whose edge is at least the binding
//              reach (largest rod half-length + largest capture distance):
//              count / exclusive start / cursor per cell; by cell slot the
//              rod index and its FP32 screening geometry (centre relative
//              to the cell origin, half-length, axis: 32 B)
//   springs    doubly bound flag and its exclusive scan per protein; the
//              springs are written into the context's link rows
#pragma once

#include "engine.cuh"

namespace alens {

// four doubles on a 32-byte boundary (one 32-byte load)
struct __align__(32) KDouble4 {
    double x, y, z, w;
};
__host__ __device__ inline KDouble4 make_kd4(double x, double y, double z, double w) { return KDouble4{x, y, z, w}; }

// Per species: the rates of Protein/ProteinModel.md with dt folded in.
struct KmcType {
    double ell0;        // rest length (freeLength)
    double c;           // centre of the S->D exponent: ell0 + D (lookupType 0), ell0 (1)
    double A;           // (1 - lambda) kappa / (2 KBT): S->D Boltzmann exponent
    double w;           // support half-width of the S->D integrand in head distance
    double rOuter;      // ell0 + D + w: farthest head distance with a non-zero S->D rate
    double Ads;         // lambda kappa / (2 KBT): D->S load sensitivity
    double rcap;        // U->S capture radius: max(rc, sqrt(6 diffUnbound dt))
    double PtoAP;       // parallel / antiparallel S->D binding ratio
    double usCoef[2];   // ko_s Ka eps * 3 / (4 pi rcap^3) * dt  (times L_c)
    double suProb[2];   // ko_s dt
    double sdCoef[2];   // ko_d Ke eps dt [/ Vb]               (times the integral)
    double koD[2];      // ko_d
    double dt;
    double kappa;       // spring constant of the D-stage spring
    // FP32 copies for the unbound / singly bound stages (the conversions
    // would issue on the FP64 pipe)
    float rcapf, rOuterf, wf, Af, cf;
    float usCoeff[2], suProbf[2], sdCoeff[2];
    float prefPar, prefAnti;  // PtoAPratio prefactor for a parallel / antiparallel rod
    float Df;                 // rod diameter (lookupType 1 stretch factor 1 - D/d)
    int lookup;               // 0: stretch r - D; 1: (1 - D/d) r (Protein/ProteinData.hpp:171-195)
    // motion step (Protein/ProteinData.hpp:318-498)
    int walkOff, vdrag[2], pad;
    double fstall, vmax[2], vmaxAP[2];
    double diffS[2], diffD[2], diffU;  // sqrt(dt D 2) of the bound heads and the free protein
    double dragD[2];                   // diffBoundD (drag velocity = load x diffBoundD / KBT)
    double KBT;
};

struct KmcRep {
    double lo[3], hi[3], L[3], cellsz[3];
    float cellszf[3];
    int pbc[3], ncell[3];
    int cellOffset, rodOffset, nRods, protOffset, nProt;
    int userLinks;      // links of alens_set_links (their rows come first)
    unsigned long long seed;
};

struct KmcDev {
    int nProt, R, nCells, nTypes;
    AlensProtein *prot;
    int *protRep;
    const KmcType *types;   // nTypes per replica (dt is per replica)
    const KmcRep *rep;
    KDouble4 *rodC;      // wrapped centre, half-length
    KDouble4 *rodA;      // axis, 1 for a sphere-shaped rod
    int *cellCount, *cellStart, *cellCursor, *cellRod;
    float4 *cellRel;     // by cell slot: centre relative to the cell origin, half-length (FP32)
    float4 *cellAx;      // by cell slot: axis, 1 for a sphere-shaped rod
    int *dFlag, *dScan;  // nProt + 1 each
    void *task;          // per protein: 64-byte task of the unbound / singly bound stages
    int *stats;          // 8 per replica: nU nS nD nUS nSU nSD nDS maxCand
    int *dCount;         // doubly bound proteins per replica
    int *err;
    long long step;
    double D;
};

constexpr int kKmcMaxCand = 64;     // candidate rods one protein may weigh in a step
constexpr int kKmcErrCand = 1;      // a protein had more candidates (its state is kept)
constexpr int kKmcErrSpring = 2;    // a spring row fell outside the link capacity

void launch_kmc_bin(const KmcDev &K, const DevState &S, cudaStream_t st);
void launch_kmc_view(const KmcDev &K, const DevState &S, cudaStream_t st);  // rod view only, no cell counts
void launch_kmc_scatter(const KmcDev &K, const DevState &S, cudaStream_t st);
int launch_kmc_bind(const KmcDev &K, cudaStream_t st);  // returns kernels launched
// one motion step (walk, drag, diffusion, walk-off, boundaries) then the
// new geometry and the per-replica counts; returns kernels launched
int launch_kmc_motion(const KmcDev &K, const DevState &S, cudaStream_t st);
// doubly bound flags, their scan and the spring rows at link offset
// userTotal (capacity linkCap); dCount per replica
int launch_kmc_springs(const KmcDev &K, const DevState &S, int userTotal, int linkCap, cudaStream_t st);

}  // namespace alens
