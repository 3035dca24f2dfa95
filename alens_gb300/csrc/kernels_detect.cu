// kernels_detect.cu - detect stage of the rod step: known (Brownian)
// velocity, cell binning, near-pair search with segment-segment closest
// points, canonical pair order, constraint assembly (Jacobian D, phi0, q,
// initial gamma) and the rod-major rows of D.
//
// The role of SimToolbox's FDPS near-neighbour search + CalcSylinderNearForce
// + DCPQuery + ConstraintCollector (called from SylinderSystem::runStep,
// SRC/TubuleSystem.cpp:223; collision buffer sylinderColBuf,
// docs/source/quickstart.md:346-348; bilateral blocks as built in
// SRC/TubuleSystem.cpp:714-742).
//
// Compiled with --fmad=false: FP64 results equal the oracle's bit for bit.
#include <cmath>

#include "engine.cuh"

namespace alens {

namespace {

__device__ __forceinline__ int flags(const DevState &S) { return ld_volatile_i32(&S.ctl->errFlags); }

__device__ __forceinline__ int cell_coord(double v, double lo, double cs, int n) {
    const double f = floor((v - lo) / cs);
    return f < 0.0 ? 0 : (f > (double)(n - 1) ? n - 1 : (int)f);
}

// ------------------------------------------------------------------ prep
__global__ void k_prep(DevState S) {
    ALENS_PDL_PROLOGUE();
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < S.nRods; r += gridDim.x * blockDim.x) {
        const int rep = S.rodRep[r];
        const RepParams &P = S.par[rep];
        double p[3] = {S.px[r], S.py[r], S.pz[r]};
        const double qx = S.qx[r], qy = S.qy[r], qz = S.qz[r], qw = S.qw[r];
        if (!isfinite(p[0]) || !isfinite(p[1]) || !isfinite(p[2]) || !isfinite(qx) ||
            !isfinite(qy) || !isfinite(qz) || !isfinite(qw)) {
            atomicOr(&S.ctl->errFlags, kErrNaN);
            S.cellOf[r] = P.cellOffset;
            atomicAdd(&S.cellCount[P.cellOffset], 1);
            continue;
        }
        for (int d = 0; d < 3; d++) {
            if (!P.pbc[d]) continue;
            const double lo = P.lo[d], hi = P.hi[d], Lb = P.L[d];
            double v = p[d];
            for (int k = 0; k < 64; k++) {
                if (v < lo)
                    v = v + Lb;
                else if (v >= hi)
                    v = v - Lb;
                else
                    break;
            }
            p[d] = v;
        }
        S.px[r] = p[0];
        S.py[r] = p[1];
        S.pz[r] = p[2];
        double a[3];
        quat_axis(qx, qy, qz, qw, a);
        S.ax[r] = a[0];
        S.ay[r] = a[1];
        S.az[r] = a[2];
        const double L = S.len[r], rad = S.rad[r];
        const bool sphere = L < 2.0 * rad;
        S.sph[r] = sphere ? 1 : 0;
        S.hcol[r] = sphere ? 0.0 : 0.5 * (L * P.colRatioL);
        S.rcol[r] = rad * P.colRatioD;
        const int cx = cell_coord(p[0], P.lo[0], P.cellsz[0], P.ncell[0]);
        const int cy = cell_coord(p[1], P.lo[1], P.cellsz[1], P.ncell[1]);
        const int cz = cell_coord(p[2], P.lo[2], P.cellsz[2], P.ncell[2]);
        const int cid = P.cellOffset + (cz * P.ncell[1] + cy) * P.ncell[0] + cx;
        S.cellOf[r] = cid;
        atomicAdd(&S.cellCount[cid], 1);
    }
}

// Known (Brownian) velocity of every rod: U_B = sqrt(2 kT / dt) M^(1/2) xi
// with xi from Philox keyed by (seed, gid, step).  Runs beside the pair
// search (it needs only the axes and flags that k_prep wrote); the
// constraint build consumes it.
__global__ void k_noise(DevState S) {
    ALENS_PDL_PROLOGUE();
    if (flags(S) & kErrNaN) return;
    const long long step = S.ctl->step;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < S.nRods; r += gridDim.x * blockDim.x) {
        const RepParams &P = S.par[S.rodRep[r]];
        const double a[3] = {S.ax[r], S.ay[r], S.az[r]};
        const bool sphere = S.sph[r] != 0;
        const bool imm = S.imm[r] != 0;
        double u[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
        if (P.kT > 0.0 && !imm) {
            const double bc = P.bcoef;
            double z[6];
            normals6(P.seed, S.gid[r], step, z);
            if (P.mono) {
                z[2] = 0.0;
                z[3] = 0.0;
                z[4] = 0.0;
            }
            double w[6];
            if (sphere) {
                const double st = S.sm0[r], sr = S.sm2[r];
                w[0] = st * z[0];
                w[1] = st * z[1];
                w[2] = st * z[2];
                w[3] = sr * z[3];
                w[4] = sr * z[4];
                w[5] = sr * z[5];
            } else {
                const double sp = S.sm0[r], sq = S.sm1[r], sr = S.sm2[r];
                const double za = a[0] * z[0] + a[1] * z[1] + a[2] * z[2];
                w[0] = sp * za * a[0] + sq * (z[0] - za * a[0]);
                w[1] = sp * za * a[1] + sq * (z[1] - za * a[1]);
                w[2] = sp * za * a[2] + sq * (z[2] - za * a[2]);
                const double ra = a[0] * z[3] + a[1] * z[4] + a[2] * z[5];
                w[3] = sr * (z[3] - ra * a[0]);
                w[4] = sr * (z[4] - ra * a[1]);
                w[5] = sr * (z[5] - ra * a[2]);
            }
            if (P.mono) {
                w[2] = 0.0;
                w[3] = 0.0;
                w[4] = 0.0;
            }
#pragma unroll
            for (int k = 0; k < 6; k++) u[k] = bc * w[k];
        }
#pragma unroll
        for (int k = 0; k < 6; k++) S.unc[(size_t)k * S.nRods + r] = u[k];
    }
}

// Start of a step: the counters the detect stage accumulates into (one
// launch instead of a memset per array).
__global__ void k_step_clear(DevState S) {
    ALENS_PDL_PROLOGUE();
    const int stride = gridDim.x * blockDim.x;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t == 0) {
        S.ctl->rawCount = 0;
        S.ctl->errFlags = 0;
        S.ctl->borderCount = 0;
    }
    for (int c = t; c < S.nCells; c += stride) {
        S.cellCount[c] = 0;
        S.cellCursor[c] = 0;
    }
    for (int r = t; r < S.nRods; r += stride) {
        S.pairCursor[r] = 0;
        S.pairCount[r] = 0;
        S.rowCount[r] = 0;
        S.rowCursor[r] = 0;
    }
}

// Drag mobilities depend only on the rod geometry: computed once per rod set.
__global__ void k_mobility(DevState S) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < S.nRods; r += gridDim.x * blockDim.x) {
        const RepParams &P = S.par[S.rodRep[r]];
        const double L = S.len[r], rad = S.rad[r];
        double m[3] = {0.0, 0.0, 0.0};
        if (!S.imm[r]) mobility_coeffs(L, rad, P.mu, L < 2.0 * rad, m);
        S.m0[r] = m[0];
        S.m1[r] = m[1];
        S.m2[r] = m[2];
        S.sm0[r] = sqrt(m[0]);
        S.sm1[r] = sqrt(m[1]);
        S.sm2[r] = sqrt(m[2]);
    }
}

// ------------------------------------------------------------------ scan
// Exclusive scan of n ints: out[0..n] (out[n] = total).  Three passes:
// per-block scan of 1024 elements, scan of block totals, add.
constexpr int kScanBlock = 256;
constexpr int kScanPer = 4;
constexpr int kScanSpan = kScanBlock * kScanPer;

__device__ __forceinline__ int block_exclusive_scan(int v, int *smem32, int *total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int incl = v;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const int o = __shfl_up_sync(0xffffffffu, incl, off);
        if (lane >= off) incl += o;
    }
    if (lane == 31) smem32[warp] = incl;
    __syncthreads();
    const int nw = blockDim.x >> 5;
    if (warp == 0) {
        int w = lane < nw ? smem32[lane] : 0;
        int wi = w;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const int o = __shfl_up_sync(0xffffffffu, wi, off);
            if (lane >= off) wi += o;
        }
        if (lane < nw) smem32[lane] = wi - w;
        if (lane == nw - 1) smem32[32] = wi;
    }
    __syncthreads();
    const int res = incl - v + smem32[warp];
    if (total) *total = smem32[32];
    __syncthreads();
    return res;
}

__global__ void k_scan_block(const int *in, int *out, int n, int *tmp) {
    ALENS_PDL_PROLOGUE();
    __shared__ int sm[33];
    const int base = blockIdx.x * kScanSpan + threadIdx.x * kScanPer;
    int v[kScanPer];
    int s = 0;
#pragma unroll
    for (int k = 0; k < kScanPer; k++) {
        v[k] = (base + k < n) ? in[base + k] : 0;
        s += v[k];
    }
    int tot;
    int ex = block_exclusive_scan(s, sm, &tot);
#pragma unroll
    for (int k = 0; k < kScanPer; k++) {
        if (base + k < n) out[base + k] = ex;
        ex += v[k];
    }
    if (threadIdx.x == 0) tmp[blockIdx.x] = tot;
}

__global__ void k_scan_top(int *tmp, int nb, int *out, int n) {
    ALENS_PDL_PROLOGUE();
    __shared__ int sm[33];
    // up to 1024 threads x 4 = 4096 block totals
    const int base = threadIdx.x * 4;
    int v[4];
    int s = 0;
    for (int k = 0; k < 4; k++) {
        v[k] = (base + k < nb) ? tmp[base + k] : 0;
        s += v[k];
    }
    int tot;
    int ex = block_exclusive_scan(s, sm, &tot);
    for (int k = 0; k < 4; k++) {
        if (base + k < nb) tmp[base + k] = ex;
        ex += v[k];
    }
    if (threadIdx.x == 0) out[n] = tot;
}

// Exclusive scan of up to kScanSingleMax ints by one 1024-thread block,
// one launch instead of three for the per-rod and per-cell counts.  Warp w owns the contiguous segment [w G, (w + 1) G) (G a
// multiple of 128); its lanes read consecutive int4 (coalesced), a round's
// loads all in flight together.  Pass 1 sums each segment, one block scan
// over the 32 segment totals gives the offsets, pass 2 writes the prefixes
// (warp scan per 128 elements plus a running carry) from the values kept
// in registers (up to kScanSingleMax counts) or read again.
constexpr int kScanSingleThreads = 1024;
constexpr int kScanSingleMax = 32768;  // above this the three-pass scan is faster
constexpr int kScanRound = 4;  // int4 loads per lane per round

__device__ __forceinline__ int4 scan_load4(const int *in, int i, int end, bool vec) {
    if (vec && i + 3 < end) return *reinterpret_cast<const int4 *>(in + i);
    int4 q;
    q.x = i < end ? in[i] : 0;
    q.y = i + 1 < end ? in[i + 1] : 0;
    q.z = i + 2 < end ? in[i + 2] : 0;
    q.w = i + 3 < end ? in[i + 3] : 0;
    return q;
}

__global__ void __launch_bounds__(kScanSingleThreads) k_scan_single(const int *in, int *out, int n, int vec,
                                                                    const int *nDev) {
    ALENS_PDL_PROLOGUE();
    // a count the device holds (the step's constraints) bounds the scan
    if (nDev) n = min(*nDev, n);
    __shared__ int sm[33];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int G = (((n + 31) / 32) + 127) & ~127;
    const int s0 = min(warp * G, n), s1 = min(s0 + G, n);
    // up to kScanSingleMax counts a warp's segment (G <= 1024) fits two
    // rounds of int4 per lane: it is read once and kept in registers
    constexpr int kIt = kScanSingleMax / 32 / (128 * kScanRound);
    const bool inRegs = n <= kScanSingleMax;
    int4 qr[kIt][kScanRound];
    int s = 0;
    if (inRegs) {
#pragma unroll
        for (int it = 0; it < kIt; it++) {
            const int r = s0 + it * 128 * kScanRound;
#pragma unroll
            for (int j = 0; j < kScanRound; j++) {
                qr[it][j] = r < s1 ? scan_load4(in, r + 128 * j + 4 * lane, s1, vec != 0) : make_int4(0, 0, 0, 0);
                s += qr[it][j].x + qr[it][j].y + qr[it][j].z + qr[it][j].w;
            }
        }
    } else {
        for (int r = s0; r < s1; r += 128 * kScanRound) {
            int4 q[kScanRound];
#pragma unroll
            for (int j = 0; j < kScanRound; j++) q[j] = scan_load4(in, r + 128 * j + 4 * lane, s1, vec != 0);
#pragma unroll
            for (int j = 0; j < kScanRound; j++) s += q[j].x + q[j].y + q[j].z + q[j].w;
        }
    }
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
    int tot;
    // every lane of a warp holds the same s: the block scan sees it once
    const int segOff = block_exclusive_scan(lane == 0 ? s : 0, sm, &tot);
    int carry = __shfl_sync(0xffffffffu, segOff, 0);
    // prefixes of one 128-element chunk (warp scan plus the running carry)
    auto emit = [&](const int4 &q, int i) {
        const int t = q.x + q.y + q.z + q.w;
        int inc = t;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const int o = __shfl_up_sync(0xffffffffu, inc, off);
            if (lane >= off) inc += o;
        }
        int ex = carry + inc - t;
        int4 o;
        o.x = ex;
        ex += q.x;
        o.y = ex;
        ex += q.y;
        o.z = ex;
        ex += q.z;
        o.w = ex;
        if (vec && i + 3 < s1) {
            *reinterpret_cast<int4 *>(out + i) = o;
        } else {
            if (i < s1) out[i] = o.x;
            if (i + 1 < s1) out[i + 1] = o.y;
            if (i + 2 < s1) out[i + 2] = o.z;
            if (i + 3 < s1) out[i + 3] = o.w;
        }
        carry += __shfl_sync(0xffffffffu, inc, 31);
    };
    if (inRegs) {
#pragma unroll
        for (int it = 0; it < kIt; it++) {
            const int r = s0 + it * 128 * kScanRound;
            if (r < s1) {
#pragma unroll
                for (int j = 0; j < kScanRound; j++) emit(qr[it][j], r + 128 * j + 4 * lane);
            }
        }
    } else {
        for (int r = s0; r < s1; r += 128 * kScanRound) {
            int4 q[kScanRound];
#pragma unroll
            for (int j = 0; j < kScanRound; j++) q[j] = scan_load4(in, r + 128 * j + 4 * lane, s1, vec != 0);
#pragma unroll
            for (int j = 0; j < kScanRound; j++) emit(q[j], r + 128 * j + 4 * lane);
        }
    }
    if (threadIdx.x == 0) out[n] = tot;
}

__global__ void k_scan_add(int *out, int n, const int *tmp) {
    ALENS_PDL_PROLOGUE();
    const int add = tmp[blockIdx.x];
    const int base = blockIdx.x * kScanSpan + threadIdx.x * kScanPer;
#pragma unroll
    for (int k = 0; k < kScanPer; k++)
        if (base + k < n) out[base + k] += add;
}

// ------------------------------------------------------------- links
// Bilateral block of every pre-bound link from the current rod state:
// anchors P = c_I + sI a_I, Q = c_J + sJ a_J, d = P - Q reduced to the
// minimum image, spring extension |d| - rest (SRC/TubuleSystem.cpp:714-736).
__global__ void k_link_blocks(DevState S) {
    ALENS_PDL_PROLOGUE();
    if (flags(S) & kErrNaN) return;
    for (int L = blockIdx.x * blockDim.x + threadIdx.x; L < S.nLinks; L += gridDim.x * blockDim.x) {
        const int rep = S.linkRep[L];
        const RepParams &P = S.par[rep];
        const int I = S.linkI[L], J = S.linkJ[L];
        const double sI = S.linkSI[L], sJ = S.linkSJ[L];
        const double aI[3] = {S.ax[I], S.ay[I], S.az[I]};
        const double aJ[3] = {S.ax[J], S.ay[J], S.az[J]};
        const double pI[3] = {S.px[I] + sI * aI[0], S.py[I] + sI * aI[1], S.pz[I] + sI * aI[2]};
        const double pJ[3] = {S.px[J] + sJ * aJ[0], S.py[J] + sJ * aJ[1], S.pz[J] + sJ * aJ[2]};
        double d[3];
        for (int c = 0; c < 3; c++) {
            d[c] = pI[c] - pJ[c];
            if (P.pbc[c]) d[c] = d[c] - P.L[c] * floor(d[c] / P.L[c] + 0.5);
        }
        const double len = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
        double n[3] = {0.0, 0.0, 1.0};
        if (len > 0.0) {
            n[0] = d[0] / len;
            n[1] = d[1] / len;
            n[2] = d[2] / len;
        }
        const int slot = S.linkSlot0[rep] + S.linkLocal[L];
        AlensBlock &B = S.blocks[slot];
        const double delta0 = len - S.linkRest[L];
        B.delta0 = delta0;
        B.gamma = -delta0 * S.linkKappa[L];
        B.gidI = S.gid[I];
        B.gidJ = S.gid[J];
        B.globalIndexI = I - P.rodOffset;
        B.globalIndexJ = J - P.rodOffset;
        for (int c = 0; c < 3; c++) {
            B.normI[c] = n[c];
            B.normJ[c] = -n[c];
            B.posI[c] = sI * aI[c];
            B.posJ[c] = sJ * aJ[c];
            B.labI[c] = pI[c];
            B.labJ[c] = pI[c] - d[c];
        }
        B.oneSide = 0;
        B.bilateral = 1;
        B.kappa = S.linkKappa[L];
        B.gammaLB = 0.0;
        for (int c = 0; c < 9; c++) B.stress[c] = 0.0;
        S.blockRep[slot] = rep;
    }
}

// ------------------------------------------------------------- scatter
// Cell-sorted FP32 search geometry: centre relative to its cell origin and
// half-length (sA), axis and collision radius (sB).  Relative coordinates
// keep the FP32 screen accurate whatever the box size.
__global__ void k_scatter(DevState S) {
    ALENS_PDL_PROLOGUE();
    if (flags(S) & kErrNaN) return;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < S.nRods; r += gridDim.x * blockDim.x) {
        const int cid = S.cellOf[r];
        const int slot = S.cellStart[cid] + atomicAdd(&S.cellCursor[cid], 1);
        const RepParams &P = S.par[S.rodRep[r]];
        const int lc = cid - P.cellOffset;
        const int cx = lc % P.ncell[0], cy = (lc / P.ncell[0]) % P.ncell[1], cz = lc / (P.ncell[0] * P.ncell[1]);
        const double ox = P.lo[0] + (double)cx * P.cellsz[0];
        const double oy = P.lo[1] + (double)cy * P.cellsz[1];
        const double oz = P.lo[2] + (double)cz * P.cellsz[2];
        S.sA[slot] = make_float4((float)(S.px[r] - ox), (float)(S.py[r] - oy), (float)(S.pz[r] - oz),
                                 (float)S.hcol[r]);
        S.sB[slot] = make_float4((float)S.ax[r], (float)S.ay[r], (float)S.az[r], (float)S.rcol[r]);
        S.sidx[slot] = r;
    }
}

// ---------------------------------------------------------- pair search
constexpr int kPairBuf = 16;
constexpr int kPairThreads = 128;
// Screening margin (um) between the FP32 separation and the FP64 decision:
// candidates with |sep32 - colBuf| < margin are decided in FP64 with the
// oracle's arithmetic, all others by the FP32 value.  FP32 errors on
// cell-relative coordinates are below 1e-5 um.
constexpr float kScreenMargin = 1e-3f;

__device__ __forceinline__ void flush_keys(const DevState &S, const unsigned long long *buf, int nb) {
    const int base = atomicAdd(&S.ctl->rawCount, nb);
    for (int e = 0; e < nb; e++) {
        const int pos = base + e;
        if (pos < S.cap)
            S.rawKeys[pos] = buf[e];
        else
            atomicOr(&S.ctl->errFlags, kErrOverflow);
    }
}

__device__ __forceinline__ float clampf_(float x, float lo, float hi) { return x < lo ? lo : (x > hi ? hi : x); }

// segment distance in FP32 (screen only)
__device__ __forceinline__ float dcp_dist32(float3 c1, float3 u1, float h1, float3 c2, float3 u2, float h2) {
    const float w0 = c1.x - c2.x, w1 = c1.y - c2.y, w2 = c1.z - c2.z;
    const float b = u1.x * u2.x + u1.y * u2.y + u1.z * u2.z;
    const float d = u1.x * w0 + u1.y * w1 + u1.z * w2;
    const float e = u2.x * w0 + u2.y * w1 + u2.z * w2;
    const float det = 1.0f - b * b;
    float s;
    if (det > 1e-6f) {
        s = clampf_((b * e - d) / det, -h1, h1);
    } else {
        const float ab = fabsf(b);
        const float lo = fmaxf(-h1, -d - ab * h2), hi = fminf(h1, -d + ab * h2);
        s = lo <= hi ? 0.5f * (lo + hi) : clampf_(-d, -h1, h1);
    }
    float t = b * s + e;
    if (t < -h2) {
        t = -h2;
        s = clampf_(b * t - d, -h1, h1);
    } else if (t > h2) {
        t = h2;
        s = clampf_(b * t - d, -h1, h1);
    }
    const float x0 = w0 + s * u1.x - t * u2.x, x1 = w1 + s * u1.y - t * u2.y, x2 = w2 + s * u1.z - t * u2.z;
    return sqrtf(x0 * x0 + x1 * x1 + x2 * x2);
}

// exact decision (the oracle's arithmetic) for a borderline candidate
__device__ __noinline__ bool exact_pair(const DevState &S, int i, int j, const RepParams &P, int sx, int sy,
                                        int sz) {
    const double pi[3] = {S.px[i], S.py[i], S.pz[i]};
    const double ai[3] = {S.ax[i], S.ay[i], S.az[i]};
    const double c2[3] = {S.px[j] + (double)sx * P.L[0], S.py[j] + (double)sy * P.L[1],
                          S.pz[j] + (double)sz * P.L[2]};
    const double aj[3] = {S.ax[j], S.ay[j], S.az[j]};
    const double hi_ = S.hcol[i], hj = S.hcol[j], ri = S.rcol[i], rj = S.rcol[j];
    const double d0 = pi[0] - c2[0], d1 = pi[1] - c2[1], d2 = pi[2] - c2[2];
    const double dd = d0 * d0 + d1 * d1 + d2 * d2;
    const double lim = hi_ + hj + ri + rj + P.colBuf;
    if (dd > lim * lim * (1.0 + 1e-10) + 1e-300) return false;
    const DcpResult R = dcp_segseg(pi, ai, hi_, c2, aj, hj);
    const double sep = R.dist - ri - rj;
    return sep < P.colBuf;
}

// One thread per (neighbour cell, cell-sorted slot) item, slot-fastest: the
// lanes of a warp hold consecutive rods of (mostly) one home cell looking
// at the same neighbour offset, so candidate loads are broadcasts.  Half
// shell: a rod looks at its home cell's later slots and at the neighbour
// offsets that follow the home cell in (z, y, x) order, so every pair and
// periodic image is met once (its mirror, from the partner's side, would
// have the negated offset); a pair met from its larger rod index is
// recorded as (smaller index, larger index, mirrored image), the
// orientation the FP64 decision and the keys use.  Two stages per warp:
// every lane runs the cheap bounding-sphere test on its cell's candidates
// and appends the pairs that pass to a warp queue in shared memory; full
// warps then take 32 queued pairs at a time through the FP32 segment
// distance, every lane busy.  FP32 screen, FP64 decision only within the
// screening margin.
constexpr int kPairQ = 64;  // per-warp queue: fewer than 32 waiting + one round of 32
__global__ void __launch_bounds__(kPairThreads) k_pairs(DevState S) {
    ALENS_PDL_PROLOGUE();
    constexpr int kW = kPairThreads / 32;
    __shared__ int qm[kW][kPairQ];             // queued candidate (cell-sorted slot)
    __shared__ unsigned char qo[kW][kPairQ];   // the lane that queued it
    __shared__ float4 oA[kPairThreads], oB[kPairThreads], oC[kPairThreads];  // per lane: (ci, h), (u, r), (off, colBuf)
    __shared__ int oI[kPairThreads], oImg[kPairThreads], oCnt[kPairThreads];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const long long item = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    // stencil of Wx x Wy x Wz cells (widths 1, 3 or 5)
    const int Wx = S.pairW[0], Wy = S.pairW[1], Wz = S.pairW[2];
    const int W3 = Wx * Wy * Wz;
    const bool valid = item < (long long)((W3 + 1) / 2) * S.nRods && !(flags(S) & kErrNaN);
    unsigned long long buf[kPairBuf];
    int nb = 0;
    int i = 0, img = kImageNone, m0 = 0, len = 0;
    float3 ci = make_float3(0.0f, 0.0f, 0.0f);
    float hi_ = 0.0f, ri = 0.0f, cutHi = 0.0f;
    float3 off = make_float3(0.0f, 0.0f, 0.0f);
    if (valid) {
        const int t = (int)(item % S.nRods);
        const int nbr = (int)(item / S.nRods) + (W3 - 1) / 2;  // the home cell and the offsets after it
        const int ox = nbr % Wx - (Wx >> 1), oy = (nbr / Wx) % Wy - (Wy >> 1), oz = nbr / (Wx * Wy) - (Wz >> 1);
        const bool home = ox == 0 && oy == 0 && oz == 0;
        i = S.sidx[t];
        const RepParams &P = S.par[S.rodRep[i]];
        const int nx = P.ncell[0], ny = P.ncell[1], nz = P.ncell[2];
        const int lc = S.cellOf[i] - P.cellOffset;
        const int cx = lc % nx, cy = (lc / nx) % ny, cz = lc / (nx * ny);
        int xx = cx + ox, y = cy + oy, z = cz + oz;
        int sx = 0, sy = 0, sz = 0;
        // offsets beyond this replica's own stencil are not needed
        const int Rp = P.stencil >> 1;
        bool ok = abs(ox) <= Rp && abs(oy) <= Rp && abs(oz) <= Rp;
        // one periodic wrap (shift of one box length); a cell still outside
        // is beyond the cutoff (the box is at least one cutoff long)
        if (xx < 0 || xx >= nx) {
            if (!P.pbc[0]) ok = false;
            else if (xx < 0) { xx += nx; sx = -1; }
            else { xx -= nx; sx = 1; }
            if (xx < 0 || xx >= nx) ok = false;
        }
        if (y < 0 || y >= ny) {
            if (!P.pbc[1]) ok = false;
            else if (y < 0) { y += ny; sy = -1; }
            else { y -= ny; sy = 1; }
            if (y < 0 || y >= ny) ok = false;
        }
        if (z < 0 || z >= nz) {
            if (!P.pbc[2]) ok = false;
            else if (z < 0) { z += nz; sz = -1; }
            else { z -= nz; sz = 1; }
            if (z < 0 || z >= nz) ok = false;
        }
        if (ok) {
            const float4 Ai = S.sA[t], Bi = S.sB[t];
            ci = make_float3(Ai.x, Ai.y, Ai.z);
            hi_ = Ai.w;
            ri = Bi.w;
            const float colBuf = P.colBuf32;
            cutHi = colBuf + kScreenMargin;
            img = (sx + 1) * 9 + (sy + 1) * 3 + (sz + 1);
            // the neighbour cell's origin relative to ours
            off = make_float3((float)ox * P.cellsz32[0], (float)oy * P.cellsz32[1], (float)oz * P.cellsz32[2]);
            // skip the whole cell when its box lies beyond any partner's reach
            // (exact: every rod centre of that cell is at least this far)
            {
                const float csx = P.cellsz32[0], csy = P.cellsz32[1], csz = P.cellsz32[2];
                const float bx = fmaxf(fmaxf(off.x - ci.x, ci.x - (off.x + csx)), 0.0f);
                const float by = fmaxf(fmaxf(off.y - ci.y, ci.y - (off.y + csy)), 0.0f);
                const float bz = fmaxf(fmaxf(off.z - ci.z, ci.z - (off.z + csz)), 0.0f);
                const float thr = hi_ + ri + P.halfReach32 + cutHi + kScreenMargin;
                if (bx * bx + by * by + bz * bz > thr * thr) ok = false;
            }
            if (ok) {
                const int cell = P.cellOffset + (z * ny + y) * nx + xx;
                m0 = home ? t + 1 : S.cellStart[cell];  // home cell: the slots after this rod's
                len = S.cellStart[cell + 1] - m0;
            }
            oA[threadIdx.x] = make_float4(ci.x, ci.y, ci.z, hi_);
            oB[threadIdx.x] = make_float4(Bi.x, Bi.y, Bi.z, ri);
            oC[threadIdx.x] = make_float4(off.x, off.y, off.z, colBuf);
        }
    }
    oI[threadIdx.x] = i;
    oImg[threadIdx.x] = img;
    oCnt[threadIdx.x] = 0;
    __syncwarp();
    // queued pairs through the FP32 segment distance, lane q taking entry q
    auto drain = [&](int n) {
        bool hit = false, border = false;
        int bi = 0, bj = 0, bimg = 0;
        unsigned long long key = 0ULL;
        if (lane < n) {
            const int m = qm[warp][lane];
            const int ow = warp * 32 + qo[warp][lane];
            const float4 A = oA[ow], B = oB[ow], C = oC[ow];
            int i2 = oI[ow], img2 = oImg[ow];
            int j = S.sidx[m];
            const float4 Aj = S.sA[m], Bj = S.sB[m];
            const float3 cj = make_float3(Aj.x + C.x, Aj.y + C.y, Aj.z + C.z);
            const float sep = dcp_dist32(make_float3(A.x, A.y, A.z), make_float3(B.x, B.y, B.z), A.w, cj,
                                         make_float3(Bj.x, Bj.y, Bj.z), Aj.w) -
                              B.w - Bj.w;
            const float cLo = C.w - kScreenMargin, cHi = C.w + kScreenMargin;
            if (sep < cHi) {
                // (smaller index, larger index, image of the larger's copy)
                if (j < i2 || (j == i2 && img2 < kImageNone)) {
                    const int tmp = i2;
                    i2 = j;
                    j = tmp;
                    img2 = 26 - img2;
                }
                if (sep >= cLo) {
                    // within the screen's margin: decided in FP64 by
                    // k_pairs_exact
                    border = true;
                    bi = i2;
                    bj = j;
                    bimg = img2;
                } else {
                    hit = true;
                    key = pair_key(i2, j, img2);
                    if (i2 == oI[ow])
                        atomicAdd(&oCnt[ow], 1);
                    else
                        atomicAdd(&S.pairCount[i2], 1);
                }
            }
        }
        const unsigned int bb = __ballot_sync(0xffffffffu, border);
        if (bb) {
            int base = 0;
            if (lane == 0) base = atomicAdd(&S.ctl->borderCount, __popc(bb));
            base = __shfl_sync(0xffffffffu, base, 0);
            if (border) {
                const int slot = base + __popc(bb & ((1u << lane) - 1u));
                if (slot < S.cap)
                    S.border[slot] = make_int4(bi, bj, bimg, 0);
                else
                    atomicOr(&S.ctl->errFlags, kErrOverflow);
            }
        }
        if (hit) {
            if (nb == kPairBuf) {
                flush_keys(S, buf, nb);
                nb = 0;
            }
            buf[nb++] = key;
        }
    };
    const int maxLen = __reduce_max_sync(0xffffffffu, len);
    int qn = 0;  // queued pairs (the same in every lane)
    for (int u = 0; u < maxLen; u++) {
        bool pass = false;
        const int m = m0 + u;
        if (u < len) {
            const float4 Aj = S.sA[m];
            const float3 cj = make_float3(Aj.x + off.x, Aj.y + off.y, Aj.z + off.z);
            const float d0 = ci.x - cj.x, d1 = ci.y - cj.y, d2 = ci.z - cj.z;
            const float4 Bj = S.sB[m];
            const float lim = hi_ + Aj.w + ri + Bj.w + cutHi;
            pass = !(d0 * d0 + d1 * d1 + d2 * d2 > lim * lim);
        }
        const unsigned int bal = __ballot_sync(0xffffffffu, pass);
        if (pass) {
            const int pos = qn + __popc(bal & ((1u << lane) - 1u));
            qm[warp][pos] = m;
            qo[warp][pos] = (unsigned char)lane;
        }
        qn += __popc(bal);
        if (qn >= 32) {
            __syncwarp();
            drain(32);
            // the rest (fewer than 32) to the front
            int mm = 0;
            unsigned char oo = 0;
            if (lane < qn - 32) {
                mm = qm[warp][32 + lane];
                oo = qo[warp][32 + lane];
            }
            __syncwarp();
            if (lane < qn - 32) {
                qm[warp][lane] = mm;
                qo[warp][lane] = oo;
            }
            qn -= 32;
            __syncwarp();
        }
    }
    __syncwarp();
    if (qn > 0) drain(qn);
    __syncwarp();
    if (oCnt[threadIdx.x]) atomicAdd(&S.pairCount[i], oCnt[threadIdx.x]);
    // warp-aggregated append of the remaining keys
    int incl = nb;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
    }
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    int base = 0;
    if (lane == 31 && total > 0) base = atomicAdd(&S.ctl->rawCount, total);
    base = __shfl_sync(0xffffffffu, base, 31);
    const int start = base + incl - nb;
    for (int e = 0; e < nb; e++) {
        const int pos = start + e;
        if (pos < S.cap)
            S.rawKeys[pos] = buf[e];
        else
            atomicOr(&S.ctl->errFlags, kErrOverflow);
    }
}

// The FP64 decision (the oracle's arithmetic) for the candidates the FP32
// screen left within its margin; accepted pairs are appended like k_pairs'.
__global__ void k_pairs_exact(DevState S) {
    ALENS_PDL_PROLOGUE();
    if (flags(S) & (kErrNaN | kErrOverflow)) return;
    const int n = min(S.ctl->borderCount, S.cap);
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < n; b += gridDim.x * blockDim.x) {
        const int4 e = S.border[b];
        const int i = e.x, j = e.y, img = e.z;
        const RepParams &P = S.par[S.rodRep[i]];
        if (!exact_pair(S, i, j, P, img / 9 - 1, (img / 3) % 3 - 1, img % 3 - 1)) continue;
        const int pos = atomicAdd(&S.ctl->rawCount, 1);
        if (pos < S.cap)
            S.rawKeys[pos] = pair_key(i, j, img);
        else
            atomicOr(&S.ctl->errFlags, kErrOverflow);
        atomicAdd(&S.pairCount[i], 1);
    }
}

// Rod-boundary contacts: every contact point of a rod closer to a boundary
// of its replica than sylinderColBuf (surface distance, FP64, the oracle's
// arithmetic) gives a key (i, b, 27 + point) in the rod's pair segment.
__global__ void k_boundary_pairs(DevState S) {
    ALENS_PDL_PROLOGUE();
    if (flags(S) & kErrNaN) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < S.nRods; i += gridDim.x * blockDim.x) {
        const int rep = S.rodRep[i];
        const int b0 = S.bndStart[rep], b1 = S.bndStart[rep + 1];
        if (b0 == b1) continue;
        const double colBuf = S.par[rep].colBuf;
        const double x[3] = {S.px[i], S.py[i], S.pz[i]};
        const double a[3] = {S.ax[i], S.ay[i], S.az[i]};
        const double h = S.hcol[i], rc = S.rcol[i];
        int cnt = 0;
        for (int b = b0; b < b1; b++) {
            const BoundaryDev &B = S.bnd[b];
            const int np = boundary_npoints(B, h);
            for (int e = 0; e < np; e++) {
                double Q[3], sd, n[3];
                boundary_contact(B, x, a, h, e, Q, sd, n);
                if (sd - rc < colBuf) {
                    const int pos = atomicAdd(&S.ctl->rawCount, 1);
                    if (pos < S.cap)
                        S.rawKeys[pos] = pair_key(i, b - b0, kImageBoundary + e);
                    else
                        atomicOr(&S.ctl->errFlags, kErrOverflow);
                    cnt++;
                }
            }
        }
        if (cnt) atomicAdd(&S.pairCount[i], cnt);
    }
}

// Bitonic sorting network over registers (ascending; N a power of two,
// every index a compile-time constant).
template <class T, int N>
__device__ __forceinline__ void sort_regs(T (&v)[N]) {
#pragma unroll
    for (int k = 2; k <= N; k <<= 1) {
#pragma unroll
        for (int j = k >> 1; j > 0; j >>= 1) {
#pragma unroll
            for (int i = 0; i < N; i++) {
                const int l = i ^ j;
                if (l > i) {
                    const T a = v[i], b = v[l];
                    const T lo = a < b ? a : b, hi = a < b ? b : a;
                    v[i] = (i & k) == 0 ? lo : hi;
                    v[l] = (i & k) == 0 ? hi : lo;
                }
            }
        }
    }
}
constexpr int kSortRegs = 16;  // rod-row entries sorted in registers
constexpr int kKeyRegs = 8;    // pair keys of one rod sorted in registers

// Place raw keys into their rod's segment, then sort each segment: the
// canonical order is (i, j, image) ascending.
__global__ void k_pair_bucket(DevState S) {
    ALENS_PDL_PROLOGUE();
    if (flags(S) & (kErrNaN | kErrOverflow)) return;
    const int n = S.ctl->rawCount;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        const unsigned long long key = S.rawKeys[p];
        const int i = (int)(key >> 32);
        const int slot = S.pairOff[i] + atomicAdd(&S.pairCursor[i], 1);
        S.keys[slot] = key;
    }
}

__global__ void k_pair_segsort(DevState S) {
    ALENS_PDL_PROLOGUE();
    if (flags(S) & (kErrNaN | kErrOverflow)) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < S.nRods; i += gridDim.x * blockDim.x) {
        const int b = S.pairOff[i], e = S.pairOff[i + 1];
        if (e - b <= kKeyRegs) {
            // loaded once, sorted in registers, stored once
            unsigned long long v[kKeyRegs];
#pragma unroll
            for (int q = 0; q < kKeyRegs; q++) v[q] = b + q < e ? S.keys[b + q] : ~0ULL;
            sort_regs<unsigned long long, kKeyRegs>(v);
#pragma unroll
            for (int q = 0; q < kKeyRegs; q++)
                if (b + q < e) S.keys[b + q] = v[q];
            continue;
        }
        for (int x = b + 1; x < e; x++) {
            const unsigned long long v = S.keys[x];
            int y = x - 1;
            while (y >= b && S.keys[y] > v) {
                S.keys[y + 1] = S.keys[y];
                y--;
            }
            S.keys[y + 1] = v;
        }
    }
}

// ---------------------------------------------------------------- ranges
// Per-replica constraint and tile ranges from the pair offsets, one thread
// per replica (a block scan gives the tile starts), then the step's totals
// and the solver's counters.
__global__ void k_ranges(DevState S) {
    ALENS_PDL_PROLOGUE();
    __shared__ int sm[33];
    __shared__ int s_tile, s_maxIte, s_ok;
    if (threadIdx.x == 0) {
        s_tile = 0;
        s_maxIte = 0;
    }
    __syncthreads();
    for (int base = 0; base < S.R; base += blockDim.x) {
        const int r = base + (int)threadIdx.x;
        int nTiles = 0;
        if (r < S.R) {
            const RepParams &P = S.par[r];
            RepDyn &d = S.dyn[r];
            d.collStart = S.pairOff[P.rodOffset];
            d.collEnd = S.pairOff[P.rodOffset + P.nRods];
            const int nBil = S.bilPrefix[r + 1] - S.bilPrefix[r];
            d.conStart = d.collStart + S.bilPrefix[r];
            d.nCon = (d.collEnd - d.collStart) + nBil;
            d.nTiles = (d.nCon + kTile - 1) / kTile;
            d.iter = 0;
            d.refineIter = 0;
            d.refined = 0;
            d.res64bits = 0ULL;
            d.active = d.nCon > 0 ? 1 : 0;
            d.converged = d.nCon > 0 ? 0 : 1;
            d.status = 0;
            d.counter = 0;
            d.alpha = 0.0;
            d.res = 0.0;
            nTiles = d.nTiles;
            atomicMax(&s_maxIte, P.maxIte);
        }
        int tot;
        const int ex = block_exclusive_scan(nTiles, sm, &tot);
        if (r < S.R) S.dyn[r].tileStart = s_tile + ex;
        __syncthreads();
        if (threadIdx.x == 0) s_tile += tot;
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        DevCtl *c = S.ctl;
        const int tile = s_tile;
        const int totalColl = S.pairOff[S.nRods];
        c->totalColl = totalColl;
        c->totalBil = S.bilPrefix[S.R];
        c->totalCon = totalColl + S.bilPrefix[S.R];
        c->nTiles = tile;
        c->activeCnt[0] = c->activeCnt[1] = c->activeCnt[2] = 0;
        c->finalParity = 1;
        c->allRefined = 0;
        c->setupDone = 0u;
        c->maxIte = s_maxIte;
        c->bar.count = 0;
        c->bar.gen = 0;
        c->bar.pass[0][0] = c->bar.pass[1][0] = c->bar.pass[2][0] = 0u;
        int ok = 1;
        if (c->totalCon > S.cap || tile > S.tileCap) {
            atomicOr(&c->errFlags, kErrOverflow);
            ok = 0;
        }
        s_ok = ok;
    }
    __syncthreads();
    if (!s_ok || (flags(S) & (kErrNaN | kErrOverflow))) return;
    // tile -> replica map, one warp per replica
    const int lane = threadIdx.x & 31;
    for (int r = threadIdx.x >> 5; r < S.R; r += blockDim.x >> 5) {
        const RepDyn &d = S.dyn[r];
        for (int t = lane; t < d.nTiles; t += 32) S.tileRep[d.tileStart + t] = r;
    }
}

// ----------------------------------------------------------------- build
__device__ __forceinline__ double dot6s(const double *J, const double *U, size_t stride, int r) {
    return J[0] * U[r] + J[1] * U[stride + r] + J[2] * U[2 * stride + r] + J[3] * U[3 * stride + r] +
           J[4] * U[4 * stride + r] + J[5] * U[5 * stride + r];
}

__device__ void finish_constraint(const DevState &S, int k, const RepParams &P, int I, int J,
                                  const double *jac, double phi0, double gamma0, double lb,
                                  double cinv) {
    const size_t st = (size_t)S.nRods;
    const double dI = dot6s(jac, S.unc, st, I);
    const double dJ = J >= 0 ? dot6s(jac + 6, S.unc, st, J) : 0.0;
    const double q = phi0 + P.dt * (dI + dJ);
    const double g0 = gamma0 < lb ? lb : gamma0;
    S.q[k] = q;
    S.st[1][k] = make_double2(g0, 0.0);  // the solver starts from the parity-1 buffer
    S.qc[k] = make_double2(q, cinv);
    S.gamma[k] = g0;
    S.lb[k] = lb;
    S.lbKind[k] = lb == 0.0 ? 0 : (lb == -INFINITY ? 1 : 2);
    S.cinv[k] = cinv;
    S.phi0[k] = phi0;
    atomicAdd(&S.rowCount[I], 1);
    if (J >= 0) atomicAdd(&S.rowCount[J], 1);
    if (S.precision == ALENS_PREC_MIXED) {
        S.qc32[k] = make_float2((float)q, (float)cinv);
        S.st32[1][k] = make_float2((float)g0, 0.0f);
    }
}

__global__ void k_build(DevState S) {
    ALENS_PDL_PROLOGUE();
    if (flags(S) & (kErrNaN | kErrOverflow)) return;
    const int totalColl = S.ctl->totalColl, totalBil = S.ctl->totalBil;
    // the previous step's multiplier of each key as the start: the
    // previous-gamma mode, and the learned mode without a network; with
    // the network its features look it up on the warm-start branch, and
    // only the boundary contacts it does not score are looked up here
    const bool warmPrev = S.warm == ALENS_WARM_PREV || (S.warm == ALENS_WARM_MLP && !S.warmNet);
    const int prevN = *S.prevCount;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < totalColl; p += gridDim.x * blockDim.x) {
        const unsigned long long key = S.keys[p];
        const int i = (int)(key >> 32), j = (int)((key >> 5) & 0x7ffffff), img = (int)(key & 31);
        const int rep = S.rodRep[i];
        const RepParams &P = S.par[rep];
        const int k = p + S.bilPrefix[rep];
        double g0 = 0.0;
        if ((warmPrev || (S.warmNet && img >= kImageBoundary)) && prevN > 0) {
            int lo = 0, hi = prevN;
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (S.prevKeys[mid] < key)
                    lo = mid + 1;
                else
                    hi = mid;
            }
            if (lo < prevN && S.prevKeys[lo] == key) g0 = S.prevGamma[lo];
        }
        if (img >= kImageBoundary) {
            // rod i against boundary j of its replica, contact point img - 27
            const BoundaryDev &B = S.bnd[S.bndStart[rep] + j];
            const double x[3] = {S.px[i], S.py[i], S.pz[i]};
            const double a[3] = {S.ax[i], S.ay[i], S.az[i]};
            double Q[3], sd, n[3];
            boundary_contact(B, x, a, S.hcol[i], img - kImageBoundary, Q, sd, n);
            const double sep = sd - S.rcol[i];
            const double r[3] = {Q[0] - x[0], Q[1] - x[1], Q[2] - x[2]};
            double J[12];
            J[0] = n[0];
            J[1] = n[1];
            J[2] = n[2];
            cross3(r, n, J + 3);
#pragma unroll
            for (int c = 6; c < 12; c++) J[c] = 0.0;
#pragma unroll
            for (int c = 0; c < 12; c++) S.jac[12 * (size_t)k + c] = J[c];
            S.conI[k] = i;
            S.conJ[k] = -1;
            S.conImg[k] = img;
            S.conST[k] = make_float2(0.0f, 0.0f);
#pragma unroll
            for (int d = 0; d < 3; d++) {
                S.lab[6 * (size_t)k + d] = Q[d];
                S.lab[6 * (size_t)k + 3 + d] = Q[d] - sd * n[d];
            }
            finish_constraint(S, k, P, i, -1, J, sep, g0, 0.0, 0.0);
            continue;
        }
        const int sv[3] = {img / 9 - 1, (img / 3) % 3 - 1, img % 3 - 1};
        const double c1[3] = {S.px[i], S.py[i], S.pz[i]};
        const double c2[3] = {S.px[j] + (double)sv[0] * P.L[0], S.py[j] + (double)sv[1] * P.L[1],
                              S.pz[j] + (double)sv[2] * P.L[2]};
        const double ai[3] = {S.ax[i], S.ay[i], S.az[i]};
        const double aj[3] = {S.ax[j], S.ay[j], S.az[j]};
        const DcpResult R = dcp_segseg(c1, ai, S.hcol[i], c2, aj, S.hcol[j]);
        double n[3];
        contact_normal(R, ai, aj, n);
        const double sep = R.dist - S.rcol[i] - S.rcol[j];
        double J[12];
        const double rI[3] = {R.s * ai[0], R.s * ai[1], R.s * ai[2]};
        const double rJ[3] = {R.t * aj[0], R.t * aj[1], R.t * aj[2]};
        const double nJ[3] = {-n[0], -n[1], -n[2]};
        J[0] = n[0];
        J[1] = n[1];
        J[2] = n[2];
        cross3(rI, n, J + 3);
        J[6] = nJ[0];
        J[7] = nJ[1];
        J[8] = nJ[2];
        cross3(rJ, nJ, J + 9);
#pragma unroll
        for (int c = 0; c < 12; c++) S.jac[12 * (size_t)k + c] = J[c];
        S.conI[k] = i;
        S.conJ[k] = j;
        S.conImg[k] = img;
        S.conST[k] = make_float2(S.hcol[i] > 0.0 ? (float)(R.s / S.hcol[i]) : 0.0f,
                                 S.hcol[j] > 0.0 ? (float)(R.t / S.hcol[j]) : 0.0f);
#pragma unroll
        for (int d = 0; d < 3; d++) {
            S.lab[6 * (size_t)k + d] = R.P[d];
            S.lab[6 * (size_t)k + 3 + d] = R.Q[d];
        }
        finish_constraint(S, k, P, i, j, J, sep, g0, 0.0, 0.0);
    }
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < totalBil; b += gridDim.x * blockDim.x) {
        const AlensBlock &B = S.blocks[b];
        const int rep = S.blockRep[b];
        const RepParams &P = S.par[rep];
        const int k = S.dyn[rep].collEnd + b;
        const int I = P.rodOffset + B.globalIndexI;
        const int Jr = B.oneSide ? -1 : P.rodOffset + B.globalIndexJ;
        double J[12];
        J[0] = B.normI[0];
        J[1] = B.normI[1];
        J[2] = B.normI[2];
        cross3(B.posI, B.normI, J + 3);
        if (!B.oneSide) {
            J[6] = B.normJ[0];
            J[7] = B.normJ[1];
            J[8] = B.normJ[2];
            cross3(B.posJ, B.normJ, J + 9);
        } else {
#pragma unroll
            for (int c = 6; c < 12; c++) J[c] = 0.0;
        }
#pragma unroll
        for (int c = 0; c < 12; c++) S.jac[12 * (size_t)k + c] = J[c];
        S.conI[k] = I;
        S.conJ[k] = Jr;
        S.conImg[k] = -1;
#pragma unroll
        for (int d = 0; d < 3; d++) {
            S.lab[6 * (size_t)k + d] = B.labI[d];
            S.lab[6 * (size_t)k + 3 + d] = B.labJ[d];
        }
        const double lb = B.bilateral ? -INFINITY : B.gammaLB;
        const double cinv = (B.bilateral && B.kappa > 0.0) ? 1.0 / B.kappa : 0.0;
        finish_constraint(S, k, P, I, Jr, J, B.delta0, B.gamma, lb, cinv);
    }
}

// ------------------------------------------------------------- rod rows
__global__ void k_rows_fill(DevState S) {
    ALENS_PDL_PROLOGUE();
    if (flags(S) & (kErrNaN | kErrOverflow)) return;
    const int nc = S.ctl->totalCon;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nc; k += gridDim.x * blockDim.x) {
        const int I = S.conI[k], J = S.conJ[k];
        S.rowEnt[S.rowPtr[I] + atomicAdd(&S.rowCursor[I], 1)] = 2 * k;
        if (J >= 0) S.rowEnt[S.rowPtr[J] + atomicAdd(&S.rowCursor[J], 1)] = 2 * k + 1;
    }
}


// Each rod's row ascending.  A row of at most kSortRegs entries is loaded
// once, sorted in registers and stored once; a longer one is sorted in
// place.  With `coupling` (the learned warm start's features) the rod's
// sum over its compressed collisions l (q_l < 0) of (-q_l) W_l at the rod's
// side is formed from the sorted row, in entry order (FP32).
__global__ void k_rows_sort(DevState S, int coupling) {
    ALENS_PDL_PROLOGUE();
    if (flags(S) & (kErrNaN | kErrOverflow)) return;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < S.nRods; r += gridDim.x * blockDim.x) {
        const int b = S.rowPtr[r], e = S.rowPtr[r + 1], len = e - b;
        float cv[6] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
        auto add = [&](int ent, float ql) {
            const double *W = S.W + 12 * (size_t)(ent >> 1) + 6 * (ent & 1);
#pragma unroll
            for (int c = 0; c < 6; c++) cv[c] = fmaf(-ql, (float)W[c], cv[c]);
        };
        if (len <= kSortRegs) {
            int v[kSortRegs];
#pragma unroll
            for (int q = 0; q < kSortRegs; q++) v[q] = q < len ? S.rowEnt[b + q] : 0x7fffffff;
            sort_regs<int, kSortRegs>(v);
#pragma unroll
            for (int q = 0; q < kSortRegs; q++)
                if (q < len) S.rowEnt[b + q] = v[q];
            if (coupling) {
                float ql[kSortRegs];
#pragma unroll
                for (int q = 0; q < kSortRegs; q++) {
                    const int l = q < len ? v[q] >> 1 : 0;  // padding: a valid index, weight 0
                    ql[q] = (q < len && S.lbKind[l] == 0) ? (float)S.q[l] : 0.0f;
                }
#pragma unroll
                for (int q = 0; q < kSortRegs; q++)
                    if (ql[q] < 0.0f) add(v[q], ql[q]);
            }
        } else {
            for (int x = b + 1; x < e; x++) {
                const int v = S.rowEnt[x];
                int y = x - 1;
                while (y >= b && S.rowEnt[y] > v) {
                    S.rowEnt[y + 1] = S.rowEnt[y];
                    y--;
                }
                S.rowEnt[y + 1] = v;
            }
            if (coupling) {
                for (int x = b; x < e; x++) {
                    const int ent = S.rowEnt[x];
                    const int l = ent >> 1;
                    if (S.lbKind[l] != 0) continue;
                    const float ql = (float)S.q[l];
                    if (ql < 0.0f) add(ent, ql);
                }
            }
        }
        if (coupling) {
#pragma unroll
            for (int c = 0; c < 6; c++) S.rodV[(size_t)c * S.nRods + r] = cv[c];
        }
    }
}

// ------------------------------------------------- host <-> device rods
// stage layout: pos[3n] then quat[4n] (x,y,z,w), interleaved per rod.
__global__ void k_unpack_rods(DevState S, int off, int n) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        const double *p = S.stage + 3 * (size_t)r;
        const double *q = S.stage + 3 * (size_t)n + 4 * (size_t)r;
        S.px[off + r] = p[0];
        S.py[off + r] = p[1];
        S.pz[off + r] = p[2];
        S.qx[off + r] = q[0];
        S.qy[off + r] = q[1];
        S.qz[off + r] = q[2];
        S.qw[off + r] = q[3];
    }
}

__global__ void k_pack_rods(DevState S, int off, int n, int what) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        if (what == 0) {
            double *p = S.stage + 3 * (size_t)r;
            double *q = S.stage + 3 * (size_t)n + 4 * (size_t)r;
            p[0] = S.px[off + r];
            p[1] = S.py[off + r];
            p[2] = S.pz[off + r];
            q[0] = S.qx[off + r];
            q[1] = S.qy[off + r];
            q[2] = S.qz[off + r];
            q[3] = S.qw[off + r];
        } else {
            double *v = S.stage + 3 * (size_t)r;
            double *w = S.stage + 3 * (size_t)n + 3 * (size_t)r;
            const size_t st = (size_t)S.nRods;
            for (int c = 0; c < 3; c++) {
                v[c] = S.vel[c * st + off + r];
                w[c] = S.vel[(c + 3) * st + off + r];
            }
        }
    }
}

int grid_for(int n, int block, int maxBlocks = 4096) {
    int g = (n + block - 1) / block;
    if (g < 1) g = 1;
    if (g > maxBlocks) g = maxBlocks;
    return g;
}

}  // namespace

void launch_step_clear(const DevState &S, cudaStream_t st) {
    k_step_clear<<<grid_for(S.nRods > S.nCells ? S.nRods : S.nCells, 256), 256, 0, st>>>(S);
}

void launch_prep(const DevState &S, cudaStream_t st) {
    launch_pdl(k_prep, dim3(grid_for(S.nRods, 32)), dim3(32), 0, st, S);
}

void launch_noise(const DevState &S, cudaStream_t st) {
    k_noise<<<grid_for(S.nRods, 32), 32, 0, st>>>(S);
}

void launch_mobility(const DevState &S, cudaStream_t st) {
    k_mobility<<<grid_for(S.nRods, 64), 64, 0, st>>>(S);
}

int launch_scan(const int *in, int *out, int n, int *tmp, cudaStream_t st) {
    if (n <= kScanSingleMax) {
        const int vec = ((reinterpret_cast<uintptr_t>(in) | reinterpret_cast<uintptr_t>(out)) & 15u) == 0 ? 1 : 0;
        launch_pdl(k_scan_single, dim3(1), dim3(kScanSingleThreads), 0, st, in, out, n, vec, (const int *)nullptr);
        return 1;
    }
    const int nb = (n + kScanSpan - 1) / kScanSpan;
    if (nb > 0) launch_pdl(k_scan_block, dim3(nb), dim3(kScanBlock), 0, st, in, out, n, tmp);
    launch_pdl(k_scan_top, dim3(1), dim3(1024), 0, st, tmp, nb, out, n);
    if (nb > 0) launch_pdl(k_scan_add, dim3(nb), dim3(kScanBlock), 0, st, out, n, tmp);
    return nb > 0 ? 3 : 1;
}

// Exclusive scan of the first *nDev of at most nMax ints (out[*nDev] = the
// total): one block while nMax is moderate (a capacity of up to 4 x
// kScanSingleMax slots; the count the device holds is typically a quarter
// to a third of it), else the three-pass scan of all nMax (the entries past
// *nDev are zeros).
int launch_scan_dev(const int *in, int *out, int nMax, const int *nDev, int *tmp, cudaStream_t st) {
    if (nMax <= 4 * kScanSingleMax) {
        const int vec = ((reinterpret_cast<uintptr_t>(in) | reinterpret_cast<uintptr_t>(out)) & 15u) == 0 ? 1 : 0;
        launch_pdl(k_scan_single, dim3(1), dim3(kScanSingleThreads), 0, st, in, out, nMax, vec, nDev);
        return 1;
    }
    return launch_scan(in, out, nMax, tmp, st);
}

void launch_link_blocks(const DevState &S, cudaStream_t st) {
    if (S.nLinks > 0) launch_pdl(k_link_blocks, dim3(grid_for(S.nLinks, 128)), dim3(128), 0, st, S);
}

void launch_scatter(const DevState &S, cudaStream_t st) {
    launch_pdl(k_scatter, dim3(grid_for(S.nRods, 256)), dim3(256), 0, st, S);
}

int sm_count_detect() {
    static int n = 0;
    if (n == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
    }
    return n;
}

void launch_pairs(const DevState &S, cudaStream_t st) {
    // half shell: the home cell and the offsets after it
    const long long items = (long long)((S.pairW[0] * S.pairW[1] * S.pairW[2] + 1) / 2) * S.nRods;
    const long long g = (items + kPairThreads - 1) / kPairThreads;
    launch_pdl(k_pairs, dim3((unsigned)(g > 0 ? g : 1)), dim3(kPairThreads), 0, st, S);
    launch_pdl(k_pairs_exact, dim3(2 * sm_count_detect()), dim3(64), 0, st, S);
}

void launch_boundary_pairs(const DevState &S, cudaStream_t st) {
    launch_pdl(k_boundary_pairs, dim3(grid_for(S.nRods, 256)), dim3(256), 0, st, S);
}

int launch_pair_sort(const DevState &S, cudaStream_t st) {
    launch_pdl(k_pair_bucket, dim3(grid_for(S.cap, 256)), dim3(256), 0, st, S);
    launch_pdl(k_pair_segsort, dim3(grid_for(S.nRods, 32)), dim3(32), 0, st, S);
    return 2;
}

void launch_ranges(const DevState &S, cudaStream_t st) { k_ranges<<<1, 1024, 0, st>>>(S); }

void launch_build(const DevState &S, cudaStream_t st) {
    k_build<<<grid_for(S.cap, 32, 8192), 32, 0, st>>>(S);
}

int launch_rows(const DevState &S, cudaStream_t st, cudaEvent_t weights) {
    const int n = launch_scan(S.rowCount, S.rowPtr, S.nRods, S.scanTmp, st);
    launch_pdl(k_rows_fill, dim3(grid_for(S.cap, 256)), dim3(256), 0, st, S);
    // the per-rod coupling sums read the weights (launched on another stream)
    if (weights) cudaStreamWaitEvent(st, weights, 0);
    launch_pdl(k_rows_sort, dim3(grid_for(S.nRods, 32)), dim3(32), 0, st, S, weights ? 1 : 0);
    return n + 2;
}

void launch_unpack_rods(const DevState &S, int rodOffset, int n, cudaStream_t st) {
    k_unpack_rods<<<grid_for(n, 256), 256, 0, st>>>(S, rodOffset, n);
}

void launch_pack_rods(const DevState &S, int rodOffset, int n, int what, cudaStream_t st) {
    k_pack_rods<<<grid_for(n, 256), 256, 0, st>>>(S, rodOffset, n, what);
}

}  // namespace alens
