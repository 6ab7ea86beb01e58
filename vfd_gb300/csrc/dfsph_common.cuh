// Shared device definitions of the GB300 DFSPH step.
//
// Layout in HBM (all per-particle arrays are structure-of-arrays, indexed by
// the particle's slot in cell-sorted order; scenes occupy fixed contiguous slot
// ranges, so a slot's scene never changes):
//   carried state, two sets A/B (ping-pong across the sort):
//     X  float4 (x, y, z, -)      V  float4 (v, -)
//     DV float4 viscosity warm start (DFSPHParticle::VelocityDifference)
//     DK float  temporal curvature (DFSPHParticle::DeltaFinalCurvature)
//     PID u32   original particle index within its scene
//   XN   float4 positions written by the integrator, read by the next search
//   per-step fields: A, AP, GB float4; RHO, ALPHA, RHOADV, KAPPA, KAPPAV, RES float
//   XB   float4 [body slot][slot] boundary sample (xb, Vb) per rigid body
//   NBR  u32 [slot][72] neighbour slots, one row per particle in the reference's
//        z, y, x cell order (at most 70 used), read by groups of G lanes
//   NCNT u32 [slot] neighbour count | flag bits
//   NG   (u32, f32) [slot][72] the row again with gradW / r of each pair beside each
//        index, written once per step by the density pass and streamed (one 8-byte load
//        per pair) by the later row loops instead of a table lookup
//   NBRC u16 [slot][72] the same row as stencil positions (only while a pass runs on
//        cell tiles, Dev::compactRows): entry (w << 6) | b is the b-th
//        candidate, in cell order, of x-run w = 3 (dz + 1) + (dy + 1) of the 27-cell
//        stencil (cells x-1, x, x+1 at y+dy, z+dz); read by the cell-tile kernels of the
//        solver loops, which stage each run contiguously in shared memory
//   X.w  mirrors kappa_v during the divergence solve and kappa during the pressure
//        solve, so the pressure-acceleration gather brings it with the position
// The reference keeps one 120-byte AoS DFSPHParticle per particle
// (Structures/DFSPHParticle.h:8-33) in original order.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace vfd {

constexpr uint32_t kMaxNeighbors = 70u;      // ParticleSearchKernels.cuh:7
constexpr uint32_t kTableRes = 10000u;       // Kernel/DFSPHKernels.h:143
constexpr uint32_t kHaltonCount = 49152u;    // HaltonVec323.cuh:4
constexpr uint32_t kBlock = 128u;            // threads per particle kernel (default)
constexpr uint32_t kMaxBlock = 256u;         // largest block a neighbour-loop kernel is launched with
constexpr uint32_t kRow = 72u;               // neighbour row length (70 rounded up to 8)
constexpr uint32_t kGroup = 8u;              // lanes per particle in neighbour loops
constexpr uint32_t kBuckets = 32u;           // reduction buckets per scene and quantity
constexpr uint32_t kAccSlots = 4u;           // FP64 accumulators per scene
constexpr float kEps = 1.0e-5f;              // Core/Math/Math.h:6

// NCNT flag bits (above the 7-bit count).
constexpr uint32_t kCountMask = 0xFFu;
constexpr uint32_t kHasBoundary = 1u << 8;   // some body gave this particle Vb > 0
constexpr uint32_t kHasBoundaryVisc = 1u << 9;
constexpr uint32_t kRowPath = 1u << 10;      // an x-run of the cell's candidates exceeds 64: no NBRC row
constexpr uint32_t kRunMax = 64u;            // candidates of one x-run an NBRC entry can address

// Neighbour-loop kernels whose lanes per particle (4, 8 or 16) the autotuner picks.
enum TunedKernel {
    kTDensity = 0, kTPAccel, kTJacobi, kTDivFinish, kTStClassify, kTStSmooth, kTViscPrecond,
    kTViscSetup, kTSpmv, kTPresInit, kTPresFinish, kTunedCount
};
// Form of the three solver-loop passes (Dev::tiles / vfd_set_tiles): 0 = neighbour rows with
// the per-pair gradient stream, kRowsNoStream = neighbour rows with gradW / r formed from
// the table per pair, >= kTileMinLog2 = cell tiles of 2^value Morton cells.
constexpr uint8_t kRowsNoStream = 1u;
constexpr uint8_t kTileMinLog2 = 3u;

// Per-scene solver loop state (one Jacobi or CG loop).
struct LoopState {
    uint32_t it;
    uint32_t active;   // 1 while this scene still iterates
    float err;
    uint32_t pad;
};

// Per scene: constants (written by the host) and solver state (device).
struct SceneDev {
    // ---- constants ----
    uint32_t begin, count;          // slot range
    uint32_t bodyBegin, bodyCount;  // rigid bodies (global body table)
    float r, diam, h, h2;
    float volume, rho0, mass, massInv;
    float dynVisc, dynBVisc, tangDist, st;
    float slope, constant, smoothing, nbrRadius;
    float mcFactor;
    int32_t temporal;
    float g[3];
    uint32_t minIterP, maxIterP, minIterD, maxIterD, minIterV, maxIterV;
    float maxErrP, maxErrD, maxErrV;
    int32_t enableDiv, enableVisc, enableST;
    uint32_t stPasses;
    int32_t csdFix, csd;
    float minDt, maxDt;
    // ---- dynamic ----
    float dt, dt2, dtInv, dt2Inv;
    uint32_t stSamples;        // sample count for the next surface-tension pass
    uint32_t stSamplesUsed;    // sample count this step's surface tension used
    float maxV2;               // CFL maximum of |v + a dt|^2 (max(0.1, ...))
    uint32_t maxV2Bits;        // the same as float bits, for atomicMax
    float frameTime, frameLength;
    uint32_t frameIndex, frameCount, iteration, frameDue;
    int32_t minCell[3], maxCell[3];
    float gridMin[3], gridDelta[3];
    uint32_t dim[3], meta[3];
    float org[3];              // cell-relative positions: corner of anchor cell (0, 0, 0)
    uint32_t cellBase, cellCount;
    uint32_t flags;            // VFD_FLAG_* of the current step
    uint32_t maxNbr;
    LoopState div, pres;
    // viscosity CG
    uint32_t cgIt, cgActive, cgDone, cgZeroG, cgUpdateP;
    double cgRhs, cgThr, cgAbsNew, cgRR;
    float cgAlpha, cgBeta;
};

// Rigid body volume map (SDFDeviceData, Utility/SDF/SDFDeviceData.cuh:549-566).
struct BodyDev {
    float dmin[3], dmax[3], cs[3], csi[3];
    uint32_t res[3];
    uint32_t nodeCount, cellCount, cellMapCount;
    const float* nodes;        // field 0 then field 1
    const uint32_t* cells;     // field 0 cells (32 per cell)
    const uint32_t* cellMap;   // field 0 cell map
};

// Device pointers and sizes of one simulation; one instance per sort parity
// (cur = state sorted by the previous step, srt = state sorted by this step).
struct Dev {
    uint32_t n, stride, nscenes, maxBodies, cellCap, scanBlocks;
    // carried state
    float4 *Xc, *Vc, *DVc;
    float* DKc;
    uint32_t* PIDc;
    float4 *X, *V, *DV;
    float* DK;
    uint32_t* PID;
    float4* XN;
    // per-step fields
    float4 *A, *AP, *GB;
    float *RHO, *ALPHA, *RHOADV, *KAPPA, *KAPPAV, *RES;
    float4* XB;
    uint32_t *NBR, *NCNT;
    uint2* NG;                 // [slot][72] (neighbour slot, gradW factor bits) of each pair (row layout)
    uint16_t* NBRC;            // [slot][kRow] stencil-position rows (null: not kept)
    // search scratch
    uint32_t *KEY, *KEYS, *TMP, *CELL_START, *CELL_COUNT, *FILL, *SCAN;
    // viscosity CG
    float4 *MINV, *BVM, *CB, *CG, *CR, *CP, *CZ, *CAP;
    // surface tension: (normal, curvature), (smoothed normal, smoothed curvature)
    float4 *STN, *STNS;
    uint16_t* SID;
    uint32_t cellRel;          // 1: positions are cell-relative (precision mode), see pair_r
    uint32_t analytic;         // 1: W and gradW from the spline itself instead of the tables
    float splK, splL;          // 8 / (pi h^3), 48 / (pi h^3)
    SceneDev* scenes;
    BodyDev* bodies;
    const float *WM, *GM;      // midpoint tables 0.5 (T[i] + T[i+1]), i < 9999
    float wZero, invStep, radius, radius2;
    const float* halton;
    uint32_t* status;          // [0] sticky error flags, [1] abort (capacity)
    // Reduction buckets, 128 B apart so that concurrent atomics land in different
    // L2 slices; blocks pick bucket blockIdx % 32, controllers fold and reset them.
    double* ACCB;              // [scene][kAccSlots][kBuckets] x16: FP64 sums
    uint32_t* MAXB;            // [scene][2][kBuckets] x32: max |v + a dt|^2 bits, max neighbours
    int32_t* MMB;              // [scene][6][kBuckets] x32: min cell xyz, max cell xyz
    unsigned long long condHandle[3];  // while-node handles (div, cg, pres); 0 = eager
    uint8_t lanes[16];                 // lanes per particle of each TunedKernel
    uint16_t blocks[16];               // threads per block of each TunedKernel's row kernels (0 = kBlock)
    // Batches: per solver loop (div, cg, pres) the controllers list the scenes still
    // iterating, [0] particles in them, [1] their count, then prefix[nscenes] (first
    // virtual index of each listed scene) and begin[nscenes] (its first slot); the loop
    // kernels of a batch walk this list with a fixed grid of batchBlocks blocks.
    uint32_t* WORK;
    uint32_t workStride, batchBlocks;
    // Cell tiles of the solver-loop kernels (pressure acceleration, Jacobi update, CG
    // product), per TunedKernel: 0 = the pass walks neighbour rows, else 2^tiles[k]
    // consecutive Morton cells per tile (3: a 2x2x2 block, 4: 4x2x2). compactRows: some
    // pass runs on tiles, so the search writes the NBRC rows.
    uint8_t tiles[16];
    uint32_t compactRows;
    // 1: the CG product walks the neighbour rows instead of cell tiles (the adjoint's CG
    // runs on recorded rows of a past step, whose cell tables are no longer current)
    uint32_t rowLoops;
};

// ---------------------------------------------------------------- float3 math
__device__ __forceinline__ float3 f3(float4 a) { return make_float3(a.x, a.y, a.z); }
__device__ __forceinline__ float3 operator+(float3 a, float3 b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 operator-(float3 a, float3 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 operator-(float3 a) { return make_float3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ float3 operator*(float s, float3 a) { return make_float3(s * a.x, s * a.y, s * a.z); }
__device__ __forceinline__ float3 operator*(float3 a, float s) { return make_float3(s * a.x, s * a.y, s * a.z); }
__device__ __forceinline__ float3& operator+=(float3& a, float3 b) { a.x += b.x; a.y += b.y; a.z += b.z; return a; }
__device__ __forceinline__ float3& operator-=(float3& a, float3 b) { a.x -= b.x; a.y -= b.y; a.z -= b.z; return a; }
__device__ __forceinline__ float dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float4 f4(float3 a, float w) { return make_float4(a.x, a.y, a.z, w); }
__device__ __forceinline__ float3 cross3(float3 a, float3 b) {
    return make_float3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
__device__ __forceinline__ float3 normalize3(float3 a) { return a * (1.0f / sqrtf(dot3(a, a))); }

// Approximate square root (PTX sqrt.approx.f32). The reference is compiled with
// -use_fast_math, which selects the same approximate instruction for its sqrt and
// divisions; the neighbour loops use it and __fdividef, the search does not.
__device__ __forceinline__ float fast_sqrt(float x) {
    float r;
    asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// -------------------------------------------------------- cell-relative positions
// Precision mode (Dev::cellRel): a particle's position is X.xyz = its offset from the
// corner of its anchor cell, a cube of edge h (the support radius) at integer
// coordinates A from the scene's origin S.org, with A packed in X.w (10 bits per axis,
// two's complement, |A| < 512). Pair vectors x_i - x_j = (o_i - o_j) + h (A_i - A_j)
// are then differences of numbers of size h instead of of absolute coordinates.
// Quantities of one particle (its boundary samples) live in its own offset frame.
__device__ __forceinline__ int3 anchor_of(float w) {
    const uint32_t b = __float_as_uint(w);
    return make_int3((int)(b << 22) >> 22, (int)((b >> 10) << 22) >> 22, (int)((b >> 20) << 22) >> 22);
}
__device__ __forceinline__ float anchor_pack(int3 a) {
    return __uint_as_float((uint32_t)(a.x & 1023) | ((uint32_t)(a.y & 1023) << 10) | ((uint32_t)(a.z & 1023) << 20));
}
// x_a - x_b of two particles of one scene; REL: positions are cell-relative (the
// neighbour-loop kernels are instantiated for both storage modes).
template <bool REL>
__device__ __forceinline__ float3 pair_r(const Dev& d, float4 a, float4 b) {
    float3 r = make_float3(a.x - b.x, a.y - b.y, a.z - b.z);
    if (REL) {
        const int3 A = anchor_of(a.w), B = anchor_of(b.w);
        const float L = d.radius;
        r.x += L * (float)(A.x - B.x);
        r.y += L * (float)(A.y - B.y);
        r.z += L * (float)(A.z - B.z);
    }
    return r;
}
// Absolute position (FP32) of a particle of scene S.
__device__ __forceinline__ float3 abs_pos(const Dev& d, const SceneDev& S, float4 x) {
    if (!d.cellRel) return make_float3(x.x, x.y, x.z);
    const int3 A = anchor_of(x.w);
    const float L = d.radius;
    return make_float3(S.org[0] + (L * (float)A.x + x.x), S.org[1] + (L * (float)A.y + x.y),
                       S.org[2] + (L * (float)A.z + x.z));
}

// -------------------------------------------------------- SPH kernel lookups
// PrecomputedDFSPHCubicKernel::GetW / GetGradientW (Kernel/DFSPHKernels.h:54-80):
// index = min(trunc(|r| / step), R - 2), value = midpoint of two table entries.
__device__ __forceinline__ uint32_t table_pos(const Dev& d, float rl) {
    const uint32_t p = __float2uint_rz(rl * d.invStep);
    return min(p, kTableRes - 2u);
}
// The cubic spline the tables sample (CalculateW / CalculateGradientW,
// Kernel/DFSPHKernels.h:86-131), evaluated at |r| itself: the analytic kernel mode, in
// which W and gradW are smooth in r (the tables are piecewise constant in |r|).
__device__ __forceinline__ float spline_w(const Dev& d, float rl) {
    const float q = rl / d.radius;
    if (q > 1.0f) return 0.0f;
    if (q <= 0.5f) {
        const float q2 = q * q, q3 = q2 * q;
        return d.splK * (6.0f * q3 - 6.0f * q2 + 1.0f);
    }
    const float f = 1.0f - q;
    return d.splK * (2.0f * (f * f * f));
}
__device__ __forceinline__ float spline_gs(const Dev& d, float rl) {  // gradW = gs * r
    const float q = rl / d.radius;
    if (!(rl > 1.0e-5f) || q > 1.0f) return 0.0f;
    const float gq = 1.0f / (rl * d.radius);
    if (q <= 0.5f) return ((d.splL * q) * (3.0f * q - 2.0f)) * gq;
    const float f = 1.0f - q;
    return (d.splL * (-f * f)) * gq;
}
__device__ __forceinline__ float kernel_w(const Dev& d, float3 r) {
    const float r2 = dot3(r, r);
    if (r2 <= d.radius2) return d.analytic ? spline_w(d, fast_sqrt(r2)) : __ldg(d.WM + table_pos(d, fast_sqrt(r2)));
    return 0.0f;
}
__device__ __forceinline__ float3 kernel_grad(const Dev& d, float3 r) {
    const float rl = fast_sqrt(dot3(r, r));
    if (rl <= d.radius) return (d.analytic ? spline_gs(d, rl) : __ldg(d.GM + table_pos(d, rl))) * r;
    return make_float3(0.f, 0.f, 0.f);
}

// gradW factor of one pair: GetGradientW(r) = gs * r (Kernel/DFSPHKernels.h:67-80),
// from the pair's squared distance r2.
__device__ __forceinline__ float grad_factor_r2(const Dev& d, float r2) {
    const float rl = fast_sqrt(r2);
    if (!(rl <= d.radius)) return 0.0f;
    return d.analytic ? spline_gs(d, rl) : __ldg(d.GM + table_pos(d, rl));
}
__device__ __forceinline__ float grad_factor(const Dev& d, float3 r) { return grad_factor_r2(d, dot3(r, r)); }

// ------------------------------------------------------------ Morton cell keys
__device__ __forceinline__ uint32_t part1by2(uint32_t x) {  // ParticleSearchKernels.cu:9-17
    x &= 0x000003ffu;
    x = (x ^ (x << 16)) & 0xff0000ffu;
    x = (x ^ (x << 8)) & 0x0300f00fu;
    x = (x ^ (x << 4)) & 0x030c30c3u;
    x = (x ^ (x << 2)) & 0x09249249u;
    return x;
}

// ToCellIndexMortonMetaGrid, ParticleSearchKernels.cu:24-38: 8^3-cell meta blocks in
// row-major order, Morton order (x lowest bit) inside each.
__device__ __forceinline__ uint32_t cell_key(const SceneDev& s, int cx, int cy, int cz) {
    const uint32_t mx = (uint32_t)cx >> 3, my = (uint32_t)cy >> 3, mz = (uint32_t)cz >> 3;
    const uint32_t meta = mz * s.meta[1] * s.meta[0] + my * s.meta[0] + mx;
    return meta * 512u + ((part1by2((uint32_t)cz & 7u) << 2) + (part1by2((uint32_t)cy & 7u) << 1) +
                          part1by2((uint32_t)cx & 7u));
}

// Inverse of the Morton interleave inside a meta block: bits 0, 3, 6 of m -> bits 0, 1, 2
// (x of m, y of m >> 1, z of m >> 2).
__device__ __forceinline__ uint32_t compact3(uint32_t m) { return (m & 1u) | ((m >> 2) & 2u) | ((m >> 4) & 4u); }

// Orthogonal vectors of a unit vector (Core/Math/Math.h:19-33).
__device__ __forceinline__ void orthogonal_vectors(float3 vec, float3& x, float3& y) {
    float3 v = make_float3(1.f, 0.f, 0.f);
    if (fabsf(dot3(v, vec)) > 0.999f) v = make_float3(0.f, 1.f, 0.f);
    x = cross3(vec, v);
    y = cross3(vec, x);
    x = normalize3(x);
    y = normalize3(y);
}

__device__ __forceinline__ uint32_t scene_of(const Dev& d, uint32_t i) { return d.nscenes == 1 ? 0u : (uint32_t)d.SID[i]; }

// ------------------------------------------------------------ reductions
__device__ __forceinline__ double* acc_bucket(const Dev& d, uint32_t s, int slot, uint32_t b) {
    return d.ACCB + ((size_t)(s * kAccSlots + (uint32_t)slot) * kBuckets + b) * 16u;
}
__device__ __forceinline__ uint32_t* max_bucket(const Dev& d, uint32_t s, int k, uint32_t b) {
    return d.MAXB + ((size_t)(s * 2u + (uint32_t)k) * kBuckets + b) * 32u;
}
__device__ __forceinline__ int32_t* mm_bucket(const Dev& d, uint32_t s, int k, uint32_t b) {
    return d.MMB + ((size_t)(s * 6u + (uint32_t)k) * kBuckets + b) * 32u;
}
// Controller side: sum (and zero) one accumulator's buckets.
// (all bucket loads are issued before the first add, so the fold costs one L2 round trip
// rather than kBuckets of them; the sum runs in bucket order as before)
__device__ __forceinline__ double fold_acc(const Dev& d, uint32_t s, int slot) {
    double* q = acc_bucket(d, s, slot, 0);
    double v[kBuckets];
#pragma unroll
    for (uint32_t b = 0; b < kBuckets; b++) v[b] = __ldcg(q + (size_t)b * 16u);
    double t = 0.0;
#pragma unroll
    for (uint32_t b = 0; b < kBuckets; b++) t += v[b];
#pragma unroll
    for (uint32_t b = 0; b < kBuckets; b++) q[(size_t)b * 16u] = 0.0;
    return t;
}
// The same fold by a whole warp (one scene's controller): lane b loads and zeroes bucket
// b, and an xor butterfly adds them, five dependent FP64 adds instead of 32 (a dependent
// FP64 add takes ~64 cycles on this GPU, an FP32 one 4). Every lane ends with the same
// sum: partners add the same two numbers, and IEEE addition is commutative.
__device__ __forceinline__ double fold_acc_warp(const Dev& d, uint32_t s, int slot, uint32_t lane) {
    static_assert(kBuckets == 32u, "one bucket per lane");
    double* q = acc_bucket(d, s, slot, lane);
    double v = __ldcg(q);
    *q = 0.0;
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ uint32_t fold_max(const Dev& d, uint32_t s, int k) {
    uint32_t* q = max_bucket(d, s, k, 0);
    uint32_t v[kBuckets];
#pragma unroll
    for (uint32_t b = 0; b < kBuckets; b++) v[b] = __ldcg(q + (size_t)b * 32u);
    uint32_t t = 0u;
#pragma unroll
    for (uint32_t b = 0; b < kBuckets; b++) t = max(t, v[b]);
#pragma unroll
    for (uint32_t b = 0; b < kBuckets; b++) q[(size_t)b * 32u] = 0u;
    return t;
}

// Warp sum of the FP32 values v over the lanes that are multiples of `step` (the others
// hold zeros), as an unevaluated pair hi + lo of FP32 numbers: each level adds the
// partners' high parts with Knuth's error-free TwoSum and carries the rounding error
// and the partners' low parts in lo, so the pair keeps ~44 significant bits (relative
// error ~1e-13 for a warp's 32 terms). FP64 arithmetic runs at a small fraction of the
// FP32 rate on this GPU (a dependent add takes ~64 cycles, and a warp instruction holds
// the FP64 pipe whatever its active lanes), so a block combines its warps' pairs the
// same way (pair_add) and widens the result to FP64 once (pair_value).
__device__ __forceinline__ void pair_add(float& hi, float& lo, float h2, float l2) {
    const float sum = __fadd_rn(hi, h2);
    const float bb = __fsub_rn(sum, hi);
    const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(sum, bb)), __fsub_rn(h2, bb));
    lo = __fadd_rn(__fadd_rn(lo, l2), err);
    hi = sum;
}
__device__ __forceinline__ float2 warp_sum_pair(float v, int step) {
    float hi = v, lo = 0.0f;
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) {
        if (o < step) break;
        const float h2 = __shfl_xor_sync(0xffffffffu, hi, o);
        const float l2 = __shfl_xor_sync(0xffffffffu, lo, o);
        pair_add(hi, lo, h2, l2);
    }
    return make_float2(hi, lo);
}
__device__ __forceinline__ double pair_value(float2 p) { return (double)p.x + (double)p.y; }

// Adds the FP32 terms `v` into scene `sid`'s FP64 accumulators `slot` (bucket
// blockIdx % 32). A block whose particles lie in one scene sums each warp as an FP32
// pair (warp_sum_pair), the warps' pairs likewise in shared memory, and issues one FP64
// atomic per accumulator; otherwise each valid thread adds its own value. Kernels running G lanes
// per particle pass G (a block then covers blockDim.x / G particles; only the first
// lane of each group contributes); all threads of the block must call this.
// Core of scene_accumulate: `uniformScene` is the scene of every particle the block
// serves, or -1 when they belong to several scenes.
template <int K, uint32_t G = 1>
__device__ __forceinline__ void scene_accumulate_core(const Dev& d, int uniformScene, uint32_t sid, bool valid,
                                                      const float (&v)[K], const int (&slot)[K]) {
    __shared__ float2 sm[32][4];  // one row per warp of a block of up to 1024 threads
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t bucket = blockIdx.x % kBuckets;
    if (uniformScene >= 0) {
        float2 s[K];
#pragma unroll
        for (int k = 0; k < K; k++) s[k] = warp_sum_pair(valid ? v[k] : 0.0f, (int)G);
        __syncthreads();
        if (lane == 0)
#pragma unroll
            for (int k = 0; k < K; k++) sm[warp][k] = s[k];
        __syncthreads();
        if (threadIdx.x == 0) {
#pragma unroll
            for (int k = 0; k < K; k++) {
                float hi = 0.0f, lo = 0.0f;
                for (uint32_t w = 0; w < blockDim.x / 32u; w++) pair_add(hi, lo, sm[w][k].x, sm[w][k].y);
                const double t = pair_value(make_float2(hi, lo));
                if (t != 0.0) atomicAdd(acc_bucket(d, (uint32_t)uniformScene, slot[k], bucket), t);
            }
        }
    } else if (valid) {
#pragma unroll
        for (int k = 0; k < K; k++) atomicAdd(acc_bucket(d, sid, slot[k], bucket), (double)v[k]);
    }
}

template <int K, uint32_t G = 1>
__device__ __forceinline__ void scene_accumulate(const Dev& d, uint32_t sid, bool valid, const float (&v)[K],
                                                 const int (&slot)[K]) {
    __shared__ float2 sm[32][4];  // one row per warp of a block of up to 1024 threads
    __shared__ int uniformBlock;
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t first = blockIdx.x * (blockDim.x / G);
    const uint32_t last = min(first + blockDim.x / G, d.n) - 1u;
    const uint32_t bucket = blockIdx.x % kBuckets;
    if (threadIdx.x == 0) uniformBlock = (first < d.n) && (scene_of(d, first) == scene_of(d, last)) ? 1 : 0;
    __syncthreads();
    if (uniformBlock) {
        float2 s[K];
#pragma unroll
        for (int k = 0; k < K; k++) s[k] = warp_sum_pair(valid ? v[k] : 0.0f, (int)G);
        if (lane == 0)
#pragma unroll
            for (int k = 0; k < K; k++) sm[warp][k] = s[k];
        __syncthreads();
        if (threadIdx.x == 0) {
            const uint32_t sc = scene_of(d, first);
#pragma unroll
            for (int k = 0; k < K; k++) {
                float hi = 0.0f, lo = 0.0f;
                for (uint32_t w = 0; w < blockDim.x / 32u; w++) pair_add(hi, lo, sm[w][k].x, sm[w][k].y);
                const double t = pair_value(make_float2(hi, lo));
                if (t != 0.0) atomicAdd(acc_bucket(d, sc, slot[k], bucket), t);
            }
        }
    } else if (valid) {
#pragma unroll
        for (int k = 0; k < K; k++) atomicAdd(acc_bucket(d, sid, slot[k], bucket), (double)v[k]);
    }
}

// Max of non-negative floats (they order like their bit patterns) into max bucket 0.
__device__ __forceinline__ void scene_max_float(const Dev& d, uint32_t sid, bool valid, float v) {
    float m = valid ? v : 0.0f;
    const uint32_t s0 = __shfl_sync(0xffffffffu, sid, 0);
    const bool uniform = __all_sync(0xffffffffu, sid == s0 || !valid);
    const uint32_t bucket = blockIdx.x % kBuckets;
    if (uniform) {
        const uint32_t mb = __reduce_max_sync(0xffffffffu, __float_as_uint(m));
        if ((threadIdx.x & 31u) == 0 && mb > 0u) atomicMax(max_bucket(d, s0, 0, bucket), mb);
    } else if (valid) {
        atomicMax(max_bucket(d, sid, 0, bucket), __float_as_uint(m));
    }
}

// Every kernel of the step counts its own launch in status[8] (block 0, thread 0),
// so graph runs with data-dependent loop counts report how many kernels ran.
#define VFD_COUNT_LAUNCH(d)                                                     \
    do {                                                                        \
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd((d).status + 8, 1u); \
    } while (0)

// Bounds-checked build (-DVFD_BOUNDS_CHECK, vfd_gb300.build.build(bounds_check=True)):
// device index checks that record a failure in the status word (VFD_FLAG_BOUNDS in
// status[0]; status[9] keeps the first offending index + 1) and substitute index 0, so
// the kernel neither faults nor traps and the host reports the failure after the step.
// The default build compiles the checks out.
__device__ __forceinline__ uint32_t checked_index(uint32_t* status, uint32_t idx, uint32_t limit) {
#ifdef VFD_BOUNDS_CHECK
    if (idx >= limit) {
        atomicOr(status, 0x80u);
        atomicCAS(status + 9, 0u, idx + 1u);
        return 0u;
    }
#else
    (void)status;
    (void)limit;
#endif
    return idx;
}

// The abort flag is raised only by the search kernels; later kernels read it through
// the read-only path (one L2 request per SM instead of one per thread).
__device__ __forceinline__ bool is_aborted(const Dev& d) { return __ldg(d.status + 1) != 0u; }

// G consecutive lanes of a warp that share one particle in a neighbour loop;
// lanes stride the neighbour row and reduce their partial sums with shuffles.
template <uint32_t G>
struct Group {
    uint32_t p, lane, mask;
    __device__ __forceinline__ Group() {
        const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
        p = t / G;
        lane = t % G;
        mask = G == 32u ? 0xffffffffu : (((1u << G) - 1u) << ((threadIdx.x & 31u) & ~(G - 1u)));
    }
    // The group of this thread serving particle slot `slot` (batch work lists).
    __device__ __forceinline__ explicit Group(uint32_t slot) {
        p = slot;
        lane = threadIdx.x % G;
        mask = G == 32u ? 0xffffffffu : (((1u << G) - 1u) << ((threadIdx.x & 31u) & ~(G - 1u)));
    }
    __device__ __forceinline__ float sum(float v) const {
#pragma unroll
        for (uint32_t o = G / 2; o > 0; o >>= 1) v += __shfl_xor_sync(mask, v, o);
        return v;
    }
    __device__ __forceinline__ float3 sum(float3 v) const { return make_float3(sum(v.x), sum(v.y), sum(v.z)); }
    __device__ __forceinline__ uint32_t sum(uint32_t v) const {
#pragma unroll
        for (uint32_t o = G / 2; o > 0; o >>= 1) v += __shfl_xor_sync(mask, v, o);
        return v;
    }
};

// Sum over the G lanes of a group (mask: the group's lanes of the warp).
template <uint32_t G>
__device__ __forceinline__ float group_sum(uint32_t mask, float v) {
#pragma unroll
    for (uint32_t o = G / 2; o > 0; o >>= 1) v += __shfl_xor_sync(mask, v, o);
    return v;
}
template <uint32_t G>
__device__ __forceinline__ float3 group_sum(uint32_t mask, float3 v) {
    return make_float3(group_sum<G>(mask, v.x), group_sum<G>(mask, v.y), group_sum<G>(mask, v.z));
}

// ------------------------------------------------------------ batch work lists
__device__ __forceinline__ const uint32_t* work_list(const Dev& d, int loop) { return d.WORK + (size_t)loop * d.workStride; }
__device__ __forceinline__ uint32_t work_total(const Dev& d, int loop) { return __ldg(work_list(d, loop)); }
// Slot of virtual index vp (< total) of a loop's work list: the listed scene whose
// prefix is the largest one <= vp, found by binary search.
__device__ __forceinline__ uint32_t work_slot(const Dev& d, int loop, uint32_t vp, uint32_t& scene) {
    const uint32_t* w = work_list(d, loop);
    const uint32_t na = __ldg(w + 1);
    const uint32_t* pre = w + 2;
    const uint32_t* beg = w + 2 + d.nscenes;
    uint32_t lo = 0, hi = na - 1u;
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1u) >> 1;
        if (__ldg(pre + mid) <= vp) lo = mid;
        else hi = mid - 1u;
    }
    const uint32_t p = __ldg(beg + lo) + (vp - __ldg(pre + lo));
    scene = scene_of(d, p);
    return p;
}

// Host-side launch helpers.
inline uint32_t blocks_for(uint32_t n, uint32_t block = kBlock) { return (n + block - 1) / block; }

// Optional per-launch timing of eagerly launched kernels (CUDA events on the launch
// stream); set only while vfd_profile_kernels runs, never during graph capture.
struct LaunchProfiler {
    virtual void begin(const char* name, cudaStream_t s) = 0;
    virtual void end(cudaStream_t s) = 0;
    virtual ~LaunchProfiler() {}
};
extern LaunchProfiler* g_profiler;
#define VFD_LAUNCH(name, stream, ...)                          \
    do {                                                       \
        if (::vfd::g_profiler) ::vfd::g_profiler->begin(name, stream); \
        __VA_ARGS__;                                           \
        if (::vfd::g_profiler) ::vfd::g_profiler->end(stream); \
    } while (0)

// Launch of a neighbour-loop kernel with the tuned lanes per particle; KERNEL(G) names
// the instantiation (a function-like macro).
// The same for a batch loop kernel: a fixed grid of d.batchBlocks blocks.
#define VFD_LAUNCH_LANES_BATCH(name, id, KERNEL)                                                     \
    do {                                                                                            \
        const uint32_t B_ = d.blocks[id] ? d.blocks[id] : kBlock;                                   \
        const uint32_t NB_ = d.batchBlocks * kBlock / B_;                                           \
        switch (d.lanes[id]) {                                                                      \
            case 4: VFD_LAUNCH(name, s, KERNEL(4)<<<NB_, B_, 0, s>>>(d)); break;                    \
            case 16: VFD_LAUNCH(name, s, KERNEL(16)<<<NB_, B_, 0, s>>>(d)); break;                  \
            default: VFD_LAUNCH(name, s, KERNEL(8)<<<NB_, B_, 0, s>>>(d)); break;                   \
        }                                                                                           \
    } while (0)

#define VFD_LAUNCH_LANES(name, id, KERNEL)                                                          \
    do {                                                                                            \
        const uint32_t B_ = d.blocks[id] ? d.blocks[id] : kBlock;                                   \
        switch (d.lanes[id]) {                                                                      \
            case 4: VFD_LAUNCH(name, s, KERNEL(4)<<<blocks_for(d.n * 4u, B_), B_, 0, s>>>(d)); break;   \
            case 16: VFD_LAUNCH(name, s, KERNEL(16)<<<blocks_for(d.n * 16u, B_), B_, 0, s>>>(d)); break; \
            default: VFD_LAUNCH(name, s, KERNEL(8)<<<blocks_for(d.n * 8u, B_), B_, 0, s>>>(d)); break;  \
        }                                                                                           \
    } while (0)

}  // namespace vfd
