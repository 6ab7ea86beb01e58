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
//   NBR  u32 [70][slot] neighbour slots (ELL, column = neighbour rank)
//   NCNT u32 [slot] neighbour count | flag bits
// The reference keeps one 120-byte AoS DFSPHParticle per particle
// (Structures/DFSPHParticle.h:8-33) in original order.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace vfd {

constexpr uint32_t kMaxNeighbors = 70u;      // ParticleSearchKernels.cuh:7
constexpr uint32_t kTableRes = 10000u;       // Kernel/DFSPHKernels.h:143
constexpr uint32_t kHaltonCount = 49152u;    // HaltonVec323.cuh:4
constexpr uint32_t kBlock = 128u;            // threads per particle kernel
constexpr float kEps = 1.0e-5f;              // Core/Math/Math.h:6

// NCNT flag bits (above the 7-bit count).
constexpr uint32_t kCountMask = 0xFFu;
constexpr uint32_t kHasBoundary = 1u << 8;   // some body gave this particle Vb > 0
constexpr uint32_t kHasBoundaryVisc = 1u << 9;

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
    uint32_t cellBase, cellCount;
    uint32_t flags;            // VFD_FLAG_* of the current step
    uint32_t maxNbr;
    LoopState div, pres;
    // viscosity CG
    uint32_t cgIt, cgActive, cgDone, cgZeroG, cgUpdateP;
    float cgErr;
    double cgRhs, cgThr, cgAbsNew, cgRR;
    float cgAlpha, cgBeta;
    double acc[4];             // FP64 reduction accumulators of the current sub-stage
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
    // search scratch
    uint32_t *KEY, *KEYS, *TMP, *CELL_START, *CELL_COUNT, *FILL, *SCAN;
    // viscosity CG
    float4 *MINV, *BVM, *CB, *CG, *CR, *CP, *CZ, *CAP;
    // surface tension: (normal, curvature), (smoothed normal, smoothed curvature)
    float4 *STN, *STNS;
    uint16_t* SID;
    SceneDev* scenes;
    BodyDev* bodies;
    const float *WM, *GM;      // midpoint tables 0.5 (T[i] + T[i+1]), i < 9999
    float wZero, invStep, radius, radius2;
    const float* halton;
    uint32_t* status;          // [0] sticky error flags, [1] abort (capacity)
    unsigned long long condHandle[3];  // while-node handles (div, cg, pres); 0 = eager
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

// -------------------------------------------------------- SPH kernel lookups
// PrecomputedDFSPHCubicKernel::GetW / GetGradientW (Kernel/DFSPHKernels.h:54-80):
// index = min(trunc(|r| / step), R - 2), value = midpoint of two table entries.
__device__ __forceinline__ uint32_t table_pos(const Dev& d, float rl) {
    const uint32_t p = __float2uint_rz(rl * d.invStep);
    return min(p, kTableRes - 2u);
}
__device__ __forceinline__ float kernel_w(const Dev& d, float3 r) {
    const float r2 = dot3(r, r);
    if (r2 <= d.radius2) return __ldg(d.WM + table_pos(d, sqrtf(r2)));
    return 0.0f;
}
__device__ __forceinline__ float3 kernel_grad(const Dev& d, float3 r) {
    const float rl = sqrtf(dot3(r, r));
    if (rl <= d.radius) return __ldg(d.GM + table_pos(d, rl)) * r;
    return make_float3(0.f, 0.f, 0.f);
}

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
// Adds `v` into scenes[sid].acc[k] (FP64). Warps whose lanes share one scene
// reduce with shuffles first; a block whose slots lie in one scene reduces in
// shared memory and issues one atomic.
template <int K>
__device__ __forceinline__ void scene_accumulate(const Dev& d, uint32_t sid, bool valid, const double (&v)[K],
                                                 const int (&slot)[K]) {
    __shared__ double sm[kBlock / 32][4];
    __shared__ int uniformBlock;
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t first = blockIdx.x * blockDim.x;
    const uint32_t last = min(first + blockDim.x, d.n) - 1u;
    if (threadIdx.x == 0) uniformBlock = (first < d.n) && (scene_of(d, first) == scene_of(d, last)) ? 1 : 0;
    __syncthreads();
    if (uniformBlock) {
        double s[K];
#pragma unroll
        for (int k = 0; k < K; k++) {
            s[k] = valid ? v[k] : 0.0;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s[k] += __shfl_xor_sync(0xffffffffu, s[k], o);
        }
        if (lane == 0)
#pragma unroll
            for (int k = 0; k < K; k++) sm[warp][k] = s[k];
        __syncthreads();
        if (threadIdx.x == 0) {
            const uint32_t sc = scene_of(d, first);
#pragma unroll
            for (int k = 0; k < K; k++) {
                double t = 0.0;
                for (uint32_t w = 0; w < blockDim.x / 32u; w++) t += sm[w][k];
                atomicAdd(&d.scenes[sc].acc[slot[k]], t);
            }
        }
    } else if (valid) {
#pragma unroll
        for (int k = 0; k < K; k++) atomicAdd(&d.scenes[sid].acc[slot[k]], v[k]);
    }
}

__device__ __forceinline__ void scene_max_float(const Dev& d, uint32_t sid, bool valid, float v) {
    // non-negative floats order like their bit patterns
    float m = valid ? v : 0.0f;
    const uint32_t s0 = __shfl_sync(0xffffffffu, sid, 0);
    const bool uniform = __all_sync(0xffffffffu, sid == s0 || !valid);
    if (uniform) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
        if ((threadIdx.x & 31u) == 0 && m > 0.0f) atomicMax(&d.scenes[s0].maxV2Bits, __float_as_uint(m));
    } else if (valid) {
        atomicMax(&d.scenes[sid].maxV2Bits, __float_as_uint(m));
    }
}

// Host-side launch helpers.
inline uint32_t blocks_for(uint32_t n, uint32_t block = kBlock) { return (n + block - 1) / block; }

}  // namespace vfd
