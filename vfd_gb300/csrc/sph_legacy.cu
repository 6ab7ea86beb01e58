// The reference's legacy SPH pipeline (Simulation/SPH: SPHSimulation.cpp, SPHSimulation.cu,
// SPHSimulationKernel.cu) on GB300: weakly compressible SPH over a uniform grid of cell
// edge 2r. Per step, as SPHSimulation::OnUpdate (SPHSimulation.cpp:71-95) orders it:
//   1. integrate (IntegrateKernel, SPHSimulationKernel.cu:61-92): wall penalties, gravity,
//      damping, position update and hard clamp, in the caller's particle order;
//   2. cell keys (CalculateHashKernel, :111-122) and a counting sort by key whose in-cell
//      order is ascending particle index -- the order the reference's stable LSD radix
//      sort of (key, index) pairs gives (SPHSimulation.cpp:84);
//   3. reorder (ReorderKernel, :124-151): the state gathered into cell order;
//   4. density and pressure (CalculateDensityKernel, :270-297) and force
//      (CalculateForceKernel, :299-334) over the 27 cells around each particle, in the
//      reference's z, y, x cell order with one partial sum per cell, at most
//      MaxParticlesInCellCount particles read per cell; the new velocity goes back to
//      the caller's order.
// Texture fetches become read-only loads of the cell-ordered arrays; the GL buffers the
// reference maps become plain device arrays; the host driver stays on one stream.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/vfd_sph.h"
#include "dfsph_sim.h"

using vfd::host::fail;

namespace {

struct SphDev {  // SPHSimulationParameters as the kernels read them
    float dt, damping, h, h2, spiky, lap, poly6, mass, rho0, stiffness, visc, minDens, minDist;
    float hardDist, softDist, boundsDamp, boundsStiff, boundsDampCrit;
    float g[3], wmin[3], wmax[3], cell;
    uint32_t gx, gy, gz, gyx, cells, maxPerCell, n;
};

__device__ __forceinline__ int3 grid_pos(const SphDev& P, float4 p) {
    // (position - WorldMin) / CellSize, floored (SPHSimulationKernel.cu:94-103)
    return make_int3((int)floorf(__fdiv_rn(__fsub_rn(p.x, P.wmin[0]), P.cell)),
                     (int)floorf(__fdiv_rn(__fsub_rn(p.y, P.wmin[1]), P.cell)),
                     (int)floorf(__fdiv_rn(__fsub_rn(p.z, P.wmin[2]), P.cell)));
}
__device__ __forceinline__ uint32_t grid_hash(const SphDev& P, int3 c) {  // :105-109
    return (uint32_t)(c.z * (int)P.gyx + c.y * (int)P.gx + c.x);
}
__device__ __forceinline__ bool in_grid(const SphDev& P, int3 c) {
    return c.x >= 0 && c.y >= 0 && c.z >= 0 && c.x < (int)P.gx && c.y < (int)P.gy && c.z < (int)P.gz;
}

// CalculateBoundary (SPHSimulationKernel.cu:17-59): penalty accelerations of the six walls
// in the order z-, z+ (critical damping), x-, x+, y-, y+.
__device__ __forceinline__ void walls(const SphDev& P, float3 x, float3& v) {
    const float b = P.softDist;
    auto add = [&](float diff, float nx, float ny, float nz, float damp) {
        if (diff > 0.00001f) {
            const float acc = __fsub_rn(__fmul_rn(P.boundsStiff, diff),
                                        __fmul_rn(damp, __fadd_rn(__fadd_rn(__fmul_rn(nx, v.x), __fmul_rn(ny, v.y)),
                                                                  __fmul_rn(nz, v.z))));
            v.x = __fadd_rn(v.x, __fmul_rn(__fmul_rn(acc, nx), P.dt));
            v.y = __fadd_rn(v.y, __fmul_rn(__fmul_rn(acc, ny), P.dt));
            v.z = __fadd_rn(v.z, __fmul_rn(__fmul_rn(acc, nz), P.dt));
        }
    };
    add(__fadd_rn(__fsub_rn(b, x.z), P.wmin[2]), 0.f, 0.f, 1.f, P.boundsDampCrit);
    add(__fsub_rn(__fadd_rn(b, x.z), P.wmax[2]), 0.f, 0.f, -1.f, P.boundsDampCrit);
    add(__fadd_rn(__fsub_rn(b, x.x), P.wmin[0]), 1.f, 0.f, 0.f, P.boundsDamp);
    add(__fsub_rn(__fadd_rn(b, x.x), P.wmax[0]), -1.f, 0.f, 0.f, P.boundsDamp);
    add(__fadd_rn(__fsub_rn(b, x.y), P.wmin[1]), 0.f, 1.f, 0.f, P.boundsDamp);
    add(__fsub_rn(__fadd_rn(b, x.y), P.wmax[1]), 0.f, -1.f, 0.f, P.boundsDamp);
}

__global__ void k_sph_integrate(SphDev P, const float4* __restrict__ xo, const float4* __restrict__ vo,
                                float4* __restrict__ xn, float4* __restrict__ vn) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    const float4 x4 = xo[i], v4 = vo[i];
    float3 x = make_float3(x4.x, x4.y, x4.z), v = make_float3(v4.x, v4.y, v4.z);
    walls(P, x, v);
    v = make_float3(__fadd_rn(v.x, __fmul_rn(P.g[0], P.dt)), __fadd_rn(v.y, __fmul_rn(P.g[1], P.dt)),
                    __fadd_rn(v.z, __fmul_rn(P.g[2], P.dt)));
    v = make_float3(__fmul_rn(v.x, P.damping), __fmul_rn(v.y, P.damping), __fmul_rn(v.z, P.damping));
    x = make_float3(__fadd_rn(x.x, __fmul_rn(v.x, P.dt)), __fadd_rn(x.y, __fmul_rn(v.y, P.dt)),
                    __fadd_rn(x.z, __fmul_rn(v.z, P.dt)));
    const float b = P.hardDist;
    float c[3] = {x.x, x.y, x.z};
    for (int k = 0; k < 3; k++) {
        const float hi = __fsub_rn(P.wmax[k], b), lo = __fadd_rn(P.wmin[k], b);
        if (c[k] > hi) c[k] = hi;
        if (c[k] < lo) c[k] = lo;
    }
    xn[i] = make_float4(c[0], c[1], c[2], x4.w);
    vn[i] = make_float4(v.x, v.y, v.z, v4.w);
}

__global__ void k_sph_keys(SphDev P, const float4* __restrict__ x, uint32_t* key, uint32_t* count,
                           uint32_t* status) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    const int3 c = grid_pos(P, x[i]);
    if (!in_grid(P, c)) {  // positions are clamped inside the world; a NaN lands here
        atomicOr(status, 1u);
        key[i] = 0u;
        atomicAdd(count, 1u);
        return;
    }
    const uint32_t k = grid_hash(P, c);
    key[i] = k;
    atomicAdd(count + k, 1u);
}

constexpr uint32_t kScanChunk = 1024u;

__global__ void __launch_bounds__(256) k_sph_scan_reduce(const uint32_t* in, uint32_t total, uint32_t* partial) {
    const uint32_t base = blockIdx.x * kScanChunk;
    uint32_t s = 0;
    for (uint32_t k = threadIdx.x; k < kScanChunk; k += 256u)
        if (base + k < total) s += in[base + k];
    s = __reduce_add_sync(0xffffffffu, s);
    __shared__ uint32_t ws[8];
    if ((threadIdx.x & 31u) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        for (int w = 0; w < 8; w++) t += ws[w];
        partial[blockIdx.x] = t;
    }
}

// Exclusive scan of the per-chunk totals in place, 1024 at a time with a running carry.
__global__ void __launch_bounds__(1024) k_sph_scan_top(uint32_t* partial, uint32_t nb) {
    __shared__ uint32_t ws[32];
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    uint32_t carry = 0;
    for (uint32_t base = 0; base < nb; base += 1024u) {
        const uint32_t k = base + threadIdx.x;
        const uint32_t v = k < nb ? partial[k] : 0u;
        uint32_t x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= (uint32_t)o) x += y;
        }
        if (lane == 31) ws[warp] = x;
        __syncthreads();
        if (warp == 0) {
            uint32_t w = ws[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
                if (lane >= (uint32_t)o) w += y;
            }
            ws[lane] = w;
        }
        __syncthreads();
        const uint32_t ex = (warp ? ws[warp - 1] : 0u) + x - v;
        const uint32_t total = ws[31];
        if (k < nb) partial[k] = carry + ex;
        carry += total;
        __syncthreads();
    }
}

__global__ void __launch_bounds__(256) k_sph_scan_down(const uint32_t* in, uint32_t total, const uint32_t* partial,
                                                       uint32_t* out) {
    __shared__ uint32_t ws[8];
    const uint32_t base = blockIdx.x * kScanChunk;
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    uint32_t v[4], s = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const uint32_t c = base + threadIdx.x * 4u + k;
        v[k] = c < total ? in[c] : 0u;
        s += v[k];
    }
    uint32_t x = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= (uint32_t)o) x += y;
    }
    if (lane == 31) ws[warp] = x;
    __syncthreads();
    uint32_t wp = 0;
    for (uint32_t w = 0; w < warp; w++) wp += ws[w];
    uint32_t run = partial[blockIdx.x] + wp + x - s;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const uint32_t c = base + threadIdx.x * 4u + k;
        if (c < total) out[c] = run;
        run += v[k];
    }
}

__global__ void k_sph_slots(SphDev P, const uint32_t* key, const uint32_t* start, uint32_t* fill, uint32_t* tmp) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    const uint32_t k = key[i];
    tmp[start[k] + atomicAdd(fill + k, 1u)] = i;
}

// In-cell rank = number of the cell's particles with a lower index; then the gather of
// position and velocity into cell order (ReorderKernel).
__global__ void k_sph_reorder(SphDev P, const uint32_t* key, const uint32_t* start, const uint32_t* count,
                              const uint32_t* tmp, const float4* __restrict__ x, const float4* __restrict__ v,
                              uint32_t* order, uint32_t* sortedKey, float4* xs, float4* vs) {
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= P.n) return;
    const uint32_t i = tmp[q];
    const uint32_t k = key[i], s = start[k], c = count[k];
    uint32_t rank = 0;
    for (uint32_t j = s; j < s + c; j++) rank += tmp[j] < i ? 1u : 0u;
    const uint32_t dst = s + rank;
    order[dst] = i;
    sortedKey[dst] = k;
    xs[dst] = x[i];
    vs[dst] = v[i];
}

// CalculateDensityKernel with CalculateCellDensity (SPHSimulationKernel.cu:153-201, 270-297).
__global__ void k_sph_density(SphDev P, const uint32_t* __restrict__ start, const uint32_t* __restrict__ count,
                              const float4* __restrict__ xs, float* rho, float* pres) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P.n) return;
    const float4 xi = xs[p];
    const int3 g = grid_pos(P, xi);
    float sum = 0.0f;
    for (int dz = -1; dz <= 1; dz++)
        for (int dy = -1; dy <= 1; dy++)
            for (int dx = -1; dx <= 1; dx++) {
                const int3 c = make_int3(g.x + dx, g.y + dy, g.z + dz);
                if (!in_grid(P, c)) continue;
                const uint32_t h = grid_hash(P, c);
                const uint32_t s = __ldg(start + h), m = min(__ldg(count + h), P.maxPerCell);
                float cell = 0.0f;
                for (uint32_t j = s; j < s + m; j++) {
                    if (j == p) continue;
                    const float4 xj = __ldg(xs + j);
                    const float rx = __fsub_rn(xi.x, xj.x), ry = __fsub_rn(xi.y, xj.y), rz = __fsub_rn(xi.z, xj.z);
                    const float r2 = __fadd_rn(__fadd_rn(__fmul_rn(rx, rx), __fmul_rn(ry, ry)), __fmul_rn(rz, rz));
                    if (r2 < P.h2) {
                        const float q = __fsub_rn(P.h2, r2);
                        cell = __fadd_rn(cell, __fmul_rn(__fmul_rn(q, q), q));
                    }
                }
                sum = __fadd_rn(sum, cell);
            }
    const float d = __fmul_rn(__fmul_rn(sum, P.poly6), P.mass);
    rho[p] = d;
    pres[p] = __fmul_rn(__fsub_rn(d, P.rho0), P.stiffness);
}

// CalculateForceKernel with CalculateCellForce and CalculatePairForce (:203-268, 299-334).
__global__ void k_sph_force(SphDev P, const uint32_t* __restrict__ start, const uint32_t* __restrict__ count,
                            const float4* __restrict__ xs, const float4* __restrict__ vs,
                            const float* __restrict__ rho, const float* __restrict__ pres,
                            const uint32_t* __restrict__ order, float4* vout) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P.n) return;
    const float4 xi = xs[p], vi = vs[p];
    const float pi = pres[p], di = rho[p];
    const int3 g = grid_pos(P, xi);
    float3 acc = make_float3(0.f, 0.f, 0.f);
    const float lapVisc = __fmul_rn(P.lap, P.visc);
    for (int dz = -1; dz <= 1; dz++)
        for (int dy = -1; dy <= 1; dy++)
            for (int dx = -1; dx <= 1; dx++) {
                const int3 c = make_int3(g.x + dx, g.y + dy, g.z + dz);
                if (!in_grid(P, c)) continue;
                const uint32_t h = grid_hash(P, c);
                const uint32_t s = __ldg(start + h), m = min(__ldg(count + h), P.maxPerCell);
                float3 cell = make_float3(0.f, 0.f, 0.f);
                for (uint32_t j = s; j < s + m; j++) {
                    if (j == p) continue;
                    const float4 xj = __ldg(xs + j), vj = __ldg(vs + j);
                    const float pj = __ldg(pres + j), dj = __ldg(rho + j);
                    const float d12 = fminf(P.minDens, __fdiv_rn(1.0f, __fmul_rn(di, dj)));
                    const float3 rp = make_float3(__fsub_rn(xi.x, xj.x), __fsub_rn(xi.y, xj.y), __fsub_rn(xi.z, xj.z));
                    const float3 rv = make_float3(__fsub_rn(vj.x, vi.x), __fsub_rn(vj.y, vi.y), __fsub_rn(vj.z, vi.z));
                    const float len = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(rp.x, rp.x), __fmul_rn(rp.y, rp.y)),
                                                           __fmul_rn(rp.z, rp.z)));
                    const float r = fmaxf(P.minDist, len);
                    if (r < P.h) {
                        const float c0 = __fsub_rn(P.h, r);
                        const float pt = __fdiv_rn(__fmul_rn(__fmul_rn(c0, P.spiky), __fadd_rn(pi, pj)), r);
                        const float sc = __fmul_rn(c0, d12);
                        cell.x = __fadd_rn(cell.x, __fmul_rn(__fadd_rn(__fmul_rn(pt, rp.x), __fmul_rn(lapVisc, rv.x)), sc));
                        cell.y = __fadd_rn(cell.y, __fmul_rn(__fadd_rn(__fmul_rn(pt, rp.y), __fmul_rn(lapVisc, rv.y)), sc));
                        cell.z = __fadd_rn(cell.z, __fmul_rn(__fadd_rn(__fmul_rn(pt, rp.z), __fmul_rn(lapVisc, rv.z)), sc));
                    }
                }
                acc = make_float3(__fadd_rn(acc.x, cell.x), __fadd_rn(acc.y, cell.y), __fadd_rn(acc.z, cell.z));
            }
    const float s = __fmul_rn(P.mass, P.dt);
    vout[order[p]] = make_float4(__fadd_rn(vi.x, __fmul_rn(acc.x, s)), __fadd_rn(vi.y, __fmul_rn(acc.y, s)),
                                 __fadd_rn(vi.z, __fmul_rn(acc.z, s)), vi.w);
}

inline uint32_t blocks(uint32_t n, uint32_t b = 256) { return (n + b - 1) / b; }

}  // namespace

struct vfd_sph {
    int device = 0;
    cudaStream_t stream = nullptr;
    vfd_sph_desc desc{};
    vfd_sph_params params{};
    SphDev P{};
    std::vector<float4> x0;
    uint32_t n = 0;
    int cur = 0, vcur = 0;  // pos[cur] and vel[vcur] hold the state
    float4 *pos[2] = {nullptr, nullptr}, *vel[2] = {nullptr, nullptr}, *xs = nullptr, *vs = nullptr;
    float *rho = nullptr, *pres = nullptr;
    uint32_t *key = nullptr, *tmp = nullptr, *order = nullptr, *skey = nullptr;
    uint32_t *cnt = nullptr, *start = nullptr, *fill = nullptr, *partial = nullptr, *status = nullptr;
    uint32_t cellCap = 0;
    bool stepped = false;
    void freeAll() {
        for (void* p : {(void*)pos[0], (void*)pos[1], (void*)vel[0], (void*)vel[1], (void*)xs, (void*)vs, (void*)rho,
                        (void*)pres, (void*)key, (void*)tmp, (void*)order, (void*)skey, (void*)cnt, (void*)start,
                        (void*)fill, (void*)partial, (void*)status})
            cudaFree(p);
        pos[0] = pos[1] = vel[0] = vel[1] = xs = vs = nullptr;
        rho = pres = nullptr;
        key = tmp = order = skey = cnt = start = fill = partial = status = nullptr;
        cellCap = 0;
    }
    ~vfd_sph() {
        freeAll();
        if (stream) cudaStreamDestroy(stream);
    }
};

namespace {

// SPHSimulation::UpdateParticles and UpdateGrid (SPHSimulation.cpp:187-214) in the
// reference's types: PI is a double literal and pow(float, int) promotes to double, so
// the kernel constants are computed in double and rounded once; pow(float, float) stays FP32.
int derive(const vfd_sph_desc& d, uint32_t n, vfd_sph_params& out, SphDev& P) {
    const double PI = 3.14159265358979323846;
    if (!(d.ParticleRadius > 0.0f) || !(d.Homogeneity > 0.0f) || !(d.TimeStep > 0.0f) || !(d.RestDensity > 0.0f))
        return fail(VFD_E_ARG, "radius, homogeneity, time step and rest density must be positive");
    if (d.MaxParticlesInCellCount == 0) return fail(VFD_E_ARG, "MaxParticlesInCellCount must be positive");
    const float h = d.Homogeneity, r = d.ParticleRadius;
    std::memset(&out, 0, sizeof(out));
    out.MinDist = r;
    out.SmoothingRadius = h * h;
    out.Poly6Kern = (float)(315.0f / (64.0f * PI * std::pow((double)h, 9)));
    out.SpikyKern = (float)((-0.5f * -45.0f) / (PI * std::pow((double)h, 6)));
    out.LapKern = (float)(45.0f / (PI * std::pow((double)h, 6)));
    out.MinDens = 1.0f / std::pow(d.RestDensity, 2.0f);
    out.ParticleMass = (float)(d.RestDensity * 4.0f / 3.0f * PI * std::pow(r, 3.0f));
    out.BoundsSoftDistance = 8 * r;
    out.BoundsHardDistance = 4 * r;
    out.CellSize = r * 2.0f;
    uint64_t cells = 1;
    for (int k = 0; k < 3; k++) {
        const float size = d.WorldMax[k] - d.WorldMin[k];
        if (!(size > 0.0f)) return fail(VFD_E_ARG, "empty world box");
        const float g = std::ceil(size / out.CellSize);
        if (!(g >= 1.0f) || g > 65535.0f) return fail(VFD_E_ARG, "grid too large");
        out.GridSize[k] = (uint32_t)g;
        cells *= out.GridSize[k];
    }
    if (cells > 0x7fffffffull) return fail(VFD_E_ARG, "grid too large (%llu cells)", (unsigned long long)cells);
    out.CellCount = (uint32_t)cells;
    out.ParticleCount = n;
    P = SphDev{};
    P.dt = d.TimeStep;
    P.damping = d.GlobalDamping;
    P.h = h;
    P.h2 = out.SmoothingRadius;
    P.spiky = out.SpikyKern;
    P.lap = out.LapKern;
    P.poly6 = out.Poly6Kern;
    P.mass = out.ParticleMass;
    P.rho0 = d.RestDensity;
    P.stiffness = d.Stiffness;
    P.visc = d.Viscosity;
    P.minDens = out.MinDens;
    P.minDist = out.MinDist;
    P.hardDist = out.BoundsHardDistance;
    P.softDist = out.BoundsSoftDistance;
    P.boundsDamp = d.BoundsDamping;
    P.boundsStiff = d.BoundsStiffness;
    P.boundsDampCrit = d.BoundsDampingCritical;
    for (int k = 0; k < 3; k++) {
        P.g[k] = d.Gravity[k];
        P.wmin[k] = d.WorldMin[k];
        P.wmax[k] = d.WorldMax[k];
    }
    P.cell = out.CellSize;
    P.gx = out.GridSize[0];
    P.gy = out.GridSize[1];
    P.gz = out.GridSize[2];
    P.gyx = out.GridSize[1] * out.GridSize[0];
    P.cells = out.CellCount;
    P.maxPerCell = d.MaxParticlesInCellCount;
    P.n = n;
    return VFD_OK;
}

#define SCK(call)                                                                                           \
    do {                                                                                                    \
        cudaError_t e_ = (call);                                                                            \
        if (e_ != cudaSuccess) return fail(VFD_E_CUDA, "%s: %s", #call, cudaGetErrorString(e_));              \
    } while (0)

int alloc_cells(vfd_sph* s) {
    const uint32_t cells = s->params.CellCount;
    if (cells <= s->cellCap) return VFD_OK;
    cudaFree(s->cnt);
    cudaFree(s->start);
    cudaFree(s->fill);
    cudaFree(s->partial);
    s->cnt = s->start = s->fill = s->partial = nullptr;
    SCK(cudaMalloc(&s->cnt, sizeof(uint32_t) * cells));
    SCK(cudaMalloc(&s->start, sizeof(uint32_t) * cells));
    SCK(cudaMalloc(&s->fill, sizeof(uint32_t) * cells));
    SCK(cudaMalloc(&s->partial, sizeof(uint32_t) * ((cells + kScanChunk - 1) / kScanChunk)));
    s->cellCap = cells;
    return VFD_OK;
}

int upload(vfd_sph* s) {
    const uint32_t n = std::max<uint32_t>(1u, s->n);
    if (!s->pos[0]) {
        for (int k = 0; k < 2; k++) {
            SCK(cudaMalloc(&s->pos[k], sizeof(float4) * n));
            SCK(cudaMalloc(&s->vel[k], sizeof(float4) * n));
        }
        SCK(cudaMalloc(&s->xs, sizeof(float4) * n));
        SCK(cudaMalloc(&s->vs, sizeof(float4) * n));
        SCK(cudaMalloc(&s->rho, sizeof(float) * n));
        SCK(cudaMalloc(&s->pres, sizeof(float) * n));
        SCK(cudaMalloc(&s->key, sizeof(uint32_t) * n));
        SCK(cudaMalloc(&s->tmp, sizeof(uint32_t) * n));
        SCK(cudaMalloc(&s->order, sizeof(uint32_t) * n));
        SCK(cudaMalloc(&s->skey, sizeof(uint32_t) * n));
        SCK(cudaMalloc(&s->status, sizeof(uint32_t)));
    }
    TRY(alloc_cells(s));
    s->cur = s->vcur = 0;
    if (s->n) {
        SCK(cudaMemcpy(s->pos[0], s->x0.data(), sizeof(float4) * s->n, cudaMemcpyHostToDevice));
        SCK(cudaMemset(s->vel[0], 0, sizeof(float4) * s->n));
        SCK(cudaMemset(s->rho, 0, sizeof(float) * s->n));
        SCK(cudaMemset(s->pres, 0, sizeof(float) * s->n));
    }
    SCK(cudaMemset(s->status, 0, sizeof(uint32_t)));
    s->stepped = false;
    return VFD_OK;
}

int step(vfd_sph* s) {
    const SphDev& P = s->P;
    const uint32_t n = s->n;
    if (n == 0) return VFD_OK;
    cudaStream_t st = s->stream;
    // the reference's buffer pairs: integrate reads one velocity buffer and writes the
    // other, the force kernel writes the first one back (SPHSimulation.cpp:80-93)
    const int a = s->cur, b = 1 - s->cur, va = s->vcur, vb = 1 - s->vcur;
    k_sph_integrate<<<blocks(n), 256, 0, st>>>(P, s->pos[a], s->vel[va], s->pos[b], s->vel[vb]);
    const uint32_t cells = P.cells, nb = (cells + kScanChunk - 1) / kScanChunk;
    SCK(cudaMemsetAsync(s->cnt, 0, sizeof(uint32_t) * cells, st));
    SCK(cudaMemsetAsync(s->fill, 0, sizeof(uint32_t) * cells, st));
    k_sph_keys<<<blocks(n), 256, 0, st>>>(P, s->pos[b], s->key, s->cnt, s->status);
    k_sph_scan_reduce<<<nb, 256, 0, st>>>(s->cnt, cells, s->partial);
    k_sph_scan_top<<<1, 1024, 0, st>>>(s->partial, nb);
    k_sph_scan_down<<<nb, 256, 0, st>>>(s->cnt, cells, s->partial, s->start);
    k_sph_slots<<<blocks(n), 256, 0, st>>>(P, s->key, s->start, s->fill, s->tmp);
    k_sph_reorder<<<blocks(n), 256, 0, st>>>(P, s->key, s->start, s->cnt, s->tmp, s->pos[b], s->vel[vb], s->order,
                                             s->skey, s->xs, s->vs);
    k_sph_density<<<blocks(n, 128), 128, 0, st>>>(P, s->start, s->cnt, s->xs, s->rho, s->pres);
    k_sph_force<<<blocks(n, 128), 128, 0, st>>>(P, s->start, s->cnt, s->xs, s->vs, s->rho, s->pres, s->order,
                                                s->vel[va]);
    SCK(cudaGetLastError());
    s->cur = b;  // the velocities stay in vel[va]
    s->stepped = true;
    return VFD_OK;
}

int check(vfd_sph* s) {
    SCK(cudaStreamSynchronize(s->stream));
    uint32_t st = 0;
    SCK(cudaMemcpy(&st, s->status, sizeof(st), cudaMemcpyDeviceToHost));
    if (st) return fail(VFD_E_NAN, "legacy SPH: a particle left the grid (non-finite state)");
    return VFD_OK;
}

}  // namespace

extern "C" {

int vfd_sph_create(const vfd_sph_desc* desc, const float* xyz, uint32_t n, vfd_sph** out) {
    if (!desc || !out || (n && !xyz)) return fail(VFD_E_ARG, "null argument");
    *out = nullptr;
    for (size_t i = 0; i < 3 * (size_t)n; i++)
        if (!std::isfinite(xyz[i])) return fail(VFD_E_NAN, "non-finite position");
    int devCount = 0;
    if (cudaGetDeviceCount(&devCount) != cudaSuccess || devCount == 0) return fail(VFD_E_NODEVICE, "no CUDA device");
    vfd_sph* s = new vfd_sph();
    s->desc = *desc;
    s->n = n;
    int rc = derive(*desc, n, s->params, s->P);
    if (rc != VFD_OK) {
        delete s;
        return rc;
    }
    s->x0.resize(n);
    for (uint32_t i = 0; i < n; i++) s->x0[i] = make_float4(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], 0.0f);
    cudaGetDevice(&s->device);
    if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete s;
        return fail(VFD_E_CUDA, "stream creation failed");
    }
    rc = upload(s);
    if (rc != VFD_OK) {
        delete s;
        return rc;
    }
    *out = s;
    return VFD_OK;
}

void vfd_sph_destroy(vfd_sph* s) {
    if (!s) return;
    cudaSetDevice(s->device);
    delete s;
}

int vfd_sph_steps(vfd_sph* s, uint32_t count) {
    if (!s) return fail(VFD_E_ARG, "null handle");
    SCK(cudaSetDevice(s->device));
    for (uint32_t k = 0; k < count; k++) TRY(step(s));
    return check(s);
}

int vfd_sph_on_update(vfd_sph* s) {
    if (!s) return fail(VFD_E_ARG, "null handle");
    return vfd_sph_steps(s, s->desc.StepCount);
}

int vfd_sph_reset(vfd_sph* s) {
    if (!s) return fail(VFD_E_ARG, "null handle");
    SCK(cudaSetDevice(s->device));
    SCK(cudaStreamSynchronize(s->stream));
    return upload(s);
}

int vfd_sph_update_description(vfd_sph* s, const vfd_sph_desc* desc) {
    if (!s || !desc) return fail(VFD_E_ARG, "null argument");
    vfd_sph_params params;
    SphDev P;
    TRY(derive(*desc, s->n, params, P));
    SCK(cudaSetDevice(s->device));
    SCK(cudaStreamSynchronize(s->stream));
    s->desc = *desc;
    s->params = params;
    s->P = P;
    return alloc_cells(s);
}

int vfd_sph_get_params(const vfd_sph* s, vfd_sph_params* out) {
    if (!s || !out) return fail(VFD_E_ARG, "null argument");
    *out = s->params;
    return VFD_OK;
}

int vfd_sph_get_state(vfd_sph* s, float* xyz, float* vel, float* density, float* pressure) {
    if (!s) return fail(VFD_E_ARG, "null handle");
    SCK(cudaSetDevice(s->device));
    SCK(cudaStreamSynchronize(s->stream));
    const uint32_t n = s->n;
    if (n == 0) return VFD_OK;
    std::vector<float4> buf(n);
    auto unpack = [&](const float4* d, float* o) -> int {
        SCK(cudaMemcpy(buf.data(), d, sizeof(float4) * n, cudaMemcpyDeviceToHost));
        for (uint32_t i = 0; i < n; i++) {
            o[3 * i] = buf[i].x;
            o[3 * i + 1] = buf[i].y;
            o[3 * i + 2] = buf[i].z;
        }
        return VFD_OK;
    };
    if (xyz) TRY(unpack(s->pos[s->cur], xyz));
    if (vel) TRY(unpack(s->vel[s->vcur], vel));
    if (density || pressure) {
        std::vector<uint32_t> order(n);
        std::vector<float> v(n);
        SCK(cudaMemcpy(order.data(), s->order, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost));
        for (int f = 0; f < 2; f++) {
            float* o = f == 0 ? density : pressure;
            if (!o) continue;
            if (!s->stepped) {
                std::fill(o, o + n, 0.0f);
                continue;
            }
            SCK(cudaMemcpy(v.data(), f == 0 ? s->rho : s->pres, sizeof(float) * n, cudaMemcpyDeviceToHost));
            for (uint32_t q = 0; q < n; q++) o[order[q]] = v[q];
        }
    }
    return VFD_OK;
}

int vfd_sph_set_velocities(vfd_sph* s, const float* vel) {
    if (!s || (!vel && s->n)) return fail(VFD_E_ARG, "null argument");
    SCK(cudaSetDevice(s->device));
    SCK(cudaStreamSynchronize(s->stream));
    std::vector<float4> buf(s->n);
    for (uint32_t i = 0; i < s->n; i++) buf[i] = make_float4(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2], 0.0f);
    if (s->n) SCK(cudaMemcpy(s->vel[s->vcur], buf.data(), sizeof(float4) * s->n, cudaMemcpyHostToDevice));
    return VFD_OK;
}

int vfd_sph_get_sort(vfd_sph* s, uint32_t* keys, uint32_t* indices) {
    if (!s) return fail(VFD_E_ARG, "null handle");
    if (!s->stepped) return fail(VFD_E_STATE, "no step has run");
    SCK(cudaSetDevice(s->device));
    SCK(cudaStreamSynchronize(s->stream));
    if (keys) SCK(cudaMemcpy(keys, s->skey, sizeof(uint32_t) * s->n, cudaMemcpyDeviceToHost));
    if (indices) SCK(cudaMemcpy(indices, s->order, sizeof(uint32_t) * s->n, cudaMemcpyDeviceToHost));
    return VFD_OK;
}

}  // extern "C"
