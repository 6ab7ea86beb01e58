// C-ABI of the GB300 DFSPH step (include/vfd_dfsph.h): the host side of
// DFSPHSimulation / DFSPHImplementation (Simulation/DFSPH/DFSPHSimulator.cpp,
// DFSPHImplementation.cu). Owns all device memory, uploads scenes, records the
// step either as one CUDA graph (conditional while nodes for the divergence,
// viscosity and pressure loops) or as eagerly launched kernels with one flag
// read per solver iteration, and converts results back to the caller's
// particle order.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstdarg>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <memory>
#include <new>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "../../include/vfd_dfsph.h"
#include "dfsph_common.cuh"

#include "dfsph_sim.h"

namespace vfd {
LaunchProfiler* g_profiler = nullptr;

// Original-order export of a per-slot float4 field (x, y, z) of slots [begin, begin + count).
__global__ void k_export3(const uint32_t* pid, const float4* src, float* out, uint32_t begin, uint32_t count) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    const uint32_t p = begin + k;
    const uint32_t o = pid[p];
    if (o >= count) return;
    const float4 v = src[p];
    out[3 * (size_t)o] = v.x;
    out[3 * (size_t)o + 1] = v.y;
    out[3 * (size_t)o + 2] = v.z;
}
// Original-order export of a scalar field (float, or component `comp` of a float4 field).
__global__ void k_export1(const uint32_t* pid, const float* src, const float4* src4, int comp, float* out,
                          uint32_t begin, uint32_t count) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    const uint32_t p = begin + k;
    const uint32_t o = pid[p];
    if (o >= count) return;
    out[o] = src4 ? (&src4[p].x)[comp] : src[p];
}
// Sets *bad when any of the n values is not finite (inputs checked on the device after
// their copy, before they are imported).
__global__ void k_check_finite(const float* a, size_t n, uint32_t* bad) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        if (!isfinite(a[i])) {
            *bad = 1u;
            return;
        }
}
// Original-order import into a float4 field (w kept).
__global__ void k_import3(const uint32_t* pid, const float* in, float4* dst, uint32_t begin, uint32_t count) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    const uint32_t p = begin + k;
    const uint32_t o = pid[p];
    if (o >= count) return;
    const float4 w = dst[p];
    dst[p] = make_float4(in[3 * (size_t)o], in[3 * (size_t)o + 1], in[3 * (size_t)o + 2], w.w);
}
// Positions out of / into the cell-relative form (Dev::cellRel): absolute FP32
// coordinates of slots [begin, begin + count) in original order; `anchors` holds each
// slot's anchor cell in .w (the positions themselves, or the state set whose frame the
// values of `src` are in).
__global__ void k_export_pos(Dev d, const float4* src, const float4* anchors, float* out, uint32_t begin,
                             uint32_t count) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    const uint32_t p = begin + k;
    const uint32_t o = d.PIDc[p];
    if (o >= count) return;
    const float4 v = src[p];
    const float3 x = abs_pos(d, d.scenes[scene_of(d, p)], make_float4(v.x, v.y, v.z, anchors[p].w));
    out[3 * (size_t)o] = x.x;
    out[3 * (size_t)o + 1] = x.y;
    out[3 * (size_t)o + 2] = x.z;
}
__global__ void k_import_pos(Dev d, const float* in, float4* dst, uint32_t begin, uint32_t count) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    const uint32_t p = begin + k;
    const uint32_t o = d.PIDc[p];
    if (o >= count) return;
    const SceneDev& S = d.scenes[scene_of(d, p)];
    const float L = d.radius;
    float3 x = make_float3(in[3 * (size_t)o] - S.org[0], in[3 * (size_t)o + 1] - S.org[1], in[3 * (size_t)o + 2] - S.org[2]);
    const float fx = floorf(x.x / L), fy = floorf(x.y / L), fz = floorf(x.z / L);
    const int3 A = make_int3((int)fx, (int)fy, (int)fz);
    dst[p] = make_float4(x.x - fx * L, x.y - fy * L, x.z - fz * L, anchor_pack(A));
}

// Frame output of vfd_simulate. When a step completes a frame (k_ctrl_end sets frameDue;
// DFSPHImplementation.cu:148-167 copies the frame there), x, v and a of the particles go
// to slot (frame - 1) % slots of a device ring, in the original particle order
// (ConvertParticlesToBuffer); the host copies the slot out asynchronously.
__global__ void k_frame_snapshot(Dev d, float* ring, uint32_t slots, uint32_t count) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= count || is_aborted(d)) return;
    const SceneDev& S = d.scenes[0];
    if (!S.frameDue) return;
    const uint32_t o = d.PIDc[p];
    if (o >= count) return;
    float* slot = ring + (size_t)((S.frameIndex - 1u) % slots) * 9u * count;
    const float4 x4 = d.XN[p];
    const float3 x = d.cellRel ? abs_pos(d, S, x4) : make_float3(x4.x, x4.y, x4.z);
    const float4 v = d.Vc[p], a = d.A[p];
    float* xs = slot + 3 * (size_t)o;
    float* vs = slot + 3 * ((size_t)count + o);
    float* as = slot + 3 * (2 * (size_t)count + o);
    xs[0] = x.x, xs[1] = x.y, xs[2] = x.z;
    vs[0] = v.x, vs[1] = v.y, vs[2] = v.z;
    as[0] = a.x, as[1] = a.y, as[2] = a.z;
}

struct FrameNote {
    uint32_t due, index, aborted, flags;
    float maxV, dt;
    uint32_t pad[2];
};

// What the host needs of a step without waiting for the ones after it: whether it made
// a frame, and the abort and error words. After the last frame the later steps already
// in the queue are turned into no-ops (abort word 2), so that the run ends on the step
// that completed the last frame, as the reference's frame loop does
// (DFSPHImplementation.cu:52-55).
__global__ void k_frame_note(Dev d, FrameNote* note, uint32_t lastFrame) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const SceneDev& S = d.scenes[0];
    FrameNote n;
    n.aborted = d.status[1];
    n.due = (n.aborted == 0u && S.frameDue) ? 1u : 0u;
    n.index = S.frameIndex;
    n.flags = d.status[0];
    n.maxV = S.maxV2;
    n.dt = S.dt;
    n.pad[0] = n.pad[1] = 0u;
    *note = n;
    if (n.due && S.frameIndex >= lastFrame) d.status[1] = 2u;
}

// Appends particles [n0, n0 + count) to the current state set (vfd_emit): positions
// converted to the storage mode (cell-relative: anchor cell of edge h around the scene
// origin, as upload does), zero warm starts, original indices n0 + k. The next step's
// search sorts them in with the others.
__global__ void k_emit(Dev d, const float* xyz, const float* vel, uint32_t n0, uint32_t count, uint32_t* status) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    const uint32_t p = n0 + k;
    const SceneDev& S = d.scenes[0];
    float3 x = make_float3(xyz[3 * (size_t)k], xyz[3 * (size_t)k + 1], xyz[3 * (size_t)k + 2]);
    float w = 0.0f;
    if (d.cellRel) {
        const float L = d.radius;
        x = make_float3(x.x - S.org[0], x.y - S.org[1], x.z - S.org[2]);
        const float fx = floorf(x.x / L), fy = floorf(x.y / L), fz = floorf(x.z / L);
        const int3 A = make_int3((int)fx, (int)fy, (int)fz);
        if (abs(A.x) > 511 || abs(A.y) > 511 || abs(A.z) > 511) atomicOr(status, 0x40u);
        x = make_float3(x.x - fx * L, x.y - fy * L, x.z - fz * L);
        w = anchor_pack(A);
    }
    d.XN[p] = make_float4(x.x, x.y, x.z, w);
    d.Vc[p] = vel ? make_float4(vel[3 * (size_t)k], vel[3 * (size_t)k + 1], vel[3 * (size_t)k + 2], 0.0f)
                  : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    d.DVc[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    d.DKc[p] = 0.0f;
    d.PIDc[p] = p;
    d.A[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (k == 0) d.scenes[0].count = n0 + count;
}
}  // namespace vfd

using namespace vfd;

namespace vfd {
namespace host {

thread_local std::string g_lastError;
int g_device = 0;

int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_lastError = buf;
    return code;
}


// Surface-tension directions (HaltonVec323.cuh:4): the Halton(2,3) points on the unit
// sphere, each component rounded to the 15 decimals the reference lists.
void halton_table(std::vector<float>& out) {
    out.assign(kHaltonCount, 0.0f);
    auto radical = [](uint32_t i, uint32_t b) {
        double inv = 1.0 / b, f = inv, r = 0.0;
        while (i > 0) { r += f * (double)(i % b); i /= b; f *= inv; }
        return r;
    };
    for (uint32_t i = 0; i < kHaltonCount / 3; i++) {
        const double z = 1.0 - 2.0 * radical(i, 3);
        const double phi = 2.0 * 3.14159265358979323846 * radical(i, 2);
        const double s = std::sqrt(std::max(0.0, 1.0 - z * z));
        const double v[3] = {s * std::cos(phi), s * std::sin(phi), z};
        for (int k = 0; k < 3; k++) out[3 * i + k] = (float)(std::nearbyint(v[k] * 1e15) / 1e15 + 0.0);  // +0.0: no negative zeros
    }
}

}  // namespace host
}  // namespace vfd

namespace vfd {
namespace host {

int check_desc(const vfd_desc* d) {
    if (!d) return fail(VFD_E_ARG, "null description");
    if (!(d->ParticleRadius > 0.0f) || !std::isfinite(d->ParticleRadius))
        return fail(VFD_E_ARG, "ParticleRadius must be positive and finite");
    if (!(d->MinTimeStepSize > 0.0f) || !(d->MaxTimeStepSize >= d->MinTimeStepSize) || !(d->TimeStepSize > 0.0f))
        return fail(VFD_E_ARG, "time step bounds must satisfy 0 < Min <= Max and TimeStepSize > 0");
    return VFD_OK;
}

// Estimated cell table size: the reference's grid for the initial bounds with 50 % headroom.
uint32_t estimate_cells(const vfd_sim* s) {
    uint64_t total = 0;
    for (const auto& sc : s->scenes) {
        const uint32_t n = (uint32_t)(sc.x0.size() / 3);
        if (n == 0) continue;
        const float R = 4.0f * sc.desc.ParticleRadius;
        uint64_t cells = 512;
        for (int k = 0; k < 3; k++) {
            float lo = FLT_MAX, hi = -FLT_MAX;
            for (uint32_t i = 0; i < n; i++) {
                lo = std::min(lo, sc.x0[3 * i + k]);
                hi = std::max(hi, sc.x0[3 * i + k]);
            }
            // the box may let the fluid spread; take the bodies' domains too
            for (const auto& b : sc.bodies) {
                lo = std::min(lo, b.dev.dmin[k]);
                hi = std::max(hi, b.dev.dmax[k]);
            }
            const uint64_t dim = (uint64_t)std::ceil((hi - lo) / R) + 6u;
            cells *= (dim + 7u) / 8u;
        }
        total += cells;
    }
    total = total + total / 2 + 4096;
    return (uint32_t)std::min<uint64_t>(total, 0xF0000000ull);
}

// Reduction buckets to their identities (sums 0, max 0, min cell INT_MAX, max cell INT_MIN).
int reset_buckets(vfd_sim* s, const Dev& d) {
    const size_t ns = d.nscenes;
    CK(cudaMemset(d.ACCB, 0, sizeof(double) * ns * kAccSlots * kBuckets * 16u));
    CK(cudaMemset(d.MAXB, 0, sizeof(uint32_t) * ns * 2u * kBuckets * 32u));
    std::vector<int32_t> mm(ns * 6u * kBuckets * 32u);
    for (size_t sc = 0; sc < ns; sc++)
        for (uint32_t k = 0; k < 6; k++)
            for (uint32_t b = 0; b < kBuckets * 32u; b++)
                mm[(sc * 6u + k) * kBuckets * 32u + b] = k < 3 ? INT_MAX : INT_MIN;
    CK(cudaMemcpy(d.MMB, mm.data(), sizeof(int32_t) * mm.size(), cudaMemcpyHostToDevice));
    return VFD_OK;
}

int allocate(vfd_sim* s) {
    s->releaseBuffers();
    uint32_t n = 0, maxBodies = 0;
    s->sceneBegin.clear();
    for (const auto& sc : s->scenes) {
        s->sceneBegin.push_back(n);
        n += sc.count();
        maxBodies = std::max<uint32_t>(maxBodies, (uint32_t)sc.bodies.size());
    }
    s->n = n;
    s->stride = std::max<uint32_t>(32u, (std::max(n, s->reserve) + 31u) & ~31u);
    s->maxBodies = maxBodies;
    if (s->cellCap == 0) s->cellCap = estimate_cells(s);
    const size_t st = s->stride;
    Dev base{};
    base.n = n;
    base.stride = s->stride;
    base.nscenes = (uint32_t)s->scenes.size();
    base.maxBodies = maxBodies;
    base.cellCap = s->cellCap;
    base.scanBlocks = scan_block_count(s->cellCap);
    std::memcpy(base.lanes, s->lanes, sizeof(base.lanes));
    float4* X[2];
    float4* V[2];
    float4* DV[2];
    float* DK[2];
    uint32_t* PID[2];
    for (int k = 0; k < 2; k++) {
        TRY(dalloc(s, &X[k], st));
        TRY(dalloc(s, &V[k], st));
        TRY(dalloc(s, &DV[k], st));
        TRY(dalloc(s, &DK[k], st));
        TRY(dalloc(s, &PID[k], st));
    }
    TRY(dalloc(s, &base.XN, st));
    TRY(dalloc(s, &base.A, st));
    TRY(dalloc(s, &base.AP, st));
    TRY(dalloc(s, &base.GB, st));
    TRY(dalloc(s, &base.RHO, st));
    TRY(dalloc(s, &base.ALPHA, st));
    TRY(dalloc(s, &base.RHOADV, st));
    TRY(dalloc(s, &base.KAPPA, st));
    TRY(dalloc(s, &base.KAPPAV, st));
    TRY(dalloc(s, &base.RES, st));
    TRY(dalloc(s, &base.XB, st * std::max<uint32_t>(1u, maxBodies)));
    TRY(dalloc(s, &base.NBR, st * kRow));
    TRY(dalloc(s, &base.NG, st * kRow));
    TRY(dalloc(s, &base.NBRC, st * kRow));
    TRY(dalloc(s, &base.NCNT, st));
    TRY(dalloc(s, &base.KEY, st));
    TRY(dalloc(s, &base.KEYS, st));
    TRY(dalloc(s, &base.TMP, st));
    TRY(dalloc(s, &base.CELL_START, s->cellCap));
    TRY(dalloc(s, &base.CELL_COUNT, s->cellCap));
    TRY(dalloc(s, &base.FILL, s->cellCap));
    TRY(dalloc(s, &base.SCAN, base.scanBlocks + 1));
    TRY(dalloc(s, &base.MINV, 3 * st));
    TRY(dalloc(s, &base.BVM, 3 * st));
    TRY(dalloc(s, &base.CB, st));
    TRY(dalloc(s, &base.CG, st));
    TRY(dalloc(s, &base.CR, st));
    TRY(dalloc(s, &base.CP, st));
    TRY(dalloc(s, &base.CZ, st));
    TRY(dalloc(s, &base.CAP, st));
    TRY(dalloc(s, &base.STN, st));
    TRY(dalloc(s, &base.STNS, st));
    TRY(dalloc(s, &base.SID, st));
    TRY(dalloc(s, &s->dScenes, base.nscenes));
    uint32_t bodyTotal = 0;
    for (const auto& sc : s->scenes) bodyTotal += (uint32_t)sc.bodies.size();
    TRY(dalloc(s, &s->dBodies, std::max<uint32_t>(1u, bodyTotal)));
    TRY(dalloc(s, &s->dStatus, 16));
    TRY(dalloc(s, &s->dStage, 3 * st));
    TRY(dalloc(s, &s->dStage2, 3 * st));
    TRY(dalloc(s, &base.ACCB, (size_t)base.nscenes * kAccSlots * kBuckets * 16u));
    TRY(dalloc(s, &base.MAXB, (size_t)base.nscenes * 2u * kBuckets * 32u));
    TRY(dalloc(s, &base.MMB, (size_t)base.nscenes * 6u * kBuckets * 32u));
    base.cellRel = s->cellRel ? 1u : 0u;
    base.analytic = s->analyticKernel ? 1u : 0u;
    base.splK = s->table.K;
    base.splL = s->table.L;
    base.workStride = 2u + 2u * base.nscenes;
    TRY(dalloc(s, &base.WORK, 3 * (size_t)base.workStride));
    {
        int sms = 0;
        CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, s->device));
        base.batchBlocks = (uint32_t)std::max(1, sms) * (2048u / kBlock);
    }
    std::memcpy(base.tiles, s->tiles, sizeof(base.tiles));
    std::memcpy(base.blocks, s->blocks, sizeof(base.blocks));
    base.compactRows = uses_tiles(s->tiles) ? 1u : 0u;
    CK(prepare_tile_kernels());
    TRY(dalloc(s, &s->dWM, kTableRes));
    TRY(dalloc(s, &s->dGM, kTableRes));
    TRY(dalloc(s, &s->dHalton, kHaltonCount));
    CK(cudaMallocHost(&s->hStatus, 16 * sizeof(uint32_t)));
    base.scenes = s->dScenes;
    base.bodies = s->dBodies;
    base.status = s->dStatus;
    base.WM = s->dWM;
    base.GM = s->dGM;
    base.halton = s->dHalton;
    base.wZero = s->table.wZero;
    base.invStep = s->table.invStep;
    base.radius = s->table.radius;
    base.radius2 = s->table.radius2;
    for (int k = 0; k < 2; k++) {
        Dev d = base;
        d.Xc = X[k]; d.Vc = V[k]; d.DVc = DV[k]; d.DKc = DK[k]; d.PIDc = PID[k];
        d.X = X[1 - k]; d.V = V[1 - k]; d.DV = DV[1 - k]; d.DK = DK[1 - k]; d.PID = PID[1 - k];
        s->dev[k] = d;
    }
    // static uploads: tables, scene ids, bodies
    std::vector<float> wm(kTableRes), gm(kTableRes);
    for (uint32_t i = 0; i + 1 < kTableRes; i++) {
        wm[i] = 0.5f * (s->table.W[i] + s->table.W[i + 1]);
        gm[i] = 0.5f * (s->table.G[i] + s->table.G[i + 1]);
    }
    wm[kTableRes - 1] = gm[kTableRes - 1] = 0.0f;
    CK(cudaMemcpy(s->dWM, wm.data(), sizeof(float) * kTableRes, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(s->dGM, gm.data(), sizeof(float) * kTableRes, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(s->dHalton, s->halton.data(), sizeof(float) * kHaltonCount, cudaMemcpyHostToDevice));
    std::vector<uint16_t> sid(st, 0);
    std::vector<BodyDev> bodies;
    for (uint32_t k = 0; k < s->scenes.size(); k++) {
        const uint32_t cnt = s->scenes[k].count();
        for (uint32_t i = 0; i < cnt; i++) sid[s->sceneBegin[k] + i] = (uint16_t)k;
        for (const auto& b : s->scenes[k].bodies) bodies.push_back(b.dev);
    }
    CK(cudaMemcpy(base.SID, sid.data(), sizeof(uint16_t) * st, cudaMemcpyHostToDevice));
    if (!bodies.empty())
        CK(cudaMemcpy(s->dBodies, bodies.data(), sizeof(BodyDev) * bodies.size(), cudaMemcpyHostToDevice));
    CK(cudaMemset(base.NCNT, 0, sizeof(uint32_t) * st));
    CK(cudaMemset(base.NBR, 0, sizeof(uint32_t) * st * kRow));
    CK(cudaMemset(base.NG, 0, sizeof(uint2) * st * kRow));
    CK(cudaMemset(base.NBRC, 0, sizeof(uint16_t) * st * kRow));
    CK(cudaMemset(base.A, 0, sizeof(float4) * st));
    CK(cudaMemset(base.AP, 0, sizeof(float4) * st));
    CK(cudaMemset(base.STN, 0, sizeof(float4) * st));
    CK(cudaMemset(base.STNS, 0, sizeof(float4) * st));
    CK(cudaMemset(base.XB, 0, sizeof(float4) * st * std::max<uint32_t>(1u, maxBodies)));
    TRY(reset_buckets(s, base));
    s->allocated = true;
    return VFD_OK;
}

SceneDev scene_constants(const vfd_desc& d, uint32_t begin, uint32_t count, uint32_t bodyBegin, uint32_t bodyCount) {
    SceneDev S;
    std::memset(&S, 0, sizeof(S));
    S.begin = begin;
    S.count = count;
    S.bodyBegin = bodyBegin;
    S.bodyCount = bodyCount;
    // DFSPHImplementation::SetDescription (DFSPHImplementation.cu:318-368)
    S.r = d.ParticleRadius;
    S.diam = 2.0f * S.r;
    S.h = 4.0f * S.r;
    S.h2 = S.h * S.h;
    S.volume = 0.8f * S.diam * S.diam * S.diam;
    S.rho0 = 1000.0f;
    S.mass = S.volume * S.rho0;
    S.massInv = 1.0f / S.mass;
    S.dynVisc = d.Viscosity * S.rho0;
    S.dynBVisc = d.BoundaryViscosity * S.rho0;
    S.tangDist = d.TangentialDistanceFactor * S.h;
    S.st = d.SurfaceTension;
    S.slope = 74.688796680497925f;
    S.constant = 12.0f;
    S.smoothing = 0.5f;
    S.nbrRadius = S.r * 0.8f;
    S.mcFactor = std::asin(S.nbrRadius / S.r);
    S.temporal = d.TemporalSmoothing ? 1 : 0;
    for (int k = 0; k < 3; k++) S.g[k] = d.Gravity[k];
    S.minIterP = d.MinPressureSolverIterations;
    S.maxIterP = d.MaxPressureSolverIterations;
    S.minIterD = d.MinDivergenceSolverIterations;
    S.maxIterD = d.MaxDivergenceSolverIterations;
    S.minIterV = d.MinViscositySolverIterations;
    S.maxIterV = d.MaxViscositySolverIterations;
    S.maxErrP = d.MaxPressureSolverError;
    S.maxErrD = d.MaxDivergenceSolverError;
    S.maxErrV = d.MaxViscositySolverError;
    S.enableDiv = d.EnableDivergenceSolverError ? 1 : 0;
    S.enableVisc = d.EnableViscositySolver ? 1 : 0;
    S.enableST = d.EnableSurfaceTensionSolver ? 1 : 0;
    S.stPasses = d.SurfaceTensionSmoothPassCount;
    S.csdFix = d.CSDFix;
    S.csd = d.CSD;
    S.minDt = d.MinTimeStepSize;
    S.maxDt = d.MaxTimeStepSize;
    // Simulate() preamble (:39-43): dt = TimeStepSize
    S.dt = d.TimeStepSize;
    S.dt2 = d.TimeStepSize * d.TimeStepSize;
    S.dtInv = 1.0f / S.dt;
    S.dt2Inv = 1.0f / S.dt2;
    // ComputeTimeStepSize sets the sample count after the first surface-tension pass
    // (:413-420); the first step uses the one of the initial dt.
    S.stSamples = d.CSDFix > 0 ? (uint32_t)d.CSDFix : (uint32_t)(int)((float)d.CSD * S.dt);
    S.stSamplesUsed = S.stSamples;
    S.frameLength = d.FrameLength;
    S.frameCount = d.FrameCount;
    for (int k = 0; k < 3; k++) {
        S.minCell[k] = INT_MAX;
        S.maxCell[k] = INT_MIN;
    }
    return S;
}

// Simulate() preamble (DFSPHImplementation.cu:33-51): initial particles to the device,
// dt and counters reset.
int upload(vfd_sim* s) {
    // the initial particles only: appended ones go, and the layout shrinks back with them
    uint32_t initial = 0, emitted = 0;
    for (auto& sc : s->scenes) {
        emitted += sc.emitted;
        sc.emitted = 0;
        initial += (uint32_t)(sc.x0.size() / 3);
    }
    if (!s->allocated || s->n != initial) TRY(allocate(s));
    const size_t st = s->stride;
    std::vector<float4> xn(st, make_float4(0, 0, 0, 0)), v(st, make_float4(0, 0, 0, 0));
    std::vector<uint32_t> pid(st, 0);
    s->hScenes.clear();
    uint32_t bodyBegin = 0;
    s->maxStPasses = 0;
    s->anyDiv = s->anyVisc = s->anyST = false;
    for (uint32_t k = 0; k < s->scenes.size(); k++) {
        const SceneHost& sc = s->scenes[k];
        const uint32_t b = s->sceneBegin[k], cnt = (uint32_t)(sc.x0.size() / 3);
        SceneDev S = scene_constants(sc.desc, b, cnt, bodyBegin, (uint32_t)sc.bodies.size());
        // cell-relative positions: anchor cells of edge h counted from the cell nearest the
        // centre of the initial positions
        double lo[3] = {DBL_MAX, DBL_MAX, DBL_MAX}, hi[3] = {-DBL_MAX, -DBL_MAX, -DBL_MAX};
        for (uint32_t i = 0; i < cnt; i++)
            for (int k = 0; k < 3; k++) {
                lo[k] = std::min(lo[k], (double)sc.x0[3 * i + k]);
                hi[k] = std::max(hi[k], (double)sc.x0[3 * i + k]);
            }
        const double L = (double)s->table.radius;
        for (int k = 0; k < 3; k++) S.org[k] = cnt ? (float)(L * std::nearbyint(0.5 * (lo[k] + hi[k]) / L)) : 0.0f;
        for (uint32_t i = 0; i < cnt; i++) {
            if (s->cellRel) {
                double o[3];
                int a[3];
                for (int k = 0; k < 3; k++) {
                    const double rel = (double)sc.x0[3 * i + k] - (double)S.org[k];
                    a[k] = (int)std::floor(rel / L);
                    o[k] = rel - a[k] * L;
                    if (std::abs(a[k]) > 511) return fail(VFD_E_CAPACITY, "cell-relative positions: a particle lies "
                                                          "more than 511 cells from its scene's centre");
                }
                const uint32_t w = (uint32_t)(a[0] & 1023) | ((uint32_t)(a[1] & 1023) << 10) |
                                   ((uint32_t)(a[2] & 1023) << 20);
                float wf;
                std::memcpy(&wf, &w, sizeof(wf));
                xn[b + i] = make_float4((float)o[0], (float)o[1], (float)o[2], wf);
            } else {
                xn[b + i] = make_float4(sc.x0[3 * i], sc.x0[3 * i + 1], sc.x0[3 * i + 2], 0.0f);
            }
            if (!sc.v0.empty()) v[b + i] = make_float4(sc.v0[3 * i], sc.v0[3 * i + 1], sc.v0[3 * i + 2], 0.0f);
            pid[b + i] = i;
        }
        s->hScenes.push_back(S);
        bodyBegin += (uint32_t)sc.bodies.size();
        if (sc.desc.EnableSurfaceTensionSolver) s->maxStPasses = std::max(s->maxStPasses, sc.desc.SurfaceTensionSmoothPassCount);
        s->anyDiv |= sc.desc.EnableDivergenceSolverError != 0;
        s->anyVisc |= sc.desc.EnableViscositySolver != 0;
        s->anyST |= sc.desc.EnableSurfaceTensionSolver != 0;
    }
    s->cs = 0;
    const Dev& d = s->dev[0];
    CK(cudaMemcpy(d.XN, xn.data(), sizeof(float4) * st, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(d.Vc, v.data(), sizeof(float4) * st, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(d.PIDc, pid.data(), sizeof(uint32_t) * st, cudaMemcpyHostToDevice));
    CK(cudaMemset(d.DVc, 0, sizeof(float4) * st));
    CK(cudaMemset(d.DKc, 0, sizeof(float) * st));
    CK(cudaMemset(d.A, 0, sizeof(float4) * st));
    CK(cudaMemcpy(s->dScenes, s->hScenes.data(), sizeof(SceneDev) * s->hScenes.size(), cudaMemcpyHostToDevice));
    CK(cudaMemset(s->dStatus, 0, 16 * sizeof(uint32_t)));
    TRY(reset_buckets(s, d));
    CK(cudaDeviceSynchronize());
    s->uploaded = true;
    s->generation++;
    if (s->fp64Mode) TRY(fp64_upload(s));
    return VFD_OK;
}

// ---------------------------------------------------------------- step recording
int build_graph(vfd_sim* s, int parity, const void* rec, cudaGraph_t* gOut, cudaGraphExec_t* execOut) {
    cudaGraph_t g;
    CK(cudaGraphCreate(&g, 0));
    // One conditional handle per while node the graph has (divergence, CG, pressure): a
    // handle that no node uses makes cudaGraphInstantiate fail with "invalid argument".
    Dev d = s->dev[parity];
    const bool used[3] = {s->anyDiv, s->anyVisc, true};
    cudaGraphConditionalHandle h[3] = {};
    for (int k = 0; k < 3; k++) {
        d.condHandle[k] = 0ull;
        if (!used[k]) continue;
        cudaError_t e = cudaGraphConditionalHandleCreate(&h[k], g, 0, 0);
        if (e != cudaSuccess) {
            cudaGraphDestroy(g);
            return fail(VFD_E_CUDA, "cudaGraphConditionalHandleCreate: %s", cudaGetErrorString(e));
        }
        d.condHandle[k] = (unsigned long long)h[k];
    }
    cudaStream_t cap = s->stream;
    std::vector<cudaGraphNode_t> leaves;
    const uint32_t passes = s->maxStPasses;
    const bool anyDiv = s->anyDiv, anyVisc = s->anyVisc, anyST = s->anyST;
    // with a recorder, tape_point() adds the adjoint's tape writes between the stages
    auto T = [&](int point, cudaStream_t st) {
        if (rec) tape_point(d, rec, point, st);
    };
    cudaError_t e = add_segment(cap, g, leaves, [&](cudaStream_t st) {
        T(kTapeBegin, st);
        launch_search(d, st);
        T(kTapeSearch, st);
        launch_boundary(d, st);
        T(kTapeBoundary, st);
        launch_density_div_init(d, st);
        T(kTapeDivInit, st);
    });
    if (e == cudaSuccess && anyDiv) e = add_while(cap, g, h[0], leaves, [&](cudaStream_t st) {
        launch_div_iter(d, st);
        T(kTapeDivIter, st);
    });
    if (e == cudaSuccess)
        e = add_segment(cap, g, leaves, [&](cudaStream_t st) {
            launch_div_finish(d, st);
            T(kTapeDivFinish, st);
            if (anyST) launch_surface_tension(d, passes, st);
            if (anyVisc) launch_visc_init(d, st);
        });
    if (e == cudaSuccess && anyVisc) e = add_while(cap, g, h[1], leaves, [&](cudaStream_t st) { launch_cg_iter(d, st); });
    if (e == cudaSuccess)
        e = add_segment(cap, g, leaves, [&](cudaStream_t st) {
            T(kTapeVisc, st);
            launch_visc_finish_dt(d, st);
            T(kTapeVelocity, st);
            launch_pres_init(d, st);
            T(kTapePresInit, st);
        });
    if (e == cudaSuccess) e = add_while(cap, g, h[2], leaves, [&](cudaStream_t st) {
        launch_pres_iter(d, st);
        T(kTapePresIter, st);
    });
    if (e == cudaSuccess) e = add_segment(cap, g, leaves, [&](cudaStream_t st) {
        launch_pres_finish(d, st);
        T(kTapeEnd, st);
    });
    cudaGraphExec_t exec = nullptr;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, g, 0);
    if (e != cudaSuccess) {
        cudaGetLastError();
        cudaGraphDestroy(g);
        return fail(VFD_E_CUDA, "step graph construction failed: %s", cudaGetErrorString(e));
    }
    *gOut = g;
    *execOut = exec;
    return VFD_OK;
}

int build_graph(vfd_sim* s, int parity) { return build_graph(s, parity, nullptr, &s->graph[parity], &s->exec[parity]); }

int read_flag(vfd_sim* s, int idx, uint32_t& v) {
    CK(cudaMemcpyAsync(s->hStatus + idx, s->dStatus + idx, sizeof(uint32_t), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    v = s->hStatus[idx];
    return VFD_OK;
}

// NVTX range of one phase of the step on the host timeline (a profiler shows the phases
// of eager steps; a graph step is one range around its launch).
struct PhaseRange {
    explicit PhaseRange(const char* name) { nvtxRangePushA(name); }
    ~PhaseRange() { nvtxRangePop(); }
    PhaseRange(const PhaseRange&) = delete;
    PhaseRange& operator=(const PhaseRange&) = delete;
};

// The reference's host-driven control flow: one flag read per solver iteration.
int launch_eager(vfd_sim* s, const void* rec) {
    const Dev& d = s->dev[s->cs];
    cudaStream_t st = s->stream;
    auto T = [&](int point) {
        if (rec) tape_point(d, rec, point, st);
    };
    uint32_t more = 0;
    PhaseRange step("vfd_step (eager)");
    T(kTapeBegin);
    {
        PhaseRange r("neighbour search");
        launch_search(d, st);
    }
    T(kTapeSearch);
    {
        PhaseRange r("boundary");
        launch_boundary(d, st);
    }
    T(kTapeBoundary);
    {
        PhaseRange r("density and factor");
        launch_density_div_init(d, st);
    }
    T(kTapeDivInit);
    if (s->anyDiv) {
        PhaseRange r("divergence solve");
        TRY(read_flag(s, 4, more));
        for (uint32_t guard = 0; more && guard < 1000000u; guard++) {
            launch_div_iter(d, st);
            T(kTapeDivIter);
            TRY(read_flag(s, 4, more));
        }
    }
    launch_div_finish(d, st);
    T(kTapeDivFinish);
    if (s->anyST) {
        PhaseRange r("surface tension");
        launch_surface_tension(d, s->maxStPasses, st);
    }
    if (s->anyVisc) {
        PhaseRange r("viscosity solve");
        launch_visc_init(d, st);
        TRY(read_flag(s, 5, more));
        for (uint32_t guard = 0; more && guard < 1000000u; guard++) {
            launch_cg_iter(d, st);
            TRY(read_flag(s, 5, more));
        }
    }
    T(kTapeVisc);
    {
        PhaseRange r("time step");
        launch_visc_finish_dt(d, st);
    }
    T(kTapeVelocity);
    {
        PhaseRange r("pressure solve");
        launch_pres_init(d, st);
        T(kTapePresInit);
        TRY(read_flag(s, 6, more));
        for (uint32_t guard = 0; more && guard < 1000000u; guard++) {
            launch_pres_iter(d, st);
            T(kTapePresIter);
            TRY(read_flag(s, 6, more));
        }
    }
    {
        PhaseRange r("integration");
        launch_pres_finish(d, st);
    }
    T(kTapeEnd);
    CK(cudaGetLastError());
    return VFD_OK;
}

int launch_eager(vfd_sim* s) { return launch_eager(s, nullptr); }

int ensure_ready(vfd_sim* s) {
    if (s->scenes.empty()) return fail(VFD_E_STATE, "no scene");
    if (!s->uploaded) TRY(upload(s));
    return VFD_OK;
}

int launch_one(vfd_sim* s) {
    if (s->graphMode && !s->graphFailed) {
        if (!s->exec[s->cs]) {
            const int rc = build_graph(s, s->cs);
            if (rc != VFD_OK) {
                // keep the kernels, drop the graph: eager launches of the same kernels
                s->graphFailed = true;
                s->releaseGraphs();
            }
        }
        if (!s->graphFailed) {
            PhaseRange r("vfd_step (graph)");
            CK(cudaGraphLaunch(s->exec[s->cs], s->stream));
            s->cs = 1 - s->cs;
            return VFD_OK;
        }
    }
    TRY(launch_eager(s));
    s->cs = 1 - s->cs;
    return VFD_OK;
}

// Handles a grid larger than the cell table: the step aborted before touching the
// carried state, so the table is grown and the same step launched again.
int finish_steps(vfd_sim* s, vfd_step_stats* stats, uint32_t& flags) {
    CK(cudaMemcpyAsync(s->hStatus, s->dStatus, 16 * sizeof(uint32_t), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    CK(cudaGetLastError());
    flags = s->hStatus[0];
    if (stats) {
        CK(cudaMemcpy(s->hScenes.data(), s->dScenes, sizeof(SceneDev) * s->hScenes.size(), cudaMemcpyDeviceToHost));
    }
    return VFD_OK;
}

void fill_stats(const SceneDev& S, vfd_step_stats* st) {
    st->IterationCount = S.iteration;
    st->DivergenceSolverIterationCount = S.enableDiv ? S.div.it : 0u;
    st->PressureSolverIterationCount = S.pres.it;
    st->ViscositySolverIterationCount = S.enableVisc ? S.cgIt : 0u;
    st->DivergenceSolverError = S.enableDiv ? S.div.err : 0.0f;
    st->PressureSolverError = S.pres.err;
    st->ViscositySolverError = (S.enableVisc && S.cgRhs > 0.0) ? (float)std::sqrt(S.cgRR / S.cgRhs) : 0.0f;
    st->FrameTime = S.frameTime;
    st->FrameIndex = S.frameIndex;
    st->TimeStepSize = S.dt;
    st->MaxVelocityMagnitude = S.maxV2;
    st->MaxNeighborCount = S.maxNbr;
    st->Flags = S.flags;
    st->SurfaceTensionSampleCount = S.stSamplesUsed;
}

int grow_cells(vfd_sim* s) {
    // keep the state: copy it out, reallocate with a larger table, copy it back
    const size_t st = s->stride;
    const Dev& d = s->dev[s->cs];
    std::vector<float4> xn(st), v(st), dv(st);
    std::vector<float> dk(st);
    std::vector<uint32_t> pid(st);
    CK(cudaMemcpy(xn.data(), d.XN, sizeof(float4) * st, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(v.data(), d.Vc, sizeof(float4) * st, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(dv.data(), d.DVc, sizeof(float4) * st, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(dk.data(), d.DKc, sizeof(float) * st, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(pid.data(), d.PIDc, sizeof(uint32_t) * st, cudaMemcpyDeviceToHost));
    std::vector<SceneDev> sc(s->hScenes.size());
    CK(cudaMemcpy(sc.data(), s->dScenes, sizeof(SceneDev) * sc.size(), cudaMemcpyDeviceToHost));
    const uint64_t want = (uint64_t)s->cellCap * 2u;
    if (want > 0xF0000000ull) return fail(VFD_E_CAPACITY, "search grid exceeds the cell table limit");
    s->cellCap = (uint32_t)want;
    TRY(allocate(s));
    const Dev& e = s->dev[0];
    s->cs = 0;
    CK(cudaMemcpy(e.XN, xn.data(), sizeof(float4) * st, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(e.Vc, v.data(), sizeof(float4) * st, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(e.DVc, dv.data(), sizeof(float4) * st, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(e.DKc, dk.data(), sizeof(float) * st, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(e.PIDc, pid.data(), sizeof(uint32_t) * st, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(s->dScenes, sc.data(), sizeof(SceneDev) * sc.size(), cudaMemcpyHostToDevice));
    CK(cudaMemset(s->dStatus, 0, 16 * sizeof(uint32_t)));
    s->uploaded = true;
    return VFD_OK;
}

int run_steps(vfd_sim* s, uint32_t count, vfd_step_stats* stats, bool wait) {
    if (!s) return fail(VFD_E_ARG, "null handle");
    TRY(ensure_ready(s));
    if (s->n == 0) return VFD_OK;
    if (s->fp64Mode) {  // the FP64 path steps synchronously
        for (uint32_t k = 0; k < count; k++) TRY(fp64_step(s, stats));
        return VFD_OK;
    }
    uint32_t remaining = count;
    for (int attempt = 0; remaining > 0 && attempt < 16; attempt++) {
        const int cs0 = s->cs;
        for (uint32_t k = 0; k < remaining; k++) TRY(launch_one(s));
        if (!wait) return VFD_OK;
        uint32_t flags = 0;
        TRY(finish_steps(s, stats, flags));
        // Only the search aborts a step (grid larger than the cell table, or a
        // non-finite position); an aborted step and the ones after it leave the
        // carried state where it was, so the state set follows the completed count.
        const uint32_t completed = s->hStatus[7];
        s->cs = (completed & 1u) ? 1 - cs0 : cs0;
        CK(cudaMemsetAsync(s->dStatus + 7, 0, sizeof(uint32_t), s->stream));
        if (!s->hStatus[1]) {
            if (stats) fill_stats(s->hScenes[0], stats);
            if (flags & 0x80u)
                return fail(VFD_E_STATE, "device bounds check failed (first index %u)", s->hStatus[9] - 1u);
            if (flags & 0x40u)
                return fail(VFD_E_CAPACITY, "cell-relative positions: a particle moved more than 511 cells from "
                                            "its scene's centre");
            return VFD_OK;
        }
        if (flags & 0x10u) return fail(VFD_E_NAN, "non-finite particle position");
        remaining -= std::min(remaining, completed);
        TRY(grow_cells(s));
    }
    return fail(VFD_E_CAPACITY, "search grid keeps exceeding the cell table");
}

int check_sim(const vfd_sim* s) { return s ? VFD_OK : fail(VFD_E_ARG, "null handle"); }

// The scatters export through one staging buffer in stream order; wait = false leaves the
// copy to a later synchronisation of the stream (the caller's).
int scatter_vec(vfd_sim* s, uint32_t scene, const float4* dsrc, float* out, bool wait) {
    const uint32_t b = s->sceneBegin[scene], cnt = s->scenes[scene].count();
    if (cnt == 0) return VFD_OK;
    k_export3<<<blocks_for(cnt, 256), 256, 0, s->stream>>>(s->dev[s->cs].PIDc, dsrc, s->dStage, b, cnt);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(out, s->dStage, sizeof(float) * 3 * (size_t)cnt, cudaMemcpyDeviceToHost, s->stream));
    if (wait) CK(cudaStreamSynchronize(s->stream));
    return VFD_OK;
}
int scatter_vec(vfd_sim* s, uint32_t scene, const float4* dsrc, float* out) { return scatter_vec(s, scene, dsrc, out, true); }

int scatter_scalar(vfd_sim* s, uint32_t scene, const float* dsrc, float* out, int comp = -1, const float4* d4 = nullptr) {
    const uint32_t b = s->sceneBegin[scene], cnt = s->scenes[scene].count();
    if (cnt == 0) return VFD_OK;
    k_export1<<<blocks_for(cnt, 256), 256, 0, s->stream>>>(s->dev[s->cs].PIDc, dsrc, d4, comp, s->dStage, b, cnt);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(out, s->dStage, sizeof(float) * (size_t)cnt, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return VFD_OK;
}

int gather_vec(vfd_sim* s, uint32_t scene, const float* in, float4* ddst) {
    const uint32_t b = s->sceneBegin[scene], cnt = s->scenes[scene].count();
    if (cnt == 0) return VFD_OK;
    CK(cudaMemcpyAsync(s->dStage, in, sizeof(float) * 3 * (size_t)cnt, cudaMemcpyHostToDevice, s->stream));
    k_import3<<<blocks_for(cnt, 256), 256, 0, s->stream>>>(s->dev[s->cs].PIDc, s->dStage, ddst, b, cnt);
    CK(cudaGetLastError());
    return VFD_OK;
}

// Positions (absolute in the caller's frame whatever the storage mode).
int scatter_pos(vfd_sim* s, uint32_t scene, const float4* dsrc, const float4* anchors, float* out, bool wait) {
    if (!s->cellRel) return scatter_vec(s, scene, dsrc, out, wait);
    const uint32_t b = s->sceneBegin[scene], cnt = s->scenes[scene].count();
    if (cnt == 0) return VFD_OK;
    k_export_pos<<<blocks_for(cnt, 256), 256, 0, s->stream>>>(s->dev[s->cs], dsrc, anchors, s->dStage, b, cnt);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(out, s->dStage, sizeof(float) * 3 * (size_t)cnt, cudaMemcpyDeviceToHost, s->stream));
    if (wait) CK(cudaStreamSynchronize(s->stream));
    return VFD_OK;
}
int scatter_pos(vfd_sim* s, uint32_t scene, const float4* dsrc, const float4* anchors, float* out) {
    return scatter_pos(s, scene, dsrc, anchors, out, true);
}

int gather_pos(vfd_sim* s, uint32_t scene, const float* in, float4* ddst) {
    if (!s->cellRel) return gather_vec(s, scene, in, ddst);
    const uint32_t b = s->sceneBegin[scene], cnt = s->scenes[scene].count();
    if (cnt == 0) return VFD_OK;
    CK(cudaMemcpyAsync(s->dStage, in, sizeof(float) * 3 * (size_t)cnt, cudaMemcpyHostToDevice, s->stream));
    k_import_pos<<<blocks_for(cnt, 256), 256, 0, s->stream>>>(s->dev[s->cs], s->dStage, ddst, b, cnt);
    CK(cudaGetLastError());
    return VFD_OK;
}

// Event-timed eager launches (vfd_profile_kernels).
struct EventProfiler : LaunchProfiler {
    struct Rec {
        std::string name;
        cudaEvent_t a, b;
    };
    std::vector<Rec> recs;
    std::vector<cudaEvent_t> pool;
    size_t used = 0;
    cudaError_t err = cudaSuccess;
    cudaEvent_t get() {
        if (used == pool.size()) {
            cudaEvent_t e;
            cudaError_t r = cudaEventCreate(&e);
            if (r != cudaSuccess) { err = r; return nullptr; }
            pool.push_back(e);
        }
        return pool[used++];
    }
    void begin(const char* name, cudaStream_t st) override {
        Rec r{name, get(), get()};
        if (r.a) cudaEventRecord(r.a, st);
        recs.push_back(r);
    }
    void end(cudaStream_t st) override {
        if (!recs.empty() && recs.back().b) cudaEventRecord(recs.back().b, st);
    }
    ~EventProfiler() override {
        for (auto e : pool) cudaEventDestroy(e);
    }
};

}  // namespace host
}  // namespace vfd

using namespace vfd::host;

// ====================================================================== C-ABI
extern "C" {

int vfd_abi_version(void) { return VFD_ABI_VERSION; }

const char* vfd_last_error(void) { return g_lastError.c_str(); }

int vfd_set_device(int32_t device) {
    int count = 0;
    CK(cudaGetDeviceCount(&count));
    if (device < 0 || device >= count) return fail(VFD_E_ARG, "device %d of %d", device, count);
    g_device = device;
    return VFD_OK;
}

int vfd_desc_default(vfd_desc* d) {
    if (!d) return fail(VFD_E_ARG, "null description");
    std::memset(d, 0, sizeof(*d));
    d->TimeStepSize = 0.001f;
    d->MinTimeStepSize = 0.0001f;
    d->MaxTimeStepSize = 0.005f;
    d->FrameLength = 0.0016f;
    d->FrameCount = 200u;
    d->MinPressureSolverIterations = 0u;
    d->MaxPressureSolverIterations = 100u;
    d->MaxPressureSolverError = 10.0f;
    d->EnableDivergenceSolverError = 1;
    d->MinDivergenceSolverIterations = 0u;
    d->MaxDivergenceSolverIterations = 100u;
    d->MaxDivergenceSolverError = 10.0f;
    d->EnableViscositySolver = 1;
    d->MinViscositySolverIterations = 0u;
    d->MaxViscositySolverIterations = 100u;
    d->MaxViscositySolverError = 0.1f;
    d->Viscosity = 10.0f;
    d->BoundaryViscosity = 10.0f;
    d->TangentialDistanceFactor = 0.5f;
    d->EnableSurfaceTensionSolver = 1;
    d->SurfaceTensionSmoothPassCount = 1u;
    d->SurfaceTension = 1.0f;
    d->TemporalSmoothing = 0;
    d->CSDFix = -1;
    d->CSD = 10000;
    d->ParticleRadius = 0.025f;
    d->Gravity[0] = 0.0f;
    d->Gravity[1] = -9.81f;
    d->Gravity[2] = 0.0f;
    return VFD_OK;
}

int vfd_create_batch(const vfd_desc* descs, uint32_t count, vfd_sim** out) {
    if (!out || !descs || count == 0 || count > 65535u) return fail(VFD_E_ARG, "invalid scene list");
    *out = nullptr;
    for (uint32_t k = 0; k < count; k++) {
        TRY(check_desc(&descs[k]));
        if (descs[k].ParticleRadius != descs[0].ParticleRadius)
            return fail(VFD_E_ARG, "all scenes of a batch share one ParticleRadius");
    }
    int devCount = 0;
    cudaError_t e = cudaGetDeviceCount(&devCount);
    if (e != cudaSuccess || devCount == 0) return fail(VFD_E_NODEVICE, "no CUDA device: %s", cudaGetErrorString(e));
    CK(cudaSetDevice(g_device));
    vfd_sim* s = new (std::nothrow) vfd_sim();
    if (!s) return fail(VFD_E_NOMEM, "host allocation");
    s->device = g_device;
    e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete s;
        return fail(VFD_E_CUDA, "cudaStreamCreate: %s", cudaGetErrorString(e));
    }
    s->scenes.resize(count);
    for (uint32_t k = 0; k < count; k++) s->scenes[k].desc = descs[k];
    s->table.setRadius(4.0f * descs[0].ParticleRadius);
    halton_table(s->halton);
    *out = s;
    return VFD_OK;
}

int vfd_create(const vfd_desc* desc, vfd_sim** out) { return vfd_create_batch(desc, 1, out); }

int vfd_destroy(vfd_sim* s) {
    if (!s) return VFD_OK;
    cudaSetDevice(s->device);
    delete s;
    return VFD_OK;
}

int vfd_get_scene_count(const vfd_sim* s, uint32_t* n) {
    TRY(check_sim(s));
    if (!n) return fail(VFD_E_ARG, "null output");
    *n = (uint32_t)s->scenes.size();
    return VFD_OK;
}

int vfd_set_description(vfd_sim* s, const vfd_desc* desc) {
    TRY(check_sim(s));
    TRY(check_desc(desc));
    if (s->scenes.size() > 1 && desc->ParticleRadius != s->scenes[0].desc.ParticleRadius)
        return fail(VFD_E_ARG, "all scenes of a batch share one ParticleRadius");
    CK(cudaSetDevice(s->device));
    const vfd_desc old = s->scenes[0].desc;
    s->scenes[0].desc = *desc;
    // parameters that change neither the table nor the step's graph structure only need
    // the next step's upload
    const bool sameShape = desc->ParticleRadius == old.ParticleRadius &&
                           desc->EnableDivergenceSolverError == old.EnableDivergenceSolverError &&
                           desc->EnableViscositySolver == old.EnableViscositySolver &&
                           desc->EnableSurfaceTensionSolver == old.EnableSurfaceTensionSolver &&
                           desc->SurfaceTensionSmoothPassCount == old.SurfaceTensionSmoothPassCount;
    if (sameShape && s->allocated) {
        s->uploaded = false;
        return VFD_OK;
    }
    if (desc->ParticleRadius != s->table.radius / 4.0f) s->table.setRadius(4.0f * desc->ParticleRadius);
    s->releaseBuffers();
    return VFD_OK;
}

int vfd_get_description(const vfd_sim* s, vfd_desc* desc) {
    TRY(check_sim(s));
    if (!desc) return fail(VFD_E_ARG, "null output");
    *desc = s->scenes[0].desc;
    return VFD_OK;
}

int vfd_scene_set_fluid(vfd_sim* s, uint32_t scene, const float* xyz, const float* vel, uint32_t n) {
    TRY(check_sim(s));
    if (scene >= s->scenes.size()) return fail(VFD_E_ARG, "scene %u out of range", scene);
    if (n > 0 && !xyz) return fail(VFD_E_ARG, "null positions");
    for (uint64_t i = 0; i < 3ull * n; i++)
        if (!std::isfinite(xyz[i]) || (vel && !std::isfinite(vel[i])))
            return fail(VFD_E_NAN, "non-finite input at element %llu", (unsigned long long)i);
    CK(cudaSetDevice(s->device));
    SceneHost& sc = s->scenes[scene];
    const bool sameCount = sc.x0.size() == 3ull * n;
    sc.x0.assign(xyz, xyz + 3ull * n);
    if (vel) sc.v0.assign(vel, vel + 3ull * n);
    else sc.v0.assign(3ull * n, 0.0f);
    if (sameCount && s->allocated) {
        // same layout: the next step uploads the new state into the existing buffers and
        // keeps the step graphs (the cell table grows if the new state needs it)
        s->uploaded = false;
        return VFD_OK;
    }
    s->releaseBuffers();
    s->cellCap = 0;
    return VFD_OK;
}

int vfd_set_fluid(vfd_sim* s, const float* xyz, const float* vel, uint32_t n) {
    return vfd_scene_set_fluid(s, 0, xyz, vel, n);
}

int vfd_scene_add_rigid_body(vfd_sim* s, uint32_t scene, const vfd_volume_map* m) {
    TRY(check_sim(s));
    if (scene >= s->scenes.size()) return fail(VFD_E_ARG, "scene %u out of range", scene);
    if (!m || !m->nodes || !m->cells || !m->cell_map) return fail(VFD_E_ARG, "incomplete volume map");
    if (m->field_count < 2) return fail(VFD_E_ARG, "a volume map needs fields 0 (distance) and 1 (volume)");
    const uint64_t cells = (uint64_t)m->resolution[0] * m->resolution[1] * m->resolution[2];
    if (cells == 0 || cells != m->cell_map_count) return fail(VFD_E_ARG, "cell map size does not match the resolution");
    for (uint64_t c = 0; c < m->cell_map_count; c++) {
        const uint32_t j = m->cell_map[c];
        if (j != UINT_MAX && j >= m->cell_count) return fail(VFD_E_ARG, "cell map entry %u out of range", j);
    }
    for (uint64_t k = 0; k < (uint64_t)m->cell_count * 32u; k++)
        if (m->cells[k] >= m->node_count) return fail(VFD_E_ARG, "cell node index out of range");
    CK(cudaSetDevice(s->device));
    BodyHost b;
    for (int k = 0; k < 3; k++) {
        b.dev.dmin[k] = m->domain_min[k];
        b.dev.dmax[k] = m->domain_max[k];
        b.dev.cs[k] = m->cell_size[k];
        b.dev.csi[k] = m->cell_size_inverse[k];
        b.dev.res[k] = m->resolution[k];
    }
    b.dev.nodeCount = m->node_count;
    b.dev.cellCount = m->cell_count;
    b.dev.cellMapCount = m->cell_map_count;
    CK(cudaMalloc(&b.nodes, sizeof(float) * 2ull * m->node_count));
    CK(cudaMalloc(&b.cells, sizeof(uint32_t) * 32ull * m->cell_count));
    CK(cudaMalloc(&b.cellMap, sizeof(uint32_t) * (size_t)m->cell_map_count));
    CK(cudaMemcpy(b.nodes, m->nodes, sizeof(float) * 2ull * m->node_count, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(b.cells, m->cells, sizeof(uint32_t) * 32ull * m->cell_count, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(b.cellMap, m->cell_map, sizeof(uint32_t) * (size_t)m->cell_map_count, cudaMemcpyHostToDevice));
    b.dev.nodes = b.nodes;
    b.dev.cells = b.cells;
    b.dev.cellMap = b.cellMap;
    s->scenes[scene].bodies.push_back(b);
    s->releaseBuffers();
    return VFD_OK;
}

int vfd_add_rigid_body(vfd_sim* s, const vfd_volume_map* m) { return vfd_scene_add_rigid_body(s, 0, m); }

int vfd_clear_rigid_bodies(vfd_sim* s) {
    TRY(check_sim(s));
    CK(cudaSetDevice(s->device));
    for (auto& sc : s->scenes) {
        for (auto& b : sc.bodies) b.release();
        sc.bodies.clear();
    }
    s->releaseBuffers();
    return VFD_OK;
}

int vfd_box_map_sizes(const uint32_t resolution[3], uint32_t* node_count, uint32_t* cell_count) {
    if (!resolution || !node_count || !cell_count) return fail(VFD_E_ARG, "null argument");
    for (int k = 0; k < 3; k++)
        if (resolution[k] == 0 || resolution[k] > 1024) return fail(VFD_E_ARG, "resolution must be in 1..1024");
    // the builders index nodes * 32 quadrature lanes and cells * 32 node slots in 32 bits
    const uint64_t r0 = resolution[0], r1 = resolution[1], r2 = resolution[2];
    const uint64_t nodes = (r0 + 1) * (r1 + 1) * (r2 + 1) +
                           2 * (r0 * (r1 + 1) * (r2 + 1) + (r0 + 1) * r1 * (r2 + 1) + (r0 + 1) * (r1 + 1) * r2);
    if (32 * nodes > 0xffffffffull) return fail(VFD_E_ARG, "resolution too fine (%llu map nodes)",
                                                (unsigned long long)nodes);
    box_map_sizes(resolution, *node_count, *cell_count);
    return VFD_OK;
}

int vfd_build_box_map(const float box_min[3], const float box_max[3], int32_t inverted, float padding,
                      const uint32_t resolution[3], float particle_radius, float* nodes, uint32_t* cells,
                      uint32_t* cell_map, vfd_volume_map* out) {
    if (!box_min || !box_max || !resolution || !nodes || !cells || !cell_map || !out)
        return fail(VFD_E_ARG, "null argument");
    if (!(particle_radius > 0.0f)) return fail(VFD_E_ARG, "particle radius must be positive");
    for (int k = 0; k < 3; k++)
        if (!(box_max[k] > box_min[k])) return fail(VFD_E_ARG, "empty box");
    uint32_t nn = 0, nc = 0;
    TRY(vfd_box_map_sizes(resolution, &nn, &nc));
    int devCount = 0;
    if (cudaGetDeviceCount(&devCount) != cudaSuccess || devCount == 0) return fail(VFD_E_NODEVICE, "no CUDA device");
    CK(cudaSetDevice(g_device));
    KernelTable t;
    t.setRadius(4.0f * particle_radius);
    const int e = build_box_map_gpu(box_min, box_max, inverted != 0, padding, resolution, particle_radius,
                                    t.W.data(), t.wZero, t.invStep, nodes, cells, cell_map, out->domain_min,
                                    out->domain_max, out->cell_size, out->cell_size_inverse);
    if (e != 0) return fail(VFD_E_CUDA, "volume map build: %s", cudaGetErrorString((cudaError_t)e));
    out->nodes = nodes;
    out->cells = cells;
    out->cell_map = cell_map;
    for (int k = 0; k < 3; k++) out->resolution[k] = resolution[k];
    out->field_count = 2;
    out->node_count = nn;
    out->cell_count = nc;
    out->cell_map_count = nc;
    return VFD_OK;
}

// Checks the mesh arguments shared by the mesh entry points and places the mesh.
static int mesh_arguments(const float* vertices, uint32_t vertexCount, const uint32_t* triangles,
                          uint32_t triangleCount, const float* transform, MeshHost& mesh) {
    if (!vertices || !triangles) return fail(VFD_E_ARG, "null mesh");
    if (vertexCount == 0 || triangleCount == 0) return fail(VFD_E_ARG, "empty mesh");
    if (prepare_mesh(vertices, vertexCount, triangles, triangleCount, transform, mesh) != 0)
        return fail(VFD_E_ARG, "triangle index out of range (vertex count %u)", vertexCount);
    for (int k = 0; k < 3; k++)
        if (!std::isfinite(mesh.bmin[k]) || !std::isfinite(mesh.bmax[k])) return fail(VFD_E_ARG, "non-finite vertex");
    return VFD_OK;
}

int vfd_build_mesh_map(const float* vertices, uint32_t vertex_count, const uint32_t* triangles,
                       uint32_t triangle_count, const float* transform, int32_t inverted, float padding,
                       const uint32_t resolution[3], float particle_radius, float* nodes, uint32_t* cells,
                       uint32_t* cell_map, vfd_volume_map* out) {
    if (!resolution || !nodes || !cells || !cell_map || !out) return fail(VFD_E_ARG, "null argument");
    if (!(particle_radius > 0.0f)) return fail(VFD_E_ARG, "particle radius must be positive");
    uint32_t nn = 0, nc = 0;
    TRY(vfd_box_map_sizes(resolution, &nn, &nc));
    MeshHost mesh;
    TRY(mesh_arguments(vertices, vertex_count, triangles, triangle_count, transform, mesh));
    int devCount = 0;
    if (cudaGetDeviceCount(&devCount) != cudaSuccess || devCount == 0) return fail(VFD_E_NODEVICE, "no CUDA device");
    CK(cudaSetDevice(g_device));
    KernelTable t;
    t.setRadius(4.0f * particle_radius);
    const int e = build_mesh_map_gpu(mesh, inverted != 0, padding, resolution, particle_radius, t.W.data(), t.wZero,
                                     t.invStep, nodes, cells, cell_map, out->domain_min, out->domain_max,
                                     out->cell_size, out->cell_size_inverse);
    if (e != 0) return fail(VFD_E_CUDA, "mesh volume map build: %s", cudaGetErrorString((cudaError_t)e));
    out->nodes = nodes;
    out->cells = cells;
    out->cell_map = cell_map;
    for (int k = 0; k < 3; k++) out->resolution[k] = resolution[k];
    out->field_count = 2;
    out->node_count = nn;
    out->cell_count = nc;
    out->cell_map_count = nc;
    return VFD_OK;
}

int vfd_sample_mesh_volume(const float* vertices, uint32_t vertex_count, const uint32_t* triangles,
                           uint32_t triangle_count, const float* transform, float particle_radius,
                           const uint32_t resolution[3], int32_t inverted, int32_t sample_mode,
                           float* positions, uint32_t capacity, uint32_t* count) {
    if (!resolution || !count) return fail(VFD_E_ARG, "null argument");
    *count = 0;
    if (!(particle_radius > 0.0f) || !std::isfinite(particle_radius))
        return fail(VFD_E_ARG, "particle radius must be positive");
    if (sample_mode < VFD_SAMPLE_MIN_DENSITY || sample_mode > VFD_SAMPLE_MAX_DENSITY)
        return fail(VFD_E_ARG, "unknown sample mode %d", sample_mode);
    uint32_t nn = 0, nc = 0;
    TRY(vfd_box_map_sizes(resolution, &nn, &nc));
    MeshHost mesh;
    TRY(mesh_arguments(vertices, vertex_count, triangles, triangle_count, transform, mesh));
    int devCount = 0;
    if (cudaGetDeviceCount(&devCount) != cudaSuccess || devCount == 0) return fail(VFD_E_NODEVICE, "no CUDA device");
    CK(cudaSetDevice(g_device));
    const int e = sample_mesh_volume_gpu(mesh, particle_radius, resolution, inverted != 0, sample_mode, positions,
                                         capacity, count);
    if (e < 0) return fail(VFD_E_CAPACITY, "sampling lattice too large for the radius");
    if (e != 0) return fail(VFD_E_CUDA, "mesh volume sampling: %s", cudaGetErrorString((cudaError_t)e));
    if (positions && *count > capacity) return fail(VFD_E_CAPACITY, "%u samples, capacity %u", *count, capacity);
    return VFD_OK;
}

int vfd_reset(vfd_sim* s) {
    TRY(check_sim(s));
    CK(cudaSetDevice(s->device));
    if (s->scenes.empty()) return fail(VFD_E_STATE, "no scene");
    return upload(s);
}

int vfd_set_position_mode(vfd_sim* s, int32_t mode) {
    TRY(check_sim(s));
    if (mode != VFD_POSITIONS_ABSOLUTE && mode != VFD_POSITIONS_CELL_RELATIVE)
        return fail(VFD_E_ARG, "unknown position mode %d", mode);
    CK(cudaSetDevice(s->device));
    s->cellRel = mode == VFD_POSITIONS_CELL_RELATIVE;
    s->releaseBuffers();
    return VFD_OK;
}

int vfd_emit(vfd_sim* s, const float* xyz, const float* vel, uint32_t count) {
    TRY(check_sim(s));
    if (s->fp64Mode) return fail(VFD_E_STATE, "vfd_emit is not available in the FP64 path");
    if (s->scenes.size() != 1) return fail(VFD_E_ARG, "vfd_emit adds to single-scene simulations");
    if (count == 0) return VFD_OK;
    if (!xyz) return fail(VFD_E_ARG, "null positions");
    for (size_t i = 0; i < 3 * (size_t)count; i++)
        if (!std::isfinite(xyz[i]) || (vel && !std::isfinite(vel[i]))) return fail(VFD_E_NAN, "non-finite input");
    if ((uint64_t)s->n + count > 0x7fffffffull) return fail(VFD_E_CAPACITY, "particle count limit");
    CK(cudaSetDevice(s->device));
    TRY(ensure_ready(s));
    vfd::adjoint_release(s);
    CK(cudaStreamSynchronize(s->stream));
    const uint32_t n0 = s->n, n1 = n0 + count;
    if (n1 > s->stride) {
        // grow with headroom for later emissions, keeping the carried state (as grow_cells)
        const size_t st = s->stride;
        const Dev& d = s->dev[s->cs];
        std::vector<float4> xn(st), v(st), dv(st), acc(st);
        std::vector<float> dk(st);
        std::vector<uint32_t> pid(st);
        CK(cudaMemcpy(xn.data(), d.XN, sizeof(float4) * st, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(v.data(), d.Vc, sizeof(float4) * st, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(dv.data(), d.DVc, sizeof(float4) * st, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(dk.data(), d.DKc, sizeof(float) * st, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(pid.data(), d.PIDc, sizeof(uint32_t) * st, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(acc.data(), d.A, sizeof(float4) * st, cudaMemcpyDeviceToHost));
        std::vector<SceneDev> sc(s->hScenes.size());
        CK(cudaMemcpy(sc.data(), s->dScenes, sizeof(SceneDev) * sc.size(), cudaMemcpyDeviceToHost));
        s->reserve = std::max<uint32_t>(n1, (uint32_t)std::min<uint64_t>(0x7fffffffull, (uint64_t)n1 + n1 / 4));
        s->scenes[0].emitted += count;  // allocate() sizes the layout for n1
        TRY(allocate(s));
        s->allocated = true;
        const Dev& e = s->dev[0];
        s->cs = 0;
        CK(cudaMemcpy(e.XN, xn.data(), sizeof(float4) * n0, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(e.Vc, v.data(), sizeof(float4) * n0, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(e.DVc, dv.data(), sizeof(float4) * n0, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(e.DKc, dk.data(), sizeof(float) * n0, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(e.PIDc, pid.data(), sizeof(uint32_t) * n0, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(e.A, acc.data(), sizeof(float4) * n0, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(s->dScenes, sc.data(), sizeof(SceneDev) * sc.size(), cudaMemcpyHostToDevice));
        CK(cudaMemset(s->dStatus, 0, 16 * sizeof(uint32_t)));
        TRY(reset_buckets(s, e));
        s->hScenes = sc;
        s->uploaded = true;
    } else {
        // same layout, more particles: the step graphs carry n, so they are rebuilt
        s->releaseGraphs();
        s->scenes[0].emitted += count;
        s->n = n1;
        for (int k = 0; k < 2; k++) s->dev[k].n = n1;
    }
    // the new particles through the staging buffer (3 floats each), in chunks of its size
    for (uint32_t done = 0; done < count;) {
        const uint32_t chunk = std::min<uint32_t>(count - done, s->stride / 2u);
        CK(cudaMemcpyAsync(s->dStage, xyz + 3 * (size_t)done, sizeof(float) * 3 * chunk, cudaMemcpyHostToDevice,
                           s->stream));
        if (vel)
            CK(cudaMemcpyAsync(s->dStage + 3 * (size_t)chunk, vel + 3 * (size_t)done, sizeof(float) * 3 * chunk,
                               cudaMemcpyHostToDevice, s->stream));
        k_emit<<<blocks_for(chunk, 256), 256, 0, s->stream>>>(s->dev[s->cs], s->dStage,
                                                              vel ? s->dStage + 3 * (size_t)chunk : nullptr,
                                                              n0 + done, chunk, s->dStatus);
        CK(cudaGetLastError());
        CK(cudaStreamSynchronize(s->stream));
        done += chunk;
    }
    uint32_t flags = 0;
    CK(cudaMemcpy(&flags, s->dStatus, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    if (flags & 0x40u) return fail(VFD_E_CAPACITY, "cell-relative positions: an emitted particle lies more than 511 "
                                                   "cells from the scene's centre");
    return VFD_OK;
}

int vfd_set_kernel_mode(vfd_sim* s, int32_t mode) {
    TRY(check_sim(s));
    if (mode != VFD_KERNEL_TABLE && mode != VFD_KERNEL_ANALYTIC) return fail(VFD_E_ARG, "unknown kernel mode %d", mode);
    CK(cudaSetDevice(s->device));
    s->analyticKernel = mode == VFD_KERNEL_ANALYTIC;
    s->releaseBuffers();
    return VFD_OK;
}

int vfd_set_precision(vfd_sim* s, int32_t mode) {
    TRY(check_sim(s));
    if (mode != VFD_PRECISION_FP32 && mode != VFD_PRECISION_FP64) return fail(VFD_E_ARG, "unknown precision %d", mode);
    if (mode == VFD_PRECISION_FP64 && s->scenes.size() != 1)
        return fail(VFD_E_STATE, "the FP64 path runs single-scene simulations");
    CK(cudaSetDevice(s->device));
    s->fp64Mode = mode == VFD_PRECISION_FP64;
    fp64_release(s);
    s->uploaded = false;  // the next call restarts from the fluid objects in the chosen precision
    return VFD_OK;
}

int vfd_get_state_f64(vfd_sim* s, double* x, double* v) {
    TRY(check_sim(s));
    if (!s->fp64Mode) return fail(VFD_E_STATE, "vfd_get_state_f64 needs VFD_PRECISION_FP64");
    CK(cudaSetDevice(s->device));
    TRY(ensure_ready(s));
    return fp64_get_state(s, x, v, nullptr, nullptr, nullptr);
}

int vfd_set_graph_mode(vfd_sim* s, int32_t enabled) {
    TRY(check_sim(s));
    s->graphMode = enabled != 0;
    s->graphFailed = false;
    return VFD_OK;
}

int vfd_get_graph_mode(const vfd_sim* s, int32_t* requested, int32_t* active) {
    TRY(check_sim(s));
    if (requested) *requested = s->graphMode ? 1 : 0;
    if (active) *active = (s->graphMode && !s->graphFailed) ? 1 : 0;
    return VFD_OK;
}

int vfd_step(vfd_sim* s, vfd_step_stats* stats) {
    TRY(check_sim(s));
    CK(cudaSetDevice(s->device));
    vfd_step_stats tmp;
    TRY(run_steps(s, 1, stats ? stats : &tmp, true));
    const uint32_t f = s->hStatus ? s->hStatus[0] : 0u;
    if (f & 0x10u) return fail(VFD_E_NAN, "non-finite particle state");
    return VFD_OK;
}

int vfd_steps(vfd_sim* s, uint32_t count, vfd_step_stats* stats) {
    TRY(check_sim(s));
    CK(cudaSetDevice(s->device));
    if (count == 0) return VFD_OK;
    vfd_step_stats tmp;
    TRY(run_steps(s, count, stats ? stats : &tmp, true));
    if (s->hStatus && (s->hStatus[0] & 0x10u)) return fail(VFD_E_NAN, "non-finite particle state");
    return VFD_OK;
}

int vfd_steps_async(vfd_sim* s, uint32_t count) {
    TRY(check_sim(s));
    CK(cudaSetDevice(s->device));
    return run_steps(s, count, nullptr, false);
}

int vfd_synchronize(vfd_sim* s, vfd_step_stats* stats) {
    TRY(check_sim(s));
    CK(cudaSetDevice(s->device));
    if (!s->uploaded) return VFD_OK;
    if (s->fp64Mode) {
        if (stats) fp64_stats(s, stats);
        return VFD_OK;
    }
    uint32_t flags = 0;
    TRY(finish_steps(s, stats, flags));
    CK(cudaMemsetAsync(s->dStatus + 7, 0, sizeof(uint32_t), s->stream));
    if (s->hStatus[1]) {
        if (flags & 0x10u) return fail(VFD_E_NAN, "non-finite particle position");
        return fail(VFD_E_CAPACITY, "search grid exceeded the cell table during an asynchronous step");
    }
    if (stats) fill_stats(s->hScenes[0], stats);
    return VFD_OK;
}

int vfd_get_state(vfd_sim* s, float* x, float* v, float* a) { return vfd_scene_get_state(s, 0, x, v, a); }

int vfd_scene_get_state(vfd_sim* s, uint32_t scene, float* x, float* v, float* a) {
    TRY(check_sim(s));
    if (scene >= s->scenes.size()) return fail(VFD_E_ARG, "scene %u out of range", scene);
    CK(cudaSetDevice(s->device));
    TRY(ensure_ready(s));
    if (s->fp64Mode) return fp64_get_state(s, nullptr, nullptr, x, v, a);
    const Dev& d = s->dev[s->cs];
    // the three exports share the staging buffer in stream order; one wait for all
    if (x) TRY(scatter_pos(s, scene, d.XN, d.XN, x, false));
    if (v) TRY(scatter_vec(s, scene, d.Vc, v, false));
    if (a) TRY(scatter_vec(s, scene, d.A, a, false));
    CK(cudaStreamSynchronize(s->stream));
    return VFD_OK;
}

int vfd_set_state(vfd_sim* s, const float* x, const float* v) {
    TRY(check_sim(s));
    if (s->fp64Mode) return fail(VFD_E_STATE, "vfd_set_state is not available in the FP64 path");
    CK(cudaSetDevice(s->device));
    TRY(ensure_ready(s));
    const uint32_t cnt = s->scenes[0].count();
    if (cnt == 0) return VFD_OK;
    const size_t bytes = sizeof(float) * 3 * (size_t)cnt;
    // both arrays are copied and checked on the device before either is imported
    uint32_t* bad = s->dStatus + 10;
    CK(cudaMemsetAsync(bad, 0, sizeof(uint32_t), s->stream));
    if (x) {
        CK(cudaMemcpyAsync(s->dStage, x, bytes, cudaMemcpyHostToDevice, s->stream));
        k_check_finite<<<blocks_for(3 * cnt, 256), 256, 0, s->stream>>>(s->dStage, 3 * (size_t)cnt, bad);
    }
    if (v) {
        CK(cudaMemcpyAsync(s->dStage2, v, bytes, cudaMemcpyHostToDevice, s->stream));
        k_check_finite<<<blocks_for(3 * cnt, 256), 256, 0, s->stream>>>(s->dStage2, 3 * (size_t)cnt, bad);
    }
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(s->hStatus + 10, bad, sizeof(uint32_t), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    if (s->hStatus[10]) return fail(VFD_E_NAN, "non-finite input");
    const Dev& d = s->dev[s->cs];
    const uint32_t b = s->sceneBegin[0];
    if (x) {
        if (s->cellRel) k_import_pos<<<blocks_for(cnt, 256), 256, 0, s->stream>>>(d, s->dStage, d.XN, b, cnt);
        else k_import3<<<blocks_for(cnt, 256), 256, 0, s->stream>>>(d.PIDc, s->dStage, d.XN, b, cnt);
    }
    if (v) k_import3<<<blocks_for(cnt, 256), 256, 0, s->stream>>>(d.PIDc, s->dStage2, d.Vc, b, cnt);
    CK(cudaGetLastError());
    // calls that write the state with default-stream copies (restore, upload) must find it settled
    CK(cudaStreamSynchronize(s->stream));
    return VFD_OK;
}

// ---------------------------------------------------------------- checkpoints
// Image layout: header, then per scene its SceneDev (the solver clock, dt and frame
// state; constants are taken from the restoring simulation), then per scene the raw
// slot ranges of the carried state: XN, Vc, DVc, A (float4), DKc (float), PIDc (u32).
namespace {
constexpr uint32_t kCkptMagic = 0x4B444656u;  // "VFDK"
constexpr uint32_t kCkptVersion = 1u;
struct CkptHeader {
    uint32_t magic, version, scenes, flags;  // flags: bit 0 cell-relative, bit 1 analytic kernel
    uint32_t stride, pad[3];
};
constexpr size_t kCkptPerParticle = 4 * sizeof(float4) + sizeof(float) + sizeof(uint32_t);
uint64_t checkpoint_bytes(const vfd_sim* s) {
    uint64_t b = sizeof(CkptHeader) + (sizeof(uint32_t) + sizeof(SceneDev)) * (uint64_t)s->scenes.size();
    for (const auto& sc : s->scenes) b += kCkptPerParticle * (uint64_t)sc.count();
    return b;
}
}  // namespace

int vfd_checkpoint_size(vfd_sim* s, uint64_t* bytes) {
    TRY(check_sim(s));
    if (s->fp64Mode) return fail(VFD_E_STATE, "vfd_checkpoint is not available in the FP64 path");
    if (!bytes) return fail(VFD_E_ARG, "null output");
    TRY(ensure_ready(s));
    *bytes = checkpoint_bytes(s);
    return VFD_OK;
}

int vfd_checkpoint(vfd_sim* s, void* buffer, uint64_t bytes) {
    TRY(check_sim(s));
    if (s->fp64Mode) return fail(VFD_E_STATE, "vfd_checkpoint is not available in the FP64 path");
    if (!buffer) return fail(VFD_E_ARG, "null buffer");
    CK(cudaSetDevice(s->device));
    TRY(ensure_ready(s));
    if (bytes < checkpoint_bytes(s)) return fail(VFD_E_CAPACITY, "checkpoint buffer too small");
    CK(cudaStreamSynchronize(s->stream));
    unsigned char* out = static_cast<unsigned char*>(buffer);
    CkptHeader h{kCkptMagic, kCkptVersion, (uint32_t)s->scenes.size(),
                 (s->cellRel ? 1u : 0u) | (s->analyticKernel ? 2u : 0u), s->stride, {0u, 0u, 0u}};
    std::memcpy(out, &h, sizeof(h));
    out += sizeof(h);
    std::vector<SceneDev> sc(s->hScenes.size());
    CK(cudaMemcpy(sc.data(), s->dScenes, sizeof(SceneDev) * sc.size(), cudaMemcpyDeviceToHost));
    for (uint32_t k = 0; k < s->scenes.size(); k++) {
        const uint32_t cnt = s->scenes[k].count();
        std::memcpy(out, &cnt, sizeof(cnt));
        std::memcpy(out + sizeof(cnt), &sc[k], sizeof(SceneDev));
        out += sizeof(cnt) + sizeof(SceneDev);
    }
    const Dev& d = s->dev[s->cs];
    for (uint32_t k = 0; k < s->scenes.size(); k++) {
        const size_t b = s->sceneBegin[k], cnt = s->scenes[k].count();
        const void* src4[4] = {d.XN + b, d.Vc + b, d.DVc + b, d.A + b};
        for (const void* p : src4) {
            CK(cudaMemcpy(out, p, sizeof(float4) * cnt, cudaMemcpyDeviceToHost));
            out += sizeof(float4) * cnt;
        }
        CK(cudaMemcpy(out, d.DKc + b, sizeof(float) * cnt, cudaMemcpyDeviceToHost));
        out += sizeof(float) * cnt;
        CK(cudaMemcpy(out, d.PIDc + b, sizeof(uint32_t) * cnt, cudaMemcpyDeviceToHost));
        out += sizeof(uint32_t) * cnt;
    }
    return VFD_OK;
}

int vfd_restore(vfd_sim* s, const void* buffer, uint64_t bytes) {
    TRY(check_sim(s));
    if (s->fp64Mode) return fail(VFD_E_STATE, "vfd_restore is not available in the FP64 path");
    if (!buffer) return fail(VFD_E_ARG, "null buffer");
    CK(cudaSetDevice(s->device));
    TRY(ensure_ready(s));
    const unsigned char* in = static_cast<const unsigned char*>(buffer);
    if (bytes < sizeof(CkptHeader)) return fail(VFD_E_ARG, "checkpoint image too short");
    CkptHeader h;
    std::memcpy(&h, in, sizeof(h));
    in += sizeof(h);
    if (h.magic != kCkptMagic || h.version != kCkptVersion) return fail(VFD_E_ARG, "not a checkpoint image");
    if (h.scenes != s->scenes.size()) return fail(VFD_E_STATE, "checkpoint has %u scenes, simulation %zu",
                                                  h.scenes, s->scenes.size());
    const uint32_t modes = (s->cellRel ? 1u : 0u) | (s->analyticKernel ? 2u : 0u);
    if (h.flags != modes) return fail(VFD_E_STATE, "checkpoint was taken in another position or kernel mode");
    if (bytes < sizeof(CkptHeader) + (sizeof(uint32_t) + sizeof(SceneDev)) * (uint64_t)h.scenes)
        return fail(VFD_E_ARG, "checkpoint image too short");
    for (uint32_t k = 0; k < h.scenes; k++) {  // particle counts first: a different scene is a state mismatch
        uint32_t cnt;
        std::memcpy(&cnt, in + k * (sizeof(uint32_t) + sizeof(SceneDev)), sizeof(cnt));
        if (cnt != s->scenes[k].count())
            return fail(VFD_E_STATE, "scene %u: checkpoint has %u particles, simulation %u", k, cnt,
                        s->scenes[k].count());
    }
    if (bytes < checkpoint_bytes(s)) return fail(VFD_E_ARG, "checkpoint image too short");
    std::vector<SceneDev> cur(s->hScenes.size());
    CK(cudaMemcpy(cur.data(), s->dScenes, sizeof(SceneDev) * cur.size(), cudaMemcpyDeviceToHost));
    const size_t dyn = offsetof(SceneDev, dt);
    for (uint32_t k = 0; k < h.scenes; k++) {
        uint32_t cnt;
        std::memcpy(&cnt, in, sizeof(cnt));
        if (cnt != s->scenes[k].count())
            return fail(VFD_E_STATE, "scene %u: checkpoint has %u particles, simulation %u", k, cnt,
                        s->scenes[k].count());
        SceneDev saved;
        std::memcpy(&saved, in + sizeof(cnt), sizeof(SceneDev));
        // the solver clock and state of the checkpoint, the constants of this simulation
        std::memcpy(reinterpret_cast<unsigned char*>(&cur[k]) + dyn, reinterpret_cast<unsigned char*>(&saved) + dyn,
                    sizeof(SceneDev) - dyn);
        in += sizeof(cnt) + sizeof(SceneDev);
    }
    const Dev& d = s->dev[s->cs];
    for (uint32_t k = 0; k < h.scenes; k++) {
        const size_t b = s->sceneBegin[k], cnt = s->scenes[k].count();
        void* dst4[4] = {d.XN + b, d.Vc + b, d.DVc + b, d.A + b};
        for (void* p : dst4) {
            CK(cudaMemcpy(p, in, sizeof(float4) * cnt, cudaMemcpyHostToDevice));
            in += sizeof(float4) * cnt;
        }
        CK(cudaMemcpy(d.DKc + b, in, sizeof(float) * cnt, cudaMemcpyHostToDevice));
        in += sizeof(float) * cnt;
        CK(cudaMemcpy(d.PIDc + b, in, sizeof(uint32_t) * cnt, cudaMemcpyHostToDevice));
        in += sizeof(uint32_t) * cnt;
    }
    CK(cudaMemcpy(s->dScenes, cur.data(), sizeof(SceneDev) * cur.size(), cudaMemcpyHostToDevice));
    s->hScenes = cur;
    s->generation++;  // a recorded adjoint run no longer matches the state
    CK(cudaDeviceSynchronize());
    return VFD_OK;
}

int vfd_get_field(vfd_sim* s, int32_t field, uint32_t body, float* out) {
    TRY(check_sim(s));
    if (!out) return fail(VFD_E_ARG, "null output");
    CK(cudaSetDevice(s->device));
    TRY(ensure_ready(s));
    if (s->fp64Mode) {
        if (field == VFD_FIELD_DENSITY) return fp64_get_density(s, out);
        return fail(VFD_E_STATE, "the FP64 path exports positions, velocities, accelerations and densities");
    }
    CK(cudaStreamSynchronize(s->stream));
    const Dev& d = s->dev[s->cs];
    const uint32_t cnt = s->scenes[0].count();
    switch (field) {
        case VFD_FIELD_DENSITY: return scatter_scalar(s, 0, d.RHO, out);
        case VFD_FIELD_FACTOR: return scatter_scalar(s, 0, d.ALPHA, out);
        case VFD_FIELD_DENSITY_ADVECTION: return scatter_scalar(s, 0, d.RHOADV, out);
        case VFD_FIELD_PRESSURE_RHO2: return scatter_scalar(s, 0, d.KAPPA, out);
        case VFD_FIELD_PRESSURE_RHO2_V: return scatter_scalar(s, 0, d.KAPPAV, out);
        case VFD_FIELD_PRESSURE_RESIDUUM: return scatter_scalar(s, 0, d.RES, out);
        case VFD_FIELD_PRESSURE_ACCELERATION: return scatter_vec(s, 0, d.AP, out);
        case VFD_FIELD_VELOCITY_DIFFERENCE: return scatter_vec(s, 0, d.DVc, out);
        case VFD_FIELD_SURFACE_NORMAL: return scatter_vec(s, 0, d.STN, out);
        case VFD_FIELD_SURFACE_CURVATURE: return scatter_scalar(s, 0, nullptr, out, 3, d.STN);
        case VFD_FIELD_DELTA_FINAL_CURVATURE: return scatter_scalar(s, 0, d.DKc, out);
        case VFD_FIELD_SURFACE_NORMAL_SMOOTH: return scatter_vec(s, 0, d.STNS, out);
        case VFD_FIELD_SURFACE_CURVATURE_SMOOTH: return scatter_scalar(s, 0, nullptr, out, 3, d.STNS);
        case VFD_FIELD_BOUNDARY_XJ:
        case VFD_FIELD_BOUNDARY_VOLUME:
            if (body >= s->scenes[0].bodies.size()) return fail(VFD_E_ARG, "body %u out of range", body);
            if (field == VFD_FIELD_BOUNDARY_XJ) return scatter_pos(s, 0, d.XB + (size_t)body * s->stride, d.Xc, out);
            return scatter_scalar(s, 0, nullptr, out, 3, d.XB + (size_t)body * s->stride);
        default:
            (void)cnt;
            return fail(VFD_E_ARG, "unknown field %d", field);
    }
}

int vfd_find_neighbors(vfd_sim* s) {
    TRY(check_sim(s));
    if (s->fp64Mode) return fail(VFD_E_STATE, "vfd_find_neighbors is not available in the FP64 path");
    CK(cudaSetDevice(s->device));
    TRY(ensure_ready(s));
    if (s->n == 0) return VFD_OK;
    for (int attempt = 0; attempt < 8; attempt++) {
        const Dev& d = s->dev[s->cs];
        launch_search(d, s->stream);
        CK(cudaGetLastError());
        uint32_t flags = 0;
        TRY(finish_steps(s, nullptr, flags));
        if (s->hStatus[1]) {
            if (flags & 0x10u) return fail(VFD_E_NAN, "non-finite particle position");
            TRY(grow_cells(s));
            continue;
        }
        // the sorted set becomes the current state; positions follow the new order
        CK(cudaMemcpyAsync(d.XN, d.X, sizeof(float4) * s->n, cudaMemcpyDeviceToDevice, s->stream));
        CK(cudaStreamSynchronize(s->stream));
        s->cs = 1 - s->cs;
        return VFD_OK;
    }
    return fail(VFD_E_CAPACITY, "search grid too large");
}

int vfd_get_neighbors(vfd_sim* s, uint32_t* counts, uint32_t* offsets, uint32_t* list, uint32_t capacity,
                      uint32_t* total, uint32_t* sort_indices, uint32_t* cell_keys) {
    TRY(check_sim(s));
    CK(cudaSetDevice(s->device));
    TRY(ensure_ready(s));
    CK(cudaStreamSynchronize(s->stream));
    const Dev& d = s->dev[s->cs];
    const uint32_t cnt = s->scenes[0].count();
    std::vector<uint32_t> pid(cnt), ncnt(cnt), keys(cnt);
    CK(cudaMemcpy(pid.data(), d.PIDc, sizeof(uint32_t) * cnt, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(ncnt.data(), d.NCNT, sizeof(uint32_t) * cnt, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(keys.data(), d.KEYS, sizeof(uint32_t) * cnt, cudaMemcpyDeviceToHost));
    std::vector<SceneDev> sc(1);
    CK(cudaMemcpy(sc.data(), s->dScenes, sizeof(SceneDev), cudaMemcpyDeviceToHost));
    std::vector<uint32_t> c(cnt), off(cnt);
    for (uint32_t p = 0; p < cnt; p++) c[pid[p]] = ncnt[p] & kCountMask;
    uint64_t tot = 0;
    for (uint32_t i = 0; i < cnt; i++) {
        off[i] = (uint32_t)tot;
        tot += c[i];
    }
    if (total) *total = (uint32_t)tot;
    if (counts) std::copy(c.begin(), c.end(), counts);
    if (offsets) std::copy(off.begin(), off.end(), offsets);
    if (sort_indices) std::copy(pid.begin(), pid.end(), sort_indices);
    if (cell_keys)
        for (uint32_t p = 0; p < cnt; p++) cell_keys[pid[p]] = keys[p] - sc[0].cellBase;
    if (list) {
        if (tot > capacity) return fail(VFD_E_CAPACITY, "list needs %llu entries", (unsigned long long)tot);
        std::vector<uint32_t> rows((size_t)cnt * kRow);
        CK(cudaMemcpy(rows.data(), d.NBR, sizeof(uint32_t) * rows.size(), cudaMemcpyDeviceToHost));
        for (uint32_t p = 0; p < cnt; p++) {
            const uint32_t o = pid[p];
            for (uint32_t j = 0; j < c[o]; j++) list[off[o] + j] = pid[rows[(size_t)p * kRow + j]];
        }
    }
    return VFD_OK;
}

int vfd_get_info(const vfd_sim* s, vfd_info* info) {
    TRY(check_sim(s));
    if (!info) return fail(VFD_E_ARG, "null output");
    const vfd_desc& d = s->scenes[0].desc;
    SceneDev S = scene_constants(d, 0, s->scenes[0].count(), 0, (uint32_t)s->scenes[0].bodies.size());
    std::memset(info, 0, sizeof(*info));
    info->ParticleCount = S.count;
    info->RigidBodyCount = S.bodyCount;
    info->SupportRadius = S.h;
    info->SupportRadius2 = S.h2;
    info->ParticleRadius = S.r;
    info->ParticleDiameter = S.diam;
    float dt = S.dt;
    if (s->uploaded && !s->hScenes.empty()) dt = s->hScenes[0].dt;
    info->TimeStepSize = dt;
    info->TimeStepSize2 = dt * dt;
    info->TimeStepSizeInverse = 1.0f / dt;
    info->TimeStepSize2Inverse = 1.0f / (dt * dt);
    info->Volume = S.volume;
    info->Density0 = S.rho0;
    info->ParticleMass = S.mass;
    info->ParticleMassInverse = S.massInv;
    info->Viscosity = d.Viscosity;
    info->BoundaryViscosity = d.BoundaryViscosity;
    info->DynamicViscosity = S.dynVisc;
    info->DynamicBoundaryViscosity = S.dynBVisc;
    info->TangentialDistanceFactor = d.TangentialDistanceFactor;
    info->TangentialDistance = S.tangDist;
    info->SurfaceTension = S.st;
    info->SurfaceTensionSampleCount = S.stSamples;
    info->ClassifierSlope = S.slope;
    info->ClassifierConstant = S.constant;
    info->TemporalSmoothing = S.temporal;
    info->SmoothingFactor = S.smoothing;
    info->Factor = 0.8f;
    info->NeighborParticleRadius = S.nbrRadius;
    info->MonteCarloFactor = S.mcFactor;
    for (int k = 0; k < 3; k++) info->Gravity[k] = S.g[k];
    return VFD_OK;
}

int vfd_get_particle_count(const vfd_sim* s, uint32_t* n) {
    TRY(check_sim(s));
    if (!n) return fail(VFD_E_ARG, "null output");
    *n = s->scenes[0].count();
    return VFD_OK;
}

int vfd_scene_get_stats(vfd_sim* s, uint32_t scene, vfd_step_stats* st) {
    TRY(check_sim(s));
    if (!st) return fail(VFD_E_ARG, "null output");
    if (scene >= s->scenes.size()) return fail(VFD_E_ARG, "scene %u out of range", scene);
    CK(cudaSetDevice(s->device));
    std::memset(st, 0, sizeof(*st));
    if (!s->uploaded) return VFD_OK;
    if (s->fp64Mode) {
        fp64_stats(s, st);
        return VFD_OK;
    }
    CK(cudaStreamSynchronize(s->stream));
    SceneDev S;
    CK(cudaMemcpy(&S, s->dScenes + scene, sizeof(SceneDev), cudaMemcpyDeviceToHost));
    fill_stats(S, st);
    return VFD_OK;
}

int vfd_get_debug_info(vfd_sim* s, vfd_step_stats* st) { return vfd_scene_get_stats(s, 0, st); }

int vfd_get_current_time_step_size(vfd_sim* s, float* dt) {
    vfd_step_stats st;
    TRY(vfd_scene_get_stats(s, 0, &st));
    if (!dt) return fail(VFD_E_ARG, "null output");
    *dt = s->uploaded ? st.TimeStepSize : s->scenes[0].desc.TimeStepSize;
    return VFD_OK;
}

int vfd_get_max_velocity_magnitude(vfd_sim* s, float* v2) {
    vfd_step_stats st;
    TRY(vfd_scene_get_stats(s, 0, &st));
    if (!v2) return fail(VFD_E_ARG, "null output");
    *v2 = st.MaxVelocityMagnitude;
    return VFD_OK;
}

int vfd_get_kernel_table(const vfd_sim* s, float* w, float* grad_w, float* radius, float* w_zero) {
    TRY(check_sim(s));
    if (w) std::copy(s->table.W.begin(), s->table.W.end(), w);
    if (grad_w) std::copy(s->table.G.begin(), s->table.G.end(), grad_w);
    if (radius) *radius = s->table.radius;
    if (w_zero) *w_zero = s->table.wZero;
    return VFD_OK;
}

// Device ring, pinned host ring, step notes and events of one vfd_simulate call.
struct FramePipe {
    static constexpr uint32_t kSlots = 4;      // frames in the rings
    static constexpr uint32_t kLookahead = 3;  // steps in flight ahead of the host (<= kSlots)
    float* dRing = nullptr;
    float* hRing = nullptr;
    FrameNote* dNotes = nullptr;
    FrameNote* hNotes = nullptr;
    cudaStream_t copy = nullptr;
    cudaStream_t main = nullptr;  // the simulation's stream
    uint32_t* status = nullptr;   // its status words
    cudaEvent_t stepDone[kLookahead] = {};
    cudaEvent_t copyDone[kSlots] = {};
    ~FramePipe() {
        // nothing of this call may still run when its buffers go; a stop word (2) left by
        // an early return would turn the simulation's next steps into no-ops
        if (main) cudaStreamSynchronize(main);
        if (copy) cudaStreamSynchronize(copy);
        if (status) {
            uint32_t w = 0;
            if (cudaMemcpy(&w, status + 1, sizeof(w), cudaMemcpyDeviceToHost) == cudaSuccess && w == 2u)
                cudaMemset(status + 1, 0, sizeof(uint32_t));
        }
        cudaFree(dRing);
        cudaFreeHost(hRing);
        cudaFree(dNotes);
        cudaFreeHost(hNotes);
        for (auto& e : stepDone)
            if (e) cudaEventDestroy(e);
        for (auto& e : copyDone)
            if (e) cudaEventDestroy(e);
        if (copy) cudaStreamDestroy(copy);
    }
};

// DFSPHImplementation::Simulate (DFSPHImplementation.cu:33-61): from the initial state,
// steps until FrameCount frames are complete, handing each frame to `cb`. The steps are
// queued up to FramePipe::kLookahead ahead of the host; a frame is copied from the device
// ring to pinned memory on a second stream while the next steps run, and `cb` runs on
// the calling thread, in frame order, once its copy has landed.
int vfd_simulate(vfd_sim* s, vfd_frame_callback cb, void* user) {
    TRY(check_sim(s));
    if (s->fp64Mode) return fail(VFD_E_STATE, "vfd_simulate is not available in the FP64 path");
    if (s->scenes.size() != 1) return fail(VFD_E_ARG, "vfd_simulate runs single-scene simulations");
    CK(cudaSetDevice(s->device));
    TRY(upload(s));
    const uint32_t n = s->scenes[0].count();
    const uint32_t frames = s->scenes[0].desc.FrameCount;
    if (frames == 0 || n == 0) return VFD_OK;
    TRY(ensure_ready(s));
    constexpr uint32_t R = FramePipe::kSlots, L = FramePipe::kLookahead;
    FramePipe fp;
    fp.main = s->stream;
    fp.status = s->dStatus;
    const size_t frameFloats = 9 * (size_t)n;
    CK(cudaMalloc(&fp.dRing, sizeof(float) * frameFloats * R));
    CK(cudaMallocHost(&fp.hRing, sizeof(float) * frameFloats * R));
    CK(cudaMalloc(&fp.dNotes, sizeof(FrameNote) * L));
    CK(cudaMallocHost(&fp.hNotes, sizeof(FrameNote) * L));
    CK(cudaStreamCreateWithFlags(&fp.copy, cudaStreamNonBlocking));
    for (auto& e : fp.stepDone) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    for (auto& e : fp.copyDone) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    CK(cudaMemsetAsync(s->dStatus + 7, 0, sizeof(uint32_t), s->stream));

    struct Pending {
        uint32_t frame;
        float maxV, dt;
    };
    std::vector<Pending> pending;  // frames copied or being copied, in order
    auto deliver = [&](bool wait, uint32_t upTo) -> int {
        size_t k = 0;
        for (; k < pending.size(); k++) {
            const Pending& f = pending[k];
            const uint32_t slot = (f.frame - 1u) % R;
            if (wait || f.frame <= upTo) {
                CK(cudaEventSynchronize(fp.copyDone[slot]));
            } else {
                const cudaError_t q = cudaEventQuery(fp.copyDone[slot]);
                if (q == cudaErrorNotReady) break;
                CK(q);
            }
            if (cb) {
                const float* base = fp.hRing + slot * frameFloats;
                cb(f.frame - 1u, n, base, base + 3 * (size_t)n, base + 6 * (size_t)n, f.maxV, f.dt, user);
            }
        }
        pending.erase(pending.begin(), pending.begin() + k);
        return VFD_OK;
    };
    // the completed-step count decides which state set holds the result (aborted steps
    // leave it where it was)
    auto settle = [&](int cs0) -> int {
        CK(cudaStreamSynchronize(s->stream));
        CK(cudaMemcpy(s->hStatus, s->dStatus, 16 * sizeof(uint32_t), cudaMemcpyDeviceToHost));
        s->cs = (s->hStatus[7] & 1u) ? 1 - cs0 : cs0;
        CK(cudaMemset(s->dStatus + 7, 0, sizeof(uint32_t)));
        return VFD_OK;
    };

    uint64_t launched = 0, processed = 0;
    int cs0 = s->cs;
    bool stop = false, searchAbort = false, finished = false;
    for (uint64_t guard = 0; guard < 100000000ull && !finished; guard++) {
        while (!stop && launched - processed < L) {
            for (uint32_t r = 0; r < R; r++) CK(cudaStreamWaitEvent(s->stream, fp.copyDone[r], 0));
            TRY(launch_one(s));
            const Dev& d = s->dev[s->cs];
            const uint32_t k = (uint32_t)(launched % L);
            k_frame_snapshot<<<blocks_for(n, 256), 256, 0, s->stream>>>(d, fp.dRing, R, n);
            k_frame_note<<<1, 32, 0, s->stream>>>(d, fp.dNotes + k, frames);
            CK(cudaGetLastError());
            CK(cudaMemcpyAsync(fp.hNotes + k, fp.dNotes + k, sizeof(FrameNote), cudaMemcpyDeviceToHost, s->stream));
            CK(cudaEventRecord(fp.stepDone[k], s->stream));
            launched++;
        }
        if (processed < launched) {
            const uint32_t k = (uint32_t)(processed % L);
            CK(cudaEventSynchronize(fp.stepDone[k]));
            const FrameNote note = fp.hNotes[k];
            processed++;
            if (note.aborted == 1u && !stop) {
                searchAbort = true;  // the search aborted: drain, grow the cell table, go on
                stop = true;
            } else if (note.due) {
                const uint32_t slot = (note.index - 1u) % R;
                TRY(deliver(false, note.index > R ? note.index - R : 0u));  // the host slot is free
                CK(cudaStreamWaitEvent(fp.copy, fp.stepDone[k], 0));
                CK(cudaMemcpyAsync(fp.hRing + slot * frameFloats, fp.dRing + slot * frameFloats,
                                   sizeof(float) * frameFloats, cudaMemcpyDeviceToHost, fp.copy));
                CK(cudaEventRecord(fp.copyDone[slot], fp.copy));
                pending.push_back({note.index, note.maxV, note.dt});
                if (note.index >= frames) stop = true;
            }
            TRY(deliver(false, 0u));
        }
        if (stop && processed == launched) {
            TRY(settle(cs0));
            if (!searchAbort) {
                finished = true;
                break;
            }
            if (s->hStatus[0] & 0x10u) return fail(VFD_E_NAN, "non-finite particle position");
            CK(cudaMemset(s->dStatus + 1, 0, sizeof(uint32_t)));
            TRY(grow_cells(s));
            cs0 = s->cs;
            stop = searchAbort = false;
        }
    }
    TRY(deliver(true, 0u));
    if (!finished) return fail(VFD_E_STATE, "frame clock did not advance");
    return VFD_OK;
}

int vfd_profile_kernels(vfd_sim* s, uint32_t steps, vfd_kernel_time* out, uint32_t capacity, uint32_t* count) {
    TRY(check_sim(s));
    if (s->fp64Mode) return fail(VFD_E_STATE, "vfd_profile_kernels is not available in the FP64 path");
    CK(cudaSetDevice(s->device));
    TRY(ensure_ready(s));
    if (count) *count = 0;
    if (s->n == 0 || steps == 0) return VFD_OK;
    EventProfiler prof;
    int rc = VFD_OK;
    g_profiler = &prof;
    for (uint32_t k = 0; k < steps && rc == VFD_OK; k++) {
        rc = launch_eager(s);
        if (rc == VFD_OK) s->cs = 1 - s->cs;
    }
    g_profiler = nullptr;
    TRY(rc);
    uint32_t flags = 0;
    TRY(finish_steps(s, nullptr, flags));
    const uint32_t completed = s->hStatus[7];
    CK(cudaMemsetAsync(s->dStatus + 7, 0, sizeof(uint32_t), s->stream));
    if (s->hStatus[1] || completed != steps) return fail(VFD_E_STATE, "a profiled step aborted; run vfd_step first");
    if (prof.err != cudaSuccess) return fail(VFD_E_CUDA, "event creation: %s", cudaGetErrorString(prof.err));
    std::vector<vfd_kernel_time> acc;
    for (const auto& r : prof.recs) {
        float ms = 0.0f;
        CK(cudaEventElapsedTime(&ms, r.a, r.b));
        auto it = std::find_if(acc.begin(), acc.end(), [&](const vfd_kernel_time& t) { return r.name == t.name; });
        if (it == acc.end()) {
            vfd_kernel_time t;
            std::memset(&t, 0, sizeof(t));
            std::snprintf(t.name, sizeof(t.name), "%s", r.name.c_str());
            acc.push_back(t);
            it = acc.end() - 1;
        }
        it->launches++;
        it->total_ms += ms;
    }
    if (count) *count = (uint32_t)std::min<size_t>(acc.size(), capacity);
    if (out) std::copy(acc.begin(), acc.begin() + std::min<size_t>(acc.size(), capacity), out);
    return VFD_OK;
}

int vfd_set_lanes(vfd_sim* s, const uint8_t* lanes, uint32_t count) {
    TRY(check_sim(s));
    if (!lanes || count == 0 || count > 16) return fail(VFD_E_ARG, "lanes: 1..16 entries");
    for (uint32_t k = 0; k < count; k++)
        if (lanes[k] != 4 && lanes[k] != 8 && lanes[k] != 16) return fail(VFD_E_ARG, "lanes must be 4, 8 or 16");
    std::memcpy(s->lanes, lanes, count);
    for (int k = 0; k < 2; k++) std::memcpy(s->dev[k].lanes, s->lanes, sizeof(s->lanes));
    s->releaseGraphs();
    return VFD_OK;
}

int vfd_get_lanes(const vfd_sim* s, uint8_t* lanes, uint32_t count) {
    TRY(check_sim(s));
    if (!lanes || count == 0 || count > 16) return fail(VFD_E_ARG, "lanes: 1..16 entries");
    std::memcpy(lanes, s->lanes, count);
    return VFD_OK;
}

int vfd_set_tiles(vfd_sim* s, const uint8_t* tiles, uint32_t count) {
    TRY(check_sim(s));
    if (!tiles || count == 0 || count > kTunedCount) return fail(VFD_E_ARG, "tiles: 1..%d values", (int)kTunedCount);
    for (uint32_t k = 0; k < count; k++)
        if (tiles[k] != 0 && tiles[k] != kRowsNoStream && tiles[k] != 3 && tiles[k] != 4)
            return fail(VFD_E_ARG, "pass form must be 0 (neighbour rows), 1 (rows, gradW recomputed), 3 (2x2x2 tiles) "
                                   "or 4 (4x2x2 tiles)");
    std::memcpy(s->tiles, tiles, count);
    for (int k = 0; k < 2; k++) {
        std::memcpy(s->dev[k].tiles, s->tiles, sizeof(s->tiles));
        s->dev[k].compactRows = uses_tiles(s->tiles) ? 1u : 0u;
    }
    s->releaseGraphs();
    return VFD_OK;
}

int vfd_set_blocks(vfd_sim* s, const uint16_t* blocks, uint32_t count) {
    TRY(check_sim(s));
    if (!blocks || count == 0 || count > kTunedCount) return fail(VFD_E_ARG, "blocks: 1..%d values", (int)kTunedCount);
    for (uint32_t k = 0; k < count; k++)
        if (blocks[k] != 64 && blocks[k] != 128 && blocks[k] != 256)
            return fail(VFD_E_ARG, "threads per block must be 64, 128 or 256");
    std::memcpy(s->blocks, blocks, count * sizeof(uint16_t));
    for (int k = 0; k < 2; k++) std::memcpy(s->dev[k].blocks, s->blocks, sizeof(s->blocks));
    s->releaseGraphs();
    return VFD_OK;
}

int vfd_get_blocks(const vfd_sim* s, uint16_t* blocks, uint32_t count) {
    TRY(check_sim(s));
    if (!blocks) return fail(VFD_E_ARG, "null output");
    for (uint32_t k = 0; k < std::min<uint32_t>(count, 16); k++) blocks[k] = s->blocks[k] ? s->blocks[k] : (uint16_t)kBlock;
    return VFD_OK;
}

int vfd_get_tiles(const vfd_sim* s, uint8_t* tiles, uint32_t count) {
    TRY(check_sim(s));
    if (!tiles) return fail(VFD_E_ARG, "null output");
    std::memcpy(tiles, s->tiles, std::min<uint32_t>(count, 16));
    return VFD_OK;
}

int vfd_autotune(vfd_sim* s, uint32_t steps, uint8_t* lanes_out, uint32_t count) {
    TRY(check_sim(s));
    if (s->fp64Mode) return fail(VFD_E_STATE, "vfd_autotune is not available in the FP64 path");
    CK(cudaSetDevice(s->device));
    TRY(ensure_ready(s));
    if (s->n == 0 || steps == 0) return VFD_OK;
    static const char* names[kTunedCount] = {"k_density_factor", "k_pressure_accel", "k_jacobi_iter",
                                             "k_div_finish", "k_st_classify", "k_st_smooth", "k_visc_precond",
                                             "k_visc_setup", "k_cg_spmv", "k_pres_init", "k_pres_finish"};
    const uint8_t cand[3] = {4, 8, 16};
    // snapshot of everything a step carries: positions, the current state set, scenes
    const size_t st = s->stride;
    const int cs0 = s->cs;
    const Dev d0 = s->dev[cs0];
    float4 *xn = nullptr, *v = nullptr, *dv = nullptr, *acc = nullptr;
    float* dk = nullptr;
    uint32_t* pid = nullptr;
    SceneDev* sc = nullptr;
    uint32_t* stat = nullptr;
    auto release = [&]() {
        cudaFree(xn); cudaFree(v); cudaFree(dv); cudaFree(acc); cudaFree(dk); cudaFree(pid); cudaFree(sc);
        cudaFree(stat);
    };
    cudaError_t e = cudaMalloc(&xn, sizeof(float4) * st);
    if (e == cudaSuccess) e = cudaMalloc(&v, sizeof(float4) * st);
    if (e == cudaSuccess) e = cudaMalloc(&dv, sizeof(float4) * st);
    if (e == cudaSuccess) e = cudaMalloc(&acc, sizeof(float4) * st);
    if (e == cudaSuccess) e = cudaMalloc(&dk, sizeof(float) * st);
    if (e == cudaSuccess) e = cudaMalloc(&pid, sizeof(uint32_t) * st);
    if (e == cudaSuccess) e = cudaMalloc(&sc, sizeof(SceneDev) * s->hScenes.size());
    if (e == cudaSuccess) e = cudaMalloc(&stat, sizeof(uint32_t) * 16);
    auto copy_all = [&](bool save) -> cudaError_t {
        cudaError_t r = cudaSuccess;
        auto cp = [&](void* a, void* b, size_t bytes) {
            if (r == cudaSuccess) r = cudaMemcpyAsync(save ? a : b, save ? b : a, bytes, cudaMemcpyDeviceToDevice, s->stream);
        };
        cp(xn, d0.XN, sizeof(float4) * st);
        cp(v, d0.Vc, sizeof(float4) * st);
        cp(dv, d0.DVc, sizeof(float4) * st);
        cp(acc, d0.A, sizeof(float4) * st);
        cp(dk, d0.DKc, sizeof(float) * st);
        cp(pid, d0.PIDc, sizeof(uint32_t) * st);
        cp(sc, s->dScenes, sizeof(SceneDev) * s->hScenes.size());
        cp(stat, s->dStatus, sizeof(uint32_t) * 16);
        if (r == cudaSuccess) r = cudaStreamSynchronize(s->stream);
        return r;
    };
    if (e == cudaSuccess) e = copy_all(true);
    if (e != cudaSuccess) {
        release();
        return fail(VFD_E_CUDA, "autotune snapshot: %s", cudaGetErrorString(e));
    }
    // every lane count with every form of the three solver-loop passes (the others ignore it)
    constexpr int kForms = 4;
    const uint8_t tileCand[kForms] = {0, kRowsNoStream, 3, 4};  // rows, rows without the gradient
                                                                // stream, 2x2x2 and 4x2x2 tiles
    const uint16_t blockCand[3] = {128, 64, 256};  // threads per block of the row kernels
    double times[kTunedCount][3][kForms][3] = {};  // [kernel][lanes][form][block]
    int rc = VFD_OK;
    for (int ct = 0; ct < 3 * kForms * 3 && rc == VFD_OK; ct++) {
        const int c = ct % 3, tl = (ct / 3) % kForms, bs = ct / (3 * kForms);
        for (int k = 0; k < 2; k++) {
            for (int t = 0; t < kTunedCount; t++) {
                s->dev[k].lanes[t] = cand[c];
                s->dev[k].tiles[t] = tileCand[tl];
                s->dev[k].blocks[t] = blockCand[bs];
            }
            s->dev[k].compactRows = tileCand[tl] >= kTileMinLog2 ? 1u : 0u;
        }
        EventProfiler prof;
        g_profiler = &prof;
        for (uint32_t k = 0; k < steps && rc == VFD_OK; k++) {
            rc = launch_eager(s);
            if (rc == VFD_OK) s->cs = 1 - s->cs;
        }
        g_profiler = nullptr;
        if (rc == VFD_OK) {
            cudaError_t r = cudaStreamSynchronize(s->stream);
            if (r != cudaSuccess) rc = fail(VFD_E_CUDA, "autotune: %s", cudaGetErrorString(r));
        }
        for (const auto& rec : prof.recs) {
            float ms = 0.0f;
            if (rc == VFD_OK && cudaEventElapsedTime(&ms, rec.a, rec.b) == cudaSuccess)
                for (int t = 0; t < kTunedCount; t++)
                    if (rec.name == names[t]) times[t][c][tl][bs] += ms;
        }
        s->cs = cs0;
        e = copy_all(false);
        if (e != cudaSuccess && rc == VFD_OK) rc = fail(VFD_E_CUDA, "autotune restore: %s", cudaGetErrorString(e));
    }
    release();
    if (rc != VFD_OK) {
        for (int k = 0; k < 2; k++) {
            std::memcpy(s->dev[k].lanes, s->lanes, sizeof(s->lanes));
            std::memcpy(s->dev[k].tiles, s->tiles, sizeof(s->tiles));
            std::memcpy(s->dev[k].blocks, s->blocks, sizeof(s->blocks));
            s->dev[k].compactRows = uses_tiles(s->tiles) ? 1u : 0u;
        }
        return rc;
    }
    for (int t = 0; t < kTunedCount; t++) {
        const bool tileable = t == kTPAccel || t == kTJacobi || t == kTSpmv;
        // A configuration is (lanes c, form tl, block bs). Kernels without forms ran the same
        // code in all the form runs: their cost is the sum of those; tile kernels run
        // kTileBlock threads whatever bs, so their block choice stays the default.
        auto cost = [&](int c, int tl, int bs) {
            if (tileable) return times[t][c][tl][bs];
            double sum = 0.0;
            for (int f = 0; f < kForms; f++) sum += times[t][c][f][bs];
            return sum;
        };
        int best = 1, bestTile = 0, bestBlock = 0;
        double bt = cost(1, 0, 0);
        for (int c = 0; c < 3; c++)
            for (int tl = 0; tl < (tileable ? kForms : 1); tl++)
                for (int bs = 0; bs < 3; bs++) {
                    const double v = cost(c, tl, bs);
                    if (v > 0.0 && v < bt) {
                        bt = v;
                        best = c;
                        bestTile = tl;
                        bestBlock = bs;
                    }
                }
        s->lanes[t] = cand[best];
        s->tiles[t] = tileable ? tileCand[bestTile] : 0;
        s->blocks[t] = tileCand[bestTile] < kTileMinLog2 ? blockCand[bestBlock] : 0;
    }
    for (int k = 0; k < 2; k++) {
        std::memcpy(s->dev[k].lanes, s->lanes, sizeof(s->lanes));
        std::memcpy(s->dev[k].tiles, s->tiles, sizeof(s->tiles));
        std::memcpy(s->dev[k].blocks, s->blocks, sizeof(s->blocks));
        s->dev[k].compactRows = uses_tiles(s->tiles) ? 1u : 0u;
    }
    s->releaseGraphs();
    if (lanes_out) std::memcpy(lanes_out, s->lanes, std::min<uint32_t>(count, 16));
    return VFD_OK;
}

int vfd_get_stream(vfd_sim* s, void** stream) {
    TRY(check_sim(s));
    if (!stream) return fail(VFD_E_ARG, "null output");
    *stream = (void*)s->stream;
    return VFD_OK;
}

int vfd_get_launch_count(vfd_sim* s, uint64_t* launches, int32_t reset) {
    TRY(check_sim(s));
    if (!launches) return fail(VFD_E_ARG, "null output");
    CK(cudaSetDevice(s->device));
    *launches = 0;
    if (!s->allocated) return VFD_OK;
    uint32_t v = 0;
    TRY(read_flag(s, 8, v));
    *launches = v;
    if (reset) CK(cudaMemsetAsync(s->dStatus + 8, 0, sizeof(uint32_t), s->stream));
    return VFD_OK;
}

}  // extern "C"
