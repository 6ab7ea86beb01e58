// Rigid-body boundary of the DFSPH step.
//   * k_boundary: ComputeVolumeAndBoundaryKernel (Simulation/DFSPH/DFSPHKernels.cu:69-150)
//     with the volume-map lookup of SDFDeviceData (Utility/SDF/SDFDeviceData.cuh:36-474):
//     one pass evaluates the 32 cubic serendipity shape functions and their gradients
//     on the fly and accumulates distance, distance gradient and volume together.
#include <cfloat>
#include <climits>
#include <cmath>
#include <vector>

#include "dfsph_common.cuh"
#include "dfsph_map.cuh"

namespace vfd {

// K1: ComputeVolumeAndBoundaryKernel (DFSPHKernels.cu:69-150).
template <bool REL>
__global__ void __launch_bounds__(kBlock) k_boundary(Dev d) {
    VFD_COUNT_LAUNCH(d);
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= d.n || is_aborted(d)) return;
    const SceneDev& S = d.scenes[scene_of(d, p)];
    uint32_t flags = d.NCNT[p] & ~kHasBoundary;
    if (S.bodyCount == 0) {
        d.NCNT[p] = flags;
        return;
    }
    float4 x4 = d.X[p];
    // x: the particle in its own frame (absolute, or its cell offset when positions are
    // cell-relative; the boundary samples are stored in that frame); xa: absolute, for
    // the map lookups
    // (with cell-relative positions the lookups take the position relative to the map's
    // corner, (origin - corner) + (anchor cell + offset), the first difference exact)
    float3 x = f3(x4);
    float3 xa = abs_pos(d, S, x4);
    float3 cell = make_float3(0.f, 0.f, 0.f);
    if (REL) {
        const int3 A = anchor_of(x4.w);
        cell = make_float3(d.radius * (float)A.x + x.x, d.radius * (float)A.y + x.y, d.radius * (float)A.z + x.z);
    }
    bool moved = false, stopped = false, any = false;
    for (uint32_t b = 0; b < S.bodyCount; b++) {
        const BodyDev& m = d.bodies[S.bodyBegin + b];
        float3 xb = make_float3(0.f, 0.f, 0.f);
        float vb = 0.0f;
        const MapSample s =
            REL ? map_lookup_rel(m, make_float3(S.org[0] - m.dmin[0], S.org[1] - m.dmin[1], S.org[2] - m.dmin[2]) + cell)
                : map_lookup(m, xa);
        const float dist = s.inside ? s.phi0 : FLT_MAX;
        float3 normal = s.grad0;
        if (dist > 0.0f && dist < S.h) {
            const float volume = s.phi1;
            if (volume > 0.0f && volume != FLT_MAX) {
                vb = volume;
                const float nl = sqrtf(dot3(normal, normal));
                if (nl > 1.0e-9f) {
                    normal = make_float3(normal.x / nl, normal.y / nl, normal.z / nl);
                    const float pd = fmaxf(dist + 0.5f * S.r, S.diam);
                    xb = x - pd * normal;
                } else {
                    vb = 0.0f;
                }
            }
        } else if (dist <= 0.0f) {
            const float nl = sqrtf(dot3(normal, normal));
            if (nl > 1.0e-5f) {
                normal = make_float3(normal.x / nl, normal.y / nl, normal.z / nl);
                const float delta = fminf(S.diam - dist, 0.1f * S.r);
                x += delta * normal;
                xa += delta * normal;
                cell += delta * normal;
                moved = true;
                stopped = true;
            }
        }
        d.XB[(size_t)b * d.stride + p] = f4(xb, vb);
        any |= vb > 0.0f;
    }
    if (moved) d.X[p] = f4(x, x4.w);
    if (stopped) d.V[p] = make_float4(0.f, 0.f, 0.f, 0.f);
    d.NCNT[p] = flags | (any ? kHasBoundary : 0u);
}

// (one instantiation per position storage mode, so that the absolute one compiles to the
// same arithmetic as before the cell-relative mode existed)
void launch_boundary(const Dev& d, cudaStream_t s) {
    if (d.cellRel) VFD_LAUNCH("k_boundary", s, k_boundary<true><<<blocks_for(d.n), kBlock, 0, s>>>(d));
    else VFD_LAUNCH("k_boundary", s, k_boundary<false><<<blocks_for(d.n), kBlock, 0, s>>>(d));
}

}  // namespace vfd
