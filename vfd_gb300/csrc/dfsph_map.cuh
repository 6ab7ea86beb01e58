// Volume-map lookup of SDFDeviceData (Utility/SDF/SDFDeviceData.cuh:36-474): the
// 32-node cubic serendipity element, evaluated on the fly with its gradients.
// Shared by the boundary kernel of the step and by its adjoint.
#pragma once

#include <climits>

#include "dfsph_common.cuh"

namespace vfd {

// Shape function k (0..31) of the 32-node cubic serendipity element at xi and its
// gradient in xi space: corners (1/64)(1+-x)(1+-y)(1+-z)(9|xi|^2 - 19), edge nodes
// (9/64)(1-t^2)(1-+3t)(1+-u)(1+-w); node numbering of SDFDeviceData::ShapeFunction.
template <int K>
__device__ __forceinline__ void shape_k(float x, float y, float z, float base, float& N, float3& dN) {
    if (K < 8) {
        const float sx = (K & 1) ? 1.f : -1.f, sy = (K & 2) ? 1.f : -1.f, sz = (K & 4) ? 1.f : -1.f;
        const float ax = 1.f + sx * x, ay = 1.f + sy * y, az = 1.f + sz * z;
        const float axyz = ax * ay * az;
        N = axyz * base * (1.0f / 64.0f);
        dN = make_float3((sx * ay * az * base + axyz * 18.f * x) * (1.0f / 64.0f),
                         (sy * ax * az * base + axyz * 18.f * y) * (1.0f / 64.0f),
                         (sz * ax * ay * base + axyz * 18.f * z) * (1.0f / 64.0f));
    } else {
        constexpr int t = (K - 8) / 8, kk = (K - 8) % 8;
        constexpr int a = kk & 1, bu = (kk >> 1) & 1, bw = (kk >> 2) & 1;
        constexpr int U = t == 0 ? 2 : (t == 1 ? 0 : 1);
        constexpr int W = t == 0 ? 1 : (t == 1 ? 2 : 0);
        const float v[3] = {x, y, z};
        const float tv = v[t], uv = v[U], wv = v[W];
        const float sa = a ? 3.f : -3.f, su = bu ? 1.f : -1.f, sw = bw ? 1.f : -1.f;
        const float ft = (1.f - tv * tv) * (1.f + sa * tv);
        const float dft = -2.f * tv * (1.f + sa * tv) + sa * (1.f - tv * tv);
        const float fu = 1.f + su * uv, fw = 1.f + sw * wv;
        const float c = 9.0f / 64.0f;
        N = c * ft * fu * fw;
        float g[3];
        g[t] = c * dft * fu * fw;
        g[U] = c * ft * su * fw;
        g[W] = c * ft * fu * sw;
        dN = make_float3(g[0], g[1], g[2]);
    }
}

struct MapSample {
    bool inside;
    float phi0, phi1;
    float3 grad0;
    float3 grad1;  // gradient of field 1, accumulated only by map_lookup<true>
};

template <int K, bool GRAD1>
__device__ __forceinline__ void accumulate_node(const BodyDev& m, const uint32_t* cell, float x, float y, float z,
                                                float base, MapSample& s) {
    float N;
    float3 dN;
    shape_k<K>(x, y, z, base, N, dN);
    const uint32_t v = __ldg(cell + K);
    const float c0 = __ldg(m.nodes + v);
    const float c1 = __ldg(m.nodes + m.nodeCount + v);
    s.phi0 += c0 * N;
    s.grad0 += c0 * dN;
    s.phi1 += c1 * N;
    if (GRAD1) s.grad1 += c1 * dN;
}

template <int K, bool GRAD1>
struct NodeLoop {
    __device__ __forceinline__ static void run(const BodyDev& m, const uint32_t* cell, float x, float y, float z,
                                               float base, MapSample& s) {
        NodeLoop<K - 1, GRAD1>::run(m, cell, x, y, z, base, s);
        accumulate_node<K - 1, GRAD1>(m, cell, x, y, z, base, s);
    }
};
template <bool GRAD1>
struct NodeLoop<0, GRAD1> {
    __device__ __forceinline__ static void run(const BodyDev&, const uint32_t*, float, float, float, float,
                                               MapSample&) {}
};

// DetermineShapeFunction + Interpolate (field 0 with gradient, field 1, and with
// GRAD1 the gradient of field 1 too) of one body.
template <bool GRAD1 = false>
__device__ __forceinline__ MapSample map_lookup(const BodyDev& m, float3 p) {
    MapSample s;
    s.inside = false;
    s.phi0 = s.phi1 = 0.0f;
    s.grad0 = make_float3(0.f, 0.f, 0.f);
    s.grad1 = make_float3(0.f, 0.f, 0.f);
    const float x[3] = {p.x, p.y, p.z};
    uint32_t mi[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        if (!(m.dmin[k] <= x[k] && m.dmax[k] >= x[k])) return s;
        mi[k] = (uint32_t)(m.csi[k] * (x[k] - m.dmin[k]));
        if (mi[k] >= m.res[k]) mi[k] = m.res[k] - 1u;
    }
    const uint32_t i = m.res[1] * m.res[0] * mi[2] + m.res[0] * mi[1] + mi[0];
    const uint32_t j = __ldg(m.cellMap + i);
    if (j == UINT_MAX) return s;
    float c0[3], xi[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const float lo = m.dmin[k] + (float)mi[k] * m.cs[k];
        const float hi = lo + m.cs[k];
        const float den = hi - lo;
        c0[k] = 2.0f / den;
        xi[k] = c0[k] * x[k] - (hi + lo) / den;
    }
    const float base = 9.f * (xi[0] * xi[0] + xi[1] * xi[1] + xi[2] * xi[2]) - 19.f;
    NodeLoop<32, GRAD1>::run(m, m.cells + (size_t)j * 32u, xi[0], xi[1], xi[2], base, s);
    s.grad0 = make_float3(s.grad0.x * c0[0], s.grad0.y * c0[1], s.grad0.z * c0[2]);
    if (GRAD1) s.grad1 = make_float3(s.grad1.x * c0[0], s.grad1.y * c0[1], s.grad1.z * c0[2]);
    s.inside = true;
    return s;
}

// The same lookup for a position given relative to the map's domain corner (p - dmin),
// so that its precision is that of the offset rather than of the absolute coordinates.
template <bool GRAD1 = false>
__device__ __forceinline__ MapSample map_lookup_rel(const BodyDev& m, float3 prel) {
    MapSample s;
    s.inside = false;
    s.phi0 = s.phi1 = 0.0f;
    s.grad0 = make_float3(0.f, 0.f, 0.f);
    s.grad1 = make_float3(0.f, 0.f, 0.f);
    const float x[3] = {prel.x, prel.y, prel.z};
    uint32_t mi[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        if (!(0.0f <= x[k] && m.dmax[k] - m.dmin[k] >= x[k])) return s;
        mi[k] = (uint32_t)(m.csi[k] * x[k]);
        if (mi[k] >= m.res[k]) mi[k] = m.res[k] - 1u;
    }
    const uint32_t i = m.res[1] * m.res[0] * mi[2] + m.res[0] * mi[1] + mi[0];
    const uint32_t j = __ldg(m.cellMap + i);
    if (j == UINT_MAX) return s;
    float c0[3], xi[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        c0[k] = 2.0f / m.cs[k];
        xi[k] = c0[k] * (x[k] - (float)mi[k] * m.cs[k]) - 1.0f;
    }
    const float base = 9.f * (xi[0] * xi[0] + xi[1] * xi[1] + xi[2] * xi[2]) - 19.f;
    NodeLoop<32, GRAD1>::run(m, m.cells + (size_t)j * 32u, xi[0], xi[1], xi[2], base, s);
    s.grad0 = make_float3(s.grad0.x * c0[0], s.grad0.y * c0[1], s.grad0.z * c0[2]);
    if (GRAD1) s.grad1 = make_float3(s.grad1.x * c0[0], s.grad1.y * c0[1], s.grad1.z * c0[2]);
    s.inside = true;
    return s;
}

}  // namespace vfd
