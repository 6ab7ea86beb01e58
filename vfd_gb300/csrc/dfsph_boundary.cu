// Rigid-body boundary of the DFSPH step.
//   * k_boundary: ComputeVolumeAndBoundaryKernel (Simulation/DFSPH/DFSPHKernels.cu:69-150)
//     with the volume-map lookup of SDFDeviceData (Utility/SDF/SDFDeviceData.cuh:36-474):
//     one pass evaluates the 32 cubic serendipity shape functions and their gradients
//     on the fly and accumulates distance, distance gradient and volume together.
//   * the box volume-map builder: RigidBody::RigidBody (RigidBody/RigidBody.cu:10-72) for
//     an axis-aligned box, i.e. SDF::AddFunction (Utility/SDF/SDF.cu:45-139) of the
//     signed distance and of the 16^3-point Gauss-Legendre boundary volume
//     (Core/Math/GaussQuadrature.cpp:5621-5656), one warp per map node.
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
    if (d.cellRel) k_boundary<true><<<blocks_for(d.n), kBlock, 0, s>>>(d);
    else k_boundary<false><<<blocks_for(d.n), kBlock, 0, s>>>(d);
}

// ---------------------------------------------------------------- box map builder
struct BoxMap {
    float dmin[3], dmax[3], cs[3], csi[3];
    uint32_t res[3];
    uint32_t nodeCount, cellCount;
    float bmin[3], bmax[3];
    float sign, tol, h;
    float w[16];        // Gauss-Legendre weights (float, as the reference stores them)
    double xq[16];      // abscissae
    float wTable[10000];  // W of the SPH table (GetW(float), Kernel/DFSPHKernels.h:43-52)
    float wInvStep, wZero;
};

// SDF::IndexToNodePosition (SDF.cu:313-373).
__device__ __host__ inline void node_position(const BoxMap& m, uint32_t i, float p[3]) {
    const uint32_t* r = m.res;
    const uint32_t nv = (r[0] + 1u) * (r[1] + 1u) * (r[2] + 1u);
    const uint32_t ne0 = r[0] * (r[1] + 1u) * (r[2] + 1u), ne1 = (r[0] + 1u) * r[1] * (r[2] + 1u);
    float idx[3];
    int axis = -1;
    uint32_t sub = 0;
    if (i < nv) {
        idx[2] = (float)(i / ((r[1] + 1u) * (r[0] + 1u)));
        const uint32_t t = i % ((r[1] + 1u) * (r[0] + 1u));
        idx[1] = (float)(t / (r[0] + 1u));
        idx[0] = (float)(t % (r[0] + 1u));
    } else if (i < nv + 2u * ne0) {
        i -= nv;
        const uint32_t e = i / 2u;
        idx[2] = (float)(e / ((r[1] + 1u) * r[0]));
        const uint32_t t = e % ((r[1] + 1u) * r[0]);
        idx[1] = (float)(t / r[0]);
        idx[0] = (float)(t % r[0]);
        axis = 0;
        sub = i % 2u;
    } else if (i < nv + 2u * (ne0 + ne1)) {
        i -= nv + 2u * ne0;
        const uint32_t e = i / 2u;
        idx[0] = (float)(e / ((r[2] + 1u) * r[1]));
        const uint32_t t = e % ((r[2] + 1u) * r[1]);
        idx[2] = (float)(t / r[1]);
        idx[1] = (float)(t % r[1]);
        axis = 1;
        sub = i % 2u;
    } else {
        i -= nv + 2u * (ne0 + ne1);
        const uint32_t e = i / 2u;
        idx[1] = (float)(e / ((r[0] + 1u) * r[2]));
        const uint32_t t = e % ((r[0] + 1u) * r[2]);
        idx[0] = (float)(t / r[2]);
        idx[2] = (float)(t % r[2]);
        axis = 2;
        sub = i % 2u;
    }
    for (int k = 0; k < 3; k++) p[k] = m.dmin[k] + m.cs[k] * idx[k];
    if (axis >= 0) p[axis] += (1.0f + (float)sub) / 3.0f * m.cs[axis];
}

__device__ inline float box_sdf(const BoxMap& m, const float p[3]) {
    double outside = 0.0, inside = -1e300;
    for (int k = 0; k < 3; k++) {
        const double c = 0.5 * ((double)m.bmin[k] + m.bmax[k]);
        const double hh = 0.5 * ((double)m.bmax[k] - m.bmin[k]);
        const double q = fabs((double)p[k] - c) - hh;
        outside += fmax(q, 0.0) * fmax(q, 0.0);
        inside = fmax(inside, q);
    }
    return (float)(sqrt(outside) + fmin(inside, 0.0));
}

__global__ void k_map_field0(BoxMap* m, float* nodes) {
    const uint32_t l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= m->nodeCount) return;
    float p[3];
    node_position(*m, l, p);
    nodes[l] = m->sign * (box_sdf(*m, p) - m->tol);
}

// Host-side SDF::Interpolate(0, x) without gradient (SDF.cu:141-188): FLT_MAX outside.
__device__ inline float map_distance(const BoxMap& m, const float* nodes, const uint32_t* cells, const float x[3]) {
    uint32_t mi[3];
    for (int k = 0; k < 3; k++) {
        if (!(m.dmin[k] <= x[k] && m.dmax[k] >= x[k])) return FLT_MAX;
        mi[k] = (uint32_t)((x[k] - m.dmin[k]) * m.csi[k]);
        if (mi[k] >= m.res[k]) mi[k] = m.res[k] - 1u;
    }
    const uint32_t i = m.res[1] * m.res[0] * mi[2] + m.res[0] * mi[1] + mi[0];
    float xi[3];
    for (int k = 0; k < 3; k++) {
        const float lo = m.dmin[k] + (float)mi[k] * m.cs[k];
        const float hi = lo + m.cs[k];
        const float den = hi - lo;
        xi[k] = 2.0f / den * x[k] - (hi + lo) / den;
    }
    const float base = 9.f * (xi[0] * xi[0] + xi[1] * xi[1] + xi[2] * xi[2]) - 19.f;
    MapSample s;
    s.phi0 = s.phi1 = 0.f;
    s.grad0 = make_float3(0.f, 0.f, 0.f);
    BodyDev b;
    b.nodes = nodes;
    b.nodeCount = 0;  // field 1 reads alias field 0 here; only phi0 is used
    NodeLoop<32, false>::run(b, cells + (size_t)i * 32u, xi[0], xi[1], xi[2], base, s);
    return s.phi0;
}

// Field 1: 0.8 * integral over the support cube of gamma(distance(x + xi)), one warp per node.
__global__ void k_map_field1(const BoxMap* mp, const float* nodes0, const uint32_t* cells, float* nodes1) {
    const BoxMap& m = *mp;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t lane = threadIdx.x & 31u;
    if (warp >= m.nodeCount) return;
    float x[3];
    node_position(m, warp, x);
    const float dx = map_distance(m, nodes0, cells, x);
    if (dx > 2.0f * m.h) {
        if (lane == 0) nodes1[warp] = 0.0f;
        return;
    }
    const double c0 = 0.5 * (double)(m.h - (-m.h));
    float acc = 0.0f;
    for (uint32_t q = lane; q < 4096u; q += 32u) {
        const uint32_t i = q >> 8, j = (q >> 4) & 15u, k = q & 15u;
        const float wijk = (m.w[i] * m.w[j]) * m.w[k];
        const float xi[3] = {(float)(c0 * m.xq[i]), (float)(c0 * m.xq[j]), (float)(c0 * m.xq[k])};
        float f = 0.0f;
        if (!(xi[0] * xi[0] + xi[1] * xi[1] + xi[2] * xi[2] > m.h * m.h)) {
            const float y[3] = {x[0] + xi[0], x[1] + xi[1], x[2] + xi[2]};
            const float dist = map_distance(m, nodes0, cells, y);
            if (dist <= 0.0f) {
                f = 1.0f;
            } else if (dist < m.h) {
                const uint32_t pos = min((uint32_t)(dist * m.wInvStep), kTableRes - 2u);
                f = 0.5f * (m.wTable[pos] + m.wTable[pos + 1]) / m.wZero;
            }
        }
        acc += wijk * f;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) nodes1[warp] = 0.8f * (float)((double)acc * (c0 * c0 * c0));
}

// Gauss-Legendre rule of n points by Newton iteration on the Legendre polynomial P_n.
static void gauss_legendre16(double* x, double* w) {
    const int n = 16;
    for (int i = 0; i < n; i++) {
        double z = std::cos(3.14159265358979323846 * (i + 0.75) / (n + 0.5)), dp = 1.0;
        for (int it = 0; it < 100; it++) {
            double p0 = 1.0, p1 = z;
            for (int k = 2; k <= n; k++) {
                const double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
                p0 = p1;
                p1 = p2;
            }
            dp = n * (z * p1 - p0) / (z * z - 1.0);
            const double dz = p1 / dp;
            z -= dz;
            if (std::fabs(dz) < 1e-17) break;
        }
        double p0 = 1.0, p1 = z;  // P_n' at the converged root
        for (int k = 2; k <= n; k++) {
            const double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
            p0 = p1;
            p1 = p2;
        }
        dp = n * (z * p1 - p0) / (z * z - 1.0);
        x[n - 1 - i] = z;
        w[n - 1 - i] = 2.0 / ((1.0 - z * z) * dp * dp);
    }
}

void box_map_sizes(const uint32_t res[3], uint32_t& nodes, uint32_t& cells) {
    const uint32_t nv = (res[0] + 1) * (res[1] + 1) * (res[2] + 1);
    const uint32_t ne = res[0] * (res[1] + 1) * (res[2] + 1) + (res[0] + 1) * res[1] * (res[2] + 1) +
                        (res[0] + 1) * (res[1] + 1) * res[2];
    nodes = nv + 2 * ne;
    cells = res[0] * res[1] * res[2];
}

// SDF::AddFunction cell table (SDF.cu:77-131): 32 node indices per cell.
void box_map_cells(const uint32_t res[3], uint32_t* cells) {
    const uint32_t nx = res[0], ny = res[1], nz = res[2];
    const uint32_t nv = (nx + 1) * (ny + 1) * (nz + 1);
    const uint32_t nex = nx * (ny + 1) * (nz + 1), ney = (nx + 1) * ny * (nz + 1);
    const uint32_t count = nx * ny * nz;
    for (uint32_t l = 0; l < count; l++) {
        const uint32_t k = l / (ny * nx), t = l % (ny * nx), j = t / nx, i = t % nx;
        uint32_t* c = cells + (size_t)l * 32u;
        const uint32_t sxy = (nx + 1) * (ny + 1);
        c[0] = sxy * k + (nx + 1) * j + i;
        c[2] = sxy * k + (nx + 1) * (j + 1) + i;
        c[4] = sxy * (k + 1) + (nx + 1) * j + i;
        c[6] = sxy * (k + 1) + (nx + 1) * (j + 1) + i;
        for (int e = 0; e < 8; e += 2) c[e + 1] = c[e] + 1;
        uint32_t off = nv;
        c[8] = off + 2 * (nx * (ny + 1) * k + nx * j + i);
        c[10] = off + 2 * (nx * (ny + 1) * (k + 1) + nx * j + i);
        c[12] = off + 2 * (nx * (ny + 1) * k + nx * (j + 1) + i);
        c[14] = off + 2 * (nx * (ny + 1) * (k + 1) + nx * (j + 1) + i);
        off += 2 * nex;
        c[16] = off + 2 * (ny * (nz + 1) * i + ny * k + j);
        c[18] = off + 2 * (ny * (nz + 1) * (i + 1) + ny * k + j);
        c[20] = off + 2 * (ny * (nz + 1) * i + ny * (k + 1) + j);
        c[22] = off + 2 * (ny * (nz + 1) * (i + 1) + ny * (k + 1) + j);
        off += 2 * ney;
        c[24] = off + 2 * (nz * (nx + 1) * j + nz * i + k);
        c[26] = off + 2 * (nz * (nx + 1) * (j + 1) + nz * i + k);
        c[28] = off + 2 * (nz * (nx + 1) * j + nz * (i + 1) + k);
        c[30] = off + 2 * (nz * (nx + 1) * (j + 1) + nz * (i + 1) + k);
        for (int e = 8; e < 32; e += 2) c[e + 1] = c[e] + 1;
    }
}

// Builds the two-field map on the current device. Host outputs: nodes (2 * nodeCount),
// cells (2 * cellCount * 32), cellMap (2 * cellCount). `table` = the FP32 SPH W table
// (10000 entries) of radius 4r. Returns a cudaError_t.
int build_box_map_gpu(const float bmin[3], const float bmax[3], bool inverted, float padding, const uint32_t res[3],
                      float r, const float* table, float wZero, float invStep, float* nodes, uint32_t* cells,
                      uint32_t* cellMap, float dminOut[3], float dmaxOut[3], float csOut[3], float csiOut[3]) {
    BoxMap* hm = new BoxMap();
    const float h = 4.0f * r;
    const float tol = padding - r;
    for (int k = 0; k < 3; k++) {
        hm->bmin[k] = bmin[k];
        hm->bmax[k] = bmax[k];
        hm->dmin[k] = bmin[k] - (8.0f * h + tol);
        hm->dmax[k] = bmax[k] + (8.0f * h + tol);
        hm->res[k] = res[k];
        hm->cs[k] = (hm->dmax[k] - hm->dmin[k]) / (float)res[k];
        hm->csi[k] = 1.0f / hm->cs[k];
    }
    box_map_sizes(res, hm->nodeCount, hm->cellCount);
    hm->sign = inverted ? -1.0f : 1.0f;
    hm->tol = tol;
    hm->h = h;
    double w[16];
    gauss_legendre16(hm->xq, w);
    for (int i = 0; i < 16; i++) hm->w[i] = (float)w[i];
    for (int i = 0; i < 10000; i++) hm->wTable[i] = table[i];
    hm->wInvStep = invStep;
    hm->wZero = wZero;
    const uint32_t nn = hm->nodeCount, nc = hm->cellCount;
    std::vector<uint32_t> hc((size_t)nc * 32u);
    box_map_cells(res, hc.data());

    BoxMap* dm = nullptr;
    float* dn = nullptr;
    uint32_t* dc = nullptr;
    cudaError_t e = cudaMalloc(&dm, sizeof(BoxMap));
    if (e == cudaSuccess) e = cudaMalloc(&dn, sizeof(float) * 2 * (size_t)nn);
    if (e == cudaSuccess) e = cudaMalloc(&dc, sizeof(uint32_t) * 32 * (size_t)nc);
    if (e == cudaSuccess) e = cudaMemcpy(dm, hm, sizeof(BoxMap), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dc, hc.data(), sizeof(uint32_t) * 32 * (size_t)nc, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        k_map_field0<<<(nn + 255) / 256, 256>>>(dm, dn);
        k_map_field1<<<(nn * 32u + 255) / 256, 256>>>(dm, dn, dc, dn + nn);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(nodes, dn, sizeof(float) * 2 * (size_t)nn, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) {
        for (int f = 0; f < 2; f++) {
            std::copy(hc.begin(), hc.end(), cells + (size_t)f * nc * 32u);
            for (uint32_t l = 0; l < nc; l++) cellMap[(size_t)f * nc + l] = l;
        }
        for (int k = 0; k < 3; k++) {
            dminOut[k] = hm->dmin[k];
            dmaxOut[k] = hm->dmax[k];
            csOut[k] = hm->cs[k];
            csiOut[k] = hm->csi[k];
        }
    }
    cudaFree(dm);
    cudaFree(dn);
    cudaFree(dc);
    delete hm;
    return (int)e;
}

}  // namespace vfd
