// Volume-map construction and mesh sampling on the GPU (scene setup, not per step).
//   * RigidBody::RigidBody (Simulation/DFSPH/RigidBody/RigidBody.cu:10-72): SDF::AddFunction
//     (Utility/SDF/SDF.cu:45-139) of field 0 = sign * (signed distance - tolerance) and of
//     field 1 = the 16^3-point Gauss-Legendre boundary volume
//     (Core/Math/GaussQuadrature.cpp:5621-5656), one warp per map node. The distance is
//     that of an axis-aligned box (analytic) or of a triangle mesh (MeshDistance).
//   * ParticleSampler::SampleMeshVolume (Utility/Sampler/ParticleSampler.cpp:7-91): lattice
//     samples kept where the mesh's signed-distance map is negative.
#include <cfloat>
#include <climits>
#include <cmath>
#include <map>
#include <memory>
#include <utility>
#include <vector>

#include "dfsph_common.cuh"
#include "dfsph_map.cuh"
#include "dfsph_sim.h"

namespace vfd {

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

// ---------------------------------------------------------------- triangle-mesh distance
// Closest point q to p on triangle (a, b, c), found by testing p against the Voronoi
// regions of the corners, the edges and the interior in turn (C. Ericson, Real-Time
// Collision Detection, 2005, sec. 5.1.5). `feature`: 0, 1, 2 = corner a, b, c; 3, 4, 5 =
// edge ab, bc, ca; 6 = interior: the closest-entity classes A..G of MeshDistance
// (MeshDistance.cpp:300-607, which finds the same point by Eberly's parametric regions).
// Returns |p - q|^2.
__device__ inline float closest_on_triangle(float3 p, float3 a, float3 b, float3 c, float3& q, int& feature) {
    const float3 ab = b - a, ac = c - a, ap = p - a;
    const float d1 = dot3(ab, ap), d2 = dot3(ac, ap);
    const float3 bp = p - b;
    const float d3 = dot3(ab, bp), d4 = dot3(ac, bp);
    const float3 cp = p - c;
    const float d5 = dot3(ab, cp), d6 = dot3(ac, cp);
    const float vc = d1 * d4 - d3 * d2, vb = d5 * d2 - d1 * d6, va = d3 * d6 - d5 * d4;
    if (d1 <= 0.0f && d2 <= 0.0f) {
        q = a;
        feature = 0;
    } else if (d3 >= 0.0f && d4 <= d3) {
        q = b;
        feature = 1;
    } else if (vc <= 0.0f && d1 >= 0.0f && d3 <= 0.0f) {
        q = a + (d1 / (d1 - d3)) * ab;
        feature = 3;
    } else if (d6 >= 0.0f && d5 <= d6) {
        q = c;
        feature = 2;
    } else if (vb <= 0.0f && d2 >= 0.0f && d6 <= 0.0f) {
        q = a + (d2 / (d2 - d6)) * ac;
        feature = 5;
    } else if (va <= 0.0f && d4 - d3 >= 0.0f && d5 - d6 >= 0.0f) {
        q = b + ((d4 - d3) / ((d4 - d3) + (d5 - d6))) * (c - b);
        feature = 4;
    } else {
        const float inv = 1.0f / (va + vb + vc);
        q = a + (vb * inv) * ab + (vc * inv) * ac;
        feature = 6;
    }
    const float3 e = p - q;
    return dot3(e, e);
}

constexpr uint32_t kMeshBlock = 128;
constexpr uint32_t kMeshTile = 256;  // faces staged in shared memory per pass

// Field 0 of a mesh map: sign * (signed distance - tolerance) at every node
// (RigidBody.cu:38-40; SDF.cu:16-36 for the sampler's map, tolerance 0). The distance is
// the minimum over all faces (MeshDistance::Distance, MeshDistance.cpp:58-118, ties to the
// lowest face index); it is negative when p - q points against the pseudo-normal of the
// closest feature (MeshDistance::SignedDistance, MeshDistance.cpp:187-228). One thread per
// node; the block walks the faces in tiles staged through shared memory.
__global__ void __launch_bounds__(kMeshBlock) k_map_field0_mesh(const BoxMap* mp, const float4* corners,
                                                                const float4* normals, uint32_t nf, float* nodes) {
    __shared__ float4 tile[kMeshTile * 3];
    const BoxMap& m = *mp;
    const uint32_t l = blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = l < m.nodeCount;
    float pv[3] = {0.0f, 0.0f, 0.0f};
    if (live) node_position(m, l, pv);
    const float3 p = make_float3(pv[0], pv[1], pv[2]);
    float best = FLT_MAX;
    uint32_t bestFace = 0;
    for (uint32_t base = 0; base < nf; base += kMeshTile) {
        const uint32_t cnt = min(kMeshTile, nf - base);
        __syncthreads();
        for (uint32_t q = threadIdx.x; q < 3u * cnt; q += blockDim.x) tile[q] = corners[3 * (size_t)base + q];
        __syncthreads();
        if (!live) continue;
        for (uint32_t f = 0; f < cnt; f++) {
            const float4 a = tile[3 * f], b = tile[3 * f + 1], c = tile[3 * f + 2];
            float3 q;
            int feature;
            const float d2 = closest_on_triangle(p, make_float3(a.x, a.y, a.z), make_float3(b.x, b.y, b.z),
                                                 make_float3(c.x, c.y, c.z), q, feature);
            if (d2 < best) {
                best = d2;
                bestFace = base + f;
            }
        }
    }
    if (!live) return;
    const float4 a = corners[3 * (size_t)bestFace], b = corners[3 * (size_t)bestFace + 1],
                 c = corners[3 * (size_t)bestFace + 2];
    float3 q;
    int feature;
    const float d2 = closest_on_triangle(p, make_float3(a.x, a.y, a.z), make_float3(b.x, b.y, b.z),
                                         make_float3(c.x, c.y, c.z), q, feature);
    const float4 n = normals[7 * (size_t)bestFace + feature];
    float dist = sqrtf(d2);
    if (dot3(p - q, make_float3(n.x, n.y, n.z)) < 0.0f) dist = -dist;
    nodes[l] = m.sign * (dist - m.tol);
}

// Host set-up of the mesh: the placement `transform * (v, 1)` of FluidObject.cpp:10-14 /
// RigidBody.cu:19-23 (glm's column-major product, summed in pairs), the bounds of the
// placed vertices, and MeshDistance's pre-computed normals (MeshDistance.cpp:27-55): the
// unit face normal, the angle-weighted sum of face normals at each vertex, and per edge the
// sum of the normals of the two faces that share it (the face's own normal on a border
// edge, MeshDistance.cpp:247-260). Edges pair a half-edge (u, v) with the first unpaired
// (v, u) in face order (EdgeMesh.cpp:97-130).
int prepare_mesh(const float* vtx, uint32_t nv, const uint32_t* tri, uint32_t nf, const float* T, MeshHost& out) {
    struct F3 {
        float x, y, z;
    };
    auto sub = [](F3 a, F3 b) { return F3{a.x - b.x, a.y - b.y, a.z - b.z}; };
    auto add = [](F3 a, F3 b) { return F3{a.x + b.x, a.y + b.y, a.z + b.z}; };
    auto scale = [](float s, F3 a) { return F3{s * a.x, s * a.y, s * a.z}; };
    auto dot = [](F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; };
    auto cross = [](F3 a, F3 b) { return F3{a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y}; };
    auto normalize = [&](F3 a) { return scale(1.0f / std::sqrt(dot(a, a)), a); };
    auto neg = [](F3 a) { return F3{-a.x, -a.y, -a.z}; };
    for (size_t i = 0; i < 3 * (size_t)nf; i++)
        if (tri[i] >= nv) return -1;
    std::vector<F3> x(nv);
    for (uint32_t v = 0; v < nv; v++) {
        const float px = vtx[3 * (size_t)v], py = vtx[3 * (size_t)v + 1], pz = vtx[3 * (size_t)v + 2];
        if (T) {
            float r[3];
            for (int k = 0; k < 3; k++) r[k] = (T[0 * 4 + k] * px + T[1 * 4 + k] * py) + (T[2 * 4 + k] * pz + T[3 * 4 + k] * 1.0f);
            x[v] = F3{r[0], r[1], r[2]};
        } else {
            x[v] = F3{px, py, pz};
        }
    }
    for (int k = 0; k < 3; k++) {
        out.bmin[k] = FLT_MAX;
        out.bmax[k] = -FLT_MAX;
    }
    for (const F3& p : x) {
        const float c[3] = {p.x, p.y, p.z};
        for (int k = 0; k < 3; k++) {
            out.bmin[k] = std::min(out.bmin[k], c[k]);
            out.bmax[k] = std::max(out.bmax[k], c[k]);
        }
    }
    std::vector<F3> faceN(nf), vertN(nv, F3{0.0f, 0.0f, 0.0f});
    for (uint32_t f = 0; f < nf; f++) {
        const F3 x0 = x[tri[3 * f]], x1 = x[tri[3 * f + 1]], x2 = x[tri[3 * f + 2]];
        const F3 n = normalize(cross(sub(x1, x0), sub(x2, x0)));
        const F3 e1 = normalize(sub(x1, x0)), e2 = normalize(sub(x2, x1)), e3 = normalize(sub(x0, x2));
        const float alpha[3] = {std::acos(dot(e1, neg(e3))), std::acos(dot(e2, neg(e1))), std::acos(dot(e3, neg(e2)))};
        for (int k = 0; k < 3; k++) vertN[tri[3 * f + k]] = add(vertN[tri[3 * f + k]], scale(alpha[k], n));
        faceN[f] = n;
    }
    // opposite face of each half-edge (face f, edge k = (tri[k], tri[(k+1)%3])); -1 on a border
    std::vector<int64_t> opp(3 * (size_t)nf, -1);
    std::multimap<std::pair<uint32_t, uint32_t>, uint32_t> open;  // unpaired half-edges by (source, target)
    for (uint32_t f = 0; f < nf; f++)
        for (uint32_t k = 0; k < 3; k++) {
            const uint32_t u = tri[3 * f + k], v = tri[3 * f + (k + 1) % 3];
            auto it = open.lower_bound({v, u});  // the earliest unpaired (v, u)
            if (it != open.end() && it->first == std::make_pair(v, u)) {
                opp[3 * (size_t)f + k] = it->second / 3;
                opp[it->second] = f;
                open.erase(it);
            } else {
                open.emplace(std::make_pair(u, v), 3 * f + k);
            }
        }
    out.corners.resize(3 * (size_t)nf);
    out.normals.resize(7 * (size_t)nf);
    auto f4 = [](F3 a) { return make_float4(a.x, a.y, a.z, 0.0f); };
    for (uint32_t f = 0; f < nf; f++) {
        for (int k = 0; k < 3; k++) {
            out.corners[3 * (size_t)f + k] = f4(x[tri[3 * f + k]]);
            out.normals[7 * (size_t)f + k] = f4(vertN[tri[3 * f + k]]);
            const int64_t o = opp[3 * (size_t)f + k];
            out.normals[7 * (size_t)f + 3 + k] = f4(o < 0 ? faceN[f] : add(faceN[f], faceN[(size_t)o]));
        }
        out.normals[7 * (size_t)f + 6] = f4(faceN[f]);
    }
    return 0;
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

// Device buffers of a map under construction.
struct MapBuild {
    BoxMap* dm = nullptr;
    float* dn = nullptr;
    uint32_t* dc = nullptr;
    float4* dcorner = nullptr;
    float4* dnormal = nullptr;
    MapBuild() = default;
    MapBuild(const MapBuild&) = delete;
    MapBuild& operator=(const MapBuild&) = delete;
    ~MapBuild() {
        cudaFree(dm);
        cudaFree(dn);
        cudaFree(dc);
        cudaFree(dcorner);
        cudaFree(dnormal);
    }
};

// Fills `hm`'s quadrature and kernel tables (field 1 only).
static void set_volume_tables(BoxMap* hm, const float* table, float wZero, float invStep) {
    double w[16];
    gauss_legendre16(hm->xq, w);
    for (int i = 0; i < 16; i++) hm->w[i] = (float)w[i];
    for (int i = 0; i < 10000; i++) hm->wTable[i] = table[i];
    hm->wInvStep = invStep;
    hm->wZero = wZero;
}

// Sets the grid of `hm` over [dmin, dmax] (SDF::SDF, SDF.cu:8-14).
static void set_grid(BoxMap* hm, const float dmin[3], const float dmax[3], const uint32_t res[3]) {
    for (int k = 0; k < 3; k++) {
        hm->dmin[k] = dmin[k];
        hm->dmax[k] = dmax[k];
        hm->res[k] = res[k];
        hm->cs[k] = (hm->dmax[k] - hm->dmin[k]) / (float)res[k];
        hm->csi[k] = 1.0f / hm->cs[k];
    }
    box_map_sizes(res, hm->nodeCount, hm->cellCount);
}

// Uploads `hm` and the cell table, evaluates field 0 (the box of `hm` when `mesh` is null,
// else the mesh) and, when `volume`, field 1, all on the device. Returns a cudaError_t.
static cudaError_t map_build_fields(const BoxMap& hm, const std::vector<uint32_t>& hc, const MeshHost* mesh,
                                    bool volume, MapBuild& b) {
    const uint32_t nn = hm.nodeCount, nc = hm.cellCount;
    cudaError_t e = cudaMalloc(&b.dm, sizeof(BoxMap));
    if (e == cudaSuccess) e = cudaMalloc(&b.dn, sizeof(float) * (volume ? 2 : 1) * (size_t)nn);
    if (e == cudaSuccess) e = cudaMalloc(&b.dc, sizeof(uint32_t) * 32 * (size_t)nc);
    if (e == cudaSuccess) e = cudaMemcpy(b.dm, &hm, sizeof(BoxMap), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(b.dc, hc.data(), sizeof(uint32_t) * 32 * (size_t)nc, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return e;
    if (mesh) {
        const uint32_t nf = (uint32_t)(mesh->corners.size() / 3);
        e = cudaMalloc(&b.dcorner, sizeof(float4) * mesh->corners.size());
        if (e == cudaSuccess) e = cudaMalloc(&b.dnormal, sizeof(float4) * mesh->normals.size());
        if (e == cudaSuccess)
            e = cudaMemcpy(b.dcorner, mesh->corners.data(), sizeof(float4) * mesh->corners.size(),
                           cudaMemcpyHostToDevice);
        if (e == cudaSuccess)
            e = cudaMemcpy(b.dnormal, mesh->normals.data(), sizeof(float4) * mesh->normals.size(),
                           cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return e;
        k_map_field0_mesh<<<(nn + kMeshBlock - 1) / kMeshBlock, kMeshBlock>>>(b.dm, b.dcorner, b.dnormal, nf, b.dn);
    } else {
        k_map_field0<<<(nn + 255) / 256, 256>>>(b.dm, b.dn);
    }
    if (volume) k_map_field1<<<(nn * 32u + 255) / 256, 256>>>(b.dm, b.dn, b.dc, b.dn + nn);
    return cudaGetLastError();
}

// Copies a finished two-field map to the host arrays of a vfd_volume_map.
static cudaError_t map_copy_out(const BoxMap& hm, const std::vector<uint32_t>& hc, const MapBuild& b, float* nodes,
                                uint32_t* cells, uint32_t* cellMap, float dminOut[3], float dmaxOut[3],
                                float csOut[3], float csiOut[3]) {
    const uint32_t nn = hm.nodeCount, nc = hm.cellCount;
    const cudaError_t e = cudaMemcpy(nodes, b.dn, sizeof(float) * 2 * (size_t)nn, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return e;
    for (int f = 0; f < 2; f++) {
        std::copy(hc.begin(), hc.end(), cells + (size_t)f * nc * 32u);
        for (uint32_t l = 0; l < nc; l++) cellMap[(size_t)f * nc + l] = l;
    }
    for (int k = 0; k < 3; k++) {
        dminOut[k] = hm.dmin[k];
        dmaxOut[k] = hm.dmax[k];
        csOut[k] = hm.cs[k];
        csiOut[k] = hm.csi[k];
    }
    return cudaSuccess;
}

// Builds the two-field map of a box on the current device. Host outputs: nodes
// (2 * nodeCount), cells (2 * cellCount * 32), cellMap (2 * cellCount). `table` = the FP32
// SPH W table (10000 entries) of radius 4r. Returns a cudaError_t.
int build_box_map_gpu(const float bmin[3], const float bmax[3], bool inverted, float padding, const uint32_t res[3],
                      float r, const float* table, float wZero, float invStep, float* nodes, uint32_t* cells,
                      uint32_t* cellMap, float dminOut[3], float dmaxOut[3], float csOut[3], float csiOut[3]) {
    std::unique_ptr<BoxMap> hm(new BoxMap());
    const float h = 4.0f * r;
    const float tol = padding - r;
    float dmin[3], dmax[3];
    for (int k = 0; k < 3; k++) {
        hm->bmin[k] = bmin[k];
        hm->bmax[k] = bmax[k];
        dmin[k] = bmin[k] - (8.0f * h + tol);
        dmax[k] = bmax[k] + (8.0f * h + tol);
    }
    set_grid(hm.get(), dmin, dmax, res);
    hm->sign = inverted ? -1.0f : 1.0f;
    hm->tol = tol;
    hm->h = h;
    set_volume_tables(hm.get(), table, wZero, invStep);
    std::vector<uint32_t> hc((size_t)hm->cellCount * 32u);
    box_map_cells(res, hc.data());
    MapBuild b;
    cudaError_t e = map_build_fields(*hm, hc, nullptr, true, b);
    if (e == cudaSuccess) e = map_copy_out(*hm, hc, b, nodes, cells, cellMap, dminOut, dmaxOut, csOut, csiOut);
    return (int)e;
}

// RigidBody::RigidBody (RigidBody.cu:10-72) for a triangle mesh already placed by its
// transform: domain = bounds of the vertices +- (8h + tolerance), field 0 =
// sign * (signed distance - tolerance), field 1 the boundary volume.
int build_mesh_map_gpu(const MeshHost& mesh, bool inverted, float padding, const uint32_t res[3], float r,
                       const float* table, float wZero, float invStep, float* nodes, uint32_t* cells,
                       uint32_t* cellMap, float dminOut[3], float dmaxOut[3], float csOut[3], float csiOut[3]) {
    std::unique_ptr<BoxMap> hm(new BoxMap());
    const float h = 4.0f * r;
    const float tol = padding - r;
    float dmin[3], dmax[3];
    for (int k = 0; k < 3; k++) {
        dmax[k] = mesh.bmax[k] + (8.0f * h + tol);
        dmin[k] = mesh.bmin[k] - (8.0f * h + tol);
    }
    set_grid(hm.get(), dmin, dmax, res);
    hm->sign = inverted ? -1.0f : 1.0f;
    hm->tol = tol;
    hm->h = h;
    set_volume_tables(hm.get(), table, wZero, invStep);
    std::vector<uint32_t> hc((size_t)hm->cellCount * 32u);
    box_map_cells(res, hc.data());
    MapBuild b;
    cudaError_t e = map_build_fields(*hm, hc, &mesh, true, b);
    if (e == cudaSuccess) e = map_copy_out(*hm, hc, b, nodes, cells, cellMap, dminOut, dmaxOut, csOut, csiOut);
    return (int)e;
}

// ---------------------------------------------------------------- mesh volume sampler
// One axis of the sampling lattice: the float sequence lo, lo + step, ... while <= hi,
// accumulated in float as ParticleSampler.cpp:32-34 does.
static bool lattice_axis(float lo, float hi, float step, std::vector<float>& out) {
    out.clear();
    for (float v = lo; v <= hi; v += step) {
        if (out.size() >= (1u << 24) || v + step == v) return false;
        out.push_back(v);
    }
    return true;
}

struct Lattice {
    uint32_t nx, ny, nz, mode;
    float radius, diameter, shiftX;
};

// Sample position of lattice point (x, y, z) with loop counters cx (x) and cy (y)
// (ParticleSampler.cpp:37-72).
__device__ inline float3 lattice_position(const Lattice& L, float x, float y, float z, uint32_t cx, uint32_t cy) {
    const float r = L.radius;
    if (L.mode == VFD_SAMPLE_MIN_DENSITY) return make_float3(__fadd_rn(x, r), __fadd_rn(y, r), __fadd_rn(z, r));
    if (L.mode == VFD_SAMPLE_MEDIUM_DENSITY) {
        if ((cy & 1u) == 0u) return make_float3(x, __fadd_rn(y, r), __fadd_rn(z, r));
        return make_float3(__fadd_rn(x, r), __fadd_rn(y, r), z);
    }
    float sx = 0.0f, sz = 0.0f;
    if (cx & 1u) sz = __fadd_rn(sz, __fdiv_rn(L.diameter, 2.0f * ((cy & 1u) ? -1.0f : 1.0f)));
    if (cy & 1u) {
        sx = __fadd_rn(sx, __fdiv_rn(L.shiftX, 2.0f));
        sz = __fadd_rn(sz, __fdiv_rn(L.diameter, 2.0f));
    }
    return make_float3(__fadd_rn(x, sx), __fadd_rn(__fadd_rn(y, r), 0.0f), __fadd_rn(__fadd_rn(z, r), sz));
}

__device__ inline float3 lattice_point(const Lattice& L, const float* xs, const float* ys, const float* zs,
                                       uint32_t f) {
    const uint32_t k = f % L.nx, t = f / L.nx, j = t % L.ny, i = t / L.ny;
    return lattice_position(L, xs[k], ys[j], zs[i], k, j);
}

// Inside test of every lattice point (SDF::GetDistance(x, 0) < 0, SDF.cu:217-225) and
// the count of kept points per block.
__global__ void __launch_bounds__(256) k_sample_flags(const BoxMap* mp, const float* nodes, const uint32_t* cells,
                                                      const float* xs, const float* ys, const float* zs, Lattice L,
                                                      uint32_t total, uint8_t* keep, uint32_t* blockCount) {
    const uint32_t f = blockIdx.x * blockDim.x + threadIdx.x;
    bool in = false;
    if (f < total) {
        const float3 p = lattice_point(L, xs, ys, zs, f);
        const float x[3] = {p.x, p.y, p.z};
        in = map_distance(*mp, nodes, cells, x) < 0.0f;
        keep[f] = in ? 1u : 0u;
    }
    const int c = __syncthreads_count(in);
    if (threadIdx.x == 0) blockCount[blockIdx.x] = (uint32_t)c;
}

// Writes the kept points in lattice order (z, then y, then x) from the per-block offsets.
__global__ void __launch_bounds__(256) k_sample_write(const float* xs, const float* ys, const float* zs, Lattice L,
                                                      uint32_t total, const uint8_t* keep,
                                                      const uint32_t* blockOffset, float* out) {
    __shared__ uint32_t warpBase[8];
    const uint32_t f = blockIdx.x * blockDim.x + threadIdx.x;
    const bool in = f < total && keep[f] != 0;
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t bal = __ballot_sync(0xffffffffu, in);
    if (lane == 0) warpBase[warp] = __popc(bal);
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t acc = 0;
        for (int w = 0; w < 8; w++) {
            const uint32_t c = warpBase[w];
            warpBase[w] = acc;
            acc += c;
        }
    }
    __syncthreads();
    if (!in) return;
    const uint32_t o = blockOffset[blockIdx.x] + warpBase[warp] + __popc(bal & ((1u << lane) - 1u));
    const float3 p = lattice_point(L, xs, ys, zs, f);
    out[3 * (size_t)o + 0] = p.x;
    out[3 * (size_t)o + 1] = p.y;
    out[3 * (size_t)o + 2] = p.z;
}

// ParticleSampler::SampleMeshVolume (ParticleSampler.cpp:7-91) of a mesh already placed
// by its transform. Writes min(count, capacity) samples to `out` (host, xyz) when `out`
// is not null and returns the count in `count`. Returns a cudaError_t, or -1 when the
// lattice does not fit (more than 2^31 points, or a step lost in the float rounding).
int sample_mesh_volume_gpu(const MeshHost& mesh, float radius, const uint32_t res[3], bool inverted, int mode,
                           float* out, uint32_t capacity, uint32_t* count) {
    // SDF::SDF(mesh, bounds, resolution, inverted) (SDF.cu:16-36): the domain grows by a
    // thousandth of its diagonal, the upper corner first (so the lower corner grows by a
    // thousandth of the already grown diagonal)
    float dmin[3] = {mesh.bmin[0], mesh.bmin[1], mesh.bmin[2]};
    float dmax[3] = {mesh.bmax[0], mesh.bmax[1], mesh.bmax[2]};
    auto diag_len = [&]() {
        const float a = dmax[0] - dmin[0], b = dmax[1] - dmin[1], c = dmax[2] - dmin[2];
        return std::sqrt(a * a + b * b + c * c);
    };
    const float growMax = 0.001f * diag_len();
    for (int k = 0; k < 3; k++) dmax[k] += growMax;
    const float growMin = 0.001f * diag_len();
    for (int k = 0; k < 3; k++) dmin[k] -= growMin;
    std::unique_ptr<BoxMap> hm(new BoxMap());
    set_grid(hm.get(), dmin, dmax, res);
    hm->sign = inverted ? -1.0f : 1.0f;
    hm->tol = 0.0f;
    std::vector<uint32_t> hc((size_t)hm->cellCount * 32u);
    box_map_cells(res, hc.data());

    const float diameter = 2.0f * radius;
    float shiftX = diameter, shiftY = diameter;
    if (mode == VFD_SAMPLE_MEDIUM_DENSITY) {
        shiftY = std::sqrt(3.0f) * radius;
    } else if (mode == VFD_SAMPLE_MAX_DENSITY) {
        shiftX = std::sqrt(3.0f) * radius;
        shiftY = std::sqrt(6.0f) * diameter / 3.0f;
    }
    std::vector<float> xs, ys, zs;
    if (!lattice_axis(mesh.bmin[0], mesh.bmax[0], shiftX, xs) || !lattice_axis(mesh.bmin[1], mesh.bmax[1], shiftY, ys) ||
        !lattice_axis(mesh.bmin[2], mesh.bmax[2], diameter, zs))
        return -1;
    const uint64_t total64 = (uint64_t)xs.size() * ys.size() * zs.size();
    if (total64 > (uint64_t)INT_MAX) return -1;
    const uint32_t total = (uint32_t)total64;
    *count = 0;
    if (total == 0) return (int)cudaSuccess;
    Lattice L{(uint32_t)xs.size(), (uint32_t)ys.size(), (uint32_t)zs.size(), (uint32_t)mode, radius, diameter,
              shiftX};

    MapBuild b;
    cudaError_t e = map_build_fields(*hm, hc, &mesh, false, b);
    const uint32_t blocks = (total + 255u) / 256u;
    float *dx = nullptr, *dout = nullptr;
    uint8_t* dkeep = nullptr;
    uint32_t* dcnt = nullptr;
    std::vector<uint32_t> cnt(blocks);
    if (e == cudaSuccess) e = cudaMalloc(&dx, sizeof(float) * (xs.size() + ys.size() + zs.size()));
    if (e == cudaSuccess) e = cudaMalloc(&dkeep, total);
    if (e == cudaSuccess) e = cudaMalloc(&dcnt, sizeof(uint32_t) * blocks);
    float* dys = dx + xs.size();
    float* dzs = dys + ys.size();
    if (e == cudaSuccess) e = cudaMemcpy(dx, xs.data(), sizeof(float) * xs.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dys, ys.data(), sizeof(float) * ys.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dzs, zs.data(), sizeof(float) * zs.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        k_sample_flags<<<blocks, 256>>>(b.dm, b.dn, b.dc, dx, dys, dzs, L, total, dkeep, dcnt);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(cnt.data(), dcnt, sizeof(uint32_t) * blocks, cudaMemcpyDeviceToHost);
    uint32_t kept = 0;
    if (e == cudaSuccess) {
        for (uint32_t i = 0; i < blocks; i++) {
            const uint32_t c = cnt[i];
            cnt[i] = kept;
            kept += c;
        }
        *count = kept;
    }
    if (e == cudaSuccess && out && kept > 0) {
        e = cudaMemcpy(dcnt, cnt.data(), sizeof(uint32_t) * blocks, cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMalloc(&dout, sizeof(float) * 3 * (size_t)kept);
        if (e == cudaSuccess) {
            k_sample_write<<<blocks, 256>>>(dx, dys, dzs, L, total, dkeep, dcnt, dout);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess)
            e = cudaMemcpy(out, dout, sizeof(float) * 3 * (size_t)std::min(kept, capacity), cudaMemcpyDeviceToHost);
    }
    cudaFree(dx);
    cudaFree(dkeep);
    cudaFree(dcnt);
    cudaFree(dout);
    return (int)e;
}

}  // namespace vfd
