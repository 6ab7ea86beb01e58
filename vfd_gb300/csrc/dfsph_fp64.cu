// FP64 GPU path of the DFSPH step (vfd_set_precision(sim, VFD_PRECISION_FP64)).
//
// The whole step of DFSPHImplementation::OnUpdate (DFSPHImplementation.cu:63-170) in
// double precision on the GPU: neighbour search, volume-map boundary (K1), density and
// factor (K2, K3), divergence solve (K4-K7), surface tension (K9-K11), implicit
// viscosity CG (K12-K15), CFL time step (T1), velocity update (K16), pressure solve
// (K17-K20) and positions (K21), with the kernels of DFSPHKernels.cu restated for
// doubles. It is the reference trajectory the FP32 paths are measured against on the
// GPU (the FP64 CPU oracle is the same method, but too slow for millions of particles):
// one scene, absolute positions, particles kept in their original order with neighbour
// rows of original indices (as the reference keeps them), one thread per particle,
// the solver loops driven from the host with one reduction read per iteration. Every
// sum over particles is a per-block partial added on the host in block order, so runs
// are reproducible. The SPH tables are built in double with the reference's formulas
// (Kernel/DFSPHKernels.h:13-131) and read with its midpoint lookup; the volume maps and
// the surface-tension direction table are the FP32 path's (their values as doubles).
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/vfd_dfsph.h"
#include "dfsph_common.cuh"
#include "dfsph_sim.h"

namespace vfd {
namespace f64 {

constexpr uint32_t kB = 256u;         // threads per block
constexpr uint32_t kCap = kMaxNeighbors;

struct D3 {
    double x, y, z;
};
__device__ __forceinline__ D3 d3(double a, double b, double c) { return D3{a, b, c}; }
__device__ __forceinline__ D3 operator+(D3 a, D3 b) { return d3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ D3 operator-(D3 a, D3 b) { return d3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ D3 operator-(D3 a) { return d3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ D3 operator*(double s, D3 a) { return d3(s * a.x, s * a.y, s * a.z); }
__device__ __forceinline__ D3 operator*(D3 a, double s) { return d3(s * a.x, s * a.y, s * a.z); }
__device__ __forceinline__ D3& operator+=(D3& a, D3 b) { a.x += b.x; a.y += b.y; a.z += b.z; return a; }
__device__ __forceinline__ D3& operator-=(D3& a, D3 b) { a.x -= b.x; a.y -= b.y; a.z -= b.z; return a; }
__device__ __forceinline__ double dot(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ D3 cross(D3 a, D3 b) {
    return d3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ D3 normalized(D3 a) { return a * (1.0 / sqrt(dot(a, a))); }
__device__ __forceinline__ bool nonzero(D3 a) { return a.x != 0.0 || a.y != 0.0 || a.z != 0.0; }

struct M3 {
    double m[3][3];
};
__device__ __forceinline__ void add_outer(M3& r, double c, D3 a, D3 b) {  // r += c a b^T
    const double av[3] = {a.x, a.y, a.z}, bv[3] = {b.x, b.y, b.z};
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) r.m[i][j] += c * av[i] * bv[j];
}
__device__ __forceinline__ D3 mul(const M3& a, D3 v) {
    return d3(a.m[0][0] * v.x + a.m[0][1] * v.y + a.m[0][2] * v.z, a.m[1][0] * v.x + a.m[1][1] * v.y + a.m[1][2] * v.z,
              a.m[2][0] * v.x + a.m[2][1] * v.y + a.m[2][2] * v.z);
}
__device__ __forceinline__ M3 inverse(const M3& a) {  // cofactors / determinant
    const double(&m)[3][3] = a.m;
    const double c00 = m[1][1] * m[2][2] - m[1][2] * m[2][1];
    const double c01 = m[1][2] * m[2][0] - m[1][0] * m[2][2];
    const double c02 = m[1][0] * m[2][1] - m[1][1] * m[2][0];
    const double id = 1.0 / (m[0][0] * c00 + m[0][1] * c01 + m[0][2] * c02);
    M3 r;
    r.m[0][0] = c00 * id;
    r.m[1][0] = c01 * id;
    r.m[2][0] = c02 * id;
    r.m[0][1] = (m[0][2] * m[2][1] - m[0][1] * m[2][2]) * id;
    r.m[1][1] = (m[0][0] * m[2][2] - m[0][2] * m[2][0]) * id;
    r.m[2][1] = (m[0][1] * m[2][0] - m[0][0] * m[2][1]) * id;
    r.m[0][2] = (m[0][1] * m[1][2] - m[0][2] * m[1][1]) * id;
    r.m[1][2] = (m[0][2] * m[1][0] - m[0][0] * m[1][2]) * id;
    r.m[2][2] = (m[0][0] * m[1][1] - m[0][1] * m[1][0]) * id;
    return r;
}

// Scene constants and the current time step (passed by value to every kernel).
struct P {
    uint32_t n, bodies, bodyBegin, analytic, stSamples, temporal;
    double r, diam, h, h2, volume, rho0, mass, massInv, dynVisc, dynBVisc, tangDist, st;
    double slope, constant, smoothing, nbrRadius, mcFactor;
    double g[3];
    double dt, dt2, dtInv, dt2Inv;
    double K, L, invStep, wZero;  // spline constants and table step
};

// Device arrays of the FP64 state, original particle order.
struct A {
    D3 *X, *V, *Acc, *AP, *DV, *N, *NS, *XB;
    double *RHO, *ALPHA, *RHOADV, *KAPPA, *KAPPAV, *RES, *CURV, *CURVS, *DK, *VB;
    D3 *CR, *CP, *CZ, *CT, *CB, *CG;
    M3* MINV;
    uint32_t *NCNT, *NBR, *KEY, *CNT, *START, *FILL, *TMP, *ORDER, *BSUM;
    int* MM;  // min cell xyz, max cell xyz
    double* PART;
    const double *W, *G;  // midpoint tables
    const float* halton;
    const BodyDev* bodyTab;
    int32_t gmin[3];
    uint32_t dim[3];
    uint32_t cells;
};

// ---------------------------------------------------------------- SPH kernel
__device__ __forceinline__ uint32_t tpos(const P& p, double rl) {
    const uint32_t q = (uint32_t)(rl * p.invStep);
    return q < kTableRes - 2u ? q : kTableRes - 2u;
}
__device__ __forceinline__ double spline_w(const P& p, double rl) {  // Kernel/DFSPHKernels.h:86-104
    const double q = rl / p.h;
    if (q > 1.0) return 0.0;
    if (q <= 0.5) return p.K * (6.0 * q * q * q - 6.0 * q * q + 1.0);
    const double f = 1.0 - q;
    return p.K * (2.0 * f * f * f);
}
__device__ __forceinline__ double spline_gs(const P& p, double rl) {  // :110-131, gradW = gs r
    const double q = rl / p.h;
    if (!(rl > 1.0e-5) || q > 1.0) return 0.0;
    const double gq = 1.0 / (rl * p.h);
    if (q <= 0.5) return (p.L * q) * (3.0 * q - 2.0) * gq;
    const double f = 1.0 - q;
    return p.L * (-f * f) * gq;
}
__device__ __forceinline__ double kw(const P& p, const A& a, D3 r) {  // GetW
    const double r2 = dot(r, r);
    if (!(r2 <= p.h2)) return 0.0;
    const double rl = sqrt(r2);
    return p.analytic ? spline_w(p, rl) : a.W[tpos(p, rl)];
}
__device__ __forceinline__ D3 kgrad(const P& p, const A& a, D3 r) {  // GetGradientW
    const double rl = sqrt(dot(r, r));
    if (!(rl <= p.h)) return d3(0, 0, 0);
    return (p.analytic ? spline_gs(p, rl) : a.G[tpos(p, rl)]) * r;
}

// ---------------------------------------------------------------- reductions
// Sum (or max) of one double per thread into PART[blockIdx.x].
__device__ __forceinline__ void block_partial(const A& a, double v, bool isMax) {
    __shared__ double s[kB / 32u];
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) {
        const double w = __shfl_xor_sync(0xffffffffu, v, o);
        v = isMax ? fmax(v, w) : v + w;
    }
    if ((threadIdx.x & 31u) == 0u) s[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = s[0];
        for (uint32_t w = 1; w < blockDim.x / 32u; w++) t = isMax ? fmax(t, s[w]) : t + s[w];
        a.PART[blockIdx.x] = t;
    }
}

// ---------------------------------------------------------------- neighbour search
__global__ void k_minmax(P p, A a) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    const D3 x = a.X[i];
    const double c[3] = {floor(x.x / p.h), floor(x.y / p.h), floor(x.z / p.h)};
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const int v = fabs(c[k]) < 1.0e9 ? (int)c[k] : 0;
        atomicMin(a.MM + k, v);
        atomicMax(a.MM + 3 + k, v);
    }
}
__device__ __forceinline__ void cell_of(const P& p, const A& a, D3 x, int c[3]) {
    c[0] = (int)floor(x.x / p.h) - a.gmin[0];
    c[1] = (int)floor(x.y / p.h) - a.gmin[1];
    c[2] = (int)floor(x.z / p.h) - a.gmin[2];
}
__global__ void k_keys(P p, A a) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    int c[3];
    cell_of(p, a, a.X[i], c);
    const uint32_t key = ((uint32_t)c[2] * a.dim[1] + (uint32_t)c[1]) * a.dim[0] + (uint32_t)c[0];
    a.KEY[i] = key;
    atomicAdd(a.CNT + key, 1u);
}
// exclusive scan of CNT into START: 1024 cells per block, block sums, then the carry
__global__ void k_scan_blocks(A a) {
    __shared__ uint32_t ws[32];
    const uint32_t c = blockIdx.x * 1024u + threadIdx.x;
    uint32_t v = c < a.cells ? a.CNT[c] : 0u;
    const uint32_t lane = threadIdx.x & 31u, w = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= (uint32_t)o) x += y;
    }
    if (lane == 31u) ws[w] = x;
    __syncthreads();
    if (w == 0) {
        uint32_t y = ws[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t z = __shfl_up_sync(0xffffffffu, y, o);
            if (lane >= (uint32_t)o) y += z;
        }
        ws[lane] = y;
    }
    __syncthreads();
    const uint32_t excl = (w ? ws[w - 1] : 0u) + x - v;
    if (c < a.cells) a.START[c] = excl;
    if (threadIdx.x == 1023u) a.BSUM[blockIdx.x] = ws[31];
}
__global__ void k_scan_carry(A a, uint32_t nblocks) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    uint32_t run = 0;
    for (uint32_t b = 0; b < nblocks; b++) {
        const uint32_t s = a.BSUM[b];
        a.BSUM[b] = run;
        run += s;
    }
}
__global__ void k_scan_add(A a) {
    const uint32_t c = blockIdx.x * 1024u + threadIdx.x;
    if (c < a.cells) a.START[c] += a.BSUM[blockIdx.x];
}
__global__ void k_slots(P p, A a) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    const uint32_t k = a.KEY[i];
    a.TMP[a.START[k] + atomicAdd(a.FILL + k, 1u)] = i;
}
// in-cell order: ascending particle index (one of the orders the reference's atomics allow)
__global__ void k_order(P p, A a) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= p.n) return;
    const uint32_t i = a.TMP[s];
    const uint32_t k = a.KEY[i], st = a.START[k], cnt = a.CNT[k];
    uint32_t rank = 0;
    for (uint32_t q = st; q < st + cnt; q++) rank += a.TMP[q] < i ? 1u : 0u;
    a.ORDER[st + rank] = i;
}
// NeighborhoodQueryWithCountsKernel (ParticleSearchKernels.cu:146-193): z, y, x cells,
// then cell order, 0 < d^2 < h^2, at most 70.
__global__ void k_neighbors(P p, A a) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    const D3 xi = a.X[i];
    int c[3];
    cell_of(p, a, xi, c);
    uint32_t cnt = 0;
    uint32_t* row = a.NBR + (size_t)i * kCap;
    for (int dz = -1; dz <= 1 && cnt < kCap; dz++)
        for (int dy = -1; dy <= 1 && cnt < kCap; dy++)
            for (int dx = -1; dx <= 1 && cnt < kCap; dx++) {
                const int x = c[0] + dx, y = c[1] + dy, z = c[2] + dz;
                if (x < 0 || y < 0 || z < 0 || x >= (int)a.dim[0] || y >= (int)a.dim[1] || z >= (int)a.dim[2]) continue;
                const uint32_t k = ((uint32_t)z * a.dim[1] + (uint32_t)y) * a.dim[0] + (uint32_t)x;
                const uint32_t st = a.START[k], n = a.CNT[k];
                for (uint32_t q = st; q < st + n && cnt < kCap; q++) {
                    const uint32_t j = a.ORDER[q];
                    const D3 e = a.X[j] - xi;
                    const double d2 = dot(e, e);
                    if (d2 < p.h2 && d2 > 0.0) row[cnt++] = j;
                }
            }
    a.NCNT[i] = cnt;
}

// ---------------------------------------------------------------- volume map
// DetermineShapeFunction + Interpolate (SDFDeviceData.cuh:36-474) in double: the 32-node
// cubic serendipity element of the FP32 path's maps, field 0 with its gradient and
// field 1.
__device__ void shape32(double x, double y, double z, double N[32], D3 dN[32]) {
    const double base = 9.0 * (x * x + y * y + z * z) - 19.0;
    for (int k = 0; k < 8; k++) {  // corners
        const double sx = (k & 1) ? 1.0 : -1.0, sy = (k & 2) ? 1.0 : -1.0, sz = (k & 4) ? 1.0 : -1.0;
        const double ax = 1.0 + sx * x, ay = 1.0 + sy * y, az = 1.0 + sz * z;
        const double axyz = ax * ay * az;
        N[k] = axyz * base / 64.0;
        dN[k] = d3((sx * ay * az * base + axyz * 18.0 * x) / 64.0, (sy * ax * az * base + axyz * 18.0 * y) / 64.0,
                   (sz * ax * ay * base + axyz * 18.0 * z) / 64.0);
    }
    const double v[3] = {x, y, z};
    for (int k = 8; k < 32; k++) {  // edge nodes at +-1/3 along an axis
        const int t = (k - 8) / 8, kk = (k - 8) % 8;
        const int a = kk & 1, bu = (kk >> 1) & 1, bw = (kk >> 2) & 1;
        const int U = t == 0 ? 2 : (t == 1 ? 0 : 1), W = t == 0 ? 1 : (t == 1 ? 2 : 0);
        const double tv = v[t], uv = v[U], wv = v[W];
        const double sa = a ? 3.0 : -3.0, su = bu ? 1.0 : -1.0, sw = bw ? 1.0 : -1.0;
        const double ft = (1.0 - tv * tv) * (1.0 + sa * tv);
        const double dft = -2.0 * tv * (1.0 + sa * tv) + sa * (1.0 - tv * tv);
        const double fu = 1.0 + su * uv, fw = 1.0 + sw * wv, c = 9.0 / 64.0;
        N[k] = c * ft * fu * fw;
        double g[3];
        g[t] = c * dft * fu * fw;
        g[U] = c * ft * su * fw;
        g[W] = c * ft * fu * sw;
        dN[k] = d3(g[0], g[1], g[2]);
    }
}
__device__ bool map_lookup(const BodyDev& m, D3 pt, double& phi0, D3& grad0, double& phi1) {
    const double x[3] = {pt.x, pt.y, pt.z};
    uint32_t mi[3];
    for (int k = 0; k < 3; k++) {
        if (!((double)m.dmin[k] <= x[k] && (double)m.dmax[k] >= x[k])) return false;
        mi[k] = (uint32_t)((double)m.csi[k] * (x[k] - (double)m.dmin[k]));
        if (mi[k] >= m.res[k]) mi[k] = m.res[k] - 1u;
    }
    const uint32_t j = m.cellMap[m.res[1] * m.res[0] * mi[2] + m.res[0] * mi[1] + mi[0]];
    if (j == UINT_MAX) return false;
    double c0[3], xi[3];
    for (int k = 0; k < 3; k++) {
        const double lo = (double)m.dmin[k] + (double)mi[k] * (double)m.cs[k];
        const double hi = lo + (double)m.cs[k];
        c0[k] = 2.0 / (hi - lo);
        xi[k] = c0[k] * x[k] - (hi + lo) / (hi - lo);
    }
    double N[32];
    D3 dN[32];
    shape32(xi[0], xi[1], xi[2], N, dN);
    const uint32_t* cell = m.cells + (size_t)j * 32u;
    phi0 = phi1 = 0.0;
    grad0 = d3(0, 0, 0);
    for (int k = 0; k < 32; k++) {
        const uint32_t v = cell[k];
        const double f0 = m.nodes[v], f1 = m.nodes[m.nodeCount + v];
        phi0 += f0 * N[k];
        grad0 += f0 * dN[k];
        phi1 += f1 * N[k];
    }
    grad0 = d3(grad0.x * c0[0], grad0.y * c0[1], grad0.z * c0[2]);
    return true;
}

// ---------------------------------------------------------------- step kernels
#define F64_THREAD                                          \
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; \
    if (i >= p.n) return;

__device__ __forceinline__ uint32_t nbr(const A& a, uint32_t i, uint32_t j) { return a.NBR[(size_t)i * kCap + j]; }

// K1 ComputeVolumeAndBoundaryKernel (DFSPHKernels.cu:69-150)
__global__ void k_boundary(P p, A a) {
    F64_THREAD
    D3 x = a.X[i];
    for (uint32_t b = 0; b < p.bodies; b++) {
        D3 xb = d3(0, 0, 0);
        double vb = 0.0;
        double dist = DBL_MAX, phi1 = 0.0;
        D3 normal = d3(0, 0, 0);
        map_lookup(a.bodyTab[p.bodyBegin + b], x, dist, normal, phi1);  // leaves dist = DBL_MAX outside the map
        if (dist > 0.0 && dist < p.h) {
            if (phi1 > 0.0 && phi1 != DBL_MAX) {
                const double nl = sqrt(dot(normal, normal));
                if (nl > 1.0e-9) {
                    vb = phi1;
                    normal = normal * (1.0 / nl);
                    xb = x - fmax(dist + 0.5 * p.r, p.diam) * normal;
                }
            }
        } else if (dist <= 0.0) {
            const double nl = sqrt(dot(normal, normal));
            if (nl > 1.0e-5) {
                normal = normal * (1.0 / nl);
                x += fmin(p.diam - dist, 0.1 * p.r) * normal;
                a.V[i] = d3(0, 0, 0);
            }
        }
        a.XB[(size_t)b * p.n + i] = xb;
        a.VB[(size_t)b * p.n + i] = vb;
    }
    a.X[i] = x;
}

// K2 ComputeDensityKernel (:152-187) + K3 ComputeDFSPHFactorKernel (:189-231)
__global__ void k_density_factor(P p, A a) {
    F64_THREAD
    const D3 xi = a.X[i];
    double rho = p.volume * p.wZero, sum = 0.0;
    D3 gi = d3(0, 0, 0);
    const uint32_t cnt = a.NCNT[i];
    for (uint32_t j = 0; j < cnt; j++) {
        const D3 r = xi - a.X[nbr(a, i, j)];
        rho += p.volume * kw(p, a, r);
        const D3 gj = -p.volume * kgrad(p, a, r);
        sum += dot(gj, gj);
        gi -= gj;
    }
    for (uint32_t b = 0; b < p.bodies; b++) {
        const double vb = a.VB[(size_t)b * p.n + i];
        if (vb > 0.0) {
            const D3 r = xi - a.XB[(size_t)b * p.n + i];
            rho += vb * kw(p, a, r);
            gi -= -vb * kgrad(p, a, r);
        }
    }
    a.RHO[i] = rho * p.rho0;
    sum += dot(gi, gi);
    a.ALPHA[i] = sum > (double)kEps ? 1.0 / sum : 0.0;
}

__device__ double velocity_divergence(const P& p, const A& a, uint32_t i) {  // K4 :498-522, K17 :253-271
    const D3 xi = a.X[i], vi = a.V[i];
    double d = 0.0;
    const uint32_t cnt = a.NCNT[i];
    for (uint32_t j = 0; j < cnt; j++) {
        const uint32_t k = nbr(a, i, j);
        d += dot(vi - a.V[k], kgrad(p, a, xi - a.X[k]));
    }
    d *= p.volume;
    for (uint32_t b = 0; b < p.bodies; b++) {
        const double vb = a.VB[(size_t)b * p.n + i];
        if (vb > 0.0) d += vb * dot(vi, kgrad(p, a, xi - a.XB[(size_t)b * p.n + i]));
    }
    return d;
}
__device__ D3 pressure_accel(const P& p, const A& a, uint32_t i, const double* kap) {  // K5/K7/K18/K20
    const D3 xi = a.X[i];
    const double ki = kap[i];
    D3 acc = d3(0, 0, 0);
    const uint32_t cnt = a.NCNT[i];
    for (uint32_t j = 0; j < cnt; j++) {
        const uint32_t k = nbr(a, i, j);
        const double s = ki + kap[k];
        if (fabs(s) > (double)kEps) acc += s * (-p.volume * kgrad(p, a, xi - a.X[k]));
    }
    if (fabs(ki) > (double)kEps)
        for (uint32_t b = 0; b < p.bodies; b++) {
            const double vb = a.VB[(size_t)b * p.n + i];
            if (vb > 0.0) acc += ki * (-vb * kgrad(p, a, xi - a.XB[(size_t)b * p.n + i]));
        }
    return acc;
}
__device__ double pressure_force(const P& p, const A& a, uint32_t i) {  // :280-315
    const D3 xi = a.X[i], ai = a.AP[i];
    double f = 0.0;
    const uint32_t cnt = a.NCNT[i];
    for (uint32_t j = 0; j < cnt; j++) {
        const uint32_t k = nbr(a, i, j);
        f += dot(ai - a.AP[k], kgrad(p, a, xi - a.X[k]));
    }
    f *= p.volume;
    for (uint32_t b = 0; b < p.bodies; b++) {
        const double vb = a.VB[(size_t)b * p.n + i];
        if (vb > 0.0) f += vb * dot(ai, kgrad(p, a, xi - a.XB[(size_t)b * p.n + i]));
    }
    return f;
}

// K4 ComputeDensityChangeKernel (:483-529)
__global__ void k_div_init(P p, A a) {
    F64_THREAD
    double d = velocity_divergence(p, a, i);
    d = a.NCNT[i] < 20u ? 0.0 : fmax(d, 0.0);
    a.RHOADV[i] = d;
    a.ALPHA[i] *= p.dtInv;
    a.KAPPAV[i] = d * a.ALPHA[i];
}
__global__ void k_paccel(P p, A a, int div) {  // K5 / K18
    F64_THREAD
    a.AP[i] = pressure_accel(p, a, i, div ? a.KAPPAV : a.KAPPA);
}
// K6 DivergenceSolveIterationKernel (:531-553) / K19 PressureSolveIterationKernel (:317-340)
__global__ void k_jacobi(P p, A a, int div) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    double res = 0.0;
    if (i < p.n) {
        if (div) {
            const double s = pressure_force(p, a, i) * p.dt;
            res = a.NCNT[i] < 20u ? 0.0 : fmin(-a.RHOADV[i] - s, 0.0);
            a.KAPPAV[i] -= res * a.ALPHA[i];
        } else {
            const double s = pressure_force(p, a, i) * p.dt2;
            res = fmin(1.0 - a.RHOADV[i] - s, 0.0);
            a.KAPPA[i] -= res * a.ALPHA[i];
        }
        a.RES[i] = res;
    }
    block_partial(a, res, false);
}
// K7 ComputePressureAccelerationAndFactorKernel (:555-602) + K8 ClearAccelerationKernel (:24-37)
__global__ void k_div_finish(P p, A a, int div) {
    F64_THREAD
    if (div) {
        const D3 ap = pressure_accel(p, a, i, a.KAPPAV);
        a.AP[i] = ap;
        a.V[i] += p.dt * ap;
        a.ALPHA[i] *= p.dt;
    }
    a.Acc[i] = d3(p.g[0], p.g[1], p.g[2]);
}

// K9 ComputeSurfaceTensionClassificationKernel (:881-958)
__global__ void k_st_classify(P p, A a) {
    F64_THREAD
    a.N[i] = d3(0, 0, 0);
    const D3 xi = a.X[i];
    const uint32_t cnt = a.NCNT[i];
    if (cnt == 0) {
        a.CURV[i] = 1.0 / p.h;
        return;
    }
    D3 com = d3(0, 0, 0);
    for (uint32_t j = 0; j < cnt; j++) com += a.X[nbr(a, i, j)] - xi;
    com = com * (1.0 / p.h);
    const double input = sqrt(dot(com, com)) / (double)cnt;
    if (!((double)cnt <= p.slope * input + p.constant + 0.0)) return;
    const uint32_t S = p.stSamples;
    const uint32_t s0 = i * S / 3u * 3u;
    const double ratio = p.nbrRadius / p.r;
    uint32_t count = 0;
    D3 nsum = d3(0, 0, 0);
    for (uint32_t q = 0; q < S; q++) {
        const uint32_t i3 = s0 + 3u * q;
        const D3 pt = p.h * d3(a.halton[i3 % kHaltonCount], a.halton[(i3 + 1u) % kHaltonCount],
                               a.halton[(i3 + 2u) % kHaltonCount]);
        bool covered = false;
        for (uint32_t j = 0; j < cnt && !covered; j++) {
            const D3 vec = pt - (a.X[nbr(a, i, j)] - xi);
            covered = dot(vec, vec) <= ratio * ratio * p.h2;
        }
        if (!covered) {
            nsum += pt;
            count++;
        }
    }
    if (count > 0) {
        if (dot(nsum, nsum) > 0.0) nsum = normalized(nsum);
        a.N[i] = nsum;
        a.CURV[i] = 1.0 / p.h * -2.0 * sqrt(1.0 - p.nbrRadius * p.nbrRadius / (p.r * p.r)) *
                    cos(acos(1.0 - 2.0 * ((double)count / (double)S)) + p.mcFactor);
    } else {
        a.CURV[i] = 0.0;
    }
}
// K10 ComputeSurfaceTensionNormalsAndCurvatureKernel (:960-1006)
__global__ void k_st_smooth(P p, A a) {
    F64_THREAD
    if (!nonzero(a.N[i])) return;
    const D3 xi = a.X[i];
    D3 nc = d3(0, 0, 0);
    double cc = 0.0, cf = 0.0;
    const uint32_t cnt = a.NCNT[i];
    for (uint32_t j = 0; j < cnt; j++) {
        const uint32_t k = nbr(a, i, j);
        if (nonzero(a.N[k])) {
            const D3 e = a.X[k] - xi;
            const double num = 1.0 - sqrt(dot(e, e)) / p.h;
            nc += a.N[k] * num;
            cc += a.CURV[k] * num;
            cf += num;
        }
    }
    if (dot(nc, nc) > 0.0) nc = normalized(nc);
    D3 ns = (1.0 - p.smoothing) * a.N[i] + p.smoothing * nc;
    if (dot(ns, ns) > 0.0) ns = normalized(ns);
    a.NS[i] = ns;
    a.CURVS[i] = ((1.0 - p.smoothing) * a.CURV[i] + p.smoothing * cc) / (1.0 - p.smoothing + p.smoothing * cf);
}
// K11 ComputeSurfaceTensionBlendingKernel (:1008-1046), one smoothing pass
__global__ void k_st_blend(P p, A a) {
    F64_THREAD
    if (nonzero(a.N[i])) {
        double fc = a.CURVS[i];
        if (p.temporal) fc = 0.05 * fc + 0.95 * a.DK[i];
        a.Acc[i] -= p.massInv * (a.NS[i] * p.st * fc);
        a.DK[i] = fc;
    } else {
        a.DK[i] = p.temporal ? 0.95 * a.DK[i] : 0.0;
    }
}

// Boundary samples of the viscosity terms (:636-681, :706-752, :793-839).
__device__ bool visc_samples(const P& p, const A& a, uint32_t i, uint32_t b, D3 dir[4], D3 grad[4], double& vol) {
    const double vb = a.VB[(size_t)b * p.n + i];
    if (!(vb > 0.0)) return false;
    const D3 xi = a.X[i], xb = a.XB[(size_t)b * p.n + i];
    D3 normal = -(xi - xb);
    const double nl = sqrt(dot(normal, normal));
    if (!(nl > 0.0001)) return false;
    normal = normal * (1.0 / nl);
    D3 v = d3(1, 0, 0);
    if (fabs(dot(v, normal)) > 0.999) v = d3(0, 1, 0);  // GetOrthogonalVectors, Core/Math/Math.h:19-33
    D3 t1 = cross(normal, v);
    D3 t2 = cross(normal, t1);
    t1 = normalized(t1);
    t2 = normalized(t2);
    const D3 pos[4] = {xb - t1 * p.tangDist, xb + t1 * p.tangDist, xb - t2 * p.tangDist, xb + t2 * p.tangDist};
    for (int k = 0; k < 4; k++) {
        dir[k] = xi - pos[k];
        grad[k] = kgrad(p, a, dir[k]);
    }
    vol = 0.25 * vb;
    return true;
}
// K12 ComputeViscosityPreconditionerKernel (:604-684) + K13's b = v and the warm start g
__global__ void k_visc_precond(P p, A a) {
    F64_THREAD
    M3 res = {};
    const D3 xi = a.X[i];
    const uint32_t cnt = a.NCNT[i];
    for (uint32_t j = 0; j < cnt; j++) {
        const uint32_t k = nbr(a, i, j);
        const D3 d = xi - a.X[k];
        add_outer(res, 10.0 * p.dynVisc * (p.mass / a.RHO[k]) / (dot(d, d) + 0.01 * p.h2), d, kgrad(p, a, d));
    }
    if (p.dynBVisc != 0.0)
        for (uint32_t b = 0; b < p.bodies; b++) {
            D3 dir[4], grad[4];
            double vol;
            if (!visc_samples(p, a, i, b, dir, grad, vol)) continue;
            for (int k = 0; k < 4; k++)  // positionDirection1 in all four terms (:674-677)
                add_outer(res, 10.0 * p.dynBVisc * vol / (dot(dir[k], dir[k]) + 0.01 * p.h2), dir[0], grad[k]);
        }
    M3 m;
    const double f = p.dt / a.RHO[i];
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) m.m[r][c] = (r == c ? 1.0 : 0.0) - f * res.m[r][c];
    a.MINV[i] = inverse(m);
    a.CB[i] = a.V[i];
    a.CG[i] = a.V[i] + a.DV[i];
}
// ComputeMatrixVecProdFunctionKernel (:758-842): out = A vec; sum of vec . out per block
__global__ void k_matvec(P p, A a, const D3* vec, D3* out, int dotWith) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    double t = 0.0;
    if (i < p.n) {
        const D3 xi = a.X[i], vi = vec[i];
        D3 acc = d3(0, 0, 0);
        const uint32_t cnt = a.NCNT[i];
        for (uint32_t j = 0; j < cnt; j++) {
            const uint32_t k = nbr(a, i, j);
            const D3 d = xi - a.X[k];
            acc += (10.0 * p.dynVisc * (p.mass / a.RHO[k]) * dot(vi - vec[k], d) / (dot(d, d) + 0.01 * p.h2)) *
                   kgrad(p, a, d);
        }
        if (p.dynBVisc != 0.0)
            for (uint32_t b = 0; b < p.bodies; b++) {
                D3 dir[4], grad[4];
                double vol;
                if (!visc_samples(p, a, i, b, dir, grad, vol)) continue;
                for (int k = 0; k < 4; k++)
                    acc += (10.0 * p.dynBVisc * vol * dot(vi, dir[k]) / (dot(dir[k], dir[k]) + 0.01 * p.h2)) * grad[k];
            }
        const D3 r = vi - (p.dt / a.RHO[i]) * acc;
        out[i] = r;
        if (dotWith) t = dot(vi, r);
    }
    block_partial(a, t, false);
}
// the CG's vector steps (DFSPHImplementation.cu:627-805); each reduces one dot product
__global__ void k_cg_residual(P p, A a) {  // r = b - A g, sum |r|^2
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    double t = 0.0;
    if (i < p.n) {
        const D3 r = a.CB[i] - a.CT[i];
        a.CR[i] = r;
        t = dot(r, r);
    }
    block_partial(a, t, false);
}
__global__ void k_dot(P p, A a, const D3* u, const D3* w) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    block_partial(a, i < p.n ? dot(u[i], w[i]) : 0.0, false);
}
__global__ void k_precondition(P p, A a, D3* out) {  // out = M^-1 r, sum r . out
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    double t = 0.0;
    if (i < p.n) {
        const D3 z = mul(a.MINV[i], a.CR[i]);
        out[i] = z;
        t = dot(a.CR[i], z);
    }
    block_partial(a, t, false);
}
__global__ void k_cg_update(P p, A a, double alpha) {  // g += alpha p, r -= alpha Ap, sum |r|^2
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    double t = 0.0;
    if (i < p.n) {
        a.CG[i] += a.CP[i] * alpha;
        a.CR[i] -= a.CT[i] * alpha;
        t = dot(a.CR[i], a.CR[i]);
    }
    block_partial(a, t, false);
}
__global__ void k_cg_p(P p, A a, double beta) {
    F64_THREAD
    a.CP[i] = a.CP[i] * beta + a.CZ[i];
}
// K15 ApplyViscosityForceKernel (:844-862)
__global__ void k_visc_apply(P p, A a, int zeroG) {
    F64_THREAD
    const D3 g = zeroG ? d3(0, 0, 0) : a.CG[i];
    a.Acc[i] += (1.0 / p.dt) * (g - a.V[i]);
    a.DV[i] = g - a.V[i];
}
// ComputeMaxVelocityMagnitude (DFSPHImplementation.cu:430-441): max |v + a dt|^2 per block
__global__ void k_cfl(P p, A a) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    double m = 0.0;
    if (i < p.n) {
        const D3 w = a.V[i] + a.Acc[i] * p.dt;
        m = dot(w, w);
    }
    block_partial(a, m, true);
}
__global__ void k_velocity(P p, A a) {  // K16 ComputeVelocityKernel (:39-52)
    F64_THREAD
    a.V[i] += p.dt * a.Acc[i];
}
__global__ void k_pres_init(P p, A a) {  // K17 ComputeDensityAdvectionKernel (:233-278)
    F64_THREAD
    const double d = velocity_divergence(p, a, i);
    const double rhoAdv = a.RHO[i] / p.rho0 + p.dt * d;
    a.RHOADV[i] = rhoAdv;
    a.ALPHA[i] *= p.dt2Inv;
    a.KAPPA[i] = -fmin(1.0 - rhoAdv, 0.0) * a.ALPHA[i];
}
// K20 ComputePressureAccelerationAndVelocityKernel (:434-481); K21 positions after all
__global__ void k_pres_finish(P p, A a) {
    F64_THREAD
    const D3 ap = pressure_accel(p, a, i, a.KAPPA);
    a.AP[i] = ap;
    a.V[i] += p.dt * ap;
}
__global__ void k_position(P p, A a) {  // K21 ComputePositionKernel (:54-67)
    F64_THREAD
    a.X[i] += p.dt * a.V[i];
}
__global__ void k_export(P p, const D3* src, float* out) {
    F64_THREAD
    const D3 v = src[i];
    out[3 * (size_t)i] = (float)v.x;
    out[3 * (size_t)i + 1] = (float)v.y;
    out[3 * (size_t)i + 2] = (float)v.z;
}

}  // namespace f64

using namespace f64;
using host::fail;

// Host side: the FP64 state of a simulation and its step.
struct Fp64State {
    f64::A a{};
    f64::P p{};
    std::vector<void*> allocs;
    void* cellAllocs[5] = {};  // CNT, START, FILL, BSUM (grown with the grid)
    uint32_t cellCap = 0, blockCap = 0;
    double frameTime = 0.0;
    vfd_step_stats stats{};
    ~Fp64State() {
        for (void* q : allocs) cudaFree(q);
        for (void* q : cellAllocs) cudaFree(q);
    }
};

namespace {

template <class T>
int falloc(Fp64State* f, T** ptr, size_t count) {
    void* q = nullptr;
    const cudaError_t e = cudaMalloc(&q, std::max<size_t>(1, count) * sizeof(T));
    if (e != cudaSuccess) return fail(VFD_E_NOMEM, "FP64 path: cudaMalloc: %s", cudaGetErrorString(e));
    f->allocs.push_back(q);
    *ptr = (T*)q;
    return VFD_OK;
}

#define FCK(call)                                                                                          \
    do {                                                                                                   \
        cudaError_t e_ = (call);                                                                           \
        if (e_ != cudaSuccess) return fail(VFD_E_CUDA, "FP64 path: %s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

// Sum (or max) of the per-block partials of the last reduction kernel, in block order.
int partials(Fp64State* f, uint32_t nb, cudaStream_t st, bool isMax, double& out) {
    std::vector<double> h(nb);
    FCK(cudaMemcpyAsync(h.data(), f->a.PART, sizeof(double) * nb, cudaMemcpyDeviceToHost, st));
    FCK(cudaStreamSynchronize(st));
    double t = 0.0;
    for (uint32_t b = 0; b < nb; b++) t = isMax ? std::max(t, h[b]) : t + h[b];
    out = t;
    return VFD_OK;
}

void set_dt(f64::P& p, double dt) {
    p.dt = dt;
    p.dt2 = dt * dt;
    p.dtInv = 1.0 / dt;
    p.dt2Inv = 1.0 / p.dt2;
}

uint32_t samples_for(const vfd_desc& d, double dt) {
    return d.CSDFix > 0 ? (uint32_t)d.CSDFix : (uint32_t)(int)((double)d.CSD * dt);
}

}  // namespace

// Creates (or rebuilds) the FP64 state from the scene's initial particles.
int fp64_upload(vfd_sim* s) {
    if (s->scenes.size() != 1) return fail(VFD_E_STATE, "the FP64 path runs single-scene simulations");
    delete s->fp64;
    s->fp64 = new Fp64State();
    Fp64State* f = s->fp64;
    const host::SceneHost& sc = s->scenes[0];
    const uint32_t n = (uint32_t)(sc.x0.size() / 3);
    const uint32_t nb = (uint32_t)sc.bodies.size();
    f64::A& a = f->a;
    f64::P& p = f->p;
    TRY(falloc(f, &a.X, n)); TRY(falloc(f, &a.V, n)); TRY(falloc(f, &a.Acc, n)); TRY(falloc(f, &a.AP, n));
    TRY(falloc(f, &a.DV, n)); TRY(falloc(f, &a.N, n)); TRY(falloc(f, &a.NS, n));
    TRY(falloc(f, &a.XB, (size_t)std::max(1u, nb) * n)); TRY(falloc(f, &a.VB, (size_t)std::max(1u, nb) * n));
    TRY(falloc(f, &a.RHO, n)); TRY(falloc(f, &a.ALPHA, n)); TRY(falloc(f, &a.RHOADV, n)); TRY(falloc(f, &a.KAPPA, n));
    TRY(falloc(f, &a.KAPPAV, n)); TRY(falloc(f, &a.RES, n)); TRY(falloc(f, &a.CURV, n)); TRY(falloc(f, &a.CURVS, n));
    TRY(falloc(f, &a.DK, n));
    TRY(falloc(f, &a.CR, n)); TRY(falloc(f, &a.CP, n)); TRY(falloc(f, &a.CZ, n)); TRY(falloc(f, &a.CT, n));
    TRY(falloc(f, &a.CB, n)); TRY(falloc(f, &a.CG, n)); TRY(falloc(f, &a.MINV, n));
    TRY(falloc(f, &a.NCNT, n)); TRY(falloc(f, &a.NBR, (size_t)n * kCap)); TRY(falloc(f, &a.KEY, n));
    TRY(falloc(f, &a.TMP, n)); TRY(falloc(f, &a.ORDER, n)); TRY(falloc(f, &a.MM, 6));
    TRY(falloc(f, &a.PART, (n + kB - 1) / kB + 1));
    // SPH tables in double (PrecomputedDFSPHCubicKernel::SetRadius, Kernel/DFSPHKernels.h:13-41)
    const double r = (double)sc.desc.ParticleRadius, h = 4.0 * r, pi = 3.14159265358979323846;
    p.h = h;
    p.h2 = h * h;
    p.K = 8.0 / (pi * h * h * h);
    p.L = 48.0 / (pi * h * h * h);
    const double step = h / (double)(kTableRes - 1);
    p.invStep = 1.0 / step;
    auto calcW = [&](double x) {
        const double q = x / h;
        if (q > 1.0) return 0.0;
        if (q <= 0.5) return p.K * (6.0 * q * q * q - 6.0 * q * q + 1.0);
        const double g = 1.0 - q;
        return p.K * (2.0 * g * g * g);
    };
    auto calcG = [&](double x) {  // CalculateGradientW({x, 0, 0}).x / x
        const double q = x / h;
        if (!(x > 1.0e-5) || q > 1.0) return 0.0;
        const double gq = x * (1.0 / (x * h));
        const double v = q <= 0.5 ? ((p.L * q) * (3.0 * q - 2.0)) * gq : (p.L * (-(1.0 - q) * (1.0 - q))) * gq;
        return v / x;
    };
    std::vector<double> W(kTableRes), G(kTableRes + 1), WM(kTableRes), GM(kTableRes);
    for (uint32_t k = 0; k < kTableRes; k++) {
        const double x = step * (double)k;
        W[k] = calcW(x);
        G[k] = x > 1.0e-9 ? calcG(x) : 0.0;
    }
    G[kTableRes] = 0.0;
    for (uint32_t k = 0; k + 1 < kTableRes; k++) {
        WM[k] = 0.5 * (W[k] + W[k + 1]);
        GM[k] = 0.5 * (G[k] + G[k + 1]);
    }
    WM[kTableRes - 1] = GM[kTableRes - 1] = 0.0;
    double *dW = nullptr, *dG = nullptr;
    TRY(falloc(f, &dW, kTableRes));
    TRY(falloc(f, &dG, kTableRes));
    FCK(cudaMemcpy(dW, WM.data(), sizeof(double) * kTableRes, cudaMemcpyHostToDevice));
    FCK(cudaMemcpy(dG, GM.data(), sizeof(double) * kTableRes, cudaMemcpyHostToDevice));
    a.W = dW;
    a.G = dG;
    p.wZero = calcW(0.0);
    a.halton = s->dHalton;
    a.bodyTab = s->dBodies;
    // constants (DFSPHImplementation::SetDescription, :318-368) in double
    const vfd_desc& d = sc.desc;
    p.n = n;
    p.bodies = nb;
    p.bodyBegin = 0;
    p.analytic = s->analyticKernel ? 1u : 0u;
    p.r = r;
    p.diam = 2.0 * r;
    p.volume = 0.8 * p.diam * p.diam * p.diam;
    p.rho0 = 1000.0;
    p.mass = p.volume * p.rho0;
    p.massInv = 1.0 / p.mass;
    p.dynVisc = (double)d.Viscosity * p.rho0;
    p.dynBVisc = (double)d.BoundaryViscosity * p.rho0;
    p.tangDist = (double)d.TangentialDistanceFactor * h;
    p.st = (double)d.SurfaceTension;
    p.slope = 74.688796680497925;
    p.constant = 12.0;
    p.temporal = d.TemporalSmoothing != 0;
    p.smoothing = 0.5;
    p.nbrRadius = r * 0.8;
    p.mcFactor = std::asin(p.nbrRadius / r);
    for (int k = 0; k < 3; k++) p.g[k] = (double)d.Gravity[k];
    set_dt(p, (double)d.TimeStepSize);
    p.stSamples = samples_for(d, p.dt);
    // initial state from the FP32 inputs
    std::vector<f64::D3> x(n), v(n);
    for (uint32_t i = 0; i < n; i++) {
        x[i] = f64::D3{sc.x0[3 * i], sc.x0[3 * i + 1], sc.x0[3 * i + 2]};
        v[i] = sc.v0.empty() ? f64::D3{0, 0, 0} : f64::D3{sc.v0[3 * i], sc.v0[3 * i + 1], sc.v0[3 * i + 2]};
    }
    FCK(cudaMemcpy(a.X, x.data(), sizeof(f64::D3) * n, cudaMemcpyHostToDevice));
    FCK(cudaMemcpy(a.V, v.data(), sizeof(f64::D3) * n, cudaMemcpyHostToDevice));
    FCK(cudaMemset(a.DV, 0, sizeof(f64::D3) * n));
    FCK(cudaMemset(a.DK, 0, sizeof(double) * n));
    FCK(cudaMemset(a.Acc, 0, sizeof(f64::D3) * n));
    f->frameTime = 0.0;
    f->stats = vfd_step_stats{};
    return VFD_OK;
}

// One OnUpdate step (DFSPHImplementation.cu:63-170) in FP64.
int fp64_step(vfd_sim* s, vfd_step_stats* out) {
    Fp64State* f = s->fp64;
    if (!f) return fail(VFD_E_STATE, "FP64 state missing");
    f64::A& a = f->a;
    f64::P& p = f->p;
    const vfd_desc& d = s->scenes[0].desc;
    cudaStream_t st = s->stream;
    const uint32_t n = p.n;
    vfd_step_stats& S = f->stats;
    S.Flags = 0;
    if (n == 0) return VFD_OK;
    const uint32_t g = (n + kB - 1) / kB;
    // ---- neighbour search (ParticleSearch::FindNeighbors)
    const int init[6] = {INT_MAX, INT_MAX, INT_MAX, INT_MIN, INT_MIN, INT_MIN};
    FCK(cudaMemcpyAsync(a.MM, init, sizeof(init), cudaMemcpyHostToDevice, st));
    f64::k_minmax<<<g, kB, 0, st>>>(p, a);
    int mm[6];
    FCK(cudaMemcpyAsync(mm, a.MM, sizeof(mm), cudaMemcpyDeviceToHost, st));
    FCK(cudaStreamSynchronize(st));
    uint64_t cells = 1;
    for (int k = 0; k < 3; k++) {
        a.gmin[k] = mm[k] - 1;
        a.dim[k] = (uint32_t)(mm[3 + k] - mm[k] + 3);
        cells *= a.dim[k];
    }
    if (cells > (1ull << 31)) return fail(VFD_E_CAPACITY, "FP64 path: search grid of %llu cells", (unsigned long long)cells);
    a.cells = (uint32_t)cells;
    const uint32_t sb = (a.cells + 1023u) / 1024u;
    if (a.cells > f->cellCap) {
        for (void*& q : f->cellAllocs) {
            cudaFree(q);
            q = nullptr;
        }
        const size_t cap = (size_t)a.cells + a.cells / 4u;
        FCK(cudaMalloc(&f->cellAllocs[0], cap * sizeof(uint32_t)));
        FCK(cudaMalloc(&f->cellAllocs[1], cap * sizeof(uint32_t)));
        FCK(cudaMalloc(&f->cellAllocs[2], cap * sizeof(uint32_t)));
        FCK(cudaMalloc(&f->cellAllocs[3], (cap / 1024u + 2u) * sizeof(uint32_t)));
        f->cellCap = (uint32_t)cap;
    }
    a.CNT = (uint32_t*)f->cellAllocs[0];
    a.START = (uint32_t*)f->cellAllocs[1];
    a.FILL = (uint32_t*)f->cellAllocs[2];
    a.BSUM = (uint32_t*)f->cellAllocs[3];
    FCK(cudaMemsetAsync(a.CNT, 0, sizeof(uint32_t) * a.cells, st));
    FCK(cudaMemsetAsync(a.FILL, 0, sizeof(uint32_t) * a.cells, st));
    f64::k_keys<<<g, kB, 0, st>>>(p, a);
    f64::k_scan_blocks<<<sb, 1024, 0, st>>>(a);
    f64::k_scan_carry<<<1, 32, 0, st>>>(a, sb);
    f64::k_scan_add<<<sb, 1024, 0, st>>>(a);
    f64::k_slots<<<g, kB, 0, st>>>(p, a);
    f64::k_order<<<g, kB, 0, st>>>(p, a);
    f64::k_neighbors<<<g, kB, 0, st>>>(p, a);
    FCK(cudaGetLastError());
    // ---- boundary, density, factor
    f64::k_boundary<<<g, kB, 0, st>>>(p, a);
    f64::k_density_factor<<<g, kB, 0, st>>>(p, a);
    // ---- divergence solve (ComputeDivergence, :506-575)
    const bool div = d.EnableDivergenceSolverError != 0;
    uint32_t itD = 0;
    double errD = 0.0;
    if (div) {
        f64::k_div_init<<<g, kB, 0, st>>>(p, a);
        const double eta = p.dtInv * (double)d.MaxDivergenceSolverError * 0.0001 * p.rho0;
        while ((errD > eta || itD < d.MinDivergenceSolverIterations) && itD < d.MaxDivergenceSolverIterations) {
            f64::k_paccel<<<g, kB, 0, st>>>(p, a, 1);
            f64::k_jacobi<<<g, kB, 0, st>>>(p, a, 1);
            double sum;
            TRY(partials(f, g, st, false, sum));
            errD = -p.rho0 * sum / (double)n;
            itD++;
        }
        if (itD >= d.MaxDivergenceSolverIterations && d.MaxDivergenceSolverIterations > 0 && errD > eta)
            S.Flags |= VFD_FLAG_DIVERGENCE_CAP;
    }
    f64::k_div_finish<<<g, kB, 0, st>>>(p, a, div ? 1 : 0);
    // ---- surface tension (:810-839)
    const uint32_t samplesUsed = p.stSamples;
    if (d.EnableSurfaceTensionSolver) {
        f64::k_st_classify<<<g, kB, 0, st>>>(p, a);
        f64::k_st_smooth<<<g, kB, 0, st>>>(p, a);
        for (uint32_t pass = 0; pass < d.SurfaceTensionSmoothPassCount; pass++) f64::k_st_blend<<<g, kB, 0, st>>>(p, a);
    }
    // ---- viscosity (ComputeViscosity + SolveViscosity, :577-808)
    uint32_t itV = 0;
    double errV = 0.0;
    if (d.EnableViscositySolver) {
        f64::k_visc_precond<<<g, kB, 0, st>>>(p, a);
        f64::k_matvec<<<g, kB, 0, st>>>(p, a, a.CG, a.CT, 0);
        f64::k_cg_residual<<<g, kB, 0, st>>>(p, a);
        double rr;
        TRY(partials(f, g, st, false, rr));
        f64::k_dot<<<g, kB, 0, st>>>(p, a, a.CB, a.CB);
        double rhs;
        TRY(partials(f, g, st, false, rhs));
        int zeroG = 0;
        if (rhs == 0.0) {
            zeroG = 1;
        } else {
            const double e = (double)d.MaxViscositySolverError;
            const double thr = std::max(e * e * 0.0001 * rhs, (double)FLT_MIN);
            if (!(rr < thr)) {
                f64::k_precondition<<<g, kB, 0, st>>>(p, a, a.CP);
                double absNew;
                TRY(partials(f, g, st, false, absNew));
                absNew = std::fabs(absNew);
                while (itV >= d.MinViscositySolverIterations && itV < d.MaxViscositySolverIterations) {
                    f64::k_matvec<<<g, kB, 0, st>>>(p, a, a.CP, a.CT, 1);
                    double pap;
                    TRY(partials(f, g, st, false, pap));
                    f64::k_cg_update<<<g, kB, 0, st>>>(p, a, absNew / pap);
                    TRY(partials(f, g, st, false, rr));
                    if (rr < thr) break;
                    f64::k_precondition<<<g, kB, 0, st>>>(p, a, a.CZ);
                    const double absOld = absNew;
                    TRY(partials(f, g, st, false, absNew));
                    absNew = std::fabs(absNew);
                    f64::k_cg_p<<<g, kB, 0, st>>>(p, a, absNew / absOld);
                    itV++;
                }
                if (itV >= d.MaxViscositySolverIterations && rr >= thr) S.Flags |= VFD_FLAG_VISCOSITY_CAP;
            }
            errV = std::sqrt(rr / rhs);
        }
        f64::k_visc_apply<<<g, kB, 0, st>>>(p, a, zeroG);
    }
    // ---- CFL time step (ComputeTimeStepSize, :395-441)
    f64::k_cfl<<<g, kB, 0, st>>>(p, a);
    double mv;
    TRY(partials(f, g, st, true, mv));
    mv = std::max(0.1, mv);
    if (mv < 1.0e-9) mv = 1.0e-9;
    double dt = 0.4 * (p.diam / std::sqrt(mv));
    dt = std::min(dt, (double)d.MaxTimeStepSize);
    dt = std::max(dt, (double)d.MinTimeStepSize);
    set_dt(p, dt);
    p.stSamples = samples_for(d, dt);
    f->frameTime += dt;
    f64::k_velocity<<<g, kB, 0, st>>>(p, a);
    // ---- pressure solve (ComputePressure, :443-504)
    f64::k_pres_init<<<g, kB, 0, st>>>(p, a);
    const double eta = (double)d.MaxPressureSolverError * 0.0001 * p.rho0;
    uint32_t itP = 0;
    double errP = 0.0;
    while ((errP > eta || itP < d.MinPressureSolverIterations) && itP < d.MaxPressureSolverIterations) {
        f64::k_paccel<<<g, kB, 0, st>>>(p, a, 0);
        f64::k_jacobi<<<g, kB, 0, st>>>(p, a, 0);
        double sum;
        TRY(partials(f, g, st, false, sum));
        errP = -p.rho0 * sum / (double)n;
        itP++;
    }
    if (itP >= d.MaxPressureSolverIterations && d.MaxPressureSolverIterations > 0 && errP > eta)
        S.Flags |= VFD_FLAG_PRESSURE_CAP;
    f64::k_pres_finish<<<g, kB, 0, st>>>(p, a);
    f64::k_position<<<g, kB, 0, st>>>(p, a);
    FCK(cudaGetLastError());
    FCK(cudaStreamSynchronize(st));
    if (S.FrameIndex < d.FrameCount && f->frameTime >= (double)d.FrameLength) {  // :148-167
        f->frameTime = 0.0;
        S.FrameIndex++;
    }
    S.IterationCount++;
    S.DivergenceSolverIterationCount = div ? itD : 0u;
    S.DivergenceSolverError = div ? (float)errD : 0.0f;
    S.PressureSolverIterationCount = itP;
    S.PressureSolverError = (float)errP;
    S.ViscositySolverIterationCount = d.EnableViscositySolver ? itV : 0u;
    S.ViscositySolverError = (float)errV;
    S.FrameTime = (float)f->frameTime;
    S.TimeStepSize = (float)dt;
    S.MaxVelocityMagnitude = (float)mv;
    S.SurfaceTensionSampleCount = samplesUsed;
    if (out) *out = S;
    return VFD_OK;
}

int fp64_get_state(vfd_sim* s, double* x, double* v, float* xf, float* vf, float* af) {
    Fp64State* f = s->fp64;
    const uint32_t n = f->p.n;
    cudaStream_t st = s->stream;
    if (x) FCK(cudaMemcpyAsync(x, f->a.X, sizeof(f64::D3) * n, cudaMemcpyDeviceToHost, st));
    if (v) FCK(cudaMemcpyAsync(v, f->a.V, sizeof(f64::D3) * n, cudaMemcpyDeviceToHost, st));
    const uint32_t g = (n + kB - 1) / kB;
    const f64::D3* src[3] = {f->a.X, f->a.V, f->a.Acc};
    float* dst[3] = {xf, vf, af};
    for (int k = 0; k < 3; k++) {
        if (!dst[k]) continue;
        f64::k_export<<<g, kB, 0, st>>>(f->p, src[k], s->dStage);
        FCK(cudaMemcpyAsync(dst[k], s->dStage, sizeof(float) * 3 * (size_t)n, cudaMemcpyDeviceToHost, st));
    }
    FCK(cudaStreamSynchronize(st));
    return VFD_OK;
}

int fp64_get_density(vfd_sim* s, float* out) {
    Fp64State* f = s->fp64;
    std::vector<double> h(f->p.n);
    FCK(cudaMemcpy(h.data(), f->a.RHO, sizeof(double) * f->p.n, cudaMemcpyDeviceToHost));
    for (uint32_t i = 0; i < f->p.n; i++) out[i] = (float)h[i];
    return VFD_OK;
}

void fp64_stats(const vfd_sim* s, vfd_step_stats* out) {
    if (s->fp64) *out = s->fp64->stats;
}

void fp64_release(vfd_sim* s) {
    delete s->fp64;
    s->fp64 = nullptr;
}

}  // namespace vfd
