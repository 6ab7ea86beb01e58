// dfsph_oracle.cpp -- CPU restatement of VFD's DFSPH step, used as TEST
// INFRASTRUCTURE ONLY: the parity checker of the CUDA library and the timed
// CPU baseline. Nothing in the product links, loads or calls this code.
//
// It restates, function by function, the reference's per-step algorithm
// (paths relative to VFD/Source/Simulation/DFSPH/ unless noted):
//   * the SPH cubic-spline table          Kernel/DFSPHKernels.h:13-131
//   * the neighbour search N1-N8          ParticleSearch/ParticleSearch.cu:29-195,
//                                         ParticleSearch/ParticleSearchKernels.cu:4-193
//   * the 22 DFSPH kernels K1-K21         DFSPHKernels.cu:6-1046
//   * the solver control flow             DFSPHImplementation.cu:63-839
//   * the volume-map lookup and build     Utility/SDF/SDFDeviceData.cuh:36-474,
//                                         Utility/SDF/SDF.cu:45-139, 313-373,
//                                         RigidBody/RigidBody.cu:10-72,
//                                         Core/Math/GaussQuadrature.cpp:5621-5656
//   * the surface-tension sample table    HaltonVec323.cuh:4 (regenerated from
//                                         its Halton(2,3) formula)
// templated on the arithmetic type: T = float is the FP32 mirror (same
// operation order as the reference, no FMA contraction: build with
// -ffp-contract=off), T = double is the FP64 oracle.
//
// Parity pinning: partial. The reference cannot be built here (Windows headers, the glm
// submodule is absent) and ships no tests or fixtures; the oracle is pinned against the
// tables and constants of the reference's source (tests/golden/reference_tables.json)
// and closed forms, not against outputs of the reference's step.
//
// Deterministic rules where the reference is not deterministic:
//   * in-cell order of the counting sort: ascending original particle index
//     (the reference's atomicAdd rank, ParticleSearchKernels.cu:78, gives any
//     order; this is one of its legal outcomes);
//   * solver error reductions: FP64 sum, error = -rho0 * sum(res) / N (the
//     reference folds with thrust::minus, DFSPHImplementation.cu:483-489,
//     whose result depends on the reduction tree);
//   * viscosity CG dot products summed in FP64 over particles (each particle's term in T).
#include "../include/vfd_dfsph.h"

#include <algorithm>
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <map>
#include <memory>
#include <utility>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace orc {

static const double kPI = 3.14159265358979323846;  // Core/Math/Math.h:4
static const double kEPS = 1.0e-5;                  // Core/Math/Math.h:6 (a double literal)

template <class T>
struct V3 {
    T x, y, z;
    V3() : x(0), y(0), z(0) {}
    V3(T a, T b, T c) : x(a), y(b), z(c) {}
    V3 operator+(const V3& o) const { return V3(x + o.x, y + o.y, z + o.z); }
    V3 operator-(const V3& o) const { return V3(x - o.x, y - o.y, z - o.z); }
    V3 operator-() const { return V3(-x, -y, -z); }
    V3 operator*(T s) const { return V3(x * s, y * s, z * s); }
    V3 operator*(const V3& o) const { return V3(x * o.x, y * o.y, z * o.z); }
    V3 operator/(T s) const { return V3(x / s, y / s, z / s); }
    V3& operator+=(const V3& o) { x += o.x; y += o.y; z += o.z; return *this; }
    V3& operator-=(const V3& o) { x -= o.x; y -= o.y; z -= o.z; return *this; }
    V3& operator*=(T s) { x *= s; y *= s; z *= s; return *this; }
    V3& operator/=(T s) { x /= s; y /= s; z /= s; return *this; }
    bool operator!=(const V3& o) const { return x != o.x || y != o.y || z != o.z; }
    T& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    T operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
template <class T> static inline V3<T> operator*(T s, const V3<T>& v) { return v * s; }
// glm::dot sums the component products left to right.
template <class T> static inline T dot(const V3<T>& a, const V3<T>& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T> static inline T length2(const V3<T>& a) { return dot(a, a); }
template <class T> static inline T length(const V3<T>& a) { return std::sqrt(dot(a, a)); }
template <class T> static inline V3<T> cross(const V3<T>& a, const V3<T>& b) {
    return V3<T>(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
template <class T> static inline V3<T> normalize(const V3<T>& a) { return a / length(a); }

// Row-major 3x3 in mathematical order: m[r][c].
template <class T>
struct M3 {
    T m[3][3];
    M3() { for (int r = 0; r < 3; r++) for (int c = 0; c < 3; c++) m[r][c] = 0; }
    V3<T> mul(const V3<T>& v) const {
        return V3<T>(m[0][0] * v.x + m[0][1] * v.y + m[0][2] * v.z,
                     m[1][0] * v.x + m[1][1] * v.y + m[1][2] * v.z,
                     m[2][0] * v.x + m[2][1] * v.y + m[2][2] * v.z);
    }
    // this += s * (a b^T): glm::outerProduct(a, b) read as a matrix.
    void add_outer(T s, const V3<T>& a, const V3<T>& b) {
        for (int r = 0; r < 3; r++)
            for (int c = 0; c < 3; c++) m[r][c] += s * (a[r] * b[c]);
    }
};

// Inverse by cofactors / determinant.
template <class T>
static M3<T> inverse(const M3<T>& a) {
    const T (&m)[3][3] = a.m;
    const T c00 = m[1][1] * m[2][2] - m[1][2] * m[2][1];
    const T c01 = m[1][2] * m[2][0] - m[1][0] * m[2][2];
    const T c02 = m[1][0] * m[2][1] - m[1][1] * m[2][0];
    const T det = m[0][0] * c00 + m[0][1] * c01 + m[0][2] * c02;
    const T id = T(1) / det;
    M3<T> r;
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

// Core/Math/Math.h:19-33 GetOrthogonalVectors.
template <class T>
static void orthogonal_vectors(const V3<T>& vec, V3<T>& x, V3<T>& y) {
    V3<T> v(T(1), T(0), T(0));
    if (std::fabs((double)dot(v, vec)) > 0.999) v = V3<T>(T(0), T(1), T(0));
    x = cross(vec, v);
    y = cross(vec, x);
    x = normalize(x);
    y = normalize(y);
}

// ---------------------------------------------------------------------------
// SPH cubic spline table: Kernel/DFSPHKernels.h:8-143 (Resolution 10000).
template <class T>
struct KernelTable {
    static const unsigned R = 10000u;
    std::vector<T> W, G;
    T radius = 0, radius2 = 0, invStep = 0, wZero = 0, K = 0, L = 0;
    bool analytic = false;  // the spline at |r| instead of the table (analytic kernel mode)

    T calcW(T r) const {  // :86-104
        T res = 0;
        const T q = r / radius;
        if (q <= T(1)) {
            if (q <= T(0.5)) {
                const T q2 = q * q;
                const T q3 = q2 * q;
                res = K * (T(6) * q3 - T(6) * q2 + T(1));
            } else {
                const T q1 = T(1) - q;
                const T q3 = q1 * q1 * q1;
                res = K * (T(2) * q3);
            }
        }
        return res;
    }
    V3<T> calcGradW(const V3<T>& r) const {  // :110-131
        V3<T> res;
        const T rl = std::sqrt(dot(r, r));
        const T q = rl / radius;
        if (rl > T(1.0e-5) && q <= T(1)) {
            const V3<T> gq = r * (T(1) / (rl * radius));
            if (q <= T(0.5)) res = ((L * q) * (T(3) * q - T(2))) * gq;
            else {
                const T f = T(1) - q;
                res = (L * (-f * f)) * gq;
            }
        }
        return res;
    }
    void setRadius(T r) {  // :13-41
        const T pi = (T)kPI;
        W.assign(R, 0);
        G.assign(R + 1, 0);
        radius = r;
        radius2 = radius * radius;
        const T r3 = radius * radius * radius;
        K = T(8) / (pi * r3);
        L = T(48) / (pi * r3);
        wZero = calcW(std::sqrt(T(0)));
        const T step = radius / (T)(R - 1);
        invStep = T(1) / step;
        for (unsigned i = 0; i < R; i++) {
            const T px = step * (T)i;
            W[i] = calcW(px);
            if (px > T(1.0e-9)) G[i] = calcGradW(V3<T>(px, 0, 0)).x / px;
            else G[i] = 0;
        }
        G[R] = 0;
    }
    unsigned pos(T rl) const {
        unsigned p = (unsigned)(rl * invStep);
        return std::min(p, R - 2u);
    }
    T getW(T r) const {  // :43-52
        if (r <= radius) {
            if (analytic) return calcW(r);
            const unsigned p = pos(r);
            return T(0.5) * (W[p] + W[p + 1]);
        }
        return 0;
    }
    T getW(const V3<T>& r) const {  // :54-65
        const T r2 = dot(r, r);
        if (r2 <= radius2) {
            if (analytic) return calcW(std::sqrt(r2));
            const unsigned p = pos(std::sqrt(r2));
            return T(0.5) * (W[p] + W[p + 1]);
        }
        return 0;
    }
    V3<T> getGradW(const V3<T>& r) const {  // :67-80
        const T rl = std::sqrt(dot(r, r));
        if (rl <= radius) {
            if (analytic) return calcGradW(r);
            const unsigned p = pos(rl);
            return (T(0.5) * (G[p] + G[p + 1])) * r;
        }
        return V3<T>();
    }
};

// ---------------------------------------------------------------------------
// Surface-tension directions, HaltonVec323.cuh:4: point i of 16384 is
// (sqrt(1-z^2) cos 2 pi h2(i), sqrt(1-z^2) sin 2 pi h2(i), z = 1 - 2 h3(i)),
// h_b the radical inverse in base b; the reference lists the values with 15
// decimals, so each is rounded to 15 decimals before the float conversion.
static double radical_inverse(unsigned i, unsigned b) {
    double inv = 1.0 / b, f = inv, r = 0.0;
    while (i > 0) { r += f * (double)(i % b); i /= b; f *= inv; }
    return r;
}
static const unsigned kHaltonCount = 49152u;
static void halton_table(float* out) {
    for (unsigned i = 0; i < kHaltonCount / 3; i++) {
        const double z = 1.0 - 2.0 * radical_inverse(i, 3);
        const double phi = 2.0 * kPI * radical_inverse(i, 2);
        const double s = std::sqrt(std::max(0.0, 1.0 - z * z));
        const double v[3] = {s * std::cos(phi), s * std::sin(phi), z};
        for (int k = 0; k < 3; k++) out[3 * i + k] = (float)(std::nearbyint(v[k] * 1e15) / 1e15 + 0.0);  // +0.0: no negative zeros
    }
}

// ---------------------------------------------------------------------------
// Morton meta-grid keys: ParticleSearchKernels.cu:9-38.
static inline uint32_t part1by2(uint32_t x) {
    x &= 0x000003ffu;
    x = (x ^ (x << 16)) & 0xff0000ffu;
    x = (x ^ (x << 8)) & 0x0300f00fu;
    x = (x ^ (x << 4)) & 0x030c30c3u;
    x = (x ^ (x << 2)) & 0x09249249u;
    return x;
}
static inline uint32_t morton3(uint32_t x, uint32_t y, uint32_t z) {
    return (part1by2(z) << 2) + (part1by2(y) << 1) + part1by2(x);
}

template <class T>
struct SearchInfo {  // ParticleSearch/SearchInfo.h:8-18
    V3<T> gridMin, gridDelta;
    uint32_t dim[3], meta[3];
    uint32_t n;
    T r2;
};

template <class T>
static inline uint32_t cell_key(const SearchInfo<T>& s, int cx, int cy, int cz) {  // :24-38
    const int mx = cx / 8, my = cy / 8, mz = cz / 8;
    cx %= 8; cy %= 8; cz %= 8;
    const uint32_t metaIndex = (uint32_t)mz * s.meta[1] * s.meta[0] + (uint32_t)my * s.meta[0] + (uint32_t)mx;
    return metaIndex * 512u + morton3((uint32_t)cx, (uint32_t)cy, (uint32_t)cz);
}

template <class T>
struct NeighborSearch {
    T radius = 0;
    SearchInfo<T> info{};
    std::vector<uint32_t> keys, cellCount, cellOffset, sortIdx, counts, offsets, list;
    uint32_t maxCount = 0;
    bool capHit = false;

    // ParticleSearch::FindNeighbors (ParticleSearch.h:80-93).
    void find(const std::vector<V3<T>>& x) {
        const uint32_t n = (uint32_t)x.size();
        if (n == 0) return;
        // ComputeMinMax, ParticleSearch.cu:29-55 + ParticleSearchKernels.cu:40-62.
        int mn[3] = {INT_MAX, INT_MAX, INT_MAX}, mx[3] = {INT_MIN, INT_MIN, INT_MIN};
        for (uint32_t i = 0; i < n; i++) {
            for (int d = 0; d < 3; d++) {
                const int c = (int)std::floor(x[i][d] / radius);
                mn[d] = std::min(mn[d], c);
                mx[d] = std::max(mx[d], c);
            }
        }
        V3<T> bmin, bmax;
        for (int d = 0; d < 3; d++) {
            bmin[d] = (T)mn[d] * radius;
            bmax[d] = (T)(mx[d] + 1) * radius;
        }
        // ComputeCellInformation, ParticleSearch.cu:57-140.
        info.n = n;
        info.r2 = radius * radius;
        info.gridMin = bmin;
        const T cellSize = radius;
        V3<T> gridSize = bmax - bmin;
        for (int d = 0; d < 3; d++) info.dim[d] = (uint32_t)std::ceil(gridSize[d] / cellSize) + 4u;
        info.gridMin -= V3<T>(cellSize, cellSize, cellSize) * T(2);
        for (int d = 0; d < 3; d++) info.meta[d] = (uint32_t)std::ceil((T)info.dim[d] / T(8));
        for (int d = 0; d < 3; d++) gridSize[d] = (T)info.dim[d] * cellSize;
        for (int d = 0; d < 3; d++) info.gridDelta[d] = (T)info.dim[d] / gridSize[d];
        const uint64_t cells = (uint64_t)info.meta[0] * info.meta[1] * info.meta[2] * 512u;
        cellCount.assign(cells, 0);
        cellOffset.assign(cells, 0);
        keys.resize(n);
        // InsertParticlesMortonKernel, ParticleSearchKernels.cu:64-78.
        for (uint32_t i = 0; i < n; i++) {
            const V3<T> g = (x[i] - info.gridMin) * info.gridDelta;
            keys[i] = cell_key(info, (int)g.x, (int)g.y, (int)g.z);
            cellCount[keys[i]]++;
        }
        // thrust::exclusive_scan, ParticleSearch.cu:111-115.
        uint32_t acc = 0;
        for (uint64_t c = 0; c < cells; c++) { cellOffset[c] = acc; acc += cellCount[c]; }
        // CountingSortIndicesKernel (:80-91) with the in-cell rank = ascending index.
        sortIdx.assign(n, 0);
        {
            std::vector<uint32_t> fill(cells, 0);
            for (uint32_t i = 0; i < n; i++) sortIdx[cellOffset[keys[i]] + fill[keys[i]]++] = i;
        }
        // ComputeCountsKernel + scan + NeighborhoodQueryWithCountsKernel (:93-193),
        // done in one pass per particle; reversedSortIndices == sortIndices (:129-137).
        counts.assign(n, 0);
        std::vector<std::vector<uint32_t>> tmp(n);
#pragma omp parallel for schedule(static)
        for (int64_t ii = 0; ii < (int64_t)n; ii++) {
            const uint32_t i = (uint32_t)ii;
            const V3<T> p = x[i];
            const V3<T> gf = (p - info.gridMin) * info.gridDelta;
            const int gc[3] = {(int)std::floor(gf.x), (int)std::floor(gf.y), (int)std::floor(gf.z)};
            uint32_t cnt = 0;
            std::vector<uint32_t>& out = tmp[i];
            out.reserve(48);
            bool done = false;
            for (int dz = -1; dz < 2 && !done; dz++)
                for (int dy = -1; dy < 2 && !done; dy++)
                    for (int dx = -1; dx < 2 && !done; dx++) {
                        const int f[3] = {gc[0] + dx, gc[1] + dy, gc[2] + dz};
                        if (f[0] < 0 || f[1] < 0 || f[2] < 0 || f[0] >= (int)info.dim[0] ||
                            f[1] >= (int)info.dim[1] || f[2] >= (int)info.dim[2])
                            continue;
                        const uint32_t c = cell_key(info, f[0], f[1], f[2]);
                        const uint32_t start = cellOffset[c], num = cellCount[c];
                        for (uint32_t k = start; k < start + num; k++) {
                            const uint32_t j = sortIdx[k];
                            const V3<T> diff = x[j] - p;
                            const T d2 = diff.x * diff.x + diff.y * diff.y + diff.z * diff.z;
                            if (d2 < info.r2 && d2 > T(0)) { out.push_back(j); cnt++; }
                            if (cnt == VFD_MAX_NEIGHBORS) { done = true; break; }
                        }
                    }
            counts[i] = cnt;
        }
        offsets.assign(n, 0);
        uint32_t tot = 0;
        maxCount = 0;
        capHit = false;
        for (uint32_t i = 0; i < n; i++) {
            offsets[i] = tot;
            tot += counts[i];
            maxCount = std::max(maxCount, counts[i]);
            if (counts[i] == VFD_MAX_NEIGHBORS) capHit = true;
        }
        list.resize(tot);
        for (uint32_t i = 0; i < n; i++) std::copy(tmp[i].begin(), tmp[i].end(), list.begin() + offsets[i]);
    }
};

// ---------------------------------------------------------------------------
// Volume map (Utility/SDF/SDFDeviceData.cuh), arrays as the reference lays them out.
struct MapData {
    std::vector<float> nodes;
    std::vector<uint32_t> cells, cellMap;
    float dmin[3], dmax[3], cs[3], csi[3];
    uint32_t res[3];
    uint32_t fieldCount = 0, nodeCount = 0, cellCount = 0, cellMapCount = 0;
};

// 32-node cubic serendipity shape functions on [-1,1]^3 and their gradients
// (SDFDeviceData.cuh:36-370 evaluates the same polynomials): corner c = bx +
// 2 by + 4 bz carries (1/64)(1+-x)(1+-y)(1+-z)(9|xi|^2 - 19); the two nodes of an
// edge along axis t carry (9/64)(1-t^2)(1 -+ 3t)(1+-u)(1+-w). Node numbering of
// the edges: x-edges 8 + a + 2 bz + 4 by, y-edges 16 + a + 2 bx + 4 bz, z-edges
// 24 + a + 2 by + 4 bx (a = 0 for the 1-3t node).
template <class T>
static void shape_functions(const V3<T>& xi, T N[32], V3<T> dN[32]) {
    const T x = xi.x, y = xi.y, z = xi.z;
    const T base = T(9) * (x * x + y * y + z * z) - T(19);
    for (int c = 0; c < 8; c++) {
        const T sx = (c & 1) ? T(1) : T(-1), sy = (c & 2) ? T(1) : T(-1), sz = (c & 4) ? T(1) : T(-1);
        const T ax = T(1) + sx * x, ay = T(1) + sy * y, az = T(1) + sz * z;
        N[c] = ax * ay * az * base / T(64);
        dN[c] = V3<T>((sx * ay * az * base + ax * ay * az * T(18) * x) / T(64),
                      (sy * ax * az * base + ax * ay * az * T(18) * y) / T(64),
                      (sz * ax * ay * base + ax * ay * az * T(18) * z) / T(64));
    }
    // axis t with the two other axes (u: bit 1 of the node offset, w: bit 2).
    const int axisU[3] = {2, 0, 1};
    const int axisW[3] = {1, 2, 0};
    for (int t = 0; t < 3; t++) {
        for (int k = 0; k < 8; k++) {
            const int a = k & 1, bu = (k >> 1) & 1, bw = (k >> 2) & 1;
            const T tv = xi[t], uv = xi[axisU[t]], wv = xi[axisW[t]];
            const T sa = a ? T(3) : T(-3), su = bu ? T(1) : T(-1), sw = bw ? T(1) : T(-1);
            const T ft = (T(1) - tv * tv) * (T(1) + sa * tv);
            const T dft = T(-2) * tv * (T(1) + sa * tv) + sa * (T(1) - tv * tv);
            const T fu = T(1) + su * uv, fw = T(1) + sw * wv;
            const int node = 8 + 8 * t + k;
            N[node] = T(9) / T(64) * ft * fu * fw;
            V3<T> g;
            g[t] = T(9) / T(64) * dft * fu * fw;
            g[axisU[t]] = T(9) / T(64) * ft * su * fw;
            g[axisW[t]] = T(9) / T(64) * ft * fu * sw;
            dN[node] = g;
        }
    }
}

// SDFDeviceData::DetermineShapeFunction (SDFDeviceData.cuh:372-419).
template <class T>
static bool determine_shape(const MapData& m, uint32_t field, const V3<T>& x, uint32_t cell[32], V3<T>& c0,
                            T N[32], V3<T> dN[32]) {
    for (int d = 0; d < 3; d++)
        if (!((T)m.dmin[d] <= x[d] && (T)m.dmax[d] >= x[d])) return false;
    uint32_t mi[3];
    for (int d = 0; d < 3; d++) {
        mi[d] = (uint32_t)((T)m.csi[d] * (x[d] - (T)m.dmin[d]));
        if (mi[d] >= m.res[d]) mi[d] = m.res[d] - 1u;
    }
    const uint32_t i = m.res[1] * m.res[0] * mi[2] + m.res[0] * mi[1] + mi[0];
    const uint32_t j = m.cellMap[field * m.cellMapCount + i];
    if (j == UINT_MAX) return false;
    // CalculateSubDomain(i) (:25-34), via SingleToMultiIndex (:14-23).
    const uint32_t n01 = m.res[0] * m.res[1];
    const uint32_t kk = i / n01, tmp = i % n01;
    const uint32_t idx[3] = {tmp % m.res[0], tmp / m.res[0], kk};
    V3<T> sdmin, sdmax;
    for (int d = 0; d < 3; d++) {
        sdmin[d] = (T)m.dmin[d] + (T)(float)idx[d] * (T)m.cs[d];
        sdmax[d] = sdmin[d] + (T)m.cs[d];
    }
    const V3<T> den = sdmax - sdmin;
    V3<T> c1;
    for (int d = 0; d < 3; d++) { c0[d] = T(2) / den[d]; c1[d] = (sdmax[d] + sdmin[d]) / den[d]; }
    const V3<T> xi = c0 * x - c1;
    for (uint32_t k = 0; k < 32; k++) cell[k] = m.cells[(size_t)field * m.cellCount * 32u + (size_t)j * 32u + k];
    shape_functions(xi, N, dN);
    return true;
}

template <class T>
static T interpolate(const MapData& m, uint32_t field, const uint32_t cell[32], const T N[32]) {  // :421-443
    T phi = 0;
    for (uint32_t j = 0; j < 32; j++) phi += (T)m.nodes[(size_t)field * m.nodeCount + cell[j]] * N[j];
    return phi;
}
template <class T>
static T interpolate_grad(const MapData& m, uint32_t field, const uint32_t cell[32], const V3<T>& c0, const T N[32],
                          V3<T>& grad, const V3<T> dN[32]) {  // :445-474
    T phi = 0;
    grad = V3<T>();
    for (uint32_t j = 0; j < 32; j++) {
        const T c = (T)m.nodes[(size_t)field * m.nodeCount + cell[j]];
        phi += c * N[j];
        grad += c * dN[j];
    }
    grad = grad * c0;
    return phi;
}

// Host SDF::Interpolate without gradient (SDF.cu:141-188), FLT_MAX outside.
static float map_interpolate_host(const MapData& m, uint32_t field, const V3<float>& p) {
    uint32_t cell[32];
    V3<float> c0, dN[32];
    float N[32];
    if (!determine_shape<float>(m, field, p, cell, c0, N, dN)) return FLT_MAX;
    float phi = 0.0f;
    for (uint32_t k = 0; k < 32; k++) {
        const float c = m.nodes[(size_t)field * m.nodeCount + cell[k]];
        if (c == FLT_MAX) return FLT_MAX;
        phi += c * N[k];
    }
    return phi;
}

// Gauss-Legendre rule of n points on [-1,1] by Newton iteration on P_n.
static void gauss_legendre(unsigned n, std::vector<double>& x, std::vector<double>& w) {
    x.assign(n, 0.0);
    w.assign(n, 0.0);
    for (unsigned i = 0; i < n; i++) {
        double z = std::cos(kPI * (i + 0.75) / (n + 0.5));
        double dp = 0.0;
        for (int it = 0; it < 100; it++) {
            double p0 = 1.0, p1 = z;
            for (unsigned k = 2; k <= n; k++) {
                const double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
                p0 = p1;
                p1 = p2;
            }
            dp = n * (z * p1 - p0) / (z * z - 1.0);
            const double dz = p1 / dp;
            z -= dz;
            if (std::fabs(dz) < 1e-17) break;
        }
        {  // P_n' at the converged root
            double p0 = 1.0, p1 = z;
            for (unsigned k = 2; k <= n; k++) {
                const double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
                p0 = p1;
                p1 = p2;
            }
            dp = n * (z * p1 - p0) / (z * z - 1.0);
        }
        x[n - 1 - i] = z;  // ascending order
        w[n - 1 - i] = 2.0 / ((1.0 - z * z) * dp * dp);
    }
}

// Signed distance of an axis-aligned box (negative inside): the value the
// reference's MeshDistance::SignedDistance gives for a box mesh.
static float box_sdf(const float bmin[3], const float bmax[3], const V3<float>& p) {
    double q[3], outside = 0.0, inside = -1e300;
    for (int d = 0; d < 3; d++) {
        const double c = 0.5 * ((double)bmin[d] + bmax[d]);
        const double h = 0.5 * ((double)bmax[d] - bmin[d]);
        q[d] = std::fabs((double)p[d] - c) - h;
        outside += std::max(q[d], 0.0) * std::max(q[d], 0.0);
        inside = std::max(inside, q[d]);
    }
    return (float)(std::sqrt(outside) + std::min(inside, 0.0));
}

static void box_map_sizes(const uint32_t res[3], uint32_t& nodes, uint32_t& cells) {
    const uint32_t nv = (res[0] + 1) * (res[1] + 1) * (res[2] + 1);
    const uint32_t ne = res[0] * (res[1] + 1) * (res[2] + 1) + (res[0] + 1) * res[1] * (res[2] + 1) +
                        (res[0] + 1) * (res[1] + 1) * res[2];
    nodes = nv + 2 * ne;
    cells = res[0] * res[1] * res[2];
}

// SDF::IndexToNodePosition (SDF.cu:313-373).
static V3<float> node_position(const MapData& m, uint32_t i) {
    const uint32_t* r = m.res;
    const uint32_t nv = (r[0] + 1u) * (r[1] + 1u) * (r[2] + 1u);
    const uint32_t ne[3] = {r[0] * (r[1] + 1u) * (r[2] + 1u), (r[0] + 1u) * r[1] * (r[2] + 1u),
                            (r[0] + 1u) * (r[1] + 1u) * r[2]};
    float idx[3];
    int axis = -1;
    uint32_t sub = 0;
    if (i < nv) {
        idx[2] = (float)(i / ((r[1] + 1u) * (r[0] + 1u)));
        const uint32_t t = i % ((r[1] + 1u) * (r[0] + 1u));
        idx[1] = (float)(t / (r[0] + 1u));
        idx[0] = (float)(t % (r[0] + 1u));
    } else if (i < nv + 2u * ne[0]) {
        i -= nv;
        const uint32_t e = i / 2u;
        idx[2] = (float)(e / ((r[1] + 1u) * r[0]));
        const uint32_t t = e % ((r[1] + 1u) * r[0]);
        idx[1] = (float)(t / r[0]);
        idx[0] = (float)(t % r[0]);
        axis = 0; sub = i % 2u;
    } else if (i < nv + 2u * (ne[0] + ne[1])) {
        i -= nv + 2u * ne[0];
        const uint32_t e = i / 2u;
        idx[0] = (float)(e / ((r[2] + 1u) * r[1]));
        const uint32_t t = e % ((r[2] + 1u) * r[1]);
        idx[2] = (float)(t / r[1]);
        idx[1] = (float)(t % r[1]);
        axis = 1; sub = i % 2u;
    } else {
        i -= nv + 2u * (ne[0] + ne[1]);
        const uint32_t e = i / 2u;
        idx[1] = (float)(e / ((r[0] + 1u) * r[2]));
        const uint32_t t = e % ((r[0] + 1u) * r[2]);
        idx[0] = (float)(t / r[2]);
        idx[2] = (float)(t % r[2]);
        axis = 2; sub = i % 2u;
    }
    V3<float> p;
    for (int d = 0; d < 3; d++) p[d] = m.dmin[d] + m.cs[d] * idx[d];
    if (axis >= 0) p[axis] += (1.0f + (float)sub) / 3.0f * m.cs[axis];
    return p;
}

// SDF::AddFunction cell table (SDF.cu:77-131).
static void build_cells(MapData& m) {
    const uint32_t nx = m.res[0], ny = m.res[1], nz = m.res[2];
    const uint32_t nv = (nx + 1) * (ny + 1) * (nz + 1);
    const uint32_t nex = nx * (ny + 1) * (nz + 1), ney = (nx + 1) * ny * (nz + 1);
    std::vector<uint32_t> cells((size_t)m.cellCount * 32u);
    for (uint32_t l = 0; l < m.cellCount; l++) {
        const uint32_t k = l / (ny * nx), t = l % (ny * nx), j = t / nx, i = t % nx;
        uint32_t* c = &cells[(size_t)l * 32u];
        c[0] = (nx + 1) * (ny + 1) * k + (nx + 1) * j + i;
        c[1] = c[0] + 1;
        c[2] = (nx + 1) * (ny + 1) * k + (nx + 1) * (j + 1) + i;
        c[3] = c[2] + 1;
        c[4] = (nx + 1) * (ny + 1) * (k + 1) + (nx + 1) * j + i;
        c[5] = c[4] + 1;
        c[6] = (nx + 1) * (ny + 1) * (k + 1) + (nx + 1) * (j + 1) + i;
        c[7] = c[6] + 1;
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
    m.cells.clear();
    for (uint32_t f = 0; f < m.fieldCount; f++) m.cells.insert(m.cells.end(), cells.begin(), cells.end());
    m.cellMap.clear();
    for (uint32_t f = 0; f < m.fieldCount; f++)
        for (uint32_t l = 0; l < m.cellCount; l++) m.cellMap.push_back(l);
}

// Grid of a map over [dmin, dmax] (SDF::SDF, SDF.cu:8-14) with `fields` fields.
static void map_grid(MapData& m, const float dmin[3], const float dmax[3], const uint32_t res[3], uint32_t fields) {
    for (int d = 0; d < 3; d++) {
        m.dmin[d] = dmin[d];
        m.dmax[d] = dmax[d];
        m.res[d] = res[d];
        m.cs[d] = (m.dmax[d] - m.dmin[d]) / (float)m.res[d];
        m.csi[d] = 1.0f / m.cs[d];
    }
    box_map_sizes(m.res, m.nodeCount, m.cellCount);
    m.cellMapCount = m.cellCount;
    m.fieldCount = fields;
    build_cells(m);
    m.nodes.assign((size_t)m.nodeCount * fields, 0.0f);
}

// Field 1 of a rigid-body map from its field 0 (RigidBody.cu:42-71): 0.8 * Gauss-Legendre
// (16 points per axis, p = 30) integral over the support cube
// (GaussQuadrature.cpp:5621-5656: float weights, float sum).
static void map_volume_field(MapData& m, float particleRadius) {
    KernelTable<float> kernel;
    kernel.setRadius(4.0f * particleRadius);
    const float supportRadius = 4.0f * particleRadius;
    std::vector<double> ga, gw;
    gauss_legendre(16, ga, gw);
    const double c0 = 0.5 * (double)(supportRadius - (-supportRadius));
    const double c1 = 0.5 * (double)(-supportRadius + supportRadius);
    const double cvol = c0 * c0 * c0;
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t l = 0; l < (int64_t)m.nodeCount; l++) {
        const V3<float> x = node_position(m, (uint32_t)l);
        const float dx = map_interpolate_host(m, 0, x);
        float value = 0.0f;
        if (!(dx > 2.0f * supportRadius)) {
            float res = 0.0f;
            for (unsigned i = 0; i < 16; i++) {
                const float wi = (float)gw[i];
                for (unsigned j = 0; j < 16; j++) {
                    const float wij = wi * (float)gw[j];
                    for (unsigned k = 0; k < 16; k++) {
                        const float wijk = wij * (float)gw[k];
                        const V3<float> xi((float)(c0 * ga[i] + c1), (float)(c0 * ga[j] + c1), (float)(c0 * ga[k] + c1));
                        float f = 0.0f;
                        if (!(length2(xi) > supportRadius * supportRadius)) {
                            const float dist = map_interpolate_host(m, 0, x + xi);
                            if (dist <= 0.0f) f = 1.0f;
                            else if (dist < supportRadius) f = kernel.getW(dist) / kernel.wZero;
                        }
                        res += wijk * f;
                    }
                }
            }
            res = (float)((double)res * cvol);
            value = 0.8f * res;
        }
        m.nodes[(size_t)m.nodeCount + (size_t)l] = value;
    }
}

// RigidBody::RigidBody for a box mesh (RigidBody.cu:10-72).
static void build_box_map(const float bmin[3], const float bmax[3], bool inverted, float padding,
                          const uint32_t res[3], float particleRadius, MapData& m) {
    const float supportRadius = 4.0f * particleRadius;
    const float tolerance = padding - particleRadius;
    const float sign = inverted ? -1.0f : 1.0f;
    float dmin[3], dmax[3];
    for (int d = 0; d < 3; d++) {
        dmin[d] = bmin[d] - (8.0f * supportRadius + tolerance);
        dmax[d] = bmax[d] + (8.0f * supportRadius + tolerance);
    }
    map_grid(m, dmin, dmax, res, 2);
    // field 0: sign * (SignedDistance - tolerance)
#pragma omp parallel for schedule(static)
    for (int64_t l = 0; l < (int64_t)m.nodeCount; l++) {
        const V3<float> x = node_position(m, (uint32_t)l);
        m.nodes[(size_t)l] = sign * (box_sdf(bmin, bmax, x) - tolerance);
    }
    map_volume_field(m, particleRadius);
}

// ---------------------------------------------------------------------------
// Triangle meshes: MeshDistance (Utility/SDF/MeshDistance.cpp) on an EdgeMesh.
struct Mesh {
    std::vector<V3<float>> x;      // placed vertices
    std::vector<uint32_t> tri;     // 3 per face
    std::vector<V3<float>> faceN;  // unit face normals
    std::vector<V3<float>> vertN;  // angle-weighted vertex normals
    std::vector<int64_t> opp;      // per half-edge (face, k): the face across it, -1 on a border
    float bmin[3], bmax[3];
};

// glm::normalize: v * inversesqrt(dot(v, v)).
static V3<float> glm_normalize(const V3<float>& v) { return v * (1.0f / std::sqrt(dot(v, v))); }

// The placement of RigidBody.cu:19-23 / FluidObject.cpp:10-14 (Transform * vec4(v, 1),
// glm's column-major product summed in pairs), BoundingBox(vertices)
// (Core/Structures/BoundingBox.h:16-21), the pre-computed normals of MeshDistance's
// constructor (MeshDistance.cpp:27-55) and the half-edge pairing of EdgeMesh
// (Renderer/Mesh/EdgeMesh.cpp:97-130: a half-edge (u, v) pairs with an unpaired (v, u)).
static bool make_mesh(const float* v, uint32_t nv, const uint32_t* tri, uint32_t nf, const float* T, Mesh& M) {
    for (size_t i = 0; i < 3 * (size_t)nf; i++)
        if (tri[i] >= nv) return false;
    M.x.resize(nv);
    for (uint32_t i = 0; i < nv; i++) {
        const float px = v[3 * i], py = v[3 * i + 1], pz = v[3 * i + 2];
        if (!T) {
            M.x[i] = V3<float>(px, py, pz);
            continue;
        }
        float r[3];
        for (int k = 0; k < 3; k++) r[k] = (T[k] * px + T[4 + k] * py) + (T[8 + k] * pz + T[12 + k] * 1.0f);
        M.x[i] = V3<float>(r[0], r[1], r[2]);
    }
    M.tri.assign(tri, tri + 3 * (size_t)nf);
    for (int d = 0; d < 3; d++) {
        M.bmin[d] = std::numeric_limits<float>::max();
        M.bmax[d] = -std::numeric_limits<float>::max();
    }
    for (const auto& p : M.x)
        for (int d = 0; d < 3; d++) {
            M.bmin[d] = std::min(M.bmin[d], p[d]);
            M.bmax[d] = std::max(M.bmax[d], p[d]);
        }
    M.faceN.assign(nf, V3<float>());
    M.vertN.assign(nv, V3<float>());
    for (uint32_t f = 0; f < nf; f++) {
        const V3<float>& x0 = M.x[tri[3 * f]];
        const V3<float>& x1 = M.x[tri[3 * f + 1]];
        const V3<float>& x2 = M.x[tri[3 * f + 2]];
        const V3<float> n = glm_normalize(cross(x1 - x0, x2 - x0));
        const V3<float> e1 = glm_normalize(x1 - x0), e2 = glm_normalize(x2 - x1), e3 = glm_normalize(x0 - x2);
        const float alpha[3] = {std::acos(dot(e1, -e3)), std::acos(dot(e2, -e1)), std::acos(dot(e3, -e2))};
        for (int k = 0; k < 3; k++) M.vertN[tri[3 * f + k]] += alpha[k] * n;
        M.faceN[f] = n;
    }
    M.opp.assign(3 * (size_t)nf, -1);
    std::map<std::pair<uint32_t, uint32_t>, std::vector<uint32_t>> open;
    for (uint32_t f = 0; f < nf; f++)
        for (uint32_t k = 0; k < 3; k++) {
            const uint32_t a = tri[3 * f + k], b = tri[3 * f + (k + 1) % 3];
            auto it = open.find({b, a});
            if (it != open.end() && !it->second.empty()) {
                const uint32_t h = it->second.front();
                it->second.erase(it->second.begin());
                M.opp[3 * (size_t)f + k] = h / 3;
                M.opp[h] = f;
            } else {
                open[{a, b}].push_back(3 * f + k);
            }
        }
    return true;
}

// Closest entity classes of MeshDistance (MeshDistance.h): corners A, B, C; edges D (01),
// E (12), F (20); interior G.
enum TriEntity { kEntA, kEntB, kEntC, kEntD, kEntE, kEntF, kEntG };

// MeshDistance::PointTriangleDistanceSquared (MeshDistance.cpp:300-607): minimises
// Q(s, t) = |t0 + s e0 + t e1 - p|^2 over s, t >= 0, s + t <= 1 by the region of the
// unconstrained minimum (D. Eberly, "Distance Between Point and Triangle in 3D"), in FP32.
// Returns Q at the minimum (clamped at 0); (s, t) and the entity of the closest point.
static float point_triangle_d2(const V3<float>& p, const V3<float>& t0, const V3<float>& t1, const V3<float>& t2,
                               float& s, float& t, int& entity) {
    const V3<float> diff = t0 - p, e0 = t1 - t0, e1 = t2 - t0;
    const float a00 = dot(e0, e0), a01 = dot(e0, e1), a11 = dot(e1, e1);
    const float b0 = dot(diff, e0), b1 = dot(diff, e1), c = dot(diff, diff);
    const float det = std::fabs(a00 * a11 - a01 * a01);
    s = a01 * b1 - a11 * b0;
    t = a01 * b0 - a00 * b1;
    float d2;
    auto quad = [&]() { return s * (a00 * s + a01 * t + 2.0f * b0) + t * (a01 * s + a11 * t + 2.0f * b1) + c; };
    auto cornerA = [&]() { s = 0.0f; t = 0.0f; entity = kEntA; return c; };
    auto cornerB = [&]() { s = 1.0f; t = 0.0f; entity = kEntB; return a00 + 2.0f * b0 + c; };
    auto cornerC = [&]() { s = 0.0f; t = 1.0f; entity = kEntC; return a11 + 2.0f * b1 + c; };
    auto edge01 = [&]() { t = 0.0f; s = -b0 / a00; entity = kEntD; return b0 * s + c; };
    auto edge20 = [&]() { s = 0.0f; t = -b1 / a11; entity = kEntF; return b1 * t + c; };
    // t = 0 side: corner A, corner B or the edge between
    auto side01 = [&]() { return b0 >= 0.0f ? cornerA() : (-b0 >= a00 ? cornerB() : edge01()); };
    // s = 0 side: corner A, corner C or the edge between
    auto side20 = [&]() { return b1 >= 0.0f ? cornerA() : (-b1 >= a11 ? cornerC() : edge20()); };
    if (s + t <= det) {
        if (s < 0.0f) {
            if (t < 0.0f) d2 = b0 < 0.0f ? (-b0 >= a00 ? cornerB() : edge01()) : side20();  // region 4
            else d2 = side20();                                                              // region 3
        } else if (t < 0.0f) {
            d2 = side01();  // region 5
        } else {            // region 0
            const float inv = 1.0f / det;
            s *= inv;
            t *= inv;
            entity = kEntG;
            d2 = quad();
        }
    } else {
        const float denom = a00 - 2.0f * a01 + a11;
        if (s < 0.0f) {  // region 2
            const float m0 = a01 + b0, m1 = a11 + b1;
            if (m1 > m0) {
                const float numer = m1 - m0;
                if (numer >= denom) d2 = cornerB();
                else { s = numer / denom; t = 1 - s; entity = kEntE; d2 = quad(); }
            } else {
                d2 = m1 <= 0.0f ? cornerC() : (b1 >= 0.0f ? cornerA() : edge20());
            }
        } else if (t < 0.0f) {  // region 6
            const float m0 = a01 + b1, m1 = a00 + b0;
            if (m1 > m0) {
                const float numer = m1 - m0;
                if (numer >= denom) d2 = cornerC();
                else { t = numer / denom; s = 1 - t; entity = kEntE; d2 = quad(); }
            } else {
                d2 = m1 <= 0.0f ? cornerB() : (b0 >= 0.0f ? cornerA() : edge01());
            }
        } else {  // region 1
            const float numer = a11 + b1 - a01 - b0;
            if (numer <= 0.0f) d2 = cornerC();
            else if (numer >= denom) d2 = cornerB();
            else { s = numer / denom; t = 1 - s; entity = kEntE; d2 = quad(); }
        }
    }
    return d2 < 0.0f ? 0.0f : d2;
}

// MeshDistance::SignedDistance (MeshDistance.cpp:187-228) with the nearest face found by
// testing every face (the bounding-sphere hierarchy only prunes; ties keep the lowest
// face index). The sign is that of dot(p - closest point, pseudo-normal of the entity).
static float mesh_signed_distance(const Mesh& M, const V3<float>& p) {
    const uint32_t nf = (uint32_t)(M.tri.size() / 3);
    float best = std::numeric_limits<float>::max();
    uint32_t face = 0;
    for (uint32_t f = 0; f < nf; f++) {
        float s, t;
        int e;
        const float d2 = point_triangle_d2(p, M.x[M.tri[3 * f]], M.x[M.tri[3 * f + 1]], M.x[M.tri[3 * f + 2]], s, t, e);
        if (best > d2) {
            best = d2;
            face = f;
        }
    }
    float s, t;
    int e;
    const V3<float>& t0 = M.x[M.tri[3 * face]];
    const float d2 = point_triangle_d2(p, t0, M.x[M.tri[3 * face + 1]], M.x[M.tri[3 * face + 2]], s, t, e);
    const V3<float> cp = t0 + s * (M.x[M.tri[3 * face + 1]] - t0) + t * (M.x[M.tri[3 * face + 2]] - t0);
    V3<float> n;
    if (e <= kEntC) {
        n = M.vertN[M.tri[3 * face + e]];
    } else if (e <= kEntF) {
        const int64_t o = M.opp[3 * (size_t)face + (e - kEntD)];
        n = o < 0 ? M.faceN[face] : M.faceN[face] + M.faceN[(size_t)o];
    } else {
        n = M.faceN[face];
    }
    float dist = std::sqrt(d2);
    if (dot(p - cp, n) < 0.0f) dist *= -1.0f;
    return dist;
}

// RigidBody::RigidBody (RigidBody.cu:10-72) for a placed triangle mesh.
static void build_mesh_map(const Mesh& M, bool inverted, float padding, const uint32_t res[3], float particleRadius,
                           MapData& m) {
    const float supportRadius = 4.0f * particleRadius;
    const float tolerance = padding - particleRadius;
    const float sign = inverted ? -1.0f : 1.0f;
    float dmin[3], dmax[3];
    for (int d = 0; d < 3; d++) {
        dmax[d] = M.bmax[d] + (8.0f * supportRadius + tolerance);
        dmin[d] = M.bmin[d] - (8.0f * supportRadius + tolerance);
    }
    map_grid(m, dmin, dmax, res, 2);
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t l = 0; l < (int64_t)m.nodeCount; l++) {
        const V3<float> x = node_position(m, (uint32_t)l);
        m.nodes[(size_t)l] = sign * (mesh_signed_distance(M, x) - tolerance);
    }
    map_volume_field(m, particleRadius);
}

// ParticleSampler::SampleMeshVolume (ParticleSampler.cpp:7-91) with SDF::SDF(mesh, bounds,
// resolution, inverted) (SDF.cu:16-36) and SDF::GetDistance(x, 0) (SDF.cu:217-225).
// Returns false when an axis step is lost in the float rounding.
static bool sample_mesh_volume(const Mesh& M, float radius, const uint32_t res[3], bool inverted, int mode,
                               std::vector<float>& out) {
    MapData m;
    float dmin[3] = {M.bmin[0], M.bmin[1], M.bmin[2]}, dmax[3] = {M.bmax[0], M.bmax[1], M.bmax[2]};
    {
        const V3<float> d0(dmax[0] - dmin[0], dmax[1] - dmin[1], dmax[2] - dmin[2]);
        const float g0 = 0.001f * std::sqrt(dot(d0, d0));
        for (int d = 0; d < 3; d++) dmax[d] += g0;
        const V3<float> d1(dmax[0] - dmin[0], dmax[1] - dmin[1], dmax[2] - dmin[2]);
        const float g1 = 0.001f * std::sqrt(dot(d1, d1));
        for (int d = 0; d < 3; d++) dmin[d] -= g1;
    }
    map_grid(m, dmin, dmax, res, 1);
    const float factor = inverted ? -1.0f : 1.0f;
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t l = 0; l < (int64_t)m.nodeCount; l++)
        m.nodes[(size_t)l] = factor * mesh_signed_distance(M, node_position(m, (uint32_t)l));

    const float diameter = 2.0f * radius;
    float shiftX = diameter, shiftY = diameter;
    if (mode == 1) {
        shiftY = std::sqrt(3.0f) * radius;
    } else if (mode == 2) {
        shiftX = std::sqrt(3.0f) * radius;
        shiftY = std::sqrt(6.0f) * diameter / 3.0f;
    }
    const float step[3] = {shiftX, shiftY, diameter};
    for (int d = 0; d < 3; d++)
        if (M.bmin[d] + step[d] == M.bmin[d] || M.bmax[d] + step[d] == M.bmax[d]) return false;
    out.clear();
    uint32_t counterY = 0;
    for (float z = M.bmin[2]; z <= M.bmax[2]; z += diameter) {
        for (float y = M.bmin[1]; y <= M.bmax[1]; y += shiftY) {
            uint32_t counterX = 0;
            for (float x = M.bmin[0]; x <= M.bmax[0]; x += shiftX) {
                V3<float> q;
                if (mode == 0) {
                    q = V3<float>(x + radius, y + radius, z + radius);
                } else if (mode == 1) {
                    q = counterY % 2 == 0 ? V3<float>(x, y + radius, z + radius) : V3<float>(x + radius, y + radius, z);
                } else {
                    q = V3<float>(x, y + radius, z + radius);
                    V3<float> shift(0.0f, 0.0f, 0.0f);
                    if (counterX % 2) shift.z += diameter / (2.0f * (counterY % 2 ? -1 : 1));
                    if (counterY % 2) {
                        shift.x += shiftX / 2.0f;
                        shift.z += diameter / 2.0f;
                    }
                    q += shift;
                }
                if (map_interpolate_host(m, 0, q) < 0.0f) {
                    out.push_back(q.x);
                    out.push_back(q.y);
                    out.push_back(q.z);
                }
                counterX++;
            }
            counterY++;
        }
        counterY = 0;
    }
    return true;
}

// ---------------------------------------------------------------------------
// Particle state: DFSPHParticle (Structures/DFSPHParticle.h:8-33).
template <class T>
struct Particle {
    V3<T> x, v, a, ap;
    T res = 0, rho = 0, rhoAdv = 0, kappa = 0, kappaV = 0, alpha = 0;
    V3<T> dv;
    V3<T> n, ns;
    T curv = 0, curvS = 0, dCurv = 0;
};

template <class T>
struct Info {  // DFSPHSimulationInfo (Structures/DFSPHSimulationInfo.h:5-44)
    uint32_t n = 0, bodies = 0;
    T h = 0, h2 = 0, r = 0, diam = 0, dt = 0, dt2 = 0, dtInv = 0, dt2Inv = 0;
    T volume = 0, rho0 = 0, mass = 0, massInv = 0;
    T visc = 0, bvisc = 0, dynVisc = 0, dynBVisc = 0, tangFactor = 0, tangDist = 0;
    T st = 0;
    uint32_t stSamples = 0;
    T slope = 0, constant = 0;
    bool temporal = false;
    T smoothing = 0, factor = 0, nbrRadius = 0, mcFactor = 0;
    V3<T> g;
};

struct Body {
    MapData map;
};

template <class T>
struct Sim {
    vfd_desc desc{};
    Info<T> info;
    KernelTable<T> kernel;
    NeighborSearch<T> search;
    std::vector<Particle<T>> init, p;
    std::vector<Body> bodies;
    std::vector<std::vector<V3<T>>> bxj;
    std::vector<std::vector<T>> bvol;
    std::vector<float> halton;
    // viscosity CG vectors (DFSPHImplementation.cu:226-233)
    std::vector<V3<T>> cgR, cgP, cgZ, cgTmp, cgB, cgG;
    std::vector<M3<T>> cgMinv;
    vfd_step_stats dbg{};
    T maxV2 = 0;
    T frameTime = 0;

    void set_description(const vfd_desc& d) {  // DFSPHImplementation.cu:318-368
        desc = d;
        if ((T)d.ParticleRadius != info.r) {
            kernel.setRadius(T(4) * (T)d.ParticleRadius);
            search.radius = T(4) * (T)d.ParticleRadius;
        }
        info.r = (T)d.ParticleRadius;
        info.diam = T(2) * info.r;
        info.h = T(4) * info.r;
        info.h2 = info.h * info.h;
        info.volume = T(0.8) * info.diam * info.diam * info.diam;
        info.rho0 = T(1000);
        info.mass = info.volume * info.rho0;
        info.massInv = T(1) / info.mass;
        info.visc = (T)d.Viscosity;
        info.bvisc = (T)d.BoundaryViscosity;
        info.dynVisc = info.visc * info.rho0;
        info.dynBVisc = info.bvisc * info.rho0;
        info.tangFactor = (T)d.TangentialDistanceFactor;
        info.tangDist = info.tangFactor * info.h;
        set_dt((T)d.TimeStepSize);
        info.st = (T)d.SurfaceTension;
        info.slope = (T)74.688796680497925;
        info.constant = T(12);
        info.temporal = d.TemporalSmoothing != 0;
        info.smoothing = T(0.5);
        info.factor = T(0.8);
        info.nbrRadius = info.r * info.factor;
        info.g = V3<T>((T)d.Gravity[0], (T)d.Gravity[1], (T)d.Gravity[2]);
        // The reference computes these two in ComputeTimeStepSize (:413-422),
        // after the first step's surface tension; they start from the initial dt.
        update_samples();
    }
    void set_dt(T dt) {
        info.dt = dt;
        info.dt2 = dt * dt;
        info.dtInv = T(1) / info.dt;
        info.dt2Inv = T(1) / info.dt2;
    }
    void update_samples() {
        if (desc.CSDFix > 0) info.stSamples = (uint32_t)desc.CSDFix;
        else info.stSamples = (uint32_t)(int)((T)desc.CSD * info.dt);
        info.mcFactor = std::asin(info.nbrRadius / info.r);
    }

    uint32_t nbrCount(uint32_t i) const { return search.counts[i]; }
    uint32_t nbr(uint32_t i, uint32_t j) const { return search.list[search.offsets[i] + j]; }

    // -------------------------------------------------------------- kernels
    void K1_boundary() {  // ComputeVolumeAndBoundaryKernel, DFSPHKernels.cu:69-150
        const uint32_t n = info.n;
#pragma omp parallel for schedule(static)
        for (int64_t ii = 0; ii < (int64_t)n; ii++) {
            const uint32_t i = (uint32_t)ii;
            V3<T>& x = p[i].x;
            for (uint32_t b = 0; b < info.bodies; b++) {
                V3<T>& xb = bxj[b][i];
                T& vb = bvol[b][i];
                xb = V3<T>();
                vb = 0;
                V3<T> normal;
                T dist = (T)FLT_MAX;
                V3<T> c0, dN[32];
                uint32_t cell[32];
                T N[32];
                const MapData& m = bodies[b].map;
                if (determine_shape(m, 0, x, cell, c0, N, dN)) dist = interpolate_grad(m, 0, cell, c0, N, normal, dN);
                if (dist > T(0) && dist < info.h) {
                    const T volume = interpolate(m, 1, cell, N);
                    if (volume > T(0) && volume != (T)FLT_MAX) {
                        vb = volume;
                        const T nl = length(normal);
                        if (nl > T(1.0e-9)) {
                            normal /= nl;
                            const T d = std::max(dist + T(0.5) * info.r, info.diam);
                            xb = x - d * normal;
                        } else vb = 0;
                    } else vb = 0;
                } else if (dist <= T(0)) {
                    if (dist != (T)FLT_MAX) {
                        const T nl = length(normal);
                        if (nl > T(1.0e-5)) {
                            normal /= nl;
                            T delta = info.diam - dist;
                            delta = std::min(delta, T(0.1) * info.r);
                            x += delta * normal;
                            p[i].v = V3<T>();
                        }
                    }
                    vb = 0;
                } else vb = 0;
            }
        }
    }

    void K2_density() {  // ComputeDensityKernel, :152-187
#pragma omp parallel for schedule(static)
        for (int64_t ii = 0; ii < (int64_t)info.n; ii++) {
            const uint32_t i = (uint32_t)ii;
            const V3<T> xi = p[i].x;
            T rho = info.volume * kernel.wZero;
            for (uint32_t j = 0; j < nbrCount(i); j++) rho += info.volume * kernel.getW(xi - p[nbr(i, j)].x);
            for (uint32_t b = 0; b < info.bodies; b++) {
                const T vb = bvol[b][i];
                if (vb > T(0)) rho += vb * kernel.getW(xi - bxj[b][i]);
            }
            p[i].rho = rho * info.rho0;
        }
    }

    void K3_factor() {  // ComputeDFSPHFactorKernel, :189-231
#pragma omp parallel for schedule(static)
        for (int64_t ii = 0; ii < (int64_t)info.n; ii++) {
            const uint32_t i = (uint32_t)ii;
            const V3<T> xi = p[i].x;
            V3<T> gi;
            T sum = 0;
            for (uint32_t j = 0; j < nbrCount(i); j++) {
                const V3<T> gj = -info.volume * kernel.getGradW(xi - p[nbr(i, j)].x);
                sum += dot(gj, gj);
                gi -= gj;
            }
            for (uint32_t b = 0; b < info.bodies; b++) {
                const T vb = bvol[b][i];
                if (vb > T(0)) {
                    const V3<T> gj = -vb * kernel.getGradW(xi - bxj[b][i]);
                    gi -= gj;
                }
            }
            sum += dot(gi, gi);
            p[i].alpha = (double)sum > kEPS ? T(1) / sum : T(0);
        }
    }

    // ComputeDensityPressureForce, :280-315
    T pressure_force(uint32_t i) const {
        const V3<T> xi = p[i].x;
        const V3<T> ai = p[i].ap;
        T f = 0;
        for (uint32_t j = 0; j < nbrCount(i); j++) {
            const uint32_t k = nbr(i, j);
            f += dot(ai - p[k].ap, kernel.getGradW(xi - p[k].x));
        }
        f *= info.volume;
        for (uint32_t b = 0; b < info.bodies; b++) {
            const T vb = bvol[b][i];
            if (vb > T(0)) f += vb * dot(ai, kernel.getGradW(xi - bxj[b][i]));
        }
        return f;
    }

    // Pressure acceleration from kappa (K5/K7/K18/K20 share this body, :342-481, :555-602).
    V3<T> pressure_accel(uint32_t i, bool divergence) const {
        const V3<T> xi = p[i].x;
        const T ki = divergence ? p[i].kappaV : p[i].kappa;
        V3<T> a;
        for (uint32_t j = 0; j < nbrCount(i); j++) {
            const uint32_t k = nbr(i, j);
            const T sum = ki + (divergence ? p[k].kappaV : p[k].kappa);
            if ((double)std::fabs(sum) > kEPS) {
                const V3<T> g = -info.volume * kernel.getGradW(xi - p[k].x);
                a += sum * g;
            }
        }
        if ((double)std::fabs(ki) > kEPS) {
            for (uint32_t b = 0; b < info.bodies; b++) {
                const T vb = bvol[b][i];
                if (vb > T(0)) {
                    const V3<T> g = -vb * kernel.getGradW(xi - bxj[b][i]);
                    a += ki * g;
                }
            }
        }
        return a;
    }

    T velocity_divergence(uint32_t i) const {  // common body of K4 (:498-522) and K17 (:253-271)
        const V3<T> xi = p[i].x, vi = p[i].v;
        T d = 0;
        for (uint32_t j = 0; j < nbrCount(i); j++) {
            const uint32_t k = nbr(i, j);
            d += dot(vi - p[k].v, kernel.getGradW(xi - p[k].x));
        }
        d *= info.volume;
        for (uint32_t b = 0; b < info.bodies; b++) {
            const T vb = bvol[b][i];
            if (vb > T(0)) d += vb * dot(vi, kernel.getGradW(xi - bxj[b][i]));
        }
        return d;
    }

    double residual_sum() const {
        double s = 0;
        for (uint32_t i = 0; i < info.n; i++) s += (double)p[i].res;
        return s;
    }

    // ComputeDivergence, DFSPHImplementation.cu:506-575
    void divergence_solve() {
        if (!desc.EnableDivergenceSolverError) {
            dbg.DivergenceSolverError = 0;
            dbg.DivergenceSolverIterationCount = 0;
            return;
        }
#pragma omp parallel for schedule(static)
        for (int64_t ii = 0; ii < (int64_t)info.n; ii++) {  // ComputeDensityChangeKernel, :483-529
            const uint32_t i = (uint32_t)ii;
            T d = velocity_divergence(i);
            d = nbrCount(i) < 20u ? T(0) : std::max(d, T(0));
            p[i].rhoAdv = d;
            p[i].alpha *= info.dtInv;
            p[i].kappaV = d * p[i].alpha;
        }
        const double eta = (double)(info.dtInv * (T)desc.MaxDivergenceSolverError * (T)0.0001 * info.rho0);
        uint32_t it = 0;
        double err = 0.0;
        while ((err > eta || it < desc.MinDivergenceSolverIterations) && it < desc.MaxDivergenceSolverIterations) {
#pragma omp parallel for schedule(static)
            for (int64_t ii = 0; ii < (int64_t)info.n; ii++) p[ii].ap = pressure_accel((uint32_t)ii, true);  // :388-432
#pragma omp parallel for schedule(static)
            for (int64_t ii = 0; ii < (int64_t)info.n; ii++) {  // DivergenceSolveIterationKernel, :531-553
                const uint32_t i = (uint32_t)ii;
                const T s = pressure_force(i) * info.dt;
                p[i].res = nbrCount(i) < 20u ? T(0) : std::min(-p[i].rhoAdv - s, T(0));
                p[i].kappaV -= p[i].res * p[i].alpha;
            }
            err = -(double)info.rho0 * residual_sum() / (double)info.n;
            it++;
        }
        dbg.DivergenceSolverIterationCount = it;
        dbg.DivergenceSolverError = (float)err;
        if (it >= desc.MaxDivergenceSolverIterations && desc.MaxDivergenceSolverIterations > 0 && err > eta)
            dbg.Flags |= VFD_FLAG_DIVERGENCE_CAP;
#pragma omp parallel for schedule(static)
        for (int64_t ii = 0; ii < (int64_t)info.n; ii++) {  // ComputePressureAccelerationAndFactorKernel, :555-602
            const uint32_t i = (uint32_t)ii;
            p[i].ap = pressure_accel(i, true);
            p[i].v += info.dt * p[i].ap;
            p[i].alpha *= info.dt;
        }
    }

    // ComputePressure, DFSPHImplementation.cu:443-504
    void pressure_solve() {
#pragma omp parallel for schedule(static)
        for (int64_t ii = 0; ii < (int64_t)info.n; ii++) {  // ComputeDensityAdvectionKernel, :233-278
            const uint32_t i = (uint32_t)ii;
            const T d = velocity_divergence(i);
            p[i].rhoAdv = p[i].rho / info.rho0 + info.dt * d;
            p[i].alpha *= info.dt2Inv;
            const T si = T(1) - p[i].rhoAdv;
            const T r = std::min(si, T(0));
            p[i].kappa = -r * p[i].alpha;
        }
        const double eta = (double)((T)desc.MaxPressureSolverError * (T)0.0001 * info.rho0);
        uint32_t it = 0;
        double err = 0.0;
        while ((err > eta || it < desc.MinPressureSolverIterations) && it < desc.MaxPressureSolverIterations) {
#pragma omp parallel for schedule(static)
            for (int64_t ii = 0; ii < (int64_t)info.n; ii++) p[ii].ap = pressure_accel((uint32_t)ii, false);  // :342-386
#pragma omp parallel for schedule(static)
            for (int64_t ii = 0; ii < (int64_t)info.n; ii++) {  // PressureSolveIterationKernel, :317-340
                const uint32_t i = (uint32_t)ii;
                const T s = pressure_force(i) * info.dt2;
                p[i].res = std::min(T(1) - p[i].rhoAdv - s, T(0));
                p[i].kappa -= p[i].res * p[i].alpha;
            }
            err = -(double)info.rho0 * residual_sum() / (double)info.n;
            it++;
        }
        dbg.PressureSolverIterationCount = it;
        dbg.PressureSolverError = (float)err;
        if (it >= desc.MaxPressureSolverIterations && desc.MaxPressureSolverIterations > 0 && err > eta)
            dbg.Flags |= VFD_FLAG_PRESSURE_CAP;
#pragma omp parallel for schedule(static)
        for (int64_t ii = 0; ii < (int64_t)info.n; ii++) {  // ComputePressureAccelerationAndVelocityKernel, :434-481
            const uint32_t i = (uint32_t)ii;
            p[i].ap = pressure_accel(i, false);
            p[i].v += info.dt * p[i].ap;
        }
    }

    // Boundary samples of the viscosity terms (:636-681, :706-752, :793-839).
    struct BSample { V3<T> dir[4]; V3<T> grad[4]; T vol; };
    bool boundary_samples(uint32_t i, uint32_t b, BSample& s) const {
        const T vb = bvol[b][i];
        if (!(vb > T(0))) return false;
        const V3<T> xi = p[i].x;
        const V3<T> xb = bxj[b][i];
        const V3<T> dir = xi - xb;
        V3<T> normal = -dir;
        const T nl = length(normal);
        if (!(nl > T(0.0001))) return false;
        normal /= nl;
        V3<T> t1, t2;
        orthogonal_vectors(normal, t1, t2);
        const V3<T> pos[4] = {xb - t1 * info.tangDist, xb + t1 * info.tangDist, xb - t2 * info.tangDist,
                              xb + t2 * info.tangDist};
        for (int k = 0; k < 4; k++) {
            s.dir[k] = xi - pos[k];
            s.grad[k] = kernel.getGradW(s.dir[k]);
        }
        s.vol = T(0.25) * vb;
        return true;
    }

    void K12_preconditioner() {  // ComputeViscosityPreconditionerKernel, :604-684
#pragma omp parallel for schedule(static)
        for (int64_t ii = 0; ii < (int64_t)info.n; ii++) {
            const uint32_t i = (uint32_t)ii;
            M3<T> res;
            const V3<T> xi = p[i].x;
            for (uint32_t j = 0; j < nbrCount(i); j++) {
                const uint32_t k = nbr(i, j);
                const V3<T> d = xi - p[k].x;
                const V3<T> g = kernel.getGradW(d);
                const T c = T(10) * info.dynVisc * (info.mass / p[k].rho) / (length2(d) + T(0.01) * info.h2);
                res.add_outer(c, d, g);
            }
            if (info.dynBVisc != T(0)) {
                for (uint32_t b = 0; b < info.bodies; b++) {
                    BSample s;
                    if (!boundary_samples(i, b, s)) continue;
                    for (int k = 0; k < 4; k++) {
                        const T c = T(10) * info.dynBVisc * s.vol / (length2(s.dir[k]) + T(0.01) * info.h2);
                        res.add_outer(c, s.dir[0], s.grad[k]);  // positionDirection1 in all four terms, :674-677
                    }
                }
            }
            M3<T> a;
            const T f = info.dt / p[i].rho;
            for (int r = 0; r < 3; r++)
                for (int c = 0; c < 3; c++) a.m[r][c] = (r == c ? T(1) : T(0)) - f * res.m[r][c];
            cgMinv[i] = inverse(a);
        }
    }

    V3<T> matvec(uint32_t i, const std::vector<V3<T>>& rhs) const {  // ComputeMatrixVecProdFunctionKernel, :758-842
        const V3<T> xi = p[i].x;
        const V3<T> vi = rhs[i];
        V3<T> acc;
        for (uint32_t j = 0; j < nbrCount(i); j++) {
            const uint32_t k = nbr(i, j);
            const V3<T> d = xi - p[k].x;
            const V3<T> g = kernel.getGradW(d);
            acc += (T(10) * info.dynVisc * (info.mass / p[k].rho) * dot(vi - rhs[k], d) / (length2(d) + T(0.01) * info.h2)) * g;
        }
        if (info.dynBVisc != T(0)) {
            for (uint32_t b = 0; b < info.bodies; b++) {
                BSample s;
                if (!boundary_samples(i, b, s)) continue;
                for (int k = 0; k < 4; k++)
                    acc += (T(10) * info.dynBVisc * s.vol * dot(vi, s.dir[k]) / (length2(s.dir[k]) + T(0.01) * info.h2)) * s.grad[k];
            }
        }
        return rhs[i] - (info.dt / p[i].rho) * acc;
    }

    // CG dot product: each particle's term in T (FP32 for the mirror: x + y then z), the
    // sum over particles in FP64.
    static double dotv(const std::vector<V3<T>>& a, const std::vector<V3<T>>& b, uint32_t n) {
        double s = 0;
        for (uint32_t i = 0; i < n; i++) s += (double)(a[i].x * b[i].x + a[i].y * b[i].y + a[i].z * b[i].z);
        return s;
    }

    // ComputeViscosity + SolveViscosity, DFSPHImplementation.cu:577-808
    void viscosity_solve() {
        if (!desc.EnableViscositySolver) {
            dbg.ViscositySolverError = 0;
            dbg.ViscositySolverIterationCount = 0;
            return;
        }
        const uint32_t n = info.n;
        K12_preconditioner();
        // ComputeViscosityGradientKernel, :686-756: the boundary term dots a zero vector.
        for (uint32_t i = 0; i < n; i++) {
            cgB[i] = p[i].v;
            cgG[i] = p[i].v + p[i].dv;
        }
        uint32_t it = 0;
#pragma omp parallel for schedule(static)
        for (int64_t ii = 0; ii < (int64_t)n; ii++) cgTmp[ii] = matvec((uint32_t)ii, cgG);
        for (uint32_t i = 0; i < n; i++) cgR[i] = cgB[i] - cgTmp[i];
        const double rhsNorm2 = dotv(cgB, cgB, n);
        bool done = false;
        double rr = 0;
        if (rhsNorm2 == 0.0) {
            for (uint32_t i = 0; i < n; i++) cgG[i] = V3<T>();
            dbg.ViscositySolverError = 0;
            done = true;
        }
        if (!done) {
            const double e = (double)desc.MaxViscositySolverError;
            const double thr = std::max(e * e * 0.0001 * rhsNorm2, (double)FLT_MIN);
            rr = dotv(cgR, cgR, n);
            if (rr < thr) {
                dbg.ViscositySolverError = (float)std::sqrt(rr / rhsNorm2);
                done = true;
            }
            if (!done) {
                for (uint32_t i = 0; i < n; i++) cgP[i] = cgMinv[i].mul(cgR[i]);
                double absNew = std::fabs(dotv(cgR, cgP, n));
                while (it >= desc.MinViscositySolverIterations && it < desc.MaxViscositySolverIterations) {
#pragma omp parallel for schedule(static)
                    for (int64_t ii = 0; ii < (int64_t)n; ii++) cgTmp[ii] = matvec((uint32_t)ii, cgP);
                    const T alpha = (T)(absNew / dotv(cgP, cgTmp, n));
                    for (uint32_t i = 0; i < n; i++) {
                        cgG[i] += cgP[i] * alpha;
                        cgR[i] -= cgTmp[i] * alpha;
                    }
                    rr = dotv(cgR, cgR, n);
                    if (rr < thr) break;
                    for (uint32_t i = 0; i < n; i++) cgZ[i] = cgMinv[i].mul(cgR[i]);
                    const double absOld = absNew;
                    absNew = std::fabs(dotv(cgR, cgZ, n));
                    const T beta = (T)(absNew / absOld);
                    for (uint32_t i = 0; i < n; i++) cgP[i] = cgP[i] * beta + cgZ[i];
                    it++;
                }
                dbg.ViscositySolverError = (float)std::sqrt(rr / rhsNorm2);
                if (it >= desc.MaxViscositySolverIterations && rr >= thr) dbg.Flags |= VFD_FLAG_VISCOSITY_CAP;
            }
        }
        dbg.ViscositySolverIterationCount = it;
        for (uint32_t i = 0; i < n; i++) {  // ApplyViscosityForceKernel, :844-862
            p[i].a += T(1) / info.dt * (cgG[i] - p[i].v);
            p[i].dv = cgG[i] - p[i].v;
        }
    }

    // Surface tension, DFSPHImplementation.cu:810-839 and DFSPHKernels.cu:864-1046
    void surface_tension() {
        if (!desc.EnableSurfaceTensionSolver) return;
        const uint32_t n = info.n;
        const uint32_t S = info.stSamples;
#pragma omp parallel for schedule(dynamic, 256)
        for (int64_t ii = 0; ii < (int64_t)n; ii++) {  // classification, :881-958
            const uint32_t i = (uint32_t)ii;
            p[i].n = V3<T>();
            const V3<T> xi = p[i].x;
            const uint32_t cnt = nbrCount(i);
            if (cnt == 0) {
                p[i].curv = T(1) / info.h;
                continue;
            }
            V3<T> com;
            for (uint32_t j = 0; j < cnt; j++) com += p[nbr(i, j)].x - xi;
            com /= info.h;
            const T input = length(com) / (T)cnt;
            if ((T)cnt <= info.slope * input + info.constant + T(0)) {
                uint32_t count = 0;
                const uint32_t s0 = i * S / 3u * 3u;
                const T ratio = info.nbrRadius / info.r;
                V3<T> nsum;
                for (uint32_t q = 0; q < S; q++) {
                    const uint32_t i3 = s0 + 3u * q;
                    const V3<T> pt = info.h * V3<T>((T)halton[i3 % kHaltonCount], (T)halton[(i3 + 1) % kHaltonCount],
                                                    (T)halton[(i3 + 2) % kHaltonCount]);
                    bool covered = false;
                    for (uint32_t j = 0; j < cnt; j++) {
                        const V3<T> d = p[nbr(i, j)].x - xi;
                        const V3<T> vec = pt - d;
                        if (length2(vec) <= ratio * ratio * info.h2) { covered = true; break; }
                    }
                    if (!covered) { nsum += pt; count++; }
                }
                if (count > 0) {
                    if (length2(nsum) > T(0)) nsum = normalize(nsum);
                    p[i].n = nsum;
                    p[i].curv = T(1) / info.h * T(-2) * std::sqrt(T(1) - info.nbrRadius * info.nbrRadius / (info.r * info.r)) *
                                std::cos(std::acos(T(1) - T(2) * ((T)count / (T)S)) + info.mcFactor);
                } else {
                    p[i].n = V3<T>();
                    p[i].curv = 0;
                }
            }
        }
        const V3<T> zero;
#pragma omp parallel for schedule(static)
        for (int64_t ii = 0; ii < (int64_t)n; ii++) {  // normals and curvature smoothing, :960-1006
            const uint32_t i = (uint32_t)ii;
            if (!(p[i].n != zero)) continue;
            const V3<T> xi = p[i].x;
            V3<T> nc;
            T cc = 0, cf = 0;
            for (uint32_t j = 0; j < nbrCount(i); j++) {
                const uint32_t k = nbr(i, j);
                if (p[k].n != zero) {
                    const T dist = length(p[k].x - xi);
                    const T num = T(1) - dist / info.h;
                    nc += p[k].n * num;
                    cc += p[k].curv * num;
                    cf += num;
                }
            }
            if (length2(nc) > T(0)) nc = normalize(nc);
            V3<T> ns = (T(1) - info.smoothing) * p[i].n + info.smoothing * nc;
            if (length2(ns) > T(0)) ns = normalize(ns);
            p[i].ns = ns;
            p[i].curvS = ((T(1) - info.smoothing) * p[i].curv + info.smoothing * cc) /
                         (T(1) - info.smoothing + info.smoothing * cf);
        }
        for (uint32_t pass = 0; pass < desc.SurfaceTensionSmoothPassCount; pass++) {
            for (uint32_t i = 0; i < n; i++) {  // blending, :1008-1046
                if (p[i].n != zero) {
                    T fc = p[i].curvS;
                    if (info.temporal) fc = T(0.05) * fc + T(0.95) * p[i].dCurv;
                    const V3<T> force = p[i].ns * info.st * fc;
                    p[i].a -= info.massInv * force;
                    p[i].dCurv = fc;
                } else {
                    T fc = 0;
                    if (info.temporal) fc = T(0.95) * p[i].dCurv;
                    p[i].dCurv = fc;
                }
            }
        }
    }

    void time_step_size() {  // ComputeTimeStepSize + ComputeMaxVelocityMagnitude, :395-441
        T mv = T(0.1);
        for (uint32_t i = 0; i < info.n; i++) mv = std::max(mv, length2(p[i].v + p[i].a * info.dt));
        if (mv < T(1.0e-9)) mv = T(1.0e-9);
        maxV2 = mv;
        T dt = T(0.4) * (info.diam / std::sqrt(mv));
        dt = std::min(dt, (T)desc.MaxTimeStepSize);
        dt = std::max(dt, (T)desc.MinTimeStepSize);
        set_dt(dt);
        update_samples();
        frameTime += info.dt;
    }

    int step(vfd_step_stats* out) {  // DFSPHImplementation::OnUpdate, :63-170
        if (info.n == 0) return VFD_OK;
        dbg.Flags = 0;
        std::vector<V3<T>> xs(info.n);
        for (uint32_t i = 0; i < info.n; i++) xs[i] = p[i].x;
        search.find(xs);
        if (search.capHit) dbg.Flags |= VFD_FLAG_NEIGHBOR_CAP;
        dbg.MaxNeighborCount = search.maxCount;
        K1_boundary();
        K2_density();
        K3_factor();
        divergence_solve();
        for (uint32_t i = 0; i < info.n; i++) p[i].a = info.g;  // ClearAccelerationKernel, :24-37
        const uint32_t samplesUsed = info.stSamples;
        surface_tension();
        viscosity_solve();
        time_step_size();
        for (uint32_t i = 0; i < info.n; i++) p[i].v += info.dt * p[i].a;  // ComputeVelocityKernel, :39-52
        pressure_solve();
        for (uint32_t i = 0; i < info.n; i++) {
            p[i].x += info.dt * p[i].v;  // ComputePositionKernel, :54-67
            if (!std::isfinite((double)p[i].x.x) || !std::isfinite((double)p[i].x.y) || !std::isfinite((double)p[i].x.z))
                dbg.Flags |= VFD_FLAG_NAN;
        }
        if (dbg.FrameIndex < desc.FrameCount && frameTime >= (T)desc.FrameLength) {  // :148-167
            frameTime = 0;
            dbg.FrameIndex++;
        }
        dbg.IterationCount++;
        dbg.FrameTime = (float)frameTime;
        dbg.TimeStepSize = (float)info.dt;
        dbg.MaxVelocityMagnitude = (float)maxV2;
        dbg.SurfaceTensionSampleCount = samplesUsed;
        if (out) *out = dbg;
        return VFD_OK;
    }

    void set_fluid(const float* x, const float* v, uint32_t n) {  // SetFluidObjects, :172-253
        init.assign(n, Particle<T>());
        for (uint32_t i = 0; i < n; i++) {
            init[i].x = V3<T>((T)x[3 * i], (T)x[3 * i + 1], (T)x[3 * i + 2]);
            if (v) init[i].v = V3<T>((T)v[3 * i], (T)v[3 * i + 1], (T)v[3 * i + 2]);
        }
        info.n = n;
        p = init;
        cgR.assign(n, V3<T>()); cgP = cgR; cgZ = cgR; cgTmp = cgR; cgB = cgR; cgG = cgR;
        cgMinv.assign(n, M3<T>());
        for (auto& b : bxj) b.assign(n, V3<T>());
        for (auto& b : bvol) b.assign(n, 0);
        reset();
    }

    // Appends particles to the running state (the GPU library's vfd_emit; the reference
    // has no emitter): zero accelerations and warm starts, original indices n, n+1, ...
    void emit(const float* x, const float* v, uint32_t k) {
        for (uint32_t i = 0; i < k; i++) {
            Particle<T> q{};
            q.x = V3<T>((T)x[3 * i], (T)x[3 * i + 1], (T)x[3 * i + 2]);
            if (v) q.v = V3<T>((T)v[3 * i], (T)v[3 * i + 1], (T)v[3 * i + 2]);
            p.push_back(q);
        }
        resize_state((uint32_t)p.size());
    }
    void resize_state(uint32_t n) {
        info.n = n;
        for (auto* a : {&cgR, &cgP, &cgZ, &cgTmp, &cgB, &cgG}) a->resize(n, V3<T>());
        cgMinv.resize(n, M3<T>());
        for (auto& b : bxj) b.resize(n, V3<T>());
        for (auto& b : bvol) b.resize(n, 0);
    }

    // The state one step carries to the next (DFSPHParticle x, v, VelocityDifference,
    // DeltaFinalCurvature; DFSPHSimulationInfo dt and the surface-tension sample count
    // derived from it), taken from another run: the next step() then starts where that
    // run stands. Arrays in original order; dv and dk may be null (zero).
    void set_carried(const float* x, const float* v, const float* dv, const float* dk, double dt) {
        for (uint32_t i = 0; i < info.n; i++) {
            p[i].x = V3<T>((T)x[3 * i], (T)x[3 * i + 1], (T)x[3 * i + 2]);
            p[i].v = V3<T>((T)v[3 * i], (T)v[3 * i + 1], (T)v[3 * i + 2]);
            p[i].dv = dv ? V3<T>((T)dv[3 * i], (T)dv[3 * i + 1], (T)dv[3 * i + 2]) : V3<T>();
            p[i].dCurv = dk ? (T)dk[i] : T(0);
        }
        set_dt((T)(float)dt);
        update_samples();
    }

    void reset() {  // Simulate preamble, :33-51
        p = init;
        if (info.n != (uint32_t)init.size()) resize_state((uint32_t)init.size());
        set_dt((T)desc.TimeStepSize);
        update_samples();
        dbg = vfd_step_stats{};
        frameTime = 0;
    }
};

struct Handle {
    int precision;
    std::unique_ptr<Sim<float>> f;
    std::unique_ptr<Sim<double>> d;
};

template <class T>
static void init_sim(Sim<T>& s, const vfd_desc& d) {
    s.halton.resize(kHaltonCount);
    halton_table(s.halton.data());
    s.info.r = -1;
    s.set_description(d);
}

template <class T>
static int get_field(Sim<T>& s, int field, uint32_t body, double* out) {
    const uint32_t n = s.info.n;
    for (uint32_t i = 0; i < n; i++) {
        const Particle<T>& q = s.p[i];
        switch (field) {
            case VFD_FIELD_DENSITY: out[i] = q.rho; break;
            case VFD_FIELD_FACTOR: out[i] = q.alpha; break;
            case VFD_FIELD_DENSITY_ADVECTION: out[i] = q.rhoAdv; break;
            case VFD_FIELD_PRESSURE_RHO2: out[i] = q.kappa; break;
            case VFD_FIELD_PRESSURE_RHO2_V: out[i] = q.kappaV; break;
            case VFD_FIELD_PRESSURE_RESIDUUM: out[i] = q.res; break;
            case VFD_FIELD_PRESSURE_ACCELERATION: for (int d = 0; d < 3; d++) out[3 * i + d] = q.ap[d]; break;
            case VFD_FIELD_VELOCITY_DIFFERENCE: for (int d = 0; d < 3; d++) out[3 * i + d] = q.dv[d]; break;
            case VFD_FIELD_SURFACE_NORMAL: for (int d = 0; d < 3; d++) out[3 * i + d] = q.n[d]; break;
            case VFD_FIELD_SURFACE_CURVATURE: out[i] = q.curv; break;
            case VFD_FIELD_DELTA_FINAL_CURVATURE: out[i] = q.dCurv; break;
            case VFD_FIELD_SURFACE_NORMAL_SMOOTH: for (int d = 0; d < 3; d++) out[3 * i + d] = q.ns[d]; break;
            case VFD_FIELD_SURFACE_CURVATURE_SMOOTH: out[i] = q.curvS; break;
            case VFD_FIELD_BOUNDARY_XJ:
                if (body >= s.info.bodies) return VFD_E_ARG;
                for (int d = 0; d < 3; d++) out[3 * i + d] = s.bxj[body][i][d];
                break;
            case VFD_FIELD_BOUNDARY_VOLUME:
                if (body >= s.info.bodies) return VFD_E_ARG;
                out[i] = s.bvol[body][i];
                break;
            default: return VFD_E_ARG;
        }
    }
    return VFD_OK;
}

template <class T>
static void add_body(Sim<T>& s, const vfd_volume_map* m) {
    Body b;
    MapData& d = b.map;
    d.fieldCount = m->field_count;
    d.nodeCount = m->node_count;
    d.cellCount = m->cell_count;
    d.cellMapCount = m->cell_map_count;
    for (int k = 0; k < 3; k++) {
        d.dmin[k] = m->domain_min[k];
        d.dmax[k] = m->domain_max[k];
        d.res[k] = m->resolution[k];
        d.cs[k] = m->cell_size[k];
        d.csi[k] = m->cell_size_inverse[k];
    }
    d.nodes.assign(m->nodes, m->nodes + (size_t)d.fieldCount * d.nodeCount);
    d.cells.assign(m->cells, m->cells + (size_t)d.fieldCount * d.cellCount * 32u);
    d.cellMap.assign(m->cell_map, m->cell_map + (size_t)d.fieldCount * d.cellMapCount);
    s.bodies.push_back(std::move(b));
    s.info.bodies = (uint32_t)s.bodies.size();
    s.bxj.emplace_back(s.info.n, V3<T>());
    s.bvol.emplace_back(s.info.n, T(0));
}

template <class T>
static int get_neighbors(Sim<T>& s, uint32_t* counts, uint32_t* offsets, uint32_t* list, uint32_t cap,
                         uint32_t* total, uint32_t* sortIdx, uint32_t* keys) {
    const NeighborSearch<T>& ns = s.search;
    const uint32_t n = (uint32_t)ns.counts.size();
    if (total) *total = (uint32_t)ns.list.size();
    if (counts) std::copy(ns.counts.begin(), ns.counts.end(), counts);
    if (offsets) std::copy(ns.offsets.begin(), ns.offsets.end(), offsets);
    if (sortIdx) std::copy(ns.sortIdx.begin(), ns.sortIdx.end(), sortIdx);
    if (keys) std::copy(ns.keys.begin(), ns.keys.end(), keys);
    if (list) {
        if (ns.list.size() > cap) return VFD_E_CAPACITY;
        std::copy(ns.list.begin(), ns.list.end(), list);
    }
    (void)n;
    return VFD_OK;
}

}  // namespace orc

using namespace orc;

extern "C" {

void* orc_create(const vfd_desc* d, int precision) {
    if (!d || (precision != 32 && precision != 64)) return nullptr;
    Handle* h = new Handle();
    h->precision = precision;
    if (precision == 32) { h->f.reset(new Sim<float>()); init_sim(*h->f, *d); }
    else { h->d.reset(new Sim<double>()); init_sim(*h->d, *d); }
    return h;
}

void orc_destroy(void* p) { delete static_cast<Handle*>(p); }

#define ORC_DISPATCH(h, call) ((h)->precision == 32 ? (*(h)->f).call : (*(h)->d).call)

int orc_set_fluid(void* p, const float* x, const float* v, uint32_t n) {
    Handle* h = static_cast<Handle*>(p);
    ORC_DISPATCH(h, set_fluid(x, v, n));
    return VFD_OK;
}

int orc_add_rigid_body(void* p, const vfd_volume_map* m) {
    Handle* h = static_cast<Handle*>(p);
    if (!m || m->field_count < 2) return VFD_E_ARG;
    if (h->precision == 32) add_body(*h->f, m); else add_body(*h->d, m);
    return VFD_OK;
}

int orc_reset(void* p) { Handle* h = static_cast<Handle*>(p); ORC_DISPATCH(h, reset()); return VFD_OK; }

int orc_emit(void* p, const float* x, const float* v, uint32_t n) {
    Handle* h = static_cast<Handle*>(p);
    if (h->f) h->f->emit(x, v, n);
    if (h->d) h->d->emit(x, v, n);
    return VFD_OK;
}

// Kernel evaluation: 0 = the reference's tables, 1 = the spline at |r| (analytic mode).
int orc_set_kernel_mode(void* p, int mode) {
    Handle* h = static_cast<Handle*>(p);
    if (h->f) h->f->kernel.analytic = mode != 0;
    if (h->d) h->d->kernel.analytic = mode != 0;
    return VFD_OK;
}

int orc_set_carried(void* p, const float* x, const float* v, const float* dv, const float* dk, double dt) {
    Handle* h = static_cast<Handle*>(p);
    if (!x || !v) return VFD_E_ARG;
    ORC_DISPATCH(h, set_carried(x, v, dv, dk, dt));
    return VFD_OK;
}

int orc_step(void* p, vfd_step_stats* st) { Handle* h = static_cast<Handle*>(p); return ORC_DISPATCH(h, step(st)); }

int orc_find_neighbors(void* p) {
    Handle* h = static_cast<Handle*>(p);
    if (h->precision == 32) {
        std::vector<V3<float>> xs(h->f->info.n);
        for (uint32_t i = 0; i < h->f->info.n; i++) xs[i] = h->f->p[i].x;
        h->f->search.find(xs);
    } else {
        std::vector<V3<double>> xs(h->d->info.n);
        for (uint32_t i = 0; i < h->d->info.n; i++) xs[i] = h->d->p[i].x;
        h->d->search.find(xs);
    }
    return VFD_OK;
}

int orc_get_neighbors(void* p, uint32_t* counts, uint32_t* offsets, uint32_t* list, uint32_t cap, uint32_t* total,
                      uint32_t* sortIdx, uint32_t* keys) {
    Handle* h = static_cast<Handle*>(p);
    if (h->precision == 32) return get_neighbors(*h->f, counts, offsets, list, cap, total, sortIdx, keys);
    return get_neighbors(*h->d, counts, offsets, list, cap, total, sortIdx, keys);
}

int orc_get_state(void* p, double* x, double* v, double* a) {
    Handle* h = static_cast<Handle*>(p);
    const uint32_t n = h->precision == 32 ? h->f->info.n : h->d->info.n;
    for (uint32_t i = 0; i < n; i++)
        for (int d = 0; d < 3; d++) {
            if (h->precision == 32) {
                if (x) x[3 * i + d] = h->f->p[i].x[d];
                if (v) v[3 * i + d] = h->f->p[i].v[d];
                if (a) a[3 * i + d] = h->f->p[i].a[d];
            } else {
                if (x) x[3 * i + d] = h->d->p[i].x[d];
                if (v) v[3 * i + d] = h->d->p[i].v[d];
                if (a) a[3 * i + d] = h->d->p[i].a[d];
            }
        }
    return VFD_OK;
}

int orc_get_field(void* p, int field, uint32_t body, double* out) {
    Handle* h = static_cast<Handle*>(p);
    if (h->precision == 32) return get_field(*h->f, field, body, out);
    return get_field(*h->d, field, body, out);
}

int orc_get_time_step(void* p, double* dt) {
    Handle* h = static_cast<Handle*>(p);
    *dt = h->precision == 32 ? (double)h->f->info.dt : h->d->info.dt;
    return VFD_OK;
}

// FP32 kernel table exactly as SetRadius builds it (Kernel/DFSPHKernels.h:13-41).
int orc_kernel_table(float radius, float* w, float* g, float* wzero) {
    KernelTable<float> k;
    k.setRadius(radius);
    if (w) std::copy(k.W.begin(), k.W.end(), w);
    if (g) std::copy(k.G.begin(), k.G.end(), g);
    if (wzero) *wzero = k.wZero;
    return VFD_OK;
}

void orc_halton(float* out) { halton_table(out); }

uint32_t orc_morton3(uint32_t x, uint32_t y, uint32_t z) { return morton3(x, y, z); }

int orc_box_map_sizes(const uint32_t res[3], uint32_t* nodes, uint32_t* cells) {
    box_map_sizes(res, *nodes, *cells);
    return VFD_OK;
}

// Builds the two-field volume map of a box into caller arrays (nodes: 2*node_count,
// cells: 2*cell_count*32, cell_map: 2*cell_count) and fills `out`.
int orc_build_box_map(const float bmin[3], const float bmax[3], int inverted, float padding, const uint32_t res[3],
                      float r, float* nodes, uint32_t* cells, uint32_t* cellMap, vfd_volume_map* out) {
    MapData m;
    build_box_map(bmin, bmax, inverted != 0, padding, res, r, m);
    std::copy(m.nodes.begin(), m.nodes.end(), nodes);
    std::copy(m.cells.begin(), m.cells.end(), cells);
    std::copy(m.cellMap.begin(), m.cellMap.end(), cellMap);
    out->nodes = nodes;
    out->cells = cells;
    out->cell_map = cellMap;
    for (int d = 0; d < 3; d++) {
        out->domain_min[d] = m.dmin[d];
        out->domain_max[d] = m.dmax[d];
        out->resolution[d] = m.res[d];
        out->cell_size[d] = m.cs[d];
        out->cell_size_inverse[d] = m.csi[d];
    }
    out->field_count = m.fieldCount;
    out->node_count = m.nodeCount;
    out->cell_count = m.cellCount;
    out->cell_map_count = m.cellMapCount;
    return VFD_OK;
}

static void export_map(const MapData& m, float* nodes, uint32_t* cells, uint32_t* cellMap, vfd_volume_map* out) {
    std::copy(m.nodes.begin(), m.nodes.end(), nodes);
    std::copy(m.cells.begin(), m.cells.end(), cells);
    std::copy(m.cellMap.begin(), m.cellMap.end(), cellMap);
    out->nodes = nodes;
    out->cells = cells;
    out->cell_map = cellMap;
    for (int d = 0; d < 3; d++) {
        out->domain_min[d] = m.dmin[d];
        out->domain_max[d] = m.dmax[d];
        out->resolution[d] = m.res[d];
        out->cell_size[d] = m.cs[d];
        out->cell_size_inverse[d] = m.csi[d];
    }
    out->field_count = m.fieldCount;
    out->node_count = m.nodeCount;
    out->cell_count = m.cellCount;
    out->cell_map_count = m.cellMapCount;
}

// Two-field volume map of a triangle mesh placed by `transform` (column-major 4x4 or null).
int orc_build_mesh_map(const float* v, uint32_t nv, const uint32_t* tri, uint32_t nf, const float* transform,
                       int inverted, float padding, const uint32_t res[3], float r, float* nodes, uint32_t* cells,
                       uint32_t* cellMap, vfd_volume_map* out) {
    Mesh M;
    if (nv == 0 || nf == 0 || !make_mesh(v, nv, tri, nf, transform, M)) return VFD_E_ARG;
    MapData m;
    build_mesh_map(M, inverted != 0, padding, res, r, m);
    export_map(m, nodes, cells, cellMap, out);
    return VFD_OK;
}

// Signed distance of a placed mesh at n points (MeshDistance::SignedDistance).
int orc_mesh_signed_distance(const float* v, uint32_t nv, const uint32_t* tri, uint32_t nf, const float* transform,
                             const float* pts, uint32_t n, float* out) {
    Mesh M;
    if (nv == 0 || nf == 0 || !make_mesh(v, nv, tri, nf, transform, M)) return VFD_E_ARG;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; i++)
        out[i] = mesh_signed_distance(M, V3<float>(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]));
    return VFD_OK;
}

// Samples of a placed mesh's volume; `count` = all samples, min(count, cap) written.
int orc_sample_mesh_volume(const float* v, uint32_t nv, const uint32_t* tri, uint32_t nf, const float* transform,
                           float radius, const uint32_t res[3], int inverted, int mode, float* out, uint32_t cap,
                           uint32_t* count) {
    Mesh M;
    if (nv == 0 || nf == 0 || mode < 0 || mode > 2 || !make_mesh(v, nv, tri, nf, transform, M)) return VFD_E_ARG;
    std::vector<float> pts;
    if (!sample_mesh_volume(M, radius, res, inverted != 0, mode, pts)) return VFD_E_CAPACITY;
    *count = (uint32_t)(pts.size() / 3);
    if (out) std::copy(pts.begin(), pts.begin() + 3 * (size_t)std::min(*count, cap), out);
    return VFD_OK;
}

// Distance and gradient of field `field` at n points (FP64 lookup of the map), the
// points given in double precision.
int orc_map_interpolate_d(const vfd_volume_map* mp, uint32_t field, const double* x, uint32_t n, double* phi,
                          double* grad) {
    MapData m;
    m.fieldCount = mp->field_count;
    m.nodeCount = mp->node_count;
    m.cellCount = mp->cell_count;
    m.cellMapCount = mp->cell_map_count;
    for (int k = 0; k < 3; k++) {
        m.dmin[k] = mp->domain_min[k]; m.dmax[k] = mp->domain_max[k]; m.res[k] = mp->resolution[k];
        m.cs[k] = mp->cell_size[k]; m.csi[k] = mp->cell_size_inverse[k];
    }
    m.nodes.assign(mp->nodes, mp->nodes + (size_t)m.fieldCount * m.nodeCount);
    m.cells.assign(mp->cells, mp->cells + (size_t)m.fieldCount * m.cellCount * 32u);
    m.cellMap.assign(mp->cell_map, mp->cell_map + (size_t)m.fieldCount * m.cellMapCount);
    for (uint32_t i = 0; i < n; i++) {
        uint32_t cell[32];
        V3<double> c0, dN[32], g;
        double N[32];
        const V3<double> p(x[3 * i], x[3 * i + 1], x[3 * i + 2]);
        if (!determine_shape(m, 0, p, cell, c0, N, dN)) {
            phi[i] = (double)FLT_MAX;
            if (grad) grad[3 * i] = grad[3 * i + 1] = grad[3 * i + 2] = 0;
            continue;
        }
        phi[i] = interpolate_grad(m, field, cell, c0, N, g, dN);
        if (grad) { grad[3 * i] = g.x; grad[3 * i + 1] = g.y; grad[3 * i + 2] = g.z; }
    }
    return VFD_OK;
}

// The same with single-precision points.
int orc_map_interpolate(const vfd_volume_map* mp, uint32_t field, const float* x, uint32_t n, double* phi,
                        double* grad) {
    std::vector<double> xd(x, x + 3 * (size_t)n);
    return orc_map_interpolate_d(mp, field, xd.data(), n, phi, grad);
}

// n-point Gauss-Legendre abscissae and weights on [-1, 1] (ascending).
int orc_gauss_legendre(unsigned n, double* x, double* w) {
    std::vector<double> a, b;
    gauss_legendre(n, a, b);
    std::copy(a.begin(), a.end(), x);
    std::copy(b.begin(), b.end(), w);
    return VFD_OK;
}

// Positions of all nodes of a map (SDF::IndexToNodePosition) into out[3 * node_count].
int orc_map_node_positions(const vfd_volume_map* mp, float* out) {
    MapData m;
    for (int k = 0; k < 3; k++) {
        m.dmin[k] = mp->domain_min[k]; m.dmax[k] = mp->domain_max[k]; m.res[k] = mp->resolution[k];
        m.cs[k] = mp->cell_size[k]; m.csi[k] = mp->cell_size_inverse[k];
    }
    for (uint32_t i = 0; i < mp->node_count; i++) {
        const V3<float> p = node_position(m, i);
        out[3 * i] = p.x; out[3 * i + 1] = p.y; out[3 * i + 2] = p.z;
    }
    return VFD_OK;
}

void orc_set_threads(int t) {
#ifdef _OPENMP
    if (t > 0) omp_set_num_threads(t);
#else
    (void)t;
#endif
}

int orc_get_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

}  // extern "C"
