// CPU oracle of the reference's legacy SPH pipeline (Simulation/SPH), test infrastructure
// only: it checks the GPU library's vfd_sph_* path and is never part of it. FP32 in the
// reference's operation order (built with -ffp-contract=off). The sort is the reference's
// own kind: a stable sort of (cell key, particle index) pairs by key, as its LSD radix
// sort orders them (SPHSimulation.cpp:84, Compute/Utility/RadixSort).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <numeric>
#include <vector>

#include "../include/vfd_sph.h"

namespace {

struct F4 {
    float x, y, z, w;
};

struct SphOracle {
    vfd_sph_desc d{};
    // SPHSimulationParameters (SPHSimulation.cpp:187-214)
    float h2 = 0, poly6 = 0, spiky = 0, lap = 0, minDens = 0, mass = 0, minDist = 0, soft = 0, hard = 0, cell = 0;
    uint32_t gx = 0, gy = 0, gz = 0, cells = 0;
    std::vector<F4> x0, pos, vel, sortedPos, sortedVel;
    std::vector<float> density, pressure;
    std::vector<std::pair<uint32_t, uint32_t>> hash;  // (key, index) after the sort
    std::vector<uint32_t> cellStart;
    bool stepped = false;

    bool derive() {
        const double PI = 3.14159265358979323846;
        const float h = d.Homogeneity, r = d.ParticleRadius;
        if (!(r > 0) || !(h > 0)) return false;
        minDist = r;
        h2 = h * h;
        poly6 = (float)(315.0f / (64.0f * PI * std::pow((double)h, 9)));
        spiky = (float)(-0.5f * -45.0f / (PI * std::pow((double)h, 6)));
        lap = (float)(45.0f / (PI * std::pow((double)h, 6)));
        minDens = 1.0f / std::pow(d.RestDensity, 2.0f);
        mass = (float)(d.RestDensity * 4.0f / 3.0f * PI * std::pow(r, 3.0f));
        soft = 8 * r;
        hard = 4 * r;
        cell = r * 2.0f;
        uint32_t g[3];
        for (int k = 0; k < 3; k++) g[k] = (uint32_t)std::ceil((d.WorldMax[k] - d.WorldMin[k]) / cell);
        gx = g[0];
        gy = g[1];
        gz = g[2];
        cells = gx * gy * gz;
        return true;
    }

    // CalculateBoundary (SPHSimulationKernel.cu:17-59)
    void boundary(const float p[3], float v[3]) const {
        auto add = [&](float diff, const float n[3], float damp) {
            if (diff > 0.00001f) {
                const float acc = d.BoundsStiffness * diff - damp * (n[0] * v[0] + n[1] * v[1] + n[2] * v[2]);
                for (int k = 0; k < 3; k++) v[k] += acc * n[k] * d.TimeStep;
            }
        };
        const float zl[3] = {0, 0, 1}, zh[3] = {0, 0, -1}, xl[3] = {1, 0, 0}, xh[3] = {-1, 0, 0}, yl[3] = {0, 1, 0},
                    yh[3] = {0, -1, 0};
        add(soft - p[2] + d.WorldMin[2], zl, d.BoundsDampingCritical);
        add(soft + p[2] - d.WorldMax[2], zh, d.BoundsDampingCritical);
        add(soft - p[0] + d.WorldMin[0], xl, d.BoundsDamping);
        add(soft + p[0] - d.WorldMax[0], xh, d.BoundsDamping);
        add(soft - p[1] + d.WorldMin[1], yl, d.BoundsDamping);
        add(soft + p[1] - d.WorldMax[1], yh, d.BoundsDamping);
    }

    void gridPos(const F4& p, int c[3]) const {
        const float q[3] = {p.x, p.y, p.z};
        for (int k = 0; k < 3; k++) c[k] = (int)std::floor((q[k] - d.WorldMin[k]) / cell);
    }
    uint32_t gridHash(const int c[3]) const { return (uint32_t)(c[2] * (int)(gy * gx) + c[1] * (int)gx + c[0]); }

    void step() {
        const uint32_t n = (uint32_t)pos.size();
        // IntegrateKernel (:61-92)
        for (uint32_t i = 0; i < n; i++) {
            float p[3] = {pos[i].x, pos[i].y, pos[i].z}, v[3] = {vel[i].x, vel[i].y, vel[i].z};
            boundary(p, v);
            for (int k = 0; k < 3; k++) {
                v[k] += d.Gravity[k] * d.TimeStep;
                v[k] *= d.GlobalDamping;
                p[k] += v[k] * d.TimeStep;
            }
            for (int k = 0; k < 3; k++) {
                if (p[k] > d.WorldMax[k] - hard) p[k] = d.WorldMax[k] - hard;
                if (p[k] < d.WorldMin[k] + hard) p[k] = d.WorldMin[k] + hard;
            }
            pos[i] = F4{p[0], p[1], p[2], pos[i].w};
            vel[i] = F4{v[0], v[1], v[2], vel[i].w};
        }
        // CalculateHashKernel (:111-122) and the stable sort by key
        hash.resize(n);
        for (uint32_t i = 0; i < n; i++) {
            int c[3];
            gridPos(pos[i], c);
            hash[i] = {gridHash(c), i};
        }
        std::stable_sort(hash.begin(), hash.end(),
                         [](const std::pair<uint32_t, uint32_t>& a, const std::pair<uint32_t, uint32_t>& b) {
                             return a.first < b.first;
                         });
        // ReorderKernel (:124-151)
        cellStart.assign(cells, 0xffffffffu);
        sortedPos.resize(n);
        sortedVel.resize(n);
        for (uint32_t q = 0; q < n; q++) {
            if (q == 0 || hash[q].first != hash[q - 1].first) cellStart[hash[q].first] = q;
            sortedPos[q] = pos[hash[q].second];
            sortedVel[q] = vel[hash[q].second];
        }
        // CalculateDensityKernel (:270-297)
        density.assign(n, 0.0f);
        pressure.assign(n, 0.0f);
        for (uint32_t q = 0; q < n; q++) {
            const F4 pi = sortedPos[q];
            int g[3];
            gridPos(pi, g);
            float sum = 0.0f;
            for (int dz = -1; dz <= 1; dz++)
                for (int dy = -1; dy <= 1; dy++)
                    for (int dx = -1; dx <= 1; dx++) {
                        const int c[3] = {g[0] + dx, g[1] + dy, g[2] + dz};
                        const uint32_t gh = gridHash(c);
                        float dens = 0.0f;
                        const uint32_t start = cellStart[gh];
                        if (start != 0xffffffffu) {
                            for (uint32_t i = 0; i < d.MaxParticlesInCellCount; i++) {
                                const uint32_t o = start + i;
                                if (o >= n || hash[o].first != gh) break;
                                if (o == q) continue;
                                const F4 po = sortedPos[o];
                                const float px = pi.x - po.x, py = pi.y - po.y, pz = pi.z - po.z;
                                const float r2 = px * px + py * py + pz * pz;
                                if (r2 < h2) {
                                    const float cc = h2 - r2;
                                    dens += cc * cc * cc;
                                }
                            }
                        }
                        sum += dens;
                    }
            const float nd = sum * poly6 * mass;
            density[q] = nd;
            pressure[q] = (nd - d.RestDensity) * d.Stiffness;
        }
        // CalculateForceKernel (:299-334)
        std::vector<F4> out(n);
        for (uint32_t q = 0; q < n; q++) {
            const F4 pi = sortedPos[q], vi = sortedVel[q];
            const float prs = pressure[q], den = density[q];
            int g[3];
            gridPos(pi, g);
            float acc[3] = {0, 0, 0};
            for (int dz = -1; dz <= 1; dz++)
                for (int dy = -1; dy <= 1; dy++)
                    for (int dx = -1; dx <= 1; dx++) {
                        const int c[3] = {g[0] + dx, g[1] + dy, g[2] + dz};
                        const uint32_t gh = gridHash(c);
                        float f[3] = {0, 0, 0};
                        const uint32_t start = cellStart[gh];
                        if (start != 0xffffffffu) {
                            for (uint32_t i = 0; i < d.MaxParticlesInCellCount; i++) {
                                const uint32_t o = start + i;
                                if (o >= n || hash[o].first != gh) break;
                                if (o == q) continue;
                                const F4 po = sortedPos[o], vo = sortedVel[o];
                                const float d12 = std::min(minDens, 1.0f / (den * density[o]));
                                const float rp[3] = {pi.x - po.x, pi.y - po.y, pi.z - po.z};
                                const float rv[3] = {vo.x - vi.x, vo.y - vi.y, vo.z - vi.z};
                                const float r = std::max(minDist, std::sqrt(rp[0] * rp[0] + rp[1] * rp[1] + rp[2] * rp[2]));
                                if (r < d.Homogeneity) {
                                    const float cc = d.Homogeneity - r;
                                    const float pt = cc * spiky * (prs + pressure[o]) / r;
                                    const float vt = lap * d.Viscosity;
                                    const float s = cc * d12;
                                    for (int k = 0; k < 3; k++) f[k] += (pt * rp[k] + vt * rv[k]) * s;
                                }
                            }
                        }
                        for (int k = 0; k < 3; k++) acc[k] += f[k];
                    }
            const float s = mass * d.TimeStep;
            out[hash[q].second] = F4{vi.x + acc[0] * s, vi.y + acc[1] * s, vi.z + acc[2] * s, vi.w};
        }
        vel = out;
        stepped = true;
    }
};

}  // namespace

extern "C" {

void* orc_sph_create(const vfd_sph_desc* d, const float* xyz, uint32_t n) {
    auto s = std::make_unique<SphOracle>();
    s->d = *d;
    if (!s->derive()) return nullptr;
    s->x0.resize(n);
    for (uint32_t i = 0; i < n; i++) s->x0[i] = F4{xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], 0.0f};
    s->pos = s->x0;
    s->vel.assign(n, F4{0, 0, 0, 0});
    return s.release();
}

void orc_sph_destroy(void* p) { delete static_cast<SphOracle*>(p); }

int orc_sph_steps(void* p, uint32_t count) {
    SphOracle* s = static_cast<SphOracle*>(p);
    for (uint32_t k = 0; k < count; k++) s->step();
    return 0;
}

int orc_sph_set_velocities(void* p, const float* v) {
    SphOracle* s = static_cast<SphOracle*>(p);
    for (size_t i = 0; i < s->vel.size(); i++) s->vel[i] = F4{v[3 * i], v[3 * i + 1], v[3 * i + 2], 0.0f};
    return 0;
}

// Positions, velocities (caller order) and density, pressure (mapped back to caller order).
int orc_sph_get_state(void* p, float* x, float* v, float* rho, float* prs) {
    SphOracle* s = static_cast<SphOracle*>(p);
    const size_t n = s->pos.size();
    for (size_t i = 0; i < n; i++) {
        if (x) {
            x[3 * i] = s->pos[i].x;
            x[3 * i + 1] = s->pos[i].y;
            x[3 * i + 2] = s->pos[i].z;
        }
        if (v) {
            v[3 * i] = s->vel[i].x;
            v[3 * i + 1] = s->vel[i].y;
            v[3 * i + 2] = s->vel[i].z;
        }
    }
    for (size_t q = 0; q < n; q++) {
        const uint32_t o = s->stepped ? s->hash[q].second : (uint32_t)q;
        if (rho) rho[o] = s->stepped ? s->density[q] : 0.0f;
        if (prs) prs[o] = s->stepped ? s->pressure[q] : 0.0f;
    }
    return 0;
}

int orc_sph_get_sort(void* p, uint32_t* keys, uint32_t* idx) {
    SphOracle* s = static_cast<SphOracle*>(p);
    for (size_t q = 0; q < s->hash.size(); q++) {
        if (keys) keys[q] = s->hash[q].first;
        if (idx) idx[q] = s->hash[q].second;
    }
    return 0;
}

int orc_sph_params(void* p, vfd_sph_params* out) {
    SphOracle* s = static_cast<SphOracle*>(p);
    std::memset(out, 0, sizeof(*out));
    out->SmoothingRadius = s->h2;
    out->Poly6Kern = s->poly6;
    out->SpikyKern = s->spiky;
    out->LapKern = s->lap;
    out->ParticleMass = s->mass;
    out->MinDens = s->minDens;
    out->MinDist = s->minDist;
    out->BoundsSoftDistance = s->soft;
    out->BoundsHardDistance = s->hard;
    out->CellSize = s->cell;
    out->GridSize[0] = s->gx;
    out->GridSize[1] = s->gy;
    out->GridSize[2] = s->gz;
    out->CellCount = s->cells;
    out->ParticleCount = (uint32_t)s->pos.size();
    return 0;
}

}  // extern "C"
