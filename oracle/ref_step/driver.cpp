// Host driver for the reference's own DFSPH step kernels, run on the CPU.
//
// Test infrastructure only (never linked into the product). The recipe in
// oracle/Makefile (target `ref`) compiles the reference's Simulation/DFSPH/DFSPHKernels.cu
// as C++ together with this file and the search driver (ref_search/driver.cpp, which runs
// the reference's ParticleSearchKernels.cu), with ref_search/pch.h and glm_subset.h
// standing in for the reference's precompiled header and its absent glm submodule. Every
// per-particle computation of the step is the reference's kernel code, run one emulated
// CUDA thread at a time. This file restates the host side around the kernels:
//   * the simulation constants (DFSPHImplementation.cu:334-367) and particle
//     initialisation (:185-222);
//   * OnUpdate (:63-170): search, boundary, density, factor, divergence solve, cleared
//     accelerations, surface tension, viscosity, time step, velocity, pressure solve,
//     positions;
//   * the loops of ComputeDivergence (:511-575), ComputePressure (:443-509),
//     ComputeViscosity / SolveViscosity (:577-805), SolveSurfaceTension (:807-838) and
//     ComputeTimeStepSize (:395-441).
// Where the reference's thrust reductions leave the result to the reduction order, the
// loops follow the deterministic rules the oracle and the CUDA library use: the sums of the
// per-particle FP32 terms are formed in FP64, a solver's error is the mean
// -rho0 * sum(residuum) / N (the reference folds with thrust::minus), and the CG step
// lengths are the FP64 ratios rounded to FP32. The first step's surface-tension sample
// count and Monte-Carlo factor, which the reference first sets in ComputeTimeStepSize, are
// taken from the initial time step, as the oracle does. The neighbour lists are the
// reference search's (original particle indices), so the particles keep their order.
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <new>
#include <vector>

#include "pch.h"
#include "Simulation/DFSPH/DFSPHKernels.cuh"
#include "vfd_dfsph.h"

extern "C" int ref_find_neighbors(const float* xyz, uint32_t n, float radius, uint32_t* counts, uint32_t* offsets,
                                  uint32_t* list, uint32_t cap, uint32_t* total, uint32_t* sortIdx, uint32_t* keys);

namespace vfd {
// The reference grants its search and SDF classes access to the members these structs
// keep private; the driver binds host arrays to them through classes of those names.
class ParticleSearch {
public:
    static void Bind(NeighborSet& s, unsigned int* counts, unsigned int* offsets, unsigned int* list) {
        s.Counts = counts;
        s.Offsets = offsets;
        s.Neighbors = list;
    }
};
class SDF {
public:
    static void Bind(SDFDeviceData& d, const vfd_volume_map& m) {
        d.m_Nodes = const_cast<float*>(m.nodes);
        d.m_Cells = const_cast<unsigned int*>(m.cells);
        d.m_CellMap = const_cast<unsigned int*>(m.cell_map);
        d.m_Domain = BoundingBox<glm::vec3>(glm::vec3(m.domain_min[0], m.domain_min[1], m.domain_min[2]),
                                            glm::vec3(m.domain_max[0], m.domain_max[1], m.domain_max[2]));
        d.m_Resolution = glm::uvec3(m.resolution[0], m.resolution[1], m.resolution[2]);
        d.m_CellSize = glm::vec3(m.cell_size[0], m.cell_size[1], m.cell_size[2]);
        d.m_CellSizeInverse = glm::vec3(m.cell_size_inverse[0], m.cell_size_inverse[1], m.cell_size_inverse[2]);
        d.m_FieldCount = m.field_count;
        d.m_NodeCount = m.node_count;
        d.m_CellCount = m.cell_count;
        d.m_CellMapCount = m.cell_map_count;
    }
};
}  // namespace vfd

namespace {

using vfd::DFSPHParticle;

// kernel<<<blocks, 256>>>(), one emulated thread after another (the kernels return for
// indices past the particle count).
template <class F>
void launch(uint32_t count, F kernel) {
    const unsigned int threads = 256;
    blockDim = RefDim3{threads, 1, 1};
    const unsigned int blocks = (count + threads - 1) / threads;
    for (unsigned int b = 0; b < blocks; b++)
        for (unsigned int t = 0; t < threads; t++) {
            blockIdx = RefDim3{b, 0, 0};
            threadIdx = RefDim3{t, 0, 0};
            kernel();
        }
}

struct Body {
    std::vector<float> nodes;
    std::vector<uint32_t> cells, cellMap;
    vfd_volume_map map{};
    vfd::SDFDeviceData sdf{};
    std::vector<glm::vec3> xj;
    std::vector<float> volume;
    vfd::RigidBodyDeviceData dev{};
};

struct RefSim {
    vfd_desc desc{};
    vfd::DFSPHSimulationInfo info{};
    vfd::PrecomputedDFSPHCubicKernel* kernel = nullptr;
    std::vector<DFSPHParticle> p;
    std::vector<Body*> bodies;
    std::vector<vfd::RigidBodyDeviceData*> bodyPtrs;
    std::vector<unsigned int> counts, offsets, list;
    vfd::NeighborSet set;
    std::vector<glm::mat3x3> precond;
    std::vector<glm::vec3> b, g, r, d, z, ad;
    float maxV2 = 0.0f;
    vfd_step_stats last{};

    ~RefSim() {
        delete kernel;
        for (Body* bd : bodies) delete bd;
    }
    uint32_t n() const { return (uint32_t)p.size(); }
    vfd::RigidBodyDeviceData** rb() { return bodyPtrs.empty() ? nullptr : bodyPtrs.data(); }

    void set_dt(float dt) {
        info.TimeStepSize = dt;
        info.TimeStepSize2 = dt * dt;
        info.TimeStepSizeInverse = 1.0f / info.TimeStepSize;
        info.TimeStepSize2Inverse = 1.0f / info.TimeStepSize2;
    }
    void update_samples() {
        if (desc.CSDFix > 0) info.SurfaceTensionSampleCount = (unsigned int)desc.CSDFix;
        else info.SurfaceTensionSampleCount = (unsigned int)(int)((float)desc.CSD * info.TimeStepSize);
        info.MonteCarloFactor = std::asin(info.NeighborParticleRadius / info.ParticleRadius);
    }
    // DFSPHImplementation.cu:334-367
    void init(const vfd_desc& d) {
        desc = d;
        info.ParticleRadius = d.ParticleRadius;
        info.ParticleDiameter = 2.0f * info.ParticleRadius;
        info.SupportRadius = 4.0f * info.ParticleRadius;
        info.SupportRadius2 = info.SupportRadius * info.SupportRadius;
        info.Volume = 0.8f * info.ParticleDiameter * info.ParticleDiameter * info.ParticleDiameter;
        info.Density0 = 1000.0f;
        info.ParticleMass = info.Volume * info.Density0;
        info.ParticleMassInverse = 1.0f / info.ParticleMass;
        info.Viscosity = d.Viscosity;
        info.BoundaryViscosity = d.BoundaryViscosity;
        info.DynamicViscosity = info.Viscosity * info.Density0;
        info.DynamicBoundaryViscosity = info.BoundaryViscosity * info.Density0;
        info.TangentialDistanceFactor = d.TangentialDistanceFactor;
        info.TangentialDistance = info.TangentialDistanceFactor * info.SupportRadius;
        set_dt(d.TimeStepSize);
        info.SurfaceTension = d.SurfaceTension;
        info.ClassifierSlope = 74.688796680497925f;
        info.ClassifierConstant = 12.0f;
        info.TemporalSmoothing = d.TemporalSmoothing != 0;
        info.SmoothingFactor = 0.5f;
        info.Factor = 0.8f;
        info.NeighborParticleRadius = info.ParticleRadius * info.Factor;
        info.Gravity = glm::vec3(d.Gravity[0], d.Gravity[1], d.Gravity[2]);
        update_samples();
        kernel = new vfd::PrecomputedDFSPHCubicKernel();
        kernel->SetRadius(info.SupportRadius);
    }
    // :185-222, one fluid object per particle's own velocity
    void set_fluid(const float* x, const float* v, uint32_t count) {
        p.assign(count, DFSPHParticle{});
        for (uint32_t i = 0; i < count; i++) {
            std::memset(&p[i], 0, sizeof(DFSPHParticle));
            p[i].Position = glm::vec3(x[3 * i], x[3 * i + 1], x[3 * i + 2]);
            if (v) p[i].Velocity = glm::vec3(v[3 * i], v[3 * i + 1], v[3 * i + 2]);
        }
        info.ParticleCount = count;
        for (Body* bd : bodies) {
            bd->xj.assign(count, glm::vec3());
            bd->volume.assign(count, 0.0f);
            bd->dev.BoundaryXJ = bd->xj.data();
            bd->dev.BoundaryVolume = bd->volume.data();
        }
        precond.assign(count, glm::mat3x3());
        for (auto* a : {&b, &g, &r, &d, &z, &ad}) a->assign(count, glm::vec3());
    }
    void add_body(const vfd_volume_map& m) {
        Body* bd = new Body();
        const size_t nn = (size_t)m.field_count * m.node_count;
        const size_t nc = (size_t)m.field_count * m.cell_count * 32u;
        const size_t nm = (size_t)m.field_count * m.cell_map_count;
        bd->nodes.assign(m.nodes, m.nodes + nn);
        bd->cells.assign(m.cells, m.cells + nc);
        bd->cellMap.assign(m.cell_map, m.cell_map + nm);
        bd->map = m;
        bd->map.nodes = bd->nodes.data();
        bd->map.cells = bd->cells.data();
        bd->map.cell_map = bd->cellMap.data();
        vfd::SDF::Bind(bd->sdf, bd->map);
        bd->dev.Map = &bd->sdf;
        bodies.push_back(bd);
        bodyPtrs.push_back(&bd->dev);
        info.RigidBodyCount = (unsigned int)bodies.size();
        set_fluid_arrays_for(bd);
    }
    void set_fluid_arrays_for(Body* bd) {
        bd->xj.assign(n(), glm::vec3());
        bd->volume.assign(n(), 0.0f);
        bd->dev.BoundaryXJ = bd->xj.data();
        bd->dev.BoundaryVolume = bd->volume.data();
    }

    int search() {
        const uint32_t N = n();
        std::vector<float> xyz(3 * (size_t)N);
        for (uint32_t i = 0; i < N; i++) {
            xyz[3 * i] = p[i].Position.x;
            xyz[3 * i + 1] = p[i].Position.y;
            xyz[3 * i + 2] = p[i].Position.z;
        }
        counts.assign(N, 0u);
        offsets.assign(N, 0u);
        uint32_t total = 0;
        int rc = ref_find_neighbors(xyz.data(), N, info.SupportRadius, counts.data(), offsets.data(), nullptr, 0,
                                    &total, nullptr, nullptr);
        if (rc) return rc;
        list.assign(std::max<uint32_t>(total, 1u), 0u);
        rc = ref_find_neighbors(xyz.data(), N, info.SupportRadius, counts.data(), offsets.data(), list.data(),
                                (uint32_t)list.size(), &total, nullptr, nullptr);
        if (rc) return rc;
        vfd::ParticleSearch::Bind(set, counts.data(), offsets.data(), list.data());
        uint32_t mx = 0;
        for (uint32_t c : counts) mx = std::max(mx, c);
        last.MaxNeighborCount = mx;
        return 0;
    }

    // The solver error of a Jacobi loop: -rho0 * sum(residuum) / N.
    float density_error() const {
        double s = 0.0;
        for (const DFSPHParticle& q : p) s += (double)q.PressureResiduum;
        return (float)(-(double)info.Density0 * s / (double)n());
    }

    // ComputeDivergence (:511-575)
    void divergence() {
        const uint32_t N = n();
        last.DivergenceSolverError = 0.0f;
        last.DivergenceSolverIterationCount = 0u;
        if (!desc.EnableDivergenceSolverError) return;
        vfd::DFSPHParticle* P = p.data();
        launch(N, [&] { ComputeDensityChangeKernel(P, &info, &set, rb(), kernel); });
        const float eta = info.TimeStepSizeInverse * desc.MaxDivergenceSolverError * 0.0001f * info.Density0;
        float err = 0.0f;
        uint32_t it = 0;
        while ((err > eta || it < desc.MinDivergenceSolverIterations) && it < desc.MaxDivergenceSolverIterations) {
            launch(N, [&] { ComputePressureAccelerationAndDivergenceKernel(P, &info, &set, rb(), kernel); });
            launch(N, [&] { DivergenceSolveIterationKernel(P, &info, &set, rb(), kernel); });
            err = density_error();
            it++;
        }
        last.DivergenceSolverError = err;
        last.DivergenceSolverIterationCount = it;
        launch(N, [&] { ComputePressureAccelerationAndFactorKernel(P, &info, &set, rb(), kernel); });
    }

    // ComputePressure (:443-509)
    void pressure() {
        const uint32_t N = n();
        vfd::DFSPHParticle* P = p.data();
        launch(N, [&] { ComputeDensityAdvectionKernel(P, &info, &set, rb(), kernel); });
        const float eta = desc.MaxPressureSolverError * 0.0001f * info.Density0;
        float err = 0.0f;
        uint32_t it = 0;
        while ((err > eta || it < desc.MinPressureSolverIterations) && it < desc.MaxPressureSolverIterations) {
            launch(N, [&] { ComputePressureAccelerationKernel(P, &info, &set, rb(), kernel); });
            launch(N, [&] { PressureSolveIterationKernel(P, &info, &set, rb(), kernel); });
            err = density_error();
            it++;
        }
        last.PressureSolverError = err;
        last.PressureSolverIterationCount = it;
        launch(N, [&] { ComputePressureAccelerationAndVelocityKernel(P, &info, &set, rb(), kernel); });
    }

    static double dot_sum(const std::vector<glm::vec3>& a, const std::vector<glm::vec3>& c) {
        double s = 0.0;
        for (size_t i = 0; i < a.size(); i++) s += (double)glm::compAdd(a[i] * c[i]);
        return s;
    }

    // ComputeViscosity / SolveViscosity (:577-805)
    void viscosity() {
        const uint32_t N = n();
        last.ViscositySolverError = 0.0f;
        last.ViscositySolverIterationCount = 0u;
        if (!desc.EnableViscositySolver) return;
        vfd::DFSPHParticle* P = p.data();
        launch(N, [&] { ComputeViscosityPreconditionerKernel(P, &info, &set, rb(), kernel, precond.data()); });
        launch(N, [&] { ComputeViscosityGradientKernel(P, &info, rb(), kernel, b.data(), g.data()); });
        solve();
        launch(N, [&] { ApplyViscosityForceKernel(P, &info, g.data()); });
    }
    void matvec(std::vector<glm::vec3>& in, std::vector<glm::vec3>& out) {
        vfd::DFSPHParticle* P = p.data();
        launch(n(), [&] { ComputeMatrixVecProdFunctionKernel(P, &info, &set, rb(), kernel, in.data(), out.data()); });
    }
    void solve() {
        const uint32_t N = n();
        uint32_t it = 0;
        matvec(g, ad);
        for (uint32_t i = 0; i < N; i++) r[i] = b[i] - ad[i];
        const double rhs = dot_sum(b, b);
        if (rhs == 0.0) {
            for (auto& e : g) e = glm::vec3();
            last.ViscositySolverError = 0.0f;
            return;
        }
        const double e = (double)desc.MaxViscositySolverError;
        const double thr = std::max(e * e * 0.0001 * rhs, (double)FLT_MIN);
        double rr = dot_sum(r, r);
        if (rr < thr) {
            last.ViscositySolverError = (float)std::sqrt(rr / rhs);
            return;
        }
        for (uint32_t i = 0; i < N; i++) d[i] = precond[i] * r[i];
        double absNew = std::fabs(dot_sum(r, d));
        while (it >= desc.MinViscositySolverIterations && it < desc.MaxViscositySolverIterations) {
            matvec(d, ad);
            const float alpha = (float)(absNew / dot_sum(d, ad));
            for (uint32_t i = 0; i < N; i++) g[i] = g[i] + d[i] * alpha;
            for (uint32_t i = 0; i < N; i++) r[i] = r[i] - ad[i] * alpha;
            rr = dot_sum(r, r);
            if (rr < thr) break;
            for (uint32_t i = 0; i < N; i++) z[i] = precond[i] * r[i];
            const double absOld = absNew;
            absNew = std::fabs(dot_sum(r, z));
            const float beta = (float)(absNew / absOld);
            for (uint32_t i = 0; i < N; i++) d[i] = d[i] * beta + z[i];
            it++;
        }
        last.ViscositySolverIterationCount = it;
        last.ViscositySolverError = (float)std::sqrt(rr / rhs);
    }

    // SolveSurfaceTension (:807-838)
    void surface_tension() {
        if (!desc.EnableSurfaceTensionSolver) return;
        const uint32_t N = n();
        vfd::DFSPHParticle* P = p.data();
        launch(N, [&] { ComputeSurfaceTensionClassificationKernel(P, &info, &set); });
        launch(N, [&] { ComputeSurfaceTensionNormalsAndCurvatureKernel(P, &info, &set); });
        for (uint32_t k = 0; k < desc.SurfaceTensionSmoothPassCount; k++)
            launch(N, [&] { ComputeSurfaceTensionBlendingKernel(P, &info); });
    }

    // ComputeTimeStepSize (:395-441): the CFL maximum of |v + a dt|^2 from 0.1.
    void time_step() {
        float m = 0.1f;
        for (const DFSPHParticle& q : p) m = std::max(m, glm::length2(q.Velocity + q.Acceleration * info.TimeStepSize));
        maxV2 = m < 1.0e-9f ? 1.0e-9f : m;
        float dt = 0.4f * (info.ParticleDiameter / std::sqrt(maxV2));
        dt = std::min(dt, desc.MaxTimeStepSize);
        dt = std::max(dt, desc.MinTimeStepSize);
        set_dt(dt);
        update_samples();
    }

    // OnUpdate (:63-170)
    int step(vfd_step_stats* st) {
        const uint32_t N = n();
        if (N == 0) return 0;
        last = vfd_step_stats{};
        last.SurfaceTensionSampleCount = info.SurfaceTensionSampleCount;
        if (int rc = search()) return rc;
        vfd::DFSPHParticle* P = p.data();
        launch(N, [&] { ComputeVolumeAndBoundaryKernel(P, &info, rb()); });
        launch(N, [&] { ComputeDensityKernel(P, &info, &set, rb(), kernel); });
        launch(N, [&] { ComputeDFSPHFactorKernel(P, &info, &set, rb(), kernel); });
        divergence();
        launch(N, [&] { ClearAccelerationKernel(P, &info); });
        surface_tension();
        viscosity();
        time_step();
        launch(N, [&] { ComputeVelocityKernel(P, &info); });
        pressure();
        launch(N, [&] { ComputePositionKernel(P, &info); });
        last.TimeStepSize = info.TimeStepSize;
        last.MaxVelocityMagnitude = maxV2;
        if (st) *st = last;
        return 0;
    }
};

}  // namespace

extern "C" {

void* ref_step_create(const vfd_desc* d) {
    if (!d) return nullptr;
    RefSim* s = new (std::nothrow) RefSim();
    if (s) s->init(*d);
    return s;
}
void ref_step_destroy(void* h) { delete static_cast<RefSim*>(h); }
int ref_step_add_rigid_body(void* h, const vfd_volume_map* m) {
    if (!h || !m) return 1;
    static_cast<RefSim*>(h)->add_body(*m);
    return 0;
}
int ref_step_set_fluid(void* h, const float* x, const float* v, uint32_t n) {
    if (!h || (n && !x)) return 1;
    static_cast<RefSim*>(h)->set_fluid(x, v, n);
    return 0;
}
int ref_step_step(void* h, vfd_step_stats* st) { return h ? static_cast<RefSim*>(h)->step(st) : 1; }
// Positions, velocities, accelerations (3 floats per particle, may be null), densities and
// DFSPH factors (1 float per particle, may be null) of the last step, original order.
int ref_step_get_state(void* h, float* x, float* v, float* a, float* rho, float* factor) {
    if (!h) return 1;
    const RefSim* s = static_cast<RefSim*>(h);
    for (uint32_t i = 0; i < s->n(); i++) {
        const DFSPHParticle& q = s->p[i];
        if (x) { x[3 * i] = q.Position.x; x[3 * i + 1] = q.Position.y; x[3 * i + 2] = q.Position.z; }
        if (v) { v[3 * i] = q.Velocity.x; v[3 * i + 1] = q.Velocity.y; v[3 * i + 2] = q.Velocity.z; }
        if (a) { a[3 * i] = q.Acceleration.x; a[3 * i + 1] = q.Acceleration.y; a[3 * i + 2] = q.Acceleration.z; }
        if (rho) rho[i] = q.Density;
        if (factor) factor[i] = q.Factor;
    }
    return 0;
}

}  // extern "C"
