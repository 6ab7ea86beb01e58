/*
 * vfd_sph.h -- C-ABI of the GB300 legacy SPH pipeline.
 *
 * The reference's earlier solver, vfd::SPHSimulation (Simulation/SPH/SPHSimulation.h:55-142,
 * SPHSimulation.cpp, SPHSimulation.cu, SPHSimulationKernel.cu): weakly compressible SPH
 * with poly6 density, spiky pressure and Laplacian viscosity forces over a uniform hash
 * grid of cell edge 2r, penalty walls of an axis-aligned world box, and a fixed time step.
 * Each entry point names the reference interface it replaces. Positions and velocities
 * are float4 in the reference; here they cross the boundary as xyz triples in the
 * caller's particle order. Status codes are those of vfd_dfsph.h.
 */
#ifndef VFD_SPH_H
#define VFD_SPH_H

#include <stdint.h>

#include "vfd_dfsph.h"

#ifdef __cplusplus
extern "C" {
#endif

/* SPHSimulationDescription (SPHSimulation.h:15-31) without the particle volumes, which
 * arrive as positions (ParticleSampler / vfd_sample_mesh_volume makes them). */
typedef struct vfd_sph_desc {
    float ParticleRadius;
    float Homogeneity;             /* support radius h */
    float RestDensity;
    float Stiffness;
    float Viscosity;
    float TimeStep;
    float GlobalDamping;
    float BoundsStiffness;
    float BoundsDamping;
    float BoundsDampingCritical;
    uint32_t MaxParticlesInCellCount;
    uint32_t StepCount;            /* steps per OnUpdate */
    float Gravity[3];
    float WorldMin[3];
    float WorldMax[3];
} vfd_sph_desc;

/* SPHSimulationParameters (SPHSimulationParameters.cuh:7-45): the derived constants. */
typedef struct vfd_sph_params {
    float SmoothingRadius;         /* h^2 */
    float Poly6Kern, SpikyKern, LapKern;
    float ParticleMass, MinDens, MinDist;
    float BoundsSoftDistance, BoundsHardDistance;
    float CellSize;
    uint32_t GridSize[3];
    uint32_t CellCount;
    uint32_t ParticleCount;
} vfd_sph_params;

typedef struct vfd_sph vfd_sph;

/* SPHSimulation::SPHSimulation (SPHSimulation.cpp:10-64): n particles at rest. */
int vfd_sph_create(const vfd_sph_desc* desc, const float* xyz, uint32_t n, vfd_sph** out);
void vfd_sph_destroy(vfd_sph* sim);

/* SPHSimulation::OnUpdate (SPHSimulation.cpp:71-95): StepCount steps of integrate, hash,
 * sort, reorder, density and force. */
int vfd_sph_on_update(vfd_sph* sim);
/* `count` steps (OnUpdate with StepCount = count). */
int vfd_sph_steps(vfd_sph* sim, uint32_t count);

/* SPHSimulation::Reset (SPHSimulation.cpp:97-114): back to the initial positions, at rest
 * (the reference re-creates its zeroed velocity mirror). */
int vfd_sph_reset(vfd_sph* sim);

/* SPHSimulation::UpdateDescription (SPHSimulation.cpp:216-240): new parameters, same particles. */
int vfd_sph_update_description(vfd_sph* sim, const vfd_sph_desc* desc);

/* GetParameters / GetParticleCount (SPHSimulation.h:70-84). */
int vfd_sph_get_params(const vfd_sph* sim, vfd_sph_params* out);

/* State in the caller's order: positions and velocities (xyz), and the density and
 * pressure of the last step (the reference keeps those in cell order; these are mapped
 * back). Any pointer may be NULL. */
int vfd_sph_get_state(vfd_sph* sim, float* xyz, float* vel, float* density, float* pressure);
/* Velocities (xyz) in the caller's order: the reference's SetArray(1, ...) (SPHSimulation.cpp:256-274). */
int vfd_sph_set_velocities(vfd_sph* sim, const float* vel);

/* Cell key and in-cell order of the last step's sort, in sorted order: key of each
 * sorted slot and the caller's index stored there (parity hook, the reference's
 * particleHash pairs after RadixSort). */
int vfd_sph_get_sort(vfd_sph* sim, uint32_t* keys, uint32_t* indices);

#ifdef __cplusplus
}
#endif

#endif /* VFD_SPH_H */
