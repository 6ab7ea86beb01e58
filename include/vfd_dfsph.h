/*
 * vfd_dfsph.h -- C-ABI of the GB300-native DFSPH simulation step.
 *
 * This is the drop-in boundary for VFD's DFSPH solver API. Each entry point
 * names the reference interface it replaces (paths are relative to the VFD
 * source tree, VFD/Source/...). Signatures use plain C types only: no CUDA,
 * torch or C++ types cross this boundary.
 *
 * Threading: one handle per host thread; calls on a handle are synchronous
 * with respect to the host unless the name says otherwise (vfd_steps_async).
 * Errors: every call returns a VFD_* status code. The library never exits,
 * traps or hangs; vfd_last_error() returns a message for the calling thread.
 *
 * Particle order: every host-side array passed in or out is in the caller's
 * original particle order (the order given to vfd_set_fluid), which is the
 * reference's particle index. Internally particles are kept sorted by cell.
 */
#ifndef VFD_DFSPH_H
#define VFD_DFSPH_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VFD_ABI_VERSION 1

/* Status codes (replace COMPUTE_SAFE -> exit(), Debug/Debug.h:107). */
enum {
    VFD_OK = 0,
    VFD_E_ARG = 1,           /* invalid argument or handle                  */
    VFD_E_CUDA = 2,          /* a CUDA runtime call failed                   */
    VFD_E_NONCONVERGED = 3,  /* a solver hit its iteration cap (flag only)   */
    VFD_E_NAN = 4,           /* non-finite particle state detected           */
    VFD_E_CAPACITY = 5,      /* grid or buffer capacity exceeded             */
    VFD_E_STATE = 6,         /* call not valid in the current state          */
    VFD_E_NOMEM = 7,         /* device or host allocation failed             */
    VFD_E_NODEVICE = 8       /* no CUDA device                               */
};

/* Bits of vfd_step_stats.Flags. */
#define VFD_FLAG_PRESSURE_CAP    0x1u  /* pressure solve stopped at its max iterations   */
#define VFD_FLAG_DIVERGENCE_CAP  0x2u  /* divergence solve stopped at its max iterations */
#define VFD_FLAG_VISCOSITY_CAP   0x4u  /* viscosity CG stopped at its max iterations     */
#define VFD_FLAG_NEIGHBOR_CAP    0x8u  /* some particle reached the 70-neighbour cap     */
#define VFD_FLAG_NAN             0x10u /* non-finite position or velocity                */
#define VFD_FLAG_GRID_CAPACITY   0x20u /* search grid larger than the cell table         */
#define VFD_FLAG_ANCHOR_RANGE    0x40u /* cell-relative positions left their anchor range */
#define VFD_FLAG_BOUNDS          0x80u /* bounds-checked build only: a device index check failed */

/* Position storage modes (vfd_set_position_mode). */
#define VFD_POSITIONS_ABSOLUTE       0  /* FP32 absolute coordinates, as the reference stores them */
#define VFD_POSITIONS_CELL_RELATIVE  1  /* FP32 offsets within anchor cells of edge h             */

/* Arithmetic of the step (vfd_set_precision). */
#define VFD_PRECISION_FP32  0  /* FP32 state and neighbour sums, FP64 reductions (the default) */
#define VFD_PRECISION_FP64  1  /* the whole step in FP64 on the GPU (a reference trajectory)   */

/* SPH kernel evaluation modes (vfd_set_kernel_mode). */
#define VFD_KERNEL_TABLE     0  /* midpoint of two 10000-entry table values, as the reference */
#define VFD_KERNEL_ANALYTIC  1  /* the cubic spline evaluated at |r| (smooth in r)            */

/* Maximum neighbours per particle, ParticleSearchKernels.cuh:7 (CUDA_MAX_NEIGHBORS). */
#define VFD_MAX_NEIGHBORS 70u

/*
 * User parameters. Field for field the reference's DFSPHSimulationDescription
 * (Simulation/DFSPH/Structures/DFSPHSimulationDescription.h:9-49), with bool
 * fields widened to int32 so the layout is plain C.
 */
typedef struct vfd_desc {
    float TimeStepSize;
    float MinTimeStepSize;
    float MaxTimeStepSize;
    float FrameLength;
    uint32_t FrameCount;

    uint32_t MinPressureSolverIterations;
    uint32_t MaxPressureSolverIterations;
    float MaxPressureSolverError;          /* [%] of rest density x 100 */

    int32_t EnableDivergenceSolverError;
    uint32_t MinDivergenceSolverIterations;
    uint32_t MaxDivergenceSolverIterations;
    float MaxDivergenceSolverError;

    int32_t EnableViscositySolver;
    uint32_t MinViscositySolverIterations;
    uint32_t MaxViscositySolverIterations;
    float MaxViscositySolverError;
    float Viscosity;                       /* kinematic; dynamic = Viscosity * 1000 */
    float BoundaryViscosity;
    float TangentialDistanceFactor;

    int32_t EnableSurfaceTensionSolver;
    uint32_t SurfaceTensionSmoothPassCount;
    float SurfaceTension;
    int32_t TemporalSmoothing;
    int32_t CSDFix;                        /* sample count per step, <= 0 = use CSD */
    int32_t CSD;                           /* sample count per particle per second  */

    float ParticleRadius;
    float Gravity[3];
} vfd_desc;

/*
 * A rigid body's volume map, in the reference's SDFDeviceData layout
 * (Utility/SDF/SDFDeviceData.cuh:549-566): field 0 is the signed distance,
 * field 1 the boundary volume; cells hold 32 node indices per cell (cubic
 * serendipity element). Arrays are host memory and are copied by the call.
 */
typedef struct vfd_volume_map {
    const float* nodes;        /* field_count * node_count                    */
    const uint32_t* cells;     /* field_count * cell_count * 32               */
    const uint32_t* cell_map;  /* field_count * cell_map_count                */
    float domain_min[3];
    float domain_max[3];
    uint32_t resolution[3];
    float cell_size[3];
    float cell_size_inverse[3];
    uint32_t field_count;
    uint32_t node_count;
    uint32_t cell_count;
    uint32_t cell_map_count;
} vfd_volume_map;

/*
 * Per-step solver statistics: DFSPHDebugInfo (Structures/DFSPHDebugInfo.h:8-28)
 * without the wall-clock timers, plus the step size and search figures.
 */
typedef struct vfd_step_stats {
    uint32_t IterationCount;
    uint32_t DivergenceSolverIterationCount;
    uint32_t PressureSolverIterationCount;
    uint32_t ViscositySolverIterationCount;
    float DivergenceSolverError;
    float PressureSolverError;
    float ViscositySolverError;
    float FrameTime;
    uint32_t FrameIndex;
    float TimeStepSize;          /* dt used by the pressure solve of the step   */
    float MaxVelocityMagnitude;  /* squared, as GetMaxVelocityMagnitude()        */
    uint32_t MaxNeighborCount;
    uint32_t Flags;              /* VFD_FLAG_* of the step                        */
    uint32_t SurfaceTensionSampleCount;
} vfd_step_stats;

/* Derived constants: DFSPHSimulationInfo (Structures/DFSPHSimulationInfo.h:5-44). */
typedef struct vfd_info {
    uint32_t ParticleCount;
    uint32_t RigidBodyCount;
    float SupportRadius;
    float SupportRadius2;
    float ParticleRadius;
    float ParticleDiameter;
    float TimeStepSize;
    float TimeStepSize2;
    float TimeStepSizeInverse;
    float TimeStepSize2Inverse;
    float Volume;
    float Density0;
    float ParticleMass;
    float ParticleMassInverse;
    float Viscosity;
    float BoundaryViscosity;
    float DynamicViscosity;
    float DynamicBoundaryViscosity;
    float TangentialDistanceFactor;
    float TangentialDistance;
    float SurfaceTension;
    uint32_t SurfaceTensionSampleCount;
    float ClassifierSlope;
    float ClassifierConstant;
    int32_t TemporalSmoothing;
    float SmoothingFactor;
    float Factor;
    float NeighborParticleRadius;
    float MonteCarloFactor;
    float Gravity[3];
} vfd_info;

/* Per-particle fields readable with vfd_get_field (DFSPHParticle, Structures/DFSPHParticle.h:8-33). */
enum {
    VFD_FIELD_DENSITY = 0,              /* float    */
    VFD_FIELD_FACTOR = 1,               /* float    */
    VFD_FIELD_DENSITY_ADVECTION = 2,    /* float    */
    VFD_FIELD_PRESSURE_RHO2 = 3,        /* float    */
    VFD_FIELD_PRESSURE_RHO2_V = 4,      /* float    */
    VFD_FIELD_PRESSURE_RESIDUUM = 5,    /* float    */
    VFD_FIELD_PRESSURE_ACCELERATION = 6,/* float[3] */
    VFD_FIELD_VELOCITY_DIFFERENCE = 7,  /* float[3] */
    VFD_FIELD_SURFACE_NORMAL = 8,       /* float[3] MonteCarloSurfaceNormal       */
    VFD_FIELD_SURFACE_CURVATURE = 9,    /* float    MonteCarloSurfaceCurvature    */
    VFD_FIELD_DELTA_FINAL_CURVATURE = 10,/* float   */
    VFD_FIELD_BOUNDARY_XJ = 11,         /* float[3] of rigid body `body`          */
    VFD_FIELD_BOUNDARY_VOLUME = 12,     /* float    of rigid body `body`          */
    VFD_FIELD_SURFACE_NORMAL_SMOOTH = 13,   /* float[3] */
    VFD_FIELD_SURFACE_CURVATURE_SMOOTH = 14 /* float    */
};

typedef struct vfd_sim vfd_sim;

/* Fill `desc` with the reference defaults (DFSPHSimulationDescription.h:11-48). */
int vfd_desc_default(vfd_desc* desc);

/* DFSPHSimulation::DFSPHSimulation (DFSPHSimulator.cpp:10-18): device check + construct. */
int vfd_create(const vfd_desc* desc, vfd_sim** out);

/* DFSPHImplementation::~DFSPHImplementation (DFSPHImplementation.cu:23-31). */
int vfd_destroy(vfd_sim* sim);

/* DFSPHSimulation::SetDescription -> DFSPHImplementation::SetDescription (DFSPHImplementation.cu:318-368). */
int vfd_set_description(vfd_sim* sim, const vfd_desc* desc);

/* DFSPHSimulation::GetDescription (DFSPHSimulator.cpp:72-75). */
int vfd_get_description(const vfd_sim* sim, vfd_desc* desc);

/*
 * DFSPHImplementation::SetFluidObjects (DFSPHImplementation.cu:172-253): the
 * concatenated positions (xyz, n*3 floats) and velocities (n*3 floats, may be
 * NULL = zero) of all fluid objects become the initial state.
 */
int vfd_set_fluid(vfd_sim* sim, const float* xyz, const float* vel, uint32_t n);

/*
 * DFSPHImplementation::SetRigidBodies (DFSPHImplementation.cu:255-271), one
 * body per call, in the reference's order. Call after vfd_set_fluid.
 */
int vfd_add_rigid_body(vfd_sim* sim, const vfd_volume_map* map);

/* Removes all rigid bodies (SetRigidBodies with an empty vector). */
int vfd_clear_rigid_bodies(vfd_sim* sim);

/*
 * Builds the volume map of an axis-aligned box on the GPU, the work of
 * RigidBody::RigidBody (RigidBody.cu:10-72) for a box mesh: distance field
 * sign*(sd - (padding - r)) and the 16^3-point Gauss-Legendre volume field.
 * Outputs go to caller buffers sized by vfd_box_map_sizes.
 */
int vfd_box_map_sizes(const uint32_t resolution[3], uint32_t* node_count, uint32_t* cell_count);
int vfd_build_box_map(const float box_min[3], const float box_max[3], int32_t inverted,
                      float padding, const uint32_t resolution[3], float particle_radius,
                      float* nodes, uint32_t* cells, uint32_t* cell_map, vfd_volume_map* map_out);

/*
 * Builds the volume map of a closed triangle mesh on the GPU: RigidBody::RigidBody
 * (Simulation/DFSPH/RigidBody/RigidBody.cu:10-72) with the signed distance of
 * MeshDistance::SignedDistance (Utility/SDF/MeshDistance.cpp:187-228, angle-weighted
 * pseudo-normals, MeshDistance.cpp:27-55). `vertices` holds vertex_count xyz triples,
 * `triangles` triangle_count index triples (counter-clockwise seen from outside, as
 * the reference's EdgeMesh expects). `transform` is the body's 4x4 placement in
 * column-major order (glm's layout; RigidBodyDescription::Transform) or NULL for the
 * identity. Domain = bounds of the placed vertices +- (8h + padding - r); buffers as
 * for vfd_build_box_map (sized by vfd_box_map_sizes).
 */
int vfd_build_mesh_map(const float* vertices, uint32_t vertex_count, const uint32_t* triangles,
                       uint32_t triangle_count, const float* transform, int32_t inverted, float padding,
                       const uint32_t resolution[3], float particle_radius, float* nodes, uint32_t* cells,
                       uint32_t* cell_map, vfd_volume_map* map_out);

/* Lattice packings of ParticleSampler (Utility/Sampler/ParticleSampler.h:7-11). */
#define VFD_SAMPLE_MIN_DENSITY 0
#define VFD_SAMPLE_MEDIUM_DENSITY 1
#define VFD_SAMPLE_MAX_DENSITY 2

/*
 * Fluid particles filling a mesh volume: FluidObject::FluidObject
 * (Simulation/DFSPH/FluidObject/FluidObject.cpp:6-25) calling
 * ParticleSampler::SampleMeshVolume (Utility/Sampler/ParticleSampler.cpp:7-91). The mesh
 * is placed by `transform` (as in vfd_build_mesh_map), its signed-distance map of
 * `resolution` cells is built on the GPU (SDF::SDF, Utility/SDF/SDF.cu:16-36), and the
 * lattice points of the chosen packing with a negative distance are kept, in the
 * reference's order (z outer, then y, then x). `count` receives the number of samples;
 * min(count, capacity) xyz triples are written to `positions` unless it is NULL (call
 * once with NULL to size the buffer). VFD_E_CAPACITY when capacity < count (the first
 * `capacity` samples are still written) or the lattice exceeds 2^31 points.
 */
int vfd_sample_mesh_volume(const float* vertices, uint32_t vertex_count, const uint32_t* triangles,
                           uint32_t triangle_count, const float* transform, float particle_radius,
                           const uint32_t resolution[3], int32_t inverted, int32_t sample_mode,
                           float* positions, uint32_t capacity, uint32_t* count);

/*
 * DFSPHImplementation::Simulate (DFSPHImplementation.cu:33-61) preamble:
 * re-uploads the initial particles, resets dt, frame time and counters.
 */
int vfd_reset(vfd_sim* sim);

/* DFSPHImplementation::OnUpdate (DFSPHImplementation.cu:63-170): one step. stats may be NULL. */
int vfd_step(vfd_sim* sim, vfd_step_stats* stats);

/*
 * `count` OnUpdate steps launched back to back without host synchronisation
 * between them; waits for the last one. stats (may be NULL) is the last step's.
 */
int vfd_steps(vfd_sim* sim, uint32_t count, vfd_step_stats* stats);

/* Same as vfd_steps but returns without waiting; vfd_synchronize waits. */
int vfd_steps_async(vfd_sim* sim, uint32_t count);
int vfd_synchronize(vfd_sim* sim, vfd_step_stats* stats);

/* Frame callback for vfd_simulate: x, v, a are n*3 floats in original order, valid
 * until the callback returns (they point into pinned staging memory). */
typedef void (*vfd_frame_callback)(uint32_t frame_index, uint32_t n, const float* x,
                                   const float* v, const float* a, float max_velocity,
                                   float time_step, void* user);

/*
 * DFSPHImplementation::Simulate (DFSPHImplementation.cu:33-61) with the frame
 * capture of OnUpdate (:148-167): resets, then steps until FrameCount frames
 * were emitted; each frame is handed to `cb` (may be NULL), in order, on the
 * calling thread. Steps are queued ahead of the host and each frame is copied
 * to pinned memory on a second stream while the next steps run; the run ends
 * on the step that completed the last frame. Single-scene simulations only.
 */
int vfd_simulate(vfd_sim* sim, vfd_frame_callback cb, void* user);

/*
 * ConvertParticlesToBuffer (DFSPHKernels.cu:6-22) + the frame D2H copy
 * (DFSPHImplementation.cu:156-162): positions, velocities, accelerations in
 * original order; any pointer may be NULL.
 */
int vfd_get_state(vfd_sim* sim, float* x, float* v, float* a);

/* Overwrites positions and velocities (original order; vel may be NULL) of the running state;
 * VFD_E_NAN for non-finite input. */
int vfd_set_state(vfd_sim* sim, const float* x, const float* v);

/*
 * Checkpoint and resume of the carried state. The reference keeps no checkpoints
 * (its only state between steps is the DFSPHParticle array and DFSPHSimulationInfo:
 * x, v, the viscosity warm start Delta v (DFSPHKernels.cu:755,861), the temporal
 * curvature delta kappa (:1034) and dt, DFSPHImplementation.cu:395-428). vfd_checkpoint
 * writes those, the last accelerations and each scene's solver clock (dt, frame time
 * and index, iteration count, surface-tension sample count) into `buffer` as an opaque
 * image of vfd_checkpoint_size bytes. vfd_restore makes a simulation with the same
 * scenes, particle counts, position mode and kernel mode continue from such an image:
 * its next steps repeat the checkpointed run's bit for bit. The description's
 * constants stay those of the restoring simulation. VFD_E_STATE when the image does
 * not match the simulation, VFD_E_CAPACITY when the buffer is too small.
 */
int vfd_checkpoint_size(vfd_sim* sim, uint64_t* bytes);
int vfd_checkpoint(vfd_sim* sim, void* buffer, uint64_t bytes);
int vfd_restore(vfd_sim* sim, const void* buffer, uint64_t bytes);

/* One per-particle field (VFD_FIELD_*) of the last step, original order. */
int vfd_get_field(vfd_sim* sim, int32_t field, uint32_t body, float* out);

/* ParticleSearch::FindNeighbors (ParticleSearch.h:80-93) on the current positions, without stepping. */
int vfd_find_neighbors(vfd_sim* sim);

/*
 * The last neighbour search (NeighborSet, NeighborSet.h:8-28, and
 * ParticleSearch::GetSortIndices, ParticleSearch.h:76-78), in the reference's
 * index space: counts[n], offsets[n] (exclusive scan), list[capacity]
 * (original indices, CSR), sort_indices[n] (sorted slot -> original index),
 * cell_keys[n] (Morton meta-grid cell of each particle). *total receives the
 * list length; VFD_E_CAPACITY if it exceeds `capacity`. Pointers may be NULL.
 */
int vfd_get_neighbors(vfd_sim* sim, uint32_t* counts, uint32_t* offsets, uint32_t* list,
                      uint32_t capacity, uint32_t* total, uint32_t* sort_indices,
                      uint32_t* cell_keys);

/* Getters of DFSPHSimulation (DFSPHSimulator.h:24-37). */
int vfd_get_info(const vfd_sim* sim, vfd_info* info);
int vfd_get_particle_count(const vfd_sim* sim, uint32_t* n);
int vfd_get_current_time_step_size(vfd_sim* sim, float* dt);
int vfd_get_max_velocity_magnitude(vfd_sim* sim, float* v2);
int vfd_get_debug_info(vfd_sim* sim, vfd_step_stats* stats);

/*
 * The SPH kernel table (PrecomputedDFSPHCubicKernel, Kernel/DFSPHKernels.h:8-143):
 * w[10000] and grad_w[10001] as built by SetRadius(4r), plus radius and W(0).
 */
int vfd_get_kernel_table(const vfd_sim* sim, float* w, float* grad_w, float* radius, float* w_zero);

/*
 * Solver execution mode: 1 (default) = the whole step is one CUDA graph with
 * device-side while loops for the three solvers; 0 = kernels launched from the
 * host with one flag read per solver iteration (the reference's control flow).
 */
int vfd_set_graph_mode(vfd_sim* sim, int32_t enabled);
/* Whether graphs are requested, and whether the steps so far ran from them (0 when the
 * step graph could not be built and the same kernels were launched from the host). */
int vfd_get_graph_mode(const vfd_sim* sim, int32_t* requested, int32_t* active);

/* Batched scenes: independent scenes advanced together, one launch per stage.
 * vfd_create_batch takes one description per scene (same ParticleRadius for all);
 * scene-scoped calls address one scene. The plain calls act on scene 0. */
int vfd_create_batch(const vfd_desc* descs, uint32_t scene_count, vfd_sim** out);
int vfd_get_scene_count(const vfd_sim* sim, uint32_t* scenes);
int vfd_scene_set_fluid(vfd_sim* sim, uint32_t scene, const float* xyz, const float* vel, uint32_t n);
int vfd_scene_add_rigid_body(vfd_sim* sim, uint32_t scene, const vfd_volume_map* map);
int vfd_scene_get_state(vfd_sim* sim, uint32_t scene, float* x, float* v, float* a);
int vfd_scene_get_stats(vfd_sim* sim, uint32_t scene, vfd_step_stats* stats);

/* Per-kernel time of eagerly launched steps (CUDA events on the launch stream). */
typedef struct vfd_kernel_time {
    char name[48];
    uint32_t launches;
    double total_ms;
} vfd_kernel_time;

/*
 * Runs `steps` steps with every kernel launched from the host and bracketed by
 * CUDA events, and reports each kernel's launch count and summed time (no
 * counterpart in the reference, whose DFSPHDebugInfo timers are host wall
 * clocks around synchronised phases, Structures/DFSPHDebugInfo.h:10-15).
 */
int vfd_profile_kernels(vfd_sim* sim, uint32_t steps, vfd_kernel_time* out, uint32_t capacity, uint32_t* count);

/*
 * Lanes per particle (4, 8 or 16) of the neighbour-loop kernels, in the order
 * density+factor (with the density change when the divergence solve runs), pressure
 * acceleration, Jacobi iteration,
 * divergence finish, surface classification, surface smoothing, viscosity
 * preconditioner, viscosity setup, CG matrix-vector product, density advection,
 * pressure finish (no counterpart in the reference, which launches every kernel
 * with 256 threads, one per particle). The neighbour search runs a warp per cell.
 */
int vfd_set_lanes(vfd_sim* sim, const uint8_t* lanes, uint32_t count);
int vfd_get_lanes(const vfd_sim* sim, uint8_t* lanes, uint32_t count);

/*
 * Form of the solver-loop kernels (pressure acceleration, Jacobi update, CG
 * matrix-vector product), in the order of vfd_set_lanes (the other entries are
 * ignored): 0 (the default) = the pass walks each particle's neighbour row and gathers
 * from global memory, as the reference's kernels do (DFSPHKernels.cu:317-432,
 * :758-842), reading each pair's gradW / r from the stream the density pass wrote;
 * 1 = the same walk over the slot rows alone, forming gradW / r from the kernel table
 * per pair (half the streamed bytes, a table lookup per pair; single scenes); 3 or 4 =
 * log2 of the cells per tile (a 2x2x2 or 4x2x2 block of cells): a block stages the
 * tile's halo of cells in shared memory and walks its particles' neighbours there. All
 * give the same results to rounding. vfd_autotune picks them with the lanes.
 */
int vfd_set_tiles(vfd_sim* sim, const uint8_t* tiles, uint32_t count);
int vfd_get_tiles(const vfd_sim* sim, uint8_t* tiles, uint32_t count);

/*
 * Threads per block (64, 128 = the default, or 256) of the neighbour-row kernels, in the
 * order of vfd_set_lanes. No counterpart in the reference, which launches 256 threads
 * (ComputeHelper.cpp:18). vfd_autotune picks them with the lanes and tiles.
 */
int vfd_set_blocks(vfd_sim* sim, const uint16_t* blocks, uint32_t count);
int vfd_get_blocks(const vfd_sim* sim, uint16_t* blocks, uint32_t count);

/*
 * Autotuner: runs `steps` steps from a snapshot of the current state once per
 * lane count, tile size and block size, times every neighbour-loop kernel with CUDA events,
 * keeps the fastest lane count (and tile size, vfd_set_tiles, and block size,
 * vfd_set_blocks) per kernel and restores the state exactly (positions,
 * velocities, accelerations and all carried solver state; the simulation does not
 * advance). Per-step diagnostics (vfd_get_field, vfd_get_neighbors) reflect the
 * last tuning step until the next step. lanes_out (may be NULL) receives the choice.
 */
int vfd_autotune(vfd_sim* sim, uint32_t steps, uint8_t* lanes_out, uint32_t count);

/* The cudaStream_t all work of `sim` is issued on (for events recorded by the caller). */
int vfd_get_stream(vfd_sim* sim, void** stream);

/* Number of kernel launches executed since creation (or the last reset), counted on the device. */
int vfd_get_launch_count(vfd_sim* sim, uint64_t* launches, int32_t reset);

/*
 * Neighbour search that allocates nothing. No counterpart in the reference.
 * For callers that cannot call cudaMalloc: code whose device memory belongs to
 * another allocator with a fixed budget, and code that must not allocate once it
 * runs. Inputs and outputs are the caller's device buffers: xyz (n*3 floats),
 * counts (n), neighbors (n * VFD_MAX_NEIGHBORS; row i holds particle i's neighbours in
 * the reference's order, original indices), sort_indices (n; sorted slot -> original
 * index). Intermediate data lives in a fixed ~10 MB __device__ array that every GPU
 * loading the library keeps until exit; limits: n <= 16384 and a search grid of at most
 * 262144 cells, else VFD_E_CAPACITY. The first call on a device looks the array up
 * (cudaGetSymbolAddress, once per CUDA context) and should come before any stream
 * capture. All calls share the array: calls that overlap on the GPU race and must be
 * serialised by the caller. Runs on `stream` (a cudaStream_t, NULL = default) and waits
 * for it before returning the status. Errors: return code only.
 */
int vfd_find_neighbors_noalloc(const float* xyz, uint32_t n, float particle_radius, uint32_t* counts,
                               uint32_t* neighbors, uint32_t* sort_indices, void* stream);

/*
 * Adjoint of the step. No counterpart in the reference (its step is not
 * differentiable code). vfd_adjoint_forward runs `steps` OnUpdate steps from the
 * current state like vfd_steps, keeping a checkpoint of the carried state every
 * `checkpoint_every` steps. vfd_adjoint_backward then takes the cotangents of the
 * final positions and velocities (x_bar, v_bar: n*3 floats, original order) and
 * returns those of the initial positions and velocities (x0_bar, v0_bar; either may
 * be NULL) and param_bar[0] = d/d Viscosity, param_bar[1] = d/d BoundaryViscosity
 * (may be NULL). It re-runs each segment from its checkpoint, recording neighbour
 * rows and solver iterates, and leaves the simulation at the end of the forward run.
 * Per step the neighbour sets, solver iteration counts and clamp decisions are those
 * of the forward run; the viscosity solve is differentiated at its converged
 * solution (a second CG solve with the same tolerance). Requires one scene, surface
 * tension off and no particle at the 70-neighbour cap (VFD_E_ARG / VFD_E_CAPACITY);
 * VFD_E_STATE if the simulation was reset after vfd_adjoint_forward.
 */
int vfd_adjoint_forward(vfd_sim* sim, uint32_t steps, uint32_t checkpoint_every, vfd_step_stats* stats);
int vfd_adjoint_backward(vfd_sim* sim, const float* x_bar, const float* v_bar, float* x0_bar, float* v0_bar,
                         float* param_bar);
/* Frees the checkpoints and tapes of the recorded run. */
int vfd_adjoint_release(vfd_sim* sim);

/*
 * Initial guess of each backward step's viscosity solve A lambda = g_bar (the steps
 * are walked from the last to the first): VFD_WARM_COLD starts from g_bar;
 * VFD_WARM_PREVIOUS (default) from the lambda of the step after; VFD_WARM_EXTRAPOLATE
 * from 2 lambda(t+1) - lambda(t+2), the linear extrapolation of the last two solutions,
 * once two exist. Every choice stops at the same residual; they differ in iteration count
 * and in the error left in lambda (the residual bounds it loosely, see
 * vfd_adjoint_set_tolerance): the previous solution carries the components of lambda that
 * change slowly from step to step, which the CG resolves last. No counterpart in the
 * reference.
 */
#define VFD_WARM_COLD 0
#define VFD_WARM_PREVIOUS 1
#define VFD_WARM_EXTRAPOLATE 2
int vfd_adjoint_set_warm_start(vfd_sim* sim, int32_t mode);

/*
 * Tolerance of the backward viscosity solves relative to the forward's: they stop at a
 * relative residual of `factor` x (MaxViscositySolverError / 100), factor in (0, 1],
 * default 1. The cotangent g_bar of a viscous step can be dominated by components the
 * viscosity damps, so that lambda = A^-1 g_bar is much smaller than g_bar and a residual
 * relative to g_bar bounds lambda's relative error only loosely; a smaller factor buys
 * gradient accuracy with iterations. No counterpart in the reference.
 */
int vfd_adjoint_set_tolerance(vfd_sim* sim, float factor);

/* Counters of the last vfd_adjoint_backward. */
typedef struct vfd_adjoint_stats {
    uint32_t Steps;                      /* steps differentiated                          */
    uint32_t ReplayedSteps;              /* steps re-run from checkpoints                 */
    uint32_t ViscositySolves;            /* adjoint viscosity solves                      */
    uint32_t ViscositySolverIterations;  /* their CG iterations, summed                   */
    uint32_t MaxViscositySolverIterations;
} vfd_adjoint_stats;
int vfd_adjoint_get_stats(vfd_sim* sim, vfd_adjoint_stats* stats);

/*
 * Position storage. No counterpart in the reference, which stores absolute FP32
 * coordinates (VFD_POSITIONS_ABSOLUTE, the default). VFD_POSITIONS_CELL_RELATIVE stores
 * each position as its FP32 offset within an anchor cell (a cube of edge h, the support
 * radius, at integer coordinates from the cell nearest the centre of the scene's initial
 * positions, at most 511 cells away); every pair vector x_i - x_j is then formed from
 * offsets and cell differences, so its rounding error scales with h instead of with the
 * distance from the origin. Inputs and outputs stay absolute. Changing the mode
 * restarts the simulation from its fluid objects, like vfd_set_description. A particle
 * leaving the anchor range fails the step with VFD_E_CAPACITY (VFD_FLAG_ANCHOR_RANGE).
 */
int vfd_set_position_mode(vfd_sim* sim, int32_t mode);

/*
 * Kernel evaluation: VFD_KERNEL_TABLE (default) looks W and gradW up in the
 * precomputed tables as PrecomputedDFSPHCubicKernel does (Kernel/DFSPHKernels.h:43-80);
 * VFD_KERNEL_ANALYTIC evaluates the same cubic spline (:86-131) at |r|, which makes the
 * step smooth in the positions, so that finite differences of it match its adjoint.
 * No counterpart in the reference. Call before the first step; like
 * vfd_set_position_mode it drops the device state.
 */
int vfd_set_kernel_mode(vfd_sim* sim, int32_t mode);

/*
 * Arithmetic of the step. No counterpart in the reference, whose step is FP32 throughout.
 * VFD_PRECISION_FP64 runs the whole step -- search, boundary, density, the three solves,
 * surface tension, CFL step, integration -- in double precision on the GPU, one thread per
 * particle with the solver loops driven from the host: the reference trajectory against
 * which the FP32 paths (absolute and cell-relative positions) are measured on scenes of
 * millions of particles. Single scene; restarts the simulation from its fluid objects.
 * In FP64 mode vfd_step / vfd_steps / vfd_get_state / vfd_get_debug_info and
 * vfd_get_field(VFD_FIELD_DENSITY) work as usual (values rounded to float), and
 * vfd_get_state_f64 returns the double positions and velocities (n*3 doubles each, original
 * order, either may be NULL); the calls that act on the FP32 state (vfd_set_state,
 * checkpoints, vfd_emit, vfd_simulate, the adjoint, the profiler and autotuner,
 * vfd_find_neighbors) return VFD_E_STATE.
 */
int vfd_set_precision(vfd_sim* sim, int32_t mode);
int vfd_get_state_f64(vfd_sim* sim, double* x, double* v);

/*
 * Appends `count` particles (xyz, and velocities or NULL for zero) to the running state
 * of a single-scene simulation: an inflow emitter's call. The particles already there
 * keep their state and their indices; the new ones take the next original indices
 * (n, n + 1, ...) and start with zero acceleration and solver warm starts. The device
 * layout grows by a quarter when it is full (the state is kept); the step graphs are
 * rebuilt at the next step. vfd_reset / vfd_simulate go back to the initial particles.
 * No counterpart in the reference, which has no emitter.
 */
int vfd_emit(vfd_sim* sim, const float* xyz, const float* vel, uint32_t count);

/* Device the library runs on (default 0, SystemInfo::InitDevice, Debug/SystemInfo.cpp:34-35). */
int vfd_set_device(int32_t device);

/* Message of the last failing call on this thread ("" if none). */
const char* vfd_last_error(void);

/* VFD_ABI_VERSION of the loaded library. */
int vfd_abi_version(void);

#ifdef __cplusplus
}
#endif

#endif /* VFD_DFSPH_H */
