// Host-side state of one simulation handle (struct vfd_sim) and the helpers that
// the C-ABI translation units share: the step launchers, the error and allocation
// helpers, and the host copies of the kernel table and the scenes. Internal to the
// library; the public interface is include/vfd_dfsph.h.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "../../include/vfd_dfsph.h"
#include "dfsph_common.cuh"

namespace vfd {
void launch_search(const Dev& d, cudaStream_t s, bool profiled = true);
uint32_t scan_block_count(uint32_t cellCap);
void launch_boundary(const Dev& d, cudaStream_t s);
void launch_density(const Dev& d, cudaStream_t s);
void launch_density_div_init(const Dev& d, cudaStream_t s);
void launch_div_iter(const Dev& d, cudaStream_t s);
void launch_div_finish(const Dev& d, cudaStream_t s);
void launch_surface_tension(const Dev& d, uint32_t maxPasses, cudaStream_t s);
void launch_visc_init(const Dev& d, cudaStream_t s);
void launch_cg_iter(const Dev& d, cudaStream_t s);
void launch_visc_finish_dt(const Dev& d, cudaStream_t s);
void launch_pres_init(const Dev& d, cudaStream_t s);
void launch_pres_iter(const Dev& d, cudaStream_t s);
void launch_pres_finish(const Dev& d, cudaStream_t s);
// Occupancy and shared-memory limits of the cell-tile kernels (once, before any capture).
cudaError_t prepare_tile_kernels();
// Whether any solver-loop pass runs on cell tiles (then the search writes NBRC rows).
inline bool uses_tiles(const uint8_t* tiles) {
    return tiles[kTPAccel] >= kTileMinLog2 || tiles[kTJacobi] >= kTileMinLog2 || tiles[kTSpmv] >= kTileMinLog2;
}
void box_map_sizes(const uint32_t res[3], uint32_t& nodes, uint32_t& cells);
int build_box_map_gpu(const float bmin[3], const float bmax[3], bool inverted, float padding, const uint32_t res[3],
                      float r, const float* table, float wZero, float invStep, float* nodes, uint32_t* cells,
                      uint32_t* cellMap, float dminOut[3], float dmaxOut[3], float csOut[3], float csiOut[3]);

// A triangle mesh placed in the world, as the distance kernels read it.
struct MeshHost {
    std::vector<float4> corners;  // 3 per face: corners A, B, C (w unused)
    std::vector<float4> normals;  // 7 per face: corner A, B, C; edge AB, BC, CA; face (w unused)
    float bmin[3], bmax[3];       // bounds of all placed vertices
};
// Places the vertices by `transform` (column-major 4x4, null = identity) and computes the
// pseudo-normals. Returns 0, or -1 when a triangle names a vertex out of range.
int prepare_mesh(const float* vertices, uint32_t vertexCount, const uint32_t* triangles, uint32_t triangleCount,
                 const float* transform, MeshHost& out);
int build_mesh_map_gpu(const MeshHost& mesh, bool inverted, float padding, const uint32_t res[3], float r,
                       const float* table, float wZero, float invStep, float* nodes, uint32_t* cells,
                       uint32_t* cellMap, float dminOut[3], float dmaxOut[3], float csOut[3], float csiOut[3]);
int sample_mesh_volume_gpu(const MeshHost& mesh, float radius, const uint32_t res[3], bool inverted, int mode,
                           float* out, uint32_t capacity, uint32_t* count);
}  // namespace vfd

namespace vfd {
namespace host {

// Records the message returned by vfd_last_error() and returns `code`.
int fail(int code, const char* fmt, ...);

#define CK(call)                                                                                       \
    do {                                                                                               \
        cudaError_t e_ = (call);                                                                       \
        if (e_ != cudaSuccess) return fail(VFD_E_CUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                                           __FILE__, __LINE__);                                        \
    } while (0)

#define TRY(x)                         \
    do {                               \
        int rc_ = (x);                 \
        if (rc_ != VFD_OK) return rc_; \
    } while (0)

// PrecomputedDFSPHCubicKernel::SetRadius (Kernel/DFSPHKernels.h:13-41) in FP32; the
// library is built with -ffp-contract=off for host code so the table matches it bit for bit.
struct KernelTable {
    std::vector<float> W, G;
    float radius = 0, radius2 = 0, invStep = 0, wZero = 0, K = 0, L = 0;
    float calcW(float r) const {
        float res = 0.0f;
        const float q = r / radius;
        if (q <= 1.0f) {
            if (q <= 0.5f) {
                const float q2 = q * q, q3 = q2 * q;
                res = K * (6.0f * q3 - 6.0f * q2 + 1.0f);
            } else {
                const float q1 = 1.0f - q, q3 = q1 * q1 * q1;
                res = K * (2.0f * q3);
            }
        }
        return res;
    }
    float calcGradWx(float px) const {  // CalculateGradientW({px, 0, 0}).x
        const float rl = std::sqrt(px * px + 0.0f * 0.0f + 0.0f * 0.0f);
        const float q = rl / radius;
        if (rl > 1.0e-5f && q <= 1.0f) {
            const float gq = px * (1.0f / (rl * radius));
            if (q <= 0.5f) return ((L * q) * (3.0f * q - 2.0f)) * gq;
            const float f = 1.0f - q;
            return (L * (-f * f)) * gq;
        }
        return 0.0f;
    }
    void setRadius(float r) {
        const float pi = (float)3.14159265358979323846;
        W.assign(kTableRes, 0.0f);
        G.assign(kTableRes + 1, 0.0f);
        radius = r;
        radius2 = radius * radius;
        const float r3 = radius * radius * radius;
        K = 8.0f / (pi * r3);
        L = 48.0f / (pi * r3);
        wZero = calcW(std::sqrt(0.0f));
        const float step = radius / (float)(kTableRes - 1);
        invStep = 1.0f / step;
        for (uint32_t i = 0; i < kTableRes; i++) {
            const float px = step * (float)i;
            W[i] = calcW(px);
            G[i] = px > 1.0e-9f ? calcGradWx(px) / px : 0.0f;
        }
        G[kTableRes] = 0.0f;
    }
};

struct BodyHost {
    BodyDev dev{};
    float* nodes = nullptr;
    uint32_t* cells = nullptr;
    uint32_t* cellMap = nullptr;
    void release() {
        cudaFree(nodes);
        cudaFree(cells);
        cudaFree(cellMap);
        nodes = nullptr;
        cells = cellMap = nullptr;
    }
};

struct SceneHost {
    vfd_desc desc{};
    std::vector<float> x0, v0;
    std::vector<BodyHost> bodies;
    uint32_t emitted = 0;  // particles appended by vfd_emit since the last upload
    uint32_t count() const { return (uint32_t)(x0.size() / 3) + emitted; }
};

}  // namespace host
}  // namespace vfd

namespace vfd {
struct AdjointState;
void adjoint_release(vfd_sim* s);  // frees the recorded forward run of the adjoint
// The FP64 GPU path (vfd_set_precision): its state, built from the scene's initial
// particles at upload, one step, and its outputs.
struct Fp64State;
int fp64_upload(vfd_sim* s);
int fp64_step(vfd_sim* s, vfd_step_stats* out);
int fp64_get_state(vfd_sim* s, double* x, double* v, float* xf, float* vf, float* af);
int fp64_get_density(vfd_sim* s, float* out);
void fp64_stats(const vfd_sim* s, vfd_step_stats* out);
void fp64_release(vfd_sim* s);
}  // namespace vfd

struct vfd_sim {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::vector<vfd::host::SceneHost> scenes;
    vfd::host::KernelTable table;
    std::vector<float> halton;
    bool graphMode = true;
    bool cellRel = false;  // VFD_POSITIONS_CELL_RELATIVE
    bool analyticKernel = false;  // VFD_KERNEL_ANALYTIC
    bool fp64Mode = false;        // VFD_PRECISION_FP64: steps run the FP64 GPU path
    bool borrowedBodies = false;  // the scenes' volume maps belong to another simulation (an adjoint's replay copy)
    vfd::Fp64State* fp64 = nullptr;
    bool graphFailed = false;
    uint8_t lanes[16] = {8, 8, 8, 8, 8, 8, 8, 8, 8, 8, 8, 8, 8, 8, 8, 8};
    // cell tiles of the solver-loop kernels per TunedKernel: 0 = neighbour rows, else log2
    // of the cells in a tile (vfd_set_tiles, vfd_autotune)
    uint8_t tiles[16] = {};
    // threads per block of each TunedKernel's neighbour-row kernels (vfd_autotune; 0 = 128)
    uint16_t blocks[16] = {};

    // layout
    bool allocated = false, uploaded = false;
    uint32_t n = 0, stride = 0, cellCap = 0, maxBodies = 0;
    uint32_t reserve = 0;  // particle capacity to allocate for (vfd_emit grows it)
    std::vector<uint32_t> sceneBegin;
    std::vector<void*> allocs;
    vfd::Dev dev[2]{};
    int cs = 0;  // set holding the current carried state
    float4* XB = nullptr;
    float* dStage = nullptr;     // 3 floats per particle, original order
    float* dStage2 = nullptr;    // a second one (velocities beside positions in vfd_set_state)
    vfd::SceneDev* dScenes = nullptr;
    vfd::BodyDev* dBodies = nullptr;
    uint32_t* dStatus = nullptr;
    float *dWM = nullptr, *dGM = nullptr, *dHalton = nullptr;
    uint32_t* hStatus = nullptr;  // pinned
    std::vector<vfd::SceneDev> hScenes;
    uint32_t maxStPasses = 0;
    bool anyDiv = false, anyVisc = false, anyST = false;

    // graphs (one per parity)
    cudaGraphExec_t exec[2] = {nullptr, nullptr};
    cudaGraph_t graph[2] = {nullptr, nullptr};
    bool searchOnlyPending = false;

    // adjoint: checkpoints and tapes of the last vfd_adjoint_forward; `generation`
    // counts uploads, so a reset after the recorded run is detected
    vfd::AdjointState* adjoint = nullptr;
    int adjWarm = 1;      // VFD_WARM_* of the adjoint viscosity solves
    float adjTol = 1.0f;  // adjoint viscosity solves' tolerance relative to the forward's
    uint64_t generation = 0;
    // kept across adjoint runs while the buffers live: the device tape set that recording
    // graphs address, those graphs (one per parity) and the backward graph of one step
    void* adjTapeSet = nullptr;
    cudaGraph_t adjRecGraph[2] = {nullptr, nullptr};
    cudaGraphExec_t adjRecExec[2] = {nullptr, nullptr};
    cudaGraph_t adjBwdGraph = nullptr;
    cudaGraphExec_t adjBwdExec = nullptr;

    ~vfd_sim() { release(); }

    void releaseGraphs() {
        for (int k = 0; k < 2; k++) {
            if (exec[k]) cudaGraphExecDestroy(exec[k]);
            if (graph[k]) cudaGraphDestroy(graph[k]);
            exec[k] = nullptr;
            graph[k] = nullptr;
            if (adjRecExec[k]) cudaGraphExecDestroy(adjRecExec[k]);
            if (adjRecGraph[k]) cudaGraphDestroy(adjRecGraph[k]);
            adjRecExec[k] = nullptr;
            adjRecGraph[k] = nullptr;
        }
        if (adjBwdExec) cudaGraphExecDestroy(adjBwdExec);
        if (adjBwdGraph) cudaGraphDestroy(adjBwdGraph);
        adjBwdExec = nullptr;
        adjBwdGraph = nullptr;
    }
    void releaseBuffers() {
        // a recorded adjoint run (and the copy of the simulation that replays it, which
        // borrows the volume maps) does not outlive the layout it was recorded on
        vfd::adjoint_release(this);
        releaseGraphs();
        for (void* p : allocs) cudaFree(p);
        allocs.clear();
        adjTapeSet = nullptr;
        if (hStatus) cudaFreeHost(hStatus);
        hStatus = nullptr;
        allocated = false;
        uploaded = false;
    }
    void release() {
        vfd::adjoint_release(this);
        vfd::fp64_release(this);
        releaseBuffers();
        if (!borrowedBodies)
            for (auto& s : scenes)
                for (auto& b : s.bodies) b.release();
        if (stream) cudaStreamDestroy(stream);
        stream = nullptr;
    }
};

namespace vfd {
namespace host {

template <class T>
int dalloc(vfd_sim* s, T** p, size_t count) {
    void* q = nullptr;
    const size_t bytes = std::max<size_t>(1, count) * sizeof(T);
    cudaError_t e = cudaMalloc(&q, bytes);
    if (e != cudaSuccess) return fail(VFD_E_NOMEM, "cudaMalloc(%zu bytes): %s", bytes, cudaGetErrorString(e));
    s->allocs.push_back(q);
    *p = (T*)q;
    return VFD_OK;
}

// Graph building blocks: a conditional WHILE node whose body `body` captures, and a
// captured segment appended after the current leaves.
template <class F>
cudaError_t add_while(cudaStream_t cap, cudaGraph_t g, cudaGraphConditionalHandle h, std::vector<cudaGraphNode_t>& leaves,
                      F body) {
    cudaGraphNodeParams np = {cudaGraphNodeTypeConditional};
    np.conditional.handle = h;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t node;
    cudaError_t e = cudaGraphAddNode(&node, g, leaves.data(), nullptr, leaves.size(), &np);
    if (e != cudaSuccess) return e;
    cudaGraph_t bodyGraph = np.conditional.phGraph_out[0];
    e = cudaStreamBeginCaptureToGraph(cap, bodyGraph, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return e;
    body(cap);
    e = cudaStreamEndCapture(cap, &bodyGraph);
    if (e != cudaSuccess) return e;
    leaves.assign(1, node);
    return cudaSuccess;
}

template <class F>
cudaError_t add_segment(cudaStream_t cap, cudaGraph_t g, std::vector<cudaGraphNode_t>& leaves, F seg) {
    cudaError_t e = cudaStreamBeginCaptureToGraph(cap, g, leaves.empty() ? nullptr : leaves.data(), nullptr,
                                                  leaves.size(), cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return e;
    seg(cap);
    cudaStreamCaptureStatus status;
    const cudaGraphNode_t* deps = nullptr;
    size_t nd = 0;
    e = cudaStreamGetCaptureInfo(cap, &status, nullptr, nullptr, &deps, nullptr, &nd);
    if (e != cudaSuccess) return e;
    std::vector<cudaGraphNode_t> next(deps, deps + nd);
    cudaGraph_t out = g;
    e = cudaStreamEndCapture(cap, &out);
    if (e != cudaSuccess) return e;
    if (!next.empty()) leaves = next;
    return cudaSuccess;
}


// Adjoint tape points of a recorded step (tape_point in dfsph_adjoint.cu).
enum TapePoint {
    kTapeBegin = 0, kTapeSearch, kTapeBoundary, kTapeDivInit, kTapeDivIter, kTapeDivFinish, kTapeVisc,
    kTapeVelocity, kTapePresInit, kTapePresIter, kTapeEnd
};
void tape_point(const Dev& d, const void* rec, int point, cudaStream_t st);

// One step as a graph (rec: the adjoint's device tape set, or null) into *gOut / *execOut.
int build_graph(vfd_sim* s, int parity, const void* rec, cudaGraph_t* gOut, cudaGraphExec_t* execOut);
// One eagerly launched step (one flag read per solver iteration), optionally recording.
int launch_eager(vfd_sim* s, const void* rec);

int ensure_ready(vfd_sim* s);
void fill_stats(const SceneDev& S, vfd_step_stats* st);
int read_flag(vfd_sim* s, int idx, uint32_t& v);
int run_steps(vfd_sim* s, uint32_t count, vfd_step_stats* stats, bool wait);
int finish_steps(vfd_sim* s, vfd_step_stats* stats, uint32_t& flags);
int scatter_vec(vfd_sim* s, uint32_t scene, const float4* dsrc, float* out);
int gather_vec(vfd_sim* s, uint32_t scene, const float* in, float4* ddst);

}  // namespace host
}  // namespace vfd
