// Neighbour search that allocates nothing (vfd_find_neighbors_noalloc).
//
// Some callers cannot call cudaMalloc: code whose device memory is owned by another
// allocator with a fixed budget (a host framework's caching allocator, a plug-in
// given a memory pool), and code that must not allocate once it is running (real-time
// loops). This entry point serves them: the caller passes device buffers for the
// input positions and the outputs, and all intermediate data (cell keys, cell tables,
// sorted copies, neighbour rows) lives in one file-scope __device__ array of fixed size,
// which every GPU that loads the library holds until the process exits.
//
// Limits: at most kNoAllocMaxParticles particles and kNoAllocMaxCells search-grid cells
// per call; larger inputs are rejected with VFD_E_CAPACITY.
// Sharing: every call uses the same array and leaves its contents behind; each call
// clears what must start at zero. Calls that overlap on the GPU (other streams,
// other host threads) race on the array and must be serialised by the caller.
// Set-up: the first call on a device looks up the array's device address with
// cudaGetSymbolAddress while that device is current; make that first call before any
// stream capture. The address is remembered per CUDA context (by the context's unique
// id), so a device reset or a second context on the same device gets its own look-up
// instead of a stale address. Each call waits for its stream before it returns the
// status. No cudaMalloc, cudaFree or allocating library call is made, and the launches
// bypass the per-kernel profiler (which would create CUDA events).
#include <cuda.h>
#include <cuda_runtime.h>

#include <climits>
#include <cstring>
#include <mutex>

#include "../../include/vfd_dfsph.h"
#include "dfsph_common.cuh"

namespace vfd {
void launch_search(const Dev& d, cudaStream_t s, bool profiled);
uint32_t scan_block_count(uint32_t cellCap);
}  // namespace vfd

using namespace vfd;

namespace {

constexpr uint32_t kNoAllocMaxParticles = 16384u;
constexpr uint32_t kNoAllocMaxCells = 262144u;

constexpr size_t align256(size_t x) { return (x + 255u) & ~size_t(255u); }

// Byte offsets of the regions inside the scratch array.
struct Layout {
    static constexpr size_t P = kNoAllocMaxParticles, C = kNoAllocMaxCells;
    static constexpr size_t f4 = align256(P * sizeof(float4)), f1 = align256(P * sizeof(float)),
                            u1 = align256(P * sizeof(uint32_t));
    static constexpr size_t XN = 0, Vc = XN + f4, DVc = Vc + f4, X = DVc + f4, V = X + f4, DV = V + f4;
    static constexpr size_t DKc = DV + f4, DK = DKc + f1;
    static constexpr size_t PIDc = DK + f1, PID = PIDc + u1, KEY = PID + u1, KEYS = KEY + u1, TMP = KEYS + u1,
                            NCNT = TMP + u1;
    static constexpr size_t NBR = NCNT + u1;
    static constexpr size_t CELL_START = NBR + align256(P * kRow * sizeof(uint32_t));
    static constexpr size_t CELL_COUNT = CELL_START + align256(C * sizeof(uint32_t));
    static constexpr size_t FILL = CELL_COUNT + align256(C * sizeof(uint32_t));
    static constexpr size_t SCAN = FILL + align256(C * sizeof(uint32_t));
    static constexpr size_t SCENE = SCAN + align256((C / 1024u + 2u) * sizeof(uint32_t));
    static constexpr size_t STATUS = SCENE + align256(sizeof(SceneDev));
    static constexpr size_t MMB = STATUS + align256(16 * sizeof(uint32_t));
    static constexpr size_t MAXB = MMB + align256(6u * kBuckets * 32u * sizeof(int32_t));
    static constexpr size_t ACCB = MAXB + align256(2u * kBuckets * 32u * sizeof(uint32_t));
    static constexpr size_t TOTAL = ACCB + align256(kAccSlots * kBuckets * 16u * sizeof(double));
};

// The scratch itself (about 10 MB).
static __device__ __align__(256) unsigned char g_noallocScratch[Layout::TOTAL];

// The array's device address per CUDA context, keyed by the context's unique id
// (cuCtxGetId; ids are never reused within a process).
struct AddrEntry {
    unsigned long long ctx;
    void* addr;
};
std::mutex g_noallocMutex;
AddrEntry g_noallocAddr[64] = {};
uint32_t g_noallocUsed = 0;

typedef CUresult (*CtxGetCurrentFn)(CUcontext*);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long*);

// Id of the calling thread's current context (the runtime's primary context once the
// device is in use), through the driver entry points the runtime hands out.
int current_context_id(unsigned long long& id) {
    static CtxGetCurrentFn getCurrent = nullptr;
    static CtxGetIdFn getId = nullptr;
    if (!getCurrent || !getId) {
        void* f1 = nullptr;
        void* f2 = nullptr;
        cudaDriverEntryPointQueryResult q1, q2;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) != cudaSuccess ||
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) != cudaSuccess ||
            q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess)
            return VFD_E_CUDA;
        getCurrent = (CtxGetCurrentFn)f1;
        getId = (CtxGetIdFn)f2;
    }
    CUcontext ctx = nullptr;
    if (getCurrent(&ctx) != CUDA_SUCCESS || !ctx) return VFD_E_CUDA;
    return getId(ctx, &id) == CUDA_SUCCESS ? VFD_OK : VFD_E_CUDA;
}

// Clears the per-call state: one scene, status words, reduction buckets.
__global__ void k_noalloc_reset(Dev d, SceneDev scene) {
    if (blockIdx.x == 0 && threadIdx.x == 0) d.scenes[0] = scene;
    for (uint32_t i = threadIdx.x; i < 16u; i += blockDim.x) d.status[i] = 0u;
    for (uint32_t i = threadIdx.x; i < 6u * kBuckets * 32u; i += blockDim.x) d.MMB[i] = (i / (kBuckets * 32u)) < 3u ? INT_MAX : INT_MIN;
    for (uint32_t i = threadIdx.x; i < 2u * kBuckets * 32u; i += blockDim.x) d.MAXB[i] = 0u;
}

// Packs the caller's positions into the search's layout (original order, zero velocities).
__global__ void k_noalloc_load(Dev d, const float* xyz) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.n) return;
    d.XN[i] = make_float4(xyz[3 * (size_t)i], xyz[3 * (size_t)i + 1], xyz[3 * (size_t)i + 2], 0.0f);
    d.Vc[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    d.DVc[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    d.DKc[i] = 0.0f;
    d.PIDc[i] = i;
}

// Sorted rows -> the caller's outputs in original order with original indices.
__global__ void k_noalloc_export(Dev d, uint32_t* counts, uint32_t* neighbors, uint32_t* sortIndices) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= d.n || __ldg(d.status + 1) != 0u) return;
    const uint32_t o = d.PID[p];
    const uint32_t c = d.NCNT[p] & kCountMask;
    sortIndices[p] = o;
    counts[o] = c;
    const uint32_t* row = d.NBR + (size_t)p * kRow;
    for (uint32_t j = 0; j < c; j++) neighbors[(size_t)o * kMaxNeighbors + j] = d.PID[row[j]];
}

// Errors are reported by status code only (no message buffer, nothing allocated).
int na_fail(int code, const char*) { return code; }

}  // namespace

extern "C" {

int vfd_find_neighbors_noalloc(const float* xyz, uint32_t n, float particle_radius, uint32_t* counts,
                               uint32_t* neighbors, uint32_t* sort_indices, void* stream) {
    if (n == 0) return VFD_OK;
    if (!xyz || !counts || !neighbors || !sort_indices) return na_fail(VFD_E_ARG, "null buffer");
    if (!(particle_radius > 0.0f)) return na_fail(VFD_E_ARG, "particle radius must be positive");
    if (n > kNoAllocMaxParticles)
        return na_fail(VFD_E_CAPACITY, "vfd_find_neighbors_noalloc handles at most 16384 particles per call");
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return na_fail(VFD_E_CUDA, "no current device");
    if (cudaSetDevice(dev) != cudaSuccess) return na_fail(VFD_E_CUDA, "no context");  // binds the primary context
    unsigned long long ctx = 0;
    if (current_context_id(ctx) != VFD_OK) return na_fail(VFD_E_CUDA, "no current context");
    void* base = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_noallocMutex);
        for (uint32_t k = 0; k < g_noallocUsed; k++)
            if (g_noallocAddr[k].ctx == ctx) base = g_noallocAddr[k].addr;
        if (!base) {  // set-up, once per context, with this device current
            void* p = nullptr;
            const cudaError_t e = cudaGetSymbolAddress(&p, g_noallocScratch);
            if (e != cudaSuccess || !p) return na_fail(VFD_E_CUDA, cudaGetErrorString(e));
            const uint32_t slot = g_noallocUsed < 64u ? g_noallocUsed++ : (uint32_t)(ctx % 64u);
            g_noallocAddr[slot] = AddrEntry{ctx, p};
            base = p;
        }
    }
    unsigned char* b = static_cast<unsigned char*>(base);
    Dev d;
    std::memset(&d, 0, sizeof(d));
    d.n = n;
    d.stride = kNoAllocMaxParticles;
    d.nscenes = 1;
    d.cellCap = kNoAllocMaxCells;
    d.scanBlocks = scan_block_count(kNoAllocMaxCells);
    d.XN = (float4*)(b + Layout::XN);
    d.Vc = (float4*)(b + Layout::Vc);
    d.DVc = (float4*)(b + Layout::DVc);
    d.X = (float4*)(b + Layout::X);
    d.V = (float4*)(b + Layout::V);
    d.DV = (float4*)(b + Layout::DV);
    d.DKc = (float*)(b + Layout::DKc);
    d.DK = (float*)(b + Layout::DK);
    d.PIDc = (uint32_t*)(b + Layout::PIDc);
    d.PID = (uint32_t*)(b + Layout::PID);
    d.KEY = (uint32_t*)(b + Layout::KEY);
    d.KEYS = (uint32_t*)(b + Layout::KEYS);
    d.TMP = (uint32_t*)(b + Layout::TMP);
    d.NCNT = (uint32_t*)(b + Layout::NCNT);
    d.NBR = (uint32_t*)(b + Layout::NBR);
    d.CELL_START = (uint32_t*)(b + Layout::CELL_START);
    d.CELL_COUNT = (uint32_t*)(b + Layout::CELL_COUNT);
    d.FILL = (uint32_t*)(b + Layout::FILL);
    d.SCAN = (uint32_t*)(b + Layout::SCAN);
    d.scenes = (SceneDev*)(b + Layout::SCENE);
    d.status = (uint32_t*)(b + Layout::STATUS);
    d.MMB = (int32_t*)(b + Layout::MMB);
    d.MAXB = (uint32_t*)(b + Layout::MAXB);
    d.ACCB = (double*)(b + Layout::ACCB);
    for (int k = 0; k < 16; k++) d.lanes[k] = 8;
    {  // the neighbour search strides a fixed grid over the cells
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        d.batchBlocks = (uint32_t)(sms > 0 ? sms : 1) * (2048u / kBlock);
    }

    // the search radius and squared radius exactly as SetDescription derives them
    SceneDev scene;
    std::memset(&scene, 0, sizeof(scene));
    scene.count = n;
    scene.r = particle_radius;
    scene.h = 4.0f * particle_radius;
    scene.h2 = scene.h * scene.h;

    cudaStream_t s = static_cast<cudaStream_t>(stream);
    k_noalloc_reset<<<1, 256, 0, s>>>(d, scene);
    k_noalloc_load<<<blocks_for(n, 256), 256, 0, s>>>(d, xyz);
    launch_search(d, s, false);
    k_noalloc_export<<<blocks_for(n, 256), 256, 0, s>>>(d, counts, neighbors, sort_indices);
    cudaError_t e = cudaGetLastError();
    uint32_t status[2] = {0u, 0u};
    if (e == cudaSuccess) e = cudaMemcpyAsync(status, d.status, sizeof(status), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return na_fail(VFD_E_CUDA, cudaGetErrorString(e));
    if (status[1]) {
        if (status[0] & 0x10u) return na_fail(VFD_E_NAN, "non-finite position");
        return na_fail(VFD_E_CAPACITY, "the search grid needs more than 262144 cells");
    }
    return VFD_OK;
}

}  // extern "C"
