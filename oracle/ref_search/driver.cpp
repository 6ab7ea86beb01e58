// Host driver for the reference's own neighbour-search kernels, run on the CPU.
//
// Test infrastructure only (never linked into the product). The recipe in
// oracle/Makefile (target `ref`) compiles the reference's
// Simulation/DFSPH/ParticleSearch/ParticleSearchKernels.cu as C++ together with this
// file, with pch.h and glm_subset.h standing in for the reference's precompiled header
// and its absent glm submodule. This file restates the host side of
// ParticleSearch::FindNeighbors (ParticleSearch.cu:29-195): the kernel launches run one
// emulated CUDA thread at a time in thread order, so every atomicAdd rank of
// InsertParticlesMortonKernel -- the in-cell order, which the GPU leaves to chance --
// comes out in ascending particle index, one of the orders the reference allows and the
// one the oracle and the CUDA library use. thrust::exclusive_scan / sequence / gather
// become their sequential definitions.
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <vector>

#include "pch.h"
#include "Simulation/DFSPH/ParticleSearch/ParticleSearchKernels.cuh"
#include "Simulation/DFSPH/ParticleSearch/SearchInfo.h"
#include "Simulation/DFSPH/Structures/DFSPHParticle.h"

RefDim3 blockIdx{0, 0, 0}, blockDim{256, 1, 1}, threadIdx{0, 0, 0};

namespace {

// kernel<<<blocks, 256>>>(args...), one thread after another.
template <class F>
void launch(unsigned int count, F kernel) {
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

void exclusive_scan(const std::vector<unsigned int>& in, std::vector<unsigned int>& out) {
    unsigned int run = 0;
    for (size_t i = 0; i < in.size(); i++) {
        out[i] = run;
        run += in[i];
    }
}

}  // namespace

extern "C" {

// Neighbour lists of n particles (xyz, original order) with search radius `radius`
// (= the support radius h): per particle its count, the exclusive-scan offsets and the
// CSR list of original indices (capacity `cap`, *total receives the length), the sort
// permutation (sorted slot -> original index) and each particle's Morton meta-grid key.
int ref_find_neighbors(const float* xyz, uint32_t n, float radius, uint32_t* counts, uint32_t* offsets,
                       uint32_t* list, uint32_t cap, uint32_t* total, uint32_t* sortIdx, uint32_t* keys) {
    std::vector<vfd::DFSPHParticle> particles(n);
    for (uint32_t i = 0; i < n; i++) {
        std::memset(&particles[i], 0, sizeof(vfd::DFSPHParticle));
        particles[i].Position = glm::vec3(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
    }
    const vfd::DFSPHParticle* pts = particles.data();

    // ComputeMinMax (ParticleSearch.cu:29-55)
    glm::ivec3 mm[2] = {glm::ivec3(std::numeric_limits<int>::max()), glm::ivec3(std::numeric_limits<int>::min())};
    launch(n, [&] { ComputeMinMaxKernel(pts, n, radius, &mm[0], &mm[1]); });
    const glm::ivec3 minCell = mm[0];
    const glm::ivec3 maxCell = mm[1] + glm::ivec3(1, 1, 1);
    const glm::vec3 bmin = static_cast<glm::vec3>(minCell) * radius;
    const glm::vec3 bmax = static_cast<glm::vec3>(maxCell) * radius;

    // ComputeCellInformation (:57-137)
    vfd::SearchInfo info;
    info.ParticleCount = n;
    info.SquaredSearchRadius = radius * radius;
    info.GridMin = bmin;
    const float cellSize = radius;
    glm::vec3 gridSize = bmax - bmin;  // BoundingBox::Diagonal
    info.GridDimension.x = static_cast<unsigned int>(std::ceil(gridSize.x / cellSize));
    info.GridDimension.y = static_cast<unsigned int>(std::ceil(gridSize.y / cellSize));
    info.GridDimension.z = static_cast<unsigned int>(std::ceil(gridSize.z / cellSize));
    info.GridDimension.x += 4;
    info.GridDimension.y += 4;
    info.GridDimension.z += 4;
    info.GridMin -= glm::vec3(cellSize, cellSize, cellSize) * 2.0f;
    info.MetaGridDimension.x = static_cast<unsigned int>(std::ceil(info.GridDimension.x / static_cast<float>(CUDA_META_GRID_GROUP_SIZE)));
    info.MetaGridDimension.y = static_cast<unsigned int>(std::ceil(info.GridDimension.y / static_cast<float>(CUDA_META_GRID_GROUP_SIZE)));
    info.MetaGridDimension.z = static_cast<unsigned int>(std::ceil(info.GridDimension.z / static_cast<float>(CUDA_META_GRID_GROUP_SIZE)));
    gridSize.x = info.GridDimension.x * cellSize;
    gridSize.y = info.GridDimension.y * cellSize;
    gridSize.z = info.GridDimension.z * cellSize;
    info.GridDelta.x = info.GridDimension.x / gridSize.x;
    info.GridDelta.y = info.GridDimension.y / gridSize.y;
    info.GridDelta.z = info.GridDimension.z / gridSize.z;
    const uint64_t cells = (uint64_t)info.MetaGridDimension.x * info.MetaGridDimension.y *
                           info.MetaGridDimension.z * CUDA_META_GRID_BLOCK_SIZE;
    if (cells > (1ull << 31)) return 5;  // VFD_E_CAPACITY
    std::vector<unsigned int> tempSort(n), cellIdx(n), sortIndices(n), reversed(n);
    std::vector<unsigned int> cellOffsets(cells), cellCounts(cells, 0u);
    launch(n, [&] { InsertParticlesMortonKernel(info, pts, cellIdx.data(), cellCounts.data(), tempSort.data()); });
    exclusive_scan(cellCounts, cellOffsets);
    launch(n, [&] {
        CountingSortIndicesKernel(info, cellIdx.data(), cellOffsets.data(), tempSort.data(), sortIndices.data());
    });
    for (uint32_t i = 0; i < n; i++) tempSort[i] = i;                  // thrust::sequence
    for (uint32_t i = 0; i < n; i++) reversed[i] = tempSort[sortIndices[i]];  // thrust::gather

    // ComputeNeighborhood (:139-195)
    std::vector<unsigned int> nbrCounts(n), nbrOffsets(n);
    launch(n, [&] {
        ComputeCountsKernel(pts, info, cellOffsets.data(), cellCounts.data(), nbrCounts.data(), reversed.data());
    });
    exclusive_scan(nbrCounts, nbrOffsets);
    const uint64_t tot = n ? (uint64_t)nbrOffsets[n - 1] + nbrCounts[n - 1] : 0u;
    std::vector<unsigned int> neighbors(std::max<uint64_t>(tot, 1));
    launch(n, [&] {
        NeighborhoodQueryWithCountsKernel(pts, info, cellOffsets.data(), cellCounts.data(), nbrOffsets.data(),
                                          neighbors.data(), reversed.data());
    });

    if (total) *total = (uint32_t)tot;
    if (counts) std::copy(nbrCounts.begin(), nbrCounts.end(), counts);
    if (offsets) std::copy(nbrOffsets.begin(), nbrOffsets.end(), offsets);
    if (sortIdx) std::copy(sortIndices.begin(), sortIndices.end(), sortIdx);
    if (keys) std::copy(cellIdx.begin(), cellIdx.end(), keys);
    if (list) {
        if (tot > cap) return 5;
        std::copy(neighbors.begin(), neighbors.begin() + tot, list);
    }
    return 0;
}

}  // extern "C"
