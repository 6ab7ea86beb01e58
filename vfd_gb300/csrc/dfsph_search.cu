// Neighbour search of the DFSPH step: ParticleSearch::FindNeighbors
// (Simulation/DFSPH/ParticleSearch/ParticleSearch.h:80-93, ParticleSearch.cu:29-195,
// ParticleSearchKernels.cu:40-193) rebuilt for GB300:
//   * the grid (bounds, dimensions, Morton meta-grid keys) is computed on the
//     device, per scene, with the reference's float arithmetic (IEEE-rounded
//     intrinsics, no contraction), so no host round trip is needed;
//   * the counting sort is deterministic: within a cell, particles are ordered
//     by original index (the reference's atomicAdd rank allows any order);
//   * the carried state is gathered into cell order (coalesced float4 rows for
//     every later kernel) instead of being read through an index;
//   * neighbour lists are ELL columns (slot-major per rank), capped at 70 in the
//     reference's z, y, x cell order; one pass, no count/scan/query split.
#include "dfsph_common.cuh"

namespace vfd {

constexpr uint32_t kScanItems = 1024u;  // cells per scan block (256 threads x 4)

__device__ __forceinline__ uint32_t part1by2(uint32_t x) {  // ParticleSearchKernels.cu:9-17
    x &= 0x000003ffu;
    x = (x ^ (x << 16)) & 0xff0000ffu;
    x = (x ^ (x << 8)) & 0x0300f00fu;
    x = (x ^ (x << 4)) & 0x030c30c3u;
    x = (x ^ (x << 2)) & 0x09249249u;
    return x;
}

// ToCellIndexMortonMetaGrid, ParticleSearchKernels.cu:24-38.
__device__ __forceinline__ uint32_t cell_key(const SceneDev& s, int cx, int cy, int cz) {
    const uint32_t mx = (uint32_t)cx >> 3, my = (uint32_t)cy >> 3, mz = (uint32_t)cz >> 3;
    const uint32_t meta = mz * s.meta[1] * s.meta[0] + my * s.meta[0] + mx;
    return meta * 512u + ((part1by2((uint32_t)cz & 7u) << 2) + (part1by2((uint32_t)cy & 7u) << 1) +
                          part1by2((uint32_t)cx & 7u));
}

__device__ __forceinline__ bool aborted(const Dev& d) { return is_aborted(d); }

// N1: ComputeMinMaxKernel (ParticleSearchKernels.cu:40-62) on the current positions.
__global__ void __launch_bounds__(kBlock) k_minmax(Dev d) {
    VFD_COUNT_LAUNCH(d);
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = i < d.n;
    const uint32_t sid = valid ? scene_of(d, i) : 0u;
    int c[3] = {INT_MAX, INT_MAX, INT_MAX};
    int cmax[3] = {INT_MIN, INT_MIN, INT_MIN};
    if (valid) {
        const float4 x4 = d.XN[i];
        const float3 x = abs_pos(d, d.scenes[sid], x4);
        const float h = d.scenes[sid].h;
        const bool finite = isfinite(x.x) && isfinite(x.y) && isfinite(x.z);
        if (!finite) {
            atomicOr(&d.scenes[sid].flags, 0x10u);
            atomicOr(d.status, 0x10u);
            atomicExch(d.status + 1, 1u);
        } else {
            const float p[3] = {x.x, x.y, x.z};
#pragma unroll
            for (int k = 0; k < 3; k++) {
                const float q = floorf(__fdiv_rn(p[k], h));
                // positions beyond +-2^30 cells cannot be gridded; flag them.
                const int v = (fabsf(q) < 1.0e9f) ? (int)q : 0;
                if (!(fabsf(q) < 1.0e9f)) { atomicOr(d.status, 0x20u); atomicExch(d.status + 1, 1u); }
                c[k] = v;
                cmax[k] = v;
            }
        }
    }
    const uint32_t s0 = __shfl_sync(0xffffffffu, sid, 0);
    const bool uniform = __all_sync(0xffffffffu, !valid || sid == s0);
    const uint32_t bucket = blockIdx.x % kBuckets;
    if (uniform) {
#pragma unroll
        for (int k = 0; k < 3; k++) {
            const int mn = __reduce_min_sync(0xffffffffu, c[k]);
            const int mx = __reduce_max_sync(0xffffffffu, cmax[k]);
            if ((threadIdx.x & 31u) == 0 && mn != INT_MAX) {
                atomicMin(mm_bucket(d, s0, k, bucket), mn);
                atomicMax(mm_bucket(d, s0, 3 + k, bucket), mx);
            }
        }
    } else if (valid) {
#pragma unroll
        for (int k = 0; k < 3; k++) {
            atomicMin(mm_bucket(d, sid, k, bucket), c[k]);
            atomicMax(mm_bucket(d, sid, 3 + k, bucket), cmax[k]);
        }
    }
}

// ParticleSearch::ComputeMinMax tail + ComputeCellInformation (ParticleSearch.cu:50-86),
// per scene, then the scene cell bases (exclusive scan) and the capacity check.
__global__ void k_grid(Dev d) {
    VFD_COUNT_LAUNCH(d);
    __shared__ uint32_t total;
    for (uint32_t s = threadIdx.x; s < d.nscenes; s += blockDim.x) {
        SceneDev& S = d.scenes[s];
        for (int k = 0; k < 3; k++) {  // fold the N1 buckets, reset them for the next step
            int mn = INT_MAX, mx = INT_MIN;
            for (uint32_t b = 0; b < kBuckets; b++) {
                int32_t* qa = mm_bucket(d, s, k, b);
                int32_t* qb = mm_bucket(d, s, 3 + k, b);
                mn = min(mn, *qa);
                mx = max(mx, *qb);
                *qa = INT_MAX;
                *qb = INT_MIN;
            }
            S.minCell[k] = mn;
            S.maxCell[k] = mx;
        }
        for (uint32_t b = 0; b < kBuckets; b++) *max_bucket(d, s, 1, b) = 0u;
        const float R = S.h;
        uint32_t cells = 1u;
        bool ok = S.count > 0;
        for (int k = 0; k < 3; k++) {
            const float bmin = __fmul_rn((float)S.minCell[k], R);
            const float bmax = __fmul_rn((float)(S.maxCell[k] + 1), R);
            const float size = __fsub_rn(bmax, bmin);
            const float q = ceilf(__fdiv_rn(size, R));
            const uint32_t dim = (ok && q >= 0.0f && q < 1.0e7f) ? (uint32_t)q + 4u : 4u;
            S.dim[k] = dim;
            S.gridMin[k] = __fsub_rn(bmin, __fmul_rn(R, 2.0f));
            S.meta[k] = (uint32_t)ceilf(__fdiv_rn((float)dim, 8.0f));
            const float gs = __fmul_rn((float)dim, R);
            S.gridDelta[k] = __fdiv_rn((float)dim, gs);
            cells = (cells > 0xFFFFFFFFu / 8u) ? 0xFFFFFFFFu : cells * S.meta[k];
        }
        S.cellCount = (!ok) ? 0u : ((cells > 0xFFFFFFFFu / 512u) ? 0xFFFFFFFFu : cells * 512u);
        S.flags = 0u;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        uint64_t acc = 0;
        for (uint32_t s = 0; s < d.nscenes; s++) {
            d.scenes[s].cellBase = (uint32_t)min(acc, (uint64_t)0xFFFFFFFFu);
            acc += d.scenes[s].cellCount;
        }
        total = (uint32_t)min(acc, (uint64_t)0xFFFFFFFFu);
        d.status[2] = total;
        if (acc > d.cellCap) {
            atomicOr(d.status, 0x20u);
            atomicExch(d.status + 1, 1u);
        }
    }
}

__global__ void __launch_bounds__(256) k_clear_cells(Dev d) {
    VFD_COUNT_LAUNCH(d);
    if (aborted(d)) return;
    const uint32_t total = d.status[2];
    for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < total; c += gridDim.x * blockDim.x) {
        d.CELL_COUNT[c] = 0u;
        d.FILL[c] = 0u;
    }
}

// N2: InsertParticlesMortonKernel (ParticleSearchKernels.cu:64-78), count part.
__global__ void __launch_bounds__(kBlock) k_keys(Dev d) {
    VFD_COUNT_LAUNCH(d);
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.n || aborted(d)) return;
    const SceneDev& S = d.scenes[scene_of(d, i)];
    const float3 x = abs_pos(d, S, d.XN[i]);
    const float p[3] = {x.x, x.y, x.z};
    int c[3];
#pragma unroll
    for (int k = 0; k < 3; k++) c[k] = (int)__fmul_rn(__fsub_rn(p[k], S.gridMin[k]), S.gridDelta[k]);
    uint32_t key = S.cellBase + cell_key(S, c[0], c[1], c[2]);
    if (key >= d.status[2] || c[0] < 0 || c[1] < 0 || c[2] < 0) {  // cannot happen for finite input
        atomicOr(d.status, 0x20u);
        atomicExch(d.status + 1, 1u);
        key = 0u;
        return;
    }
    d.KEY[i] = key;
    atomicAdd(d.CELL_COUNT + key, 1u);
}

// N3: exclusive scan of the cell counts (thrust::exclusive_scan, ParticleSearch.cu:111-115),
// three phases over the device-known number of cells.
__global__ void __launch_bounds__(256) k_scan_reduce(Dev d) {
    VFD_COUNT_LAUNCH(d);
    if (aborted(d)) return;
    const uint32_t total = d.status[2];
    const uint32_t base = blockIdx.x * kScanItems;
    if (base >= total) return;
    uint32_t s = 0;
    for (uint32_t k = threadIdx.x; k < kScanItems; k += 256u) {
        const uint32_t c = base + k;
        if (c < total) s += d.CELL_COUNT[c];
    }
    s = __reduce_add_sync(0xffffffffu, s);
    __shared__ uint32_t ws[8];
    if ((threadIdx.x & 31u) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        for (int w = 0; w < 8; w++) t += ws[w];
        d.SCAN[blockIdx.x] = t;
    }
}

__device__ __forceinline__ uint32_t block_exclusive_scan_1024(uint32_t v, uint32_t& blockTotal) {
    // 1024 threads; returns the exclusive prefix of v within the block
    __shared__ uint32_t ws[32];
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= (uint32_t)o) x += y;
    }
    if (lane == 31) ws[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = ws[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= (uint32_t)o) w += y;
        }
        ws[lane] = w;
    }
    __syncthreads();
    const uint32_t warpPrefix = warp ? ws[warp - 1] : 0u;
    blockTotal = ws[31];
    __syncthreads();
    return warpPrefix + x - v;
}

__global__ void __launch_bounds__(1024) k_scan_top(Dev d) {
    VFD_COUNT_LAUNCH(d);
    if (aborted(d)) return;
    const uint32_t total = d.status[2];
    const uint32_t nb = (total + kScanItems - 1) / kScanItems;
    uint32_t carry = 0;
    for (uint32_t base = 0; base < nb; base += 1024u) {
        const uint32_t k = base + threadIdx.x;
        const uint32_t v = k < nb ? d.SCAN[k] : 0u;
        uint32_t tot;
        const uint32_t ex = block_exclusive_scan_1024(v, tot);
        if (k < nb) d.SCAN[k] = carry + ex;
        carry += tot;
    }
}

__global__ void __launch_bounds__(256) k_scan_down(Dev d) {
    VFD_COUNT_LAUNCH(d);
    if (aborted(d)) return;
    const uint32_t total = d.status[2];
    const uint32_t base = blockIdx.x * kScanItems;
    if (base >= total) return;
    __shared__ uint32_t ws[8];
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    // each thread owns 4 consecutive cells
    uint32_t v[4], s = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const uint32_t c = base + threadIdx.x * 4u + k;
        v[k] = c < total ? d.CELL_COUNT[c] : 0u;
        s += v[k];
    }
    uint32_t x = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= (uint32_t)o) x += y;
    }
    if (lane == 31) ws[warp] = x;
    __syncthreads();
    uint32_t wp = 0;
    for (uint32_t w = 0; w < warp; w++) wp += ws[w];
    uint32_t run = d.SCAN[blockIdx.x] + wp + x - s;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const uint32_t c = base + threadIdx.x * 4u + k;
        if (c < total) d.CELL_START[c] = run;
        run += v[k];
    }
}

// N4 (first half): CountingSortIndicesKernel's slot, here through a per-cell fill counter.
__global__ void __launch_bounds__(kBlock) k_slots(Dev d) {
    VFD_COUNT_LAUNCH(d);
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.n || aborted(d)) return;
    const uint32_t key = d.KEY[i];
    const uint32_t s = atomicAdd(d.FILL + key, 1u);
    d.TMP[d.CELL_START[key] + s] = i;
}

// N4 (second half): the deterministic in-cell rank (ascending original index) and the
// gather of the carried state into the new cell order.
__global__ void __launch_bounds__(kBlock) k_rank_gather(Dev d) {
    VFD_COUNT_LAUNCH(d);
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= d.n || aborted(d)) return;
    const uint32_t i = d.TMP[p];
    const uint32_t key = d.KEY[i];
    const uint32_t start = d.CELL_START[key], cnt = d.CELL_COUNT[key];
    const uint32_t pid = d.PIDc[i];
    uint32_t rank = 0;
    for (uint32_t q = start; q < start + cnt; q++) rank += (d.PIDc[d.TMP[q]] < pid) ? 1u : 0u;
    const uint32_t dst = start + rank;
    d.X[dst] = d.XN[i];
    d.V[dst] = d.Vc[i];
    d.DV[dst] = d.DVc[i];
    d.DK[dst] = d.DKc[i];
    d.PID[dst] = pid;
    d.KEYS[dst] = key;
}

// N6-N8: ComputeCountsKernel + NeighborhoodQueryWithCountsKernel (ParticleSearchKernels.cu:93-193)
// in one pass. G lanes test consecutive candidates of a cell together and compact the
// hits with a ballot, so the row keeps the reference's order (z, y, x cells, then cell
// order) and its cap of 70. The squared distance is computed without contraction,
// x^2 + y^2 + z^2 left to right, as the FP32 oracle does.
template <uint32_t G, bool REL>
__global__ void __launch_bounds__(kBlock) k_neighbors(Dev d) {
    VFD_COUNT_LAUNCH(d);
    const Group<G> grp;
    const uint32_t p = grp.p;
    if (p >= d.n || aborted(d)) return;
    const uint32_t sid = scene_of(d, p);
    const SceneDev& S = d.scenes[sid];
    const float4 xi = d.X[p];
    const float3 xa = abs_pos(d, S, xi);
    const float pos[3] = {xa.x, xa.y, xa.z};
    int gc[3];
#pragma unroll
    for (int k = 0; k < 3; k++) gc[k] = (int)floorf(__fmul_rn(__fsub_rn(pos[k], S.gridMin[k]), S.gridDelta[k]));
    const float h2 = S.h2;
    const uint32_t shift = (threadIdx.x & 31u) & ~(G - 1u);
    const uint32_t below = (1u << grp.lane) - 1u;
    uint32_t count = 0;
    uint32_t* row = d.NBR + (size_t)p * kRow;
    for (int dz = -1; dz < 2; dz++) {
        for (int dy = -1; dy < 2; dy++) {
            for (int dx = -1; dx < 2; dx++) {
                const int fx = gc[0] + dx, fy = gc[1] + dy, fz = gc[2] + dz;
                if (fx < 0 || fy < 0 || fz < 0 || fx >= (int)S.dim[0] || fy >= (int)S.dim[1] || fz >= (int)S.dim[2])
                    continue;
                const uint32_t c = S.cellBase + cell_key(S, fx, fy, fz);
                const uint32_t start = d.CELL_START[c], end = start + d.CELL_COUNT[c];
                for (uint32_t base = start; base < end; base += G) {
                    const uint32_t q = base + grp.lane;
                    bool hit = false;
                    if (q < end) {
                        const float3 e = pair_r<REL>(d, d.X[q], xi);
                        const float ex = e.x, ey = e.y, ez = e.z;
                        const float d2 =
                            __fadd_rn(__fadd_rn(__fmul_rn(ex, ex), __fmul_rn(ey, ey)), __fmul_rn(ez, ez));
                        hit = d2 < h2 && d2 > 0.0f;
                    }
                    const uint32_t bits = (__ballot_sync(grp.mask, hit) >> shift) & (G == 32u ? 0xffffffffu : ((1u << G) - 1u));
                    const uint32_t at = count + __popc(bits & below);
                    if (hit && at < kMaxNeighbors) row[at] = q;
                    count += __popc(bits);
                    if (count >= kMaxNeighbors) {
                        count = kMaxNeighbors;
                        goto done;
                    }
                }
            }
        }
    }
done:
    if (grp.lane == 0) {
        d.NCNT[p] = count;
        if (count == kMaxNeighbors) atomicOr(&d.scenes[sid].flags, 0x8u);
    }
    // one max per warp (per scene) into the bucket
    const uint32_t active = __activemask();
    const uint32_t leader = __ffs(active) - 1u;
    const uint32_t s0 = __shfl_sync(active, sid, leader);
    if (__all_sync(active, sid == s0)) {
        const uint32_t m = __reduce_max_sync(active, count);
        if ((threadIdx.x & 31u) == leader) atomicMax(max_bucket(d, s0, 1, blockIdx.x % kBuckets), m);
    } else if (grp.lane == 0) {
        atomicMax(max_bucket(d, sid, 1, blockIdx.x % kBuckets), count);
    }
}

// ---------------------------------------------------------------- launchers
void launch_search(const Dev& d, cudaStream_t s) {
    const uint32_t nb = blocks_for(d.n);
    VFD_LAUNCH("k_minmax", s, k_minmax<<<nb, kBlock, 0, s>>>(d));
    VFD_LAUNCH("k_grid", s, k_grid<<<1, 256, 0, s>>>(d));
    VFD_LAUNCH("k_clear_cells", s, k_clear_cells<<<1216, 256, 0, s>>>(d));
    VFD_LAUNCH("k_keys", s, k_keys<<<nb, kBlock, 0, s>>>(d));
    VFD_LAUNCH("k_scan_reduce", s, k_scan_reduce<<<d.scanBlocks, 256, 0, s>>>(d));
    VFD_LAUNCH("k_scan_top", s, k_scan_top<<<1, 1024, 0, s>>>(d));
    VFD_LAUNCH("k_scan_down", s, k_scan_down<<<d.scanBlocks, 256, 0, s>>>(d));
    VFD_LAUNCH("k_slots", s, k_slots<<<nb, kBlock, 0, s>>>(d));
    VFD_LAUNCH("k_rank_gather", s, k_rank_gather<<<nb, kBlock, 0, s>>>(d));
#define K_NEIGHBORS(G) k_neighbors<G, false>
#define K_NEIGHBORS_R(G) k_neighbors<G, true>
    if (d.cellRel) VFD_LAUNCH_LANES("k_neighbors", kTNeighbors, K_NEIGHBORS_R);
    else VFD_LAUNCH_LANES("k_neighbors", kTNeighbors, K_NEIGHBORS);
}

uint32_t scan_block_count(uint32_t cellCap) { return (cellCap + kScanItems - 1) / kScanItems; }

}  // namespace vfd
