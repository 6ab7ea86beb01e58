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
//   * neighbour lists are rows of kRow slots per particle (row-major), capped at 70
//     in the reference's z, y, x cell order; one pass, no count/scan/query split.
#include "dfsph_common.cuh"

namespace vfd {

constexpr uint32_t kScanItems = 1024u;  // cells per scan block (256 threads x 4)

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
// per scene, then the scene cell bases (exclusive scan) and the capacity check. With one
// scene the first warp folds the N1 buckets (lane b takes bucket b, an xor butterfly of
// min / max) instead of one thread walking them: 192 dependent L2 round trips were ~27 us,
// most of a small scene's search.
__global__ void k_grid(Dev d) {
    VFD_COUNT_LAUNCH(d);
    __shared__ uint32_t total;
    __shared__ int foldMin[3], foldMax[3];
    const bool one = d.nscenes == 1;
    if (one && threadIdx.x < 32u) {
        const uint32_t b = threadIdx.x;
        for (int k = 0; k < 3; k++) {  // fold the N1 buckets, reset them for the next step
            int32_t* qa = mm_bucket(d, 0, k, b);
            int32_t* qb = mm_bucket(d, 0, 3 + k, b);
            int mn = *qa, mx = *qb;
            *qa = INT_MAX;
            *qb = INT_MIN;
#pragma unroll
            for (int o = 16; o >= 1; o >>= 1) {
                mn = min(mn, __shfl_xor_sync(0xffffffffu, mn, o));
                mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
            }
            if (b == 0) {
                foldMin[k] = mn;
                foldMax[k] = mx;
            }
        }
        *max_bucket(d, 0, 1, b) = 0u;
    }
    __syncthreads();
    for (uint32_t s = threadIdx.x; s < d.nscenes; s += blockDim.x) {
        SceneDev& S = d.scenes[s];
        if (one) {
            for (int k = 0; k < 3; k++) {
                S.minCell[k] = foldMin[k];
                S.maxCell[k] = foldMax[k];
            }
        } else {
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
        }
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
// in one pass, one warp per cell. The particles of a cell share their 27 candidate cells,
// so the warp walks that candidate set once, 32 candidates per round (lane j < 27 holds
// cell j's range, a prefix over the lanes flattens them), and tests each candidate
// against every particle of the cell, whose positions sit in shared memory. A ballot per
// particle appends its hits in candidate order, so each row keeps the reference's order
// (z, y, x cells, then cell order) and its cap of 70. The squared distance is computed
// without contraction, x^2 + y^2 + z^2 left to right, as the FP32 oracle does. The
// cell's grid coordinates come from its first particle by the same formula a
// per-particle search would use on each of them (they agree: it is how they were binned).
// Each hit also goes into the particle's NBRC row (when kept) as its stencil position: the
// candidates of cells 3w, 3w + 1, 3w + 2 (an x-run) are positions 0.. of run w, and the entry
// is (w << 6) | position. A cell with an x-run of more than 64 candidates gets no NBRC rows;
// its particles are flagged kRowPath.
template <bool REL>
__global__ void __launch_bounds__(kBlock) k_neighbors(Dev d) {
    VFD_COUNT_LAUNCH(d);
    if (aborted(d)) return;
    __shared__ float4 sx[kBlock / 32u][32];
    const uint32_t lane = threadIdx.x & 31u, w = threadIdx.x >> 5;
    const uint32_t below = (1u << lane) - 1u;
    const uint32_t total = d.status[2];
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < total; c += warps) {
        const uint32_t cnt = d.CELL_COUNT[c];
        if (cnt == 0u) continue;
        const uint32_t start = d.CELL_START[c];
        const uint32_t sid = scene_of(d, start);
        const SceneDev& S = d.scenes[sid];
        const float3 xa = abs_pos(d, S, d.X[start]);
        const float pos[3] = {xa.x, xa.y, xa.z};
        int gc[3];
#pragma unroll
        for (int k = 0; k < 3; k++) gc[k] = (int)floorf(__fmul_rn(__fsub_rn(pos[k], S.gridMin[k]), S.gridDelta[k]));
        // lane j < 27: candidate cell j (dz, dy, dx = j / 9, j / 3 % 3, j % 3, each minus 1)
        uint32_t cs = 0u, cc = 0u;
        if (lane < 27u) {
            const int fx = gc[0] + (int)(lane % 3u) - 1, fy = gc[1] + (int)(lane / 3u % 3u) - 1,
                      fz = gc[2] + (int)(lane / 9u) - 1;
            if (fx >= 0 && fy >= 0 && fz >= 0 && fx < (int)S.dim[0] && fy < (int)S.dim[1] && fz < (int)S.dim[2]) {
                const uint32_t key = S.cellBase + cell_key(S, fx, fy, fz);
                cs = d.CELL_START[key];
                cc = d.CELL_COUNT[key];
            }
        }
        uint32_t incl = cc;
#pragma unroll
        for (uint32_t o = 1; o < 32u; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        const uint32_t ncand = __shfl_sync(0xffffffffu, incl, 31);
        const uint32_t excl = incl - cc;
        const float h2 = S.h2;
        // x-run w (lanes 3w, 3w + 1, 3w + 2): its candidate total decides whether masks fit
        const uint32_t runEnd = __shfl_sync(0xffffffffu, incl, min(3u * lane + 2u, 31u));
        const uint32_t runBeg = __shfl_sync(0xffffffffu, excl, min(3u * lane, 31u));
        const bool want = d.NBRC != nullptr && d.compactRows != 0u;
        const bool compact = want && !__any_sync(0xffffffffu, lane < 9u && runEnd - runBeg > kRunMax);
        const uint32_t rowFlag = (want && !compact) ? kRowPath : 0u;
        uint32_t mx = 0u;
        for (uint32_t k0 = 0; k0 < cnt; k0 += 32u) {
            const uint32_t kk = min(32u, cnt - k0);
            __syncwarp();
            if (lane < kk) sx[w][lane] = d.X[start + k0 + lane];
            __syncwarp();
            uint32_t count = 0u;  // neighbours so far of particle start + k0 + lane
            for (uint32_t base = 0; base < ncand; base += 32u) {
                const uint32_t i = base + lane;
                // candidate i lies in the last cell j whose flattened start is <= i
                uint32_t j = 0u;
#pragma unroll
                for (uint32_t step = 16u; step > 0u; step >>= 1) {
                    const uint32_t e = __shfl_sync(0xffffffffu, excl, min(j + step, 26u));
                    if (j + step <= 26u && e <= i) j += step;
                }
                const bool valid = i < ncand;
                const uint32_t q = checked_index(d.status, __shfl_sync(0xffffffffu, cs, j) +
                                                 (i - __shfl_sync(0xffffffffu, excl, j)), valid ? d.n : 0xFFFFFFFFu);
                // stencil position of this candidate: its x-run and place in the run
                const uint32_t run = j / 3u;
                const uint32_t entry = (run << 6) | (i - __shfl_sync(0xffffffffu, excl, 3u * run));
                const float4 xq = valid ? d.X[q] : make_float4(0.f, 0.f, 0.f, 0.f);
                for (uint32_t k = 0; k < kk; k++) {
                    const float3 e = pair_r<REL>(d, xq, sx[w][k]);
                    const float d2 = __fadd_rn(__fadd_rn(__fmul_rn(e.x, e.x), __fmul_rn(e.y, e.y)), __fmul_rn(e.z, e.z));
                    const bool hit = valid && d2 < h2 && d2 > 0.0f;
                    const uint32_t bits = __ballot_sync(0xffffffffu, hit);
                    const uint32_t ck = __shfl_sync(0xffffffffu, count, k);
                    const uint32_t at = ck + __popc(bits & below);
                    if (hit && at < kMaxNeighbors) {
                        d.NBR[(size_t)(start + k0 + k) * kRow + at] = q;
                        if (compact) d.NBRC[(size_t)(start + k0 + k) * kRow + at] = (uint16_t)entry;
                    }
                    if (lane == k) count = min(kMaxNeighbors, ck + __popc(bits));
                }
            }
            if (lane < kk) {
                d.NCNT[start + k0 + lane] = count | rowFlag;
                if (count == kMaxNeighbors) atomicOr(&d.scenes[sid].flags, 0x8u);
            }
            mx = max(mx, __reduce_max_sync(0xffffffffu, lane < kk ? count : 0u));
        }
        if (lane == 0) atomicMax(max_bucket(d, sid, 1, blockIdx.x % kBuckets), mx);
    }
}

// ---------------------------------------------------------------- launchers
// `profiled` = false launches without the per-kernel profiler hook (the allocation-free
// search must not create CUDA events, whatever another thread is profiling).
#define SEARCH_LAUNCH(name, ...)                 \
    do {                                         \
        if (profiled) VFD_LAUNCH(name, s, __VA_ARGS__); \
        else { __VA_ARGS__; }                    \
    } while (0)
void launch_search(const Dev& d, cudaStream_t s, bool profiled) {
    const uint32_t nb = blocks_for(d.n);
    SEARCH_LAUNCH("k_minmax", k_minmax<<<nb, kBlock, 0, s>>>(d));
    SEARCH_LAUNCH("k_grid", k_grid<<<1, 256, 0, s>>>(d));
    SEARCH_LAUNCH("k_clear_cells", k_clear_cells<<<1216, 256, 0, s>>>(d));
    SEARCH_LAUNCH("k_keys", k_keys<<<nb, kBlock, 0, s>>>(d));
    SEARCH_LAUNCH("k_scan_reduce", k_scan_reduce<<<d.scanBlocks, 256, 0, s>>>(d));
    SEARCH_LAUNCH("k_scan_top", k_scan_top<<<1, 1024, 0, s>>>(d));
    SEARCH_LAUNCH("k_scan_down", k_scan_down<<<d.scanBlocks, 256, 0, s>>>(d));
    SEARCH_LAUNCH("k_slots", k_slots<<<nb, kBlock, 0, s>>>(d));
    SEARCH_LAUNCH("k_rank_gather", k_rank_gather<<<nb, kBlock, 0, s>>>(d));
    // a warp per cell, a fixed grid striding over the cells the device counted
    const uint32_t nbrBlocks = 4u * d.batchBlocks;
    if (d.cellRel) SEARCH_LAUNCH("k_neighbors", k_neighbors<true><<<nbrBlocks, kBlock, 0, s>>>(d));
    else SEARCH_LAUNCH("k_neighbors", k_neighbors<false><<<nbrBlocks, kBlock, 0, s>>>(d));
}
#undef SEARCH_LAUNCH

uint32_t scan_block_count(uint32_t cellCap) { return (cellCap + kScanItems - 1) / kScanItems; }

}  // namespace vfd
