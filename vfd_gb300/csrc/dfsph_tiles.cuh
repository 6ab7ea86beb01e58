// Cell-tile neighbour loops of the solver iterations (pressure acceleration K5/K18, the
// Jacobi update K6/K19 and the viscosity CG product K14, DFSPHKernels.cu:317-432 and
// :758-842), the passes a step repeats tens of times.
//
// A block takes a tile of 2^L consecutive Morton cells (a 2x2x2 or 4x2x2 block of cells of
// edge h), stages the positions and the pass's neighbour field of every particle in the
// tile's halo (the tile grown by one cell on every side) into shared memory, and walks each
// particle's neighbours there. The halo is staged in z, y, x cell order, so the candidates
// of the three cells (x-1, x, x+1) of one (y, z) row -- an x-run -- are contiguous; the
// search gives every neighbour its stencil position (x-run w, place b in the run), stored
// as a 16-bit NBRC row beside the slot row, and the neighbour's staged index is then the
// run's first staged index (nine per particle, kept in shared memory) plus b. No per-pair
// slot or gradient is read from memory; gradW / r is recomputed from the table (the same
// midpoint lookup the row loops use). Each particle's data is read from L2 once per tile
// whose halo holds it ((TX+2)(TY+2)(TZ+2) / (TX TY TZ) times per pass, 8x for a 2x2x2
// tile, 6x for 4x2x2) instead of once per neighbour.
//
// G lanes share a particle and walk its row in lockstep rounds: lane l takes entries
// l, l + G, ..., U entries per round (as the row loops do), so no lane runs a loop of its
// own length; the group's partial sums meet in a shuffle tree and lane 0 writes the
// results. Particles flagged kRowPath by the search (an x-run of more than 64 candidates),
// and every particle of a tile whose halo holds more than the shared-memory capacity, walk
// their slot rows from global memory instead; both walks evaluate the same pair terms.
//
// Reductions (Jacobi residual, p . Ap): each lane 0 accumulates its particles' FP32 terms
// as an FP32 pair across the block's tiles; the block folds them (warp_sum_pair
// arithmetic) and adds one FP64 atomic per scene it served.
#pragma once

#include "dfsph_common.cuh"

namespace vfd {

constexpr uint32_t kTileBlock = 128u;  // threads per tile block

// A tile of 2^L consecutive Morton keys: the local Morton bits go to x, y, z in turn.
template <uint32_t L>
struct TileShape {
    static constexpr uint32_t T = 1u << L;
    static constexpr uint32_t TX = 1u << ((L + 2u) / 3u), TY = 1u << ((L + 1u) / 3u), TZ = 1u << (L / 3u);
    static constexpr uint32_t HX = TX + 2u, HY = TY + 2u, HZ = TZ + 2u, HALO = HX * HY * HZ;
    // staged particles: 12 per halo cell on average (cells of the configurations hold ~10
    // on average and 18 at most; a halo sums 64-96 of them); a fuller halo walks rows
    static constexpr uint32_t CAP = 12u * HALO;
};

// Per-thread FP32-pair accumulation of a pass's reduction term across tiles, folded per
// scene into the FP64 buckets (one atomic per block and scene).
struct TileSum {
    float hi = 0.0f, lo = 0.0f;
    int scene = -1;
    __device__ __forceinline__ void add(float v) { pair_add(hi, lo, v, 0.0f); }
    // All threads of the block call this with the same arguments.
    __device__ void flush(const Dev& d, int slot) {
        __shared__ float2 part[kTileBlock / 32u];
        float h = hi, l = lo;
#pragma unroll
        for (int o = 16; o >= 1; o >>= 1) {
            const float h2 = __shfl_xor_sync(0xffffffffu, h, o);
            const float l2 = __shfl_xor_sync(0xffffffffu, l, o);
            pair_add(h, l, h2, l2);
        }
        if ((threadIdx.x & 31u) == 0u) part[threadIdx.x >> 5] = make_float2(h, l);
        __syncthreads();
        if (threadIdx.x == 0 && scene >= 0) {
            float a = 0.0f, b = 0.0f;
            for (uint32_t w = 0; w < kTileBlock / 32u; w++) pair_add(a, b, part[w].x, part[w].y);
            const double t = pair_value(make_float2(a, b));
            if (t != 0.0) atomicAdd(acc_bucket(d, (uint32_t)scene, slot, blockIdx.x % kBuckets), t);
        }
        __syncthreads();
        hi = lo = 0.0f;
    }
};

// The tile loop (the calling kernel counts its launch). Op supplies, as static device
// functions and members:
//   kField            whether a per-particle float4 field is staged beside the position
//   kReduce, kSlot    whether finish() returns a term summed into accumulator kSlot
//   active(S)         whether scene S runs this pass
//   field(d, q)       the staged field of particle q
//   Own, Acc          per-particle own data and the pair-sum type (float or float3)
//   load(d, p, S, o)  the particle's own data
//   pair(d, o, xq, fq, acc)  one neighbour's term
//   finish(d, p, S, o, acc, ncnt)  lane 0, after the group sum: writes the outputs and
//                     returns the reduction term
template <class Op, uint32_t L, uint32_t G, bool REL>
__device__ __forceinline__ void tile_pass(const Dev& d) {
    using TS = TileShape<L>;
    constexpr uint32_t CAP = TS::CAP;
    constexpr uint32_t U = 4u;                   // row entries per lane and round
    constexpr uint32_t PER = kTileBlock / G;     // particles per chunk
    static_assert(TS::HALO <= 255u, "staged cell index is one byte");
    extern __shared__ float4 tileSmem[];
    float4* sx = tileSmem;
    float4* sf = tileSmem + CAP;
    __shared__ uint32_t hStart[TS::HALO], hOff[TS::HALO + 1u];
    __shared__ uint8_t cellOf[CAP];              // halo cell of each staged particle
    __shared__ uint32_t runBase[PER][9];         // first staged index of each x-run, per particle
    __shared__ uint32_t tInfo[4];                // first, last, scene, skip
    if (is_aborted(d)) return;
    const uint32_t nTiles = d.status[2] >> L;
    const uint32_t gl = threadIdx.x % G, pp = threadIdx.x / G;
    const uint32_t gmask = G == 32u ? 0xffffffffu : (((1u << G) - 1u) << ((threadIdx.x & 31u) & ~(G - 1u)));
    TileSum sum;
    for (uint32_t tile = blockIdx.x; tile < nTiles; tile += gridDim.x) {
        const uint32_t k0 = tile << L;
        if (threadIdx.x == 0) {
            const uint32_t first = d.CELL_START[k0];
            const uint32_t kl = k0 + TS::T - 1u;
            const uint32_t last = d.CELL_START[kl] + d.CELL_COUNT[kl];
            uint32_t skip = first >= last ? 1u : 0u, sid = 0u;
            if (!skip) {
                sid = scene_of(d, first);
                if (!Op::active(d.scenes[sid])) skip = 1u;
            }
            tInfo[0] = first;
            tInfo[1] = last;
            tInfo[2] = sid;
            tInfo[3] = skip;
        }
        __syncthreads();
        const uint32_t first = tInfo[0], last = tInfo[1], sid = tInfo[2];
        if (tInfo[3]) {
            __syncthreads();  // tInfo is rewritten by the next tile
            continue;
        }
        if (Op::kReduce && (int)sid != sum.scene) {
            sum.flush(d, Op::kSlot);
            sum.scene = (int)sid;
        }
        const SceneDev& S = d.scenes[sid];
        // the tile's corner cell: meta block of the key, then the Morton bits inside it
        const uint32_t kl = k0 - S.cellBase, meta = kl >> 9, low = kl & 511u;
        const uint32_t mx = meta % S.meta[0], myz = meta / S.meta[0];
        const int ox = (int)(mx * 8u + compact3(low)) - 1;
        const int oy = (int)((myz % S.meta[1]) * 8u + compact3(low >> 1)) - 1;
        const int oz = (int)((myz / S.meta[1]) * 8u + compact3(low >> 2)) - 1;
        // halo cells in z, y, x order: ranges, then offsets (one warp scans)
        for (uint32_t t = threadIdx.x; t < TS::HALO; t += kTileBlock) {
            const int cx = ox + (int)(t % TS::HX), cy = oy + (int)((t / TS::HX) % TS::HY),
                      cz = oz + (int)(t / (TS::HX * TS::HY));
            uint32_t cs = 0u, cc = 0u;
            if (cx >= 0 && cy >= 0 && cz >= 0 && cx < (int)S.dim[0] && cy < (int)S.dim[1] && cz < (int)S.dim[2]) {
                const uint32_t key = S.cellBase + cell_key(S, cx, cy, cz);
                cs = d.CELL_START[key];
                cc = d.CELL_COUNT[key];
            }
            hStart[t] = cs;
            hOff[t + 1u] = cc;
        }
        __syncthreads();
        if (threadIdx.x < 32u) {
            const uint32_t lane = threadIdx.x;
            uint32_t carry = 0u;
            for (uint32_t b = 0; b < TS::HALO; b += 32u) {
                const uint32_t t = b + lane;
                uint32_t v = t < TS::HALO ? hOff[t + 1u] : 0u;
#pragma unroll
                for (uint32_t o = 1; o < 32u; o <<= 1) {
                    const uint32_t u = __shfl_up_sync(0xffffffffu, v, o);
                    if (lane >= o) v += u;
                }
                if (t < TS::HALO) hOff[t + 1u] = carry + v;
                carry += __shfl_sync(0xffffffffu, v, 31);
            }
            if (lane == 0) hOff[0] = 0u;
        }
        __syncthreads();
        const uint32_t staged = hOff[TS::HALO];
        const bool fits = staged <= CAP;
        if (fits) {
            // each halo cell marks its staged range, then every thread copies its elements
            for (uint32_t t = threadIdx.x; t < TS::HALO; t += kTileBlock)
                for (uint32_t i = hOff[t]; i < hOff[t + 1u]; i++) cellOf[i] = (uint8_t)t;
            __syncthreads();
            for (uint32_t i = threadIdx.x; i < staged; i += kTileBlock) {
                const uint32_t c = cellOf[i];
                const uint32_t q = checked_index(d.status, hStart[c] + (i - hOff[c]), d.n);
                sx[i] = d.X[q];
                if (Op::kField) sf[i] = Op::field(d, q);
            }
        }
        __syncthreads();
        for (uint32_t pb = first; pb < last; pb += PER) {
            const uint32_t p = pb + pp;
            if (p < last) {  // whole groups take this branch together
                typename Op::Own own;
                Op::load(d, p, S, own);
                typename Op::Acc acc{};
                const uint32_t ncnt = d.NCNT[p];
                const uint32_t cnt = ncnt & kCountMask;
                if (fits && !(ncnt & kRowPath)) {
                    const uint32_t m = d.KEYS[p] - k0;  // local Morton index of the particle's cell
                    const uint32_t lx = compact3(m), ly = compact3(m >> 1), lz = compact3(m >> 2);
                    for (uint32_t w = gl; w < 9u; w += G)
                        runBase[pp][w] = hOff[((lz + w / 3u) * TS::HY + ly + w % 3u) * TS::HX + lx];
                    __syncwarp(gmask);
                    const uint16_t* row = d.NBRC + (size_t)p * kRow;
                    for (uint32_t base = 0; base < cnt; base += U * G) {
                        uint32_t e[U];
#pragma unroll
                        for (uint32_t u = 0; u < U; u++) {
                            const uint32_t j = base + gl + u * G;
                            e[u] = j < cnt ? (uint32_t)__ldcs(row + j) : 0xFFFFu;
                        }
#pragma unroll
                        for (uint32_t u = 0; u < U; u++) {
                            if (e[u] == 0xFFFFu) continue;
                            const uint32_t jj = checked_index(d.status, runBase[pp][e[u] >> 6] + (e[u] & 63u), staged);
                            Op::pair(d, own, sx[jj], Op::kField ? sf[jj] : make_float4(0.f, 0.f, 0.f, 0.f), acc);
                        }
                    }
                } else {
                    const uint32_t* row = d.NBR + (size_t)p * kRow;
                    for (uint32_t j = gl; j < cnt; j += G) {
                        const uint32_t q = checked_index(d.status, __ldg(row + j), d.n);
                        Op::pair(d, own, d.X[q], Op::kField ? Op::field(d, q) : make_float4(0.f, 0.f, 0.f, 0.f), acc);
                    }
                }
                acc = group_sum<G>(gmask, acc);
                if (gl == 0u) {
                    const float term = Op::finish(d, p, S, own, acc, ncnt);
                    if (Op::kReduce) sum.add(term);
                }
            }
            __syncwarp();  // runBase of this chunk is reused by the next
        }
        __syncthreads();  // the halo and tInfo are rewritten by the next tile
    }
    if (Op::kReduce) sum.flush(d, Op::kSlot);
}

}  // namespace vfd
