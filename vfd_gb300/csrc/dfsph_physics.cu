// DFSPH physics kernels of one step (Simulation/DFSPH/DFSPHKernels.cu:24-1046)
// and the device-side control of its three solver loops
// (DFSPHImplementation.cu:443-808).
//
// Neighbour loops run G lanes per particle (Group<G>): the lanes stride the
// particle's neighbour row, so one warp-wide gather reads a few runs of
// consecutive cell-sorted slots instead of 32 scattered ones, and the partial
// sums meet in a shuffle tree. Element-wise kernels run one thread per particle.
//
// Fusions relative to the reference's 22 kernels:
//   K2+K3 (density, factor) -> k_density_factor, which also stores the summed
//         boundary gradient GB = sum_b Vb gradW(x - xb) that K4-K7, K17-K20 reuse;
//   K7+K8 -> k_div_finish; K15+T1 (CFL max) -> k_visc_finish;
//   K20+K21 -> k_pres_finish; K6/K19 fused with their FP64 residual reduction;
//   the CG's thrust transforms and reductions -> k_cg_update / k_cg_p (FP64 dots);
//   the boundary part of the viscosity SpMV is a per-particle 3x3 matrix built once
//   per step by k_visc_precond.
// Loop control: after each iteration a one-block controller updates every
// scene's iteration count, error and active flag and sets the CUDA-graph while
// condition (or, in eager mode, a flag the host reads).
#include <cfloat>

#include "dfsph_common.cuh"
#include "dfsph_tiles.cuh"

namespace vfd {

enum LoopId { kLoopDiv = 0, kLoopCG = 1, kLoopPres = 2 };

__device__ __forceinline__ bool aborted_p(const Dev& d) { return is_aborted(d); }

__device__ __forceinline__ void set_condition(const Dev& d, int loop, uint32_t value) {
    if (d.condHandle[loop]) cudaGraphSetConditional((cudaGraphConditionalHandle)d.condHandle[loop], value);
    d.status[4 + loop] = value;
}

// Batches: lists the scenes for which active(s) holds into loop `loop`'s work list
// (prefix sums of their particle counts by a block-wide scan). One block of 256 threads,
// called by all of them after the scenes' flags are final.
template <class F>
__device__ void build_work_list(const Dev& d, int loop, F active) {
    __shared__ uint32_t scanP[256], scanA[256];
    __shared__ uint32_t runP, runA;
    uint32_t* w = d.WORK + (size_t)loop * d.workStride;
    uint32_t* pre = w + 2;
    uint32_t* beg = w + 2 + d.nscenes;
    if (threadIdx.x == 0) runP = runA = 0u;
    __syncthreads();
    for (uint32_t c = 0; c < d.nscenes; c += blockDim.x) {
        const uint32_t sc = c + threadIdx.x;
        const bool a = sc < d.nscenes && active(sc);
        const uint32_t cnt = a ? d.scenes[sc].count : 0u;
        scanP[threadIdx.x] = cnt;
        scanA[threadIdx.x] = a ? 1u : 0u;
        __syncthreads();
        for (uint32_t off = 1; off < blockDim.x; off <<= 1) {
            const uint32_t tp = threadIdx.x >= off ? scanP[threadIdx.x - off] : 0u;
            const uint32_t ta = threadIdx.x >= off ? scanA[threadIdx.x - off] : 0u;
            __syncthreads();
            scanP[threadIdx.x] += tp;
            scanA[threadIdx.x] += ta;
            __syncthreads();
        }
        if (a) {
            const uint32_t idx = runA + scanA[threadIdx.x] - 1u;
            pre[idx] = runP + scanP[threadIdx.x] - cnt;
            beg[idx] = d.scenes[sc].begin;
        }
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1u) {
            runP += scanP[threadIdx.x];
            runA += scanA[threadIdx.x];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        w[0] = runP;
        w[1] = runA;
    }
}

// Grid-stride walk of a batch loop's work list: base_ is the first virtual index of the
// block's current chunk of per_ particles (blockDim.x / G of them).
#define BATCH_LOOP(LOOP, G)                                  \
    const uint32_t per_ = blockDim.x / (G);                  \
    const uint32_t total_ = work_total(d, (LOOP));           \
    for (uint32_t base_ = blockIdx.x * per_; base_ < total_; base_ += gridDim.x * per_)

// Scene of the whole chunk, or -1 when it spans several.
__device__ __forceinline__ int chunk_scene(const Dev& d, int loop, uint32_t base, uint32_t per, uint32_t total) {
    uint32_t s0, s1;
    work_slot(d, loop, base, s0);
    work_slot(d, loop, min(base + per, total) - 1u, s1);
    return s0 == s1 ? (int)s0 : -1;
}

struct Nbr {
    const uint32_t* row;
    const uint2* ng;
    uint32_t count, flags;
#ifdef VFD_BOUNDS_CHECK
    uint32_t n;
    uint32_t* status;
    __device__ __forceinline__ uint32_t check(uint32_t q) const { return checked_index(status, q, n); }
#else
    __device__ __forceinline__ uint32_t check(uint32_t q) const { return q; }
#endif
    __device__ __forceinline__ uint32_t operator[](uint32_t j) const { return check(__ldg(row + j)); }
};
__device__ __forceinline__ Nbr neighbors(const Dev& d, uint32_t p) {
    const uint32_t w = d.NCNT[p];
#ifdef VFD_BOUNDS_CHECK
    return Nbr{d.NBR + (size_t)p * kRow, d.NG + (size_t)p * kRow, w & kCountMask, w, d.n, d.status};
#else
    return Nbr{d.NBR + (size_t)p * kRow, d.NG + (size_t)p * kRow, w & kCountMask, w};
#endif
}

// kappa (or kappa_v) of particle p, mirrored into X[p].w for the neighbours' gathers.
// (Cell-relative positions keep their anchor in X.w; the neighbours then read kappa itself.)
__device__ __forceinline__ void set_kappa(const Dev& d, uint32_t p, float k) {
    if (!d.cellRel) reinterpret_cast<float*>(d.X)[4 * (size_t)p + 3] = k;
}

// Row entries per lane and round of a neighbour loop (other depths measured slower).
constexpr uint32_t kUnroll = 4u;

// Neighbour loop of one group. In a round the group covers U*G consecutive row
// entries and lane l takes entries l, l + G, ..., l + (U-1)G, so at each step the
// group's lanes read consecutive entries -- usually consecutive slots of one cell,
// which the gathers then fetch in one or two sectors. The first round's index loads do
// not wait for the count (rows have 72 slots, entries past the count are masked), so
// the count, the indices and the particle's own fields are fetched together; within a
// round the U gathers per lane are independent. Masked entries use the particle itself
// as a stand-in index. The row and gradient streams are read once per pass, so they
// are loaded with the evict-first hint (ld.global.cs) to leave L2 to the gathered
// fields.
template <uint32_t G, bool WITH_GS, class F>
__device__ __forceinline__ void for_neighbors(const Group<G>& grp, const Nbr& nb, uint32_t self, F&& f) {
    constexpr uint32_t U = kUnroll;
    static_assert(U * G <= kRow, "first round must stay inside the row");
    uint32_t q[U];
    float g[U];
#pragma unroll
    for (uint32_t u = 0; u < U; u++) {
        if (WITH_GS) {
            const uint2 e = __ldcs(nb.ng + grp.lane + u * G);
            q[u] = e.x;
            g[u] = __uint_as_float(e.y);
        } else {
            q[u] = __ldcs(nb.row + grp.lane + u * G);
            g[u] = 0.0f;
        }
    }
    for (uint32_t base = 0; base < nb.count; base += U * G) {
        if (base > 0) {
#pragma unroll
            for (uint32_t u = 0; u < U; u++) {
                const uint32_t j = base + grp.lane + u * G;
                if (WITH_GS) {
                    const uint2 e = j < nb.count ? __ldcs(nb.ng + j) : make_uint2(self, 0u);
                    q[u] = e.x;
                    g[u] = __uint_as_float(e.y);
                } else {
                    q[u] = j < nb.count ? __ldcs(nb.row + j) : self;
                    g[u] = 0.0f;
                }
            }
        }
#pragma unroll
        for (uint32_t u = 0; u < U; u++) {
            const uint32_t j = base + grp.lane + u * G;
            const bool ok = j < nb.count;
            f(ok ? nb.check(q[u]) : self, g[u], j, ok);
        }
    }
}

// One particle's term of a CG dot product: the FP32 dot of its two vectors (no
// contraction, x + y then z, as the FP32 oracle forms it); the sum over particles is
// FP64-accurate (scene_accumulate). FP64 arithmetic runs at a small fraction of the
// FP32 rate on this GPU, so the per-particle terms stay FP32, as every per-particle sum
// of the reference does.
__device__ __forceinline__ float dot_term(float3 a, float3 b) {
    return __fadd_rn(__fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)), __fmul_rn(a.z, b.z));
}

// W and gradW of one pair from one table position (GetW / GetGradientW keep their own
// range tests: |r|^2 <= R^2 for W, |r| <= R for gradW).
__device__ __forceinline__ void kernel_wg(const Dev& d, float3 r, float& w, float& gs) {
    const float r2 = dot3(r, r);
    const float rl = fast_sqrt(r2);
    if (d.analytic) {
        w = r2 <= d.radius2 ? spline_w(d, rl) : 0.0f;
        gs = rl <= d.radius ? spline_gs(d, rl) : 0.0f;
        return;
    }
    const uint32_t pos = table_pos(d, rl);
    w = r2 <= d.radius2 ? __ldg(d.WM + pos) : 0.0f;
    gs = rl <= d.radius ? __ldg(d.GM + pos) : 0.0f;
}

#define GROUP_PROLOGUE(G)                    \
    const Group<G> grp;                      \
    const uint32_t p = grp.p;                \
    if (p >= d.n || aborted_p(d)) return;

// ---------------------------------------------------------------------------
// K2 + K3: ComputeDensityKernel (:152-187) and ComputeDFSPHFactorKernel (:189-231).
// With DIV, also K4 (ComputeDensityChangeKernel, :483-529) for the scenes that run the
// divergence solve: it walks the same pairs and needs only the particle's own factor
// and boundary gradient and each pair's gradW, so it rides along (the terms and order of
// velocity_divergence, which K17 uses).
template <uint32_t G, bool REL, bool DIV = false>
__global__ void __launch_bounds__(kMaxBlock) k_density_factor(Dev d) {
    VFD_COUNT_LAUNCH(d);
    GROUP_PROLOGUE(G)
    const SceneDev& S = d.scenes[scene_of(d, p)];
    const float4 xi4 = d.X[p];
    const float3 xi = f3(xi4);
    const Nbr nb = neighbors(d, p);
    float wsum = 0.0f, g2 = 0.0f, sdiv = 0.0f;
    float3 gi = make_float3(0.f, 0.f, 0.f);
    const float V = S.volume;
    const bool div = DIV && S.enableDiv;
    const float3 vi = div ? f3(d.V[p]) : make_float3(0.f, 0.f, 0.f);
    uint2* ngRow = d.NG + (size_t)p * kRow;
    for_neighbors<G, false>(grp, nb, p, [&](uint32_t q, float, uint32_t j, bool ok) {
        const float3 r = pair_r<REL>(d, xi4, d.X[q]);
        float w, gs;
        kernel_wg(d, r, w, gs);
        const float3 vq = div ? f3(d.V[q]) : make_float3(0.f, 0.f, 0.f);
        if (!ok) return;
        __stcs(ngRow + j, make_uint2(q, __float_as_uint(gs)));
        wsum += w;
        const float3 gj = (-V * gs) * r;
        g2 += dot3(gj, gj);
        gi -= gj;
        if (div) sdiv += dot3(vi - vq, gs * r);
    });
    wsum = grp.sum(wsum);
    g2 = grp.sum(g2);
    gi = grp.sum(gi);
    if (DIV) sdiv = grp.sum(sdiv);
    if (grp.lane != 0) return;
    float rhoB = 0.0f;
    float3 gb = make_float3(0.f, 0.f, 0.f);
    if (nb.flags & kHasBoundary) {
        for (uint32_t b = 0; b < S.bodyCount; b++) {
            const float4 xb = d.XB[(size_t)b * d.stride + p];
            if (xb.w > 0.0f) {
                const float3 r = xi - f3(xb);
                float w, gs;
                kernel_wg(d, r, w, gs);
                rhoB += xb.w * w;
                gb += (xb.w * gs) * r;
            }
        }
    }
    gi += gb;
    d.RHO[p] = (V * d.wZero + V * wsum + rhoB) * S.rho0;
    g2 += dot3(gi, gi);
    const float alpha = g2 > kEps ? 1.0f / g2 : 0.0f;
    d.GB[p] = f4(gb, 0.0f);
    if (!div) {
        d.ALPHA[p] = alpha;
        return;
    }
    // K4 (:498-528)
    float rhoAdv = sdiv * V;
    if (nb.flags & kHasBoundary) rhoAdv += dot3(vi, gb);
    rhoAdv = nb.count < 20u ? 0.0f : fmaxf(rhoAdv, 0.0f);
    d.RHOADV[p] = rhoAdv;
    const float alphaDt = alpha * S.dtInv;
    d.ALPHA[p] = alphaDt;
    d.KAPPAV[p] = rhoAdv * alphaDt;
    set_kappa(d, p, rhoAdv * alphaDt);
}

// Sum_j (vi - vj) . gradW_ij * V + vi . GB  (K4 :498-522, K17 :253-271); valid on lane 0.
template <uint32_t G, bool REL>
__device__ __forceinline__ float velocity_divergence(const Dev& d, const Group<G>& grp, uint32_t p, const SceneDev& S,
                                                     const Nbr& nb, float4 xi, float3 vi) {
    float s = 0.0f;
    for_neighbors<G, true>(grp, nb, p, [&](uint32_t q, float gs, uint32_t, bool ok) {
        const float3 r = pair_r<REL>(d, xi, d.X[q]);
        const float3 vq = f3(d.V[q]);
        const float t = dot3(vi - vq, gs * r);
        if (ok) s += t;
    });
    s = grp.sum(s) * S.volume;
    if (nb.flags & kHasBoundary) s += dot3(vi, f3(d.GB[p]));
    return s;
}

// Pressure acceleration from kappa (K5 :388-432, K7 :555-602, K18 :342-386, K20 :434-481);
// valid on lane 0. NS: the pass reads the slot rows only and forms each pair's gradW / r
// from the table itself (as the density pass did), instead of reading it from the
// per-pair stream: half the streamed bytes for a table lookup per pair.
template <bool DIV, uint32_t G, bool REL, bool NS = false>
__device__ __forceinline__ float3 pressure_accel(const Dev& d, const Group<G>& grp, uint32_t p, const SceneDev& S,
                                                 const Nbr& nb) {
    const float* kap = DIV ? d.KAPPAV : d.KAPPA;
    const float ki = kap[p];
    const float4 xi = d.X[p];
    const float V = S.volume;
    float3 a = make_float3(0.f, 0.f, 0.f);
    for_neighbors<G, !NS>(grp, nb, p, [&](uint32_t q, float gsStream, uint32_t, bool ok) {
        const float4 xq = d.X[q];
        const float sum = ki + (REL ? kap[q] : xq.w);
        const float3 r = pair_r<REL>(d, xi, xq);
        const float gs = NS ? grad_factor(d, r) : gsStream;
        if (ok && fabsf(sum) > kEps) a += (sum * (-V * gs)) * r;
    });
    a = grp.sum(a);
    if (fabsf(ki) > kEps && (nb.flags & kHasBoundary)) a += ki * (-f3(d.GB[p]));
    return a;
}

// K5 / K18.
template <bool DIV, uint32_t G, bool REL, bool NS = false>
__global__ void __launch_bounds__(kMaxBlock) k_pressure_accel(Dev d) {
    VFD_COUNT_LAUNCH(d);
    GROUP_PROLOGUE(G)
    const SceneDev& S = d.scenes[scene_of(d, p)];
    if (!(DIV ? S.div.active : S.pres.active)) return;
    const Nbr nb = neighbors(d, p);
    const float3 a = pressure_accel<DIV, G, REL, NS>(d, grp, p, S, nb);
    if (grp.lane == 0) d.AP[p] = f4(a, 0.0f);
}

// K5 / K18 of a batch: the scenes still iterating, from the loop's work list.
template <bool DIV, uint32_t G, bool REL>
__global__ void __launch_bounds__(kMaxBlock) k_pressure_accel_b(Dev d) {
    VFD_COUNT_LAUNCH(d);
    if (aborted_p(d)) return;
    const int L = DIV ? kLoopDiv : kLoopPres;
    BATCH_LOOP(L, G) {
        const uint32_t vp = base_ + threadIdx.x / G;
        if (vp >= total_) continue;
        uint32_t sid;
        const uint32_t p = work_slot(d, L, vp, sid);
        const Group<G> grp(p);
        const Nbr nb = neighbors(d, p);
        const float3 a = pressure_accel<DIV, G, REL>(d, grp, p, d.scenes[sid], nb);
        if (grp.lane == 0) d.AP[p] = f4(a, 0.0f);
    }
}

// K6 DivergenceSolveIterationKernel (:531-553) / K19 PressureSolveIterationKernel (:317-340),
// each with ComputeDensityPressureForce (:280-315) and the FP64-accurate residual sum.
template <bool DIV, uint32_t G, bool REL, bool NS = false>
__device__ __forceinline__ float jacobi_item(const Dev& d, const Group<G>& grp, uint32_t p, const SceneDev& S) {
    float res = 0.0f;
    const Nbr nb = neighbors(d, p);
    const float4 xi = d.X[p];
    const float3 ai = f3(d.AP[p]);
    float f = 0.0f;
    for_neighbors<G, !NS>(grp, nb, p, [&](uint32_t q, float gsStream, uint32_t, bool ok) {
        const float3 r = pair_r<REL>(d, xi, d.X[q]);
        const float gs = NS ? grad_factor(d, r) : gsStream;
        const float3 aq = f3(d.AP[q]);
        const float t = dot3(ai - aq, gs * r);
        if (ok) f += t;
    });
    f = grp.sum(f) * S.volume;
    if (grp.lane == 0) {
        if (nb.flags & kHasBoundary) f += dot3(ai, f3(d.GB[p]));
        float r;
        if (DIV) {
            f *= S.dt;
            r = nb.count < 20u ? 0.0f : fminf(-d.RHOADV[p] - f, 0.0f);
            const float k = d.KAPPAV[p] - r * d.ALPHA[p];
            d.KAPPAV[p] = k;
            set_kappa(d, p, k);
        } else {
            f *= S.dt2;
            r = fminf(1.0f - d.RHOADV[p] - f, 0.0f);
            const float k = d.KAPPA[p] - r * d.ALPHA[p];
            d.KAPPA[p] = k;
            set_kappa(d, p, k);
        }
        d.RES[p] = r;
        res = r;
    }
    return res;
}

template <bool DIV, uint32_t G, bool REL, bool NS = false>
__global__ void __launch_bounds__(kMaxBlock) k_jacobi_iter(Dev d) {
    VFD_COUNT_LAUNCH(d);
    const Group<G> grp;
    const uint32_t p = grp.p;
    const bool inRange = p < d.n && !aborted_p(d);
    const uint32_t sid = inRange ? scene_of(d, p) : 0u;
    const SceneDev& S = d.scenes[sid];
    const bool active = inRange && (DIV ? S.div.active : S.pres.active);
    float res = 0.0f;
    if (active) res = jacobi_item<DIV, G, REL, NS>(d, grp, p, S);
    const float v[1] = {res};
    const int slot[1] = {0};
    scene_accumulate<1, G>(d, sid, active && grp.lane == 0, v, slot);
}

// The same for a batch (work list of the loop).
template <bool DIV, uint32_t G, bool REL>
__global__ void __launch_bounds__(kMaxBlock) k_jacobi_iter_b(Dev d) {
    VFD_COUNT_LAUNCH(d);
    if (aborted_p(d)) return;
    const int L = DIV ? kLoopDiv : kLoopPres;
    BATCH_LOOP(L, G) {
        const uint32_t vp = base_ + threadIdx.x / G;
        const bool in = vp < total_;
        uint32_t sid = 0;
        const uint32_t p = in ? work_slot(d, L, vp, sid) : 0u;
        float res = 0.0f;
        if (in) {
            const Group<G> grp(p);
            res = jacobi_item<DIV, G, REL>(d, grp, p, d.scenes[sid]);
        }
        const float v[1] = {res};
        const int slot[1] = {0};
        scene_accumulate_core<1, G>(d, chunk_scene(d, L, base_, per_, total_), sid, in && threadIdx.x % G == 0u, v, slot);
    }
}

// Loop start: the reference's while condition evaluated with error 0, iteration 0
// (DFSPHImplementation.cu:461, :532).
template <bool DIV>
__global__ void k_ctrl_jacobi_init(Dev d) {
    VFD_COUNT_LAUNCH(d);
    __shared__ uint32_t any;
    if (threadIdx.x == 0) any = 0;
    __syncthreads();
    const bool ab = aborted_p(d);
    for (uint32_t s = threadIdx.x; s < d.nscenes; s += blockDim.x) {
        SceneDev& S = d.scenes[s];
        LoopState& L = DIV ? S.div : S.pres;
        L.it = 0;
        L.err = 0.0f;
        const uint32_t mn = DIV ? S.minIterD : S.minIterP, mx = DIV ? S.maxIterD : S.maxIterP;
        const bool enabled = (DIV ? S.enableDiv != 0 : true) && S.count > 0 && !ab;
        const float eta = DIV ? S.dtInv * S.maxErrD * 0.0001f * S.rho0 : S.maxErrP * 0.0001f * S.rho0;
        L.active = (enabled && ((0.0f > eta) || 0u < mn) && 0u < mx) ? 1u : 0u;
        if (L.active) atomicOr(&any, 1u);
    }
    __syncthreads();
    if (d.nscenes > 1)
        build_work_list(d, DIV ? kLoopDiv : kLoopPres,
                        [&](uint32_t sc) { return (DIV ? d.scenes[sc].div.active : d.scenes[sc].pres.active) != 0u; });
    if (threadIdx.x == 0) set_condition(d, DIV ? kLoopDiv : kLoopPres, any);
}

// After an iteration: error = -rho0 * sum(res) / N (order-independent form of the
// reference's thrust::minus fold, DFSPHImplementation.cu:483-491, :554-563). Returns
// whether the scene runs another iteration.
template <bool DIV>
__device__ __forceinline__ bool jacobi_control(SceneDev& S, double sum) {
    LoopState& L = DIV ? S.div : S.pres;
    const double err = -(double)S.rho0 * sum / (double)S.count;
    L.err = (float)err;
    L.it++;
    const uint32_t mn = DIV ? S.minIterD : S.minIterP, mx = DIV ? S.maxIterD : S.maxIterP;
    const float eta = DIV ? S.dtInv * S.maxErrD * 0.0001f * S.rho0 : S.maxErrP * 0.0001f * S.rho0;
    const bool again = (err > (double)eta || L.it < mn) && L.it < mx;
    if (!again && L.it >= mx && err > (double)eta) S.flags |= DIV ? 0x2u : 0x1u;
    L.active = again ? 1u : 0u;
    return again;
}

// The loop controllers run as one block. With one scene its first warp folds the
// buckets together (fold_acc_warp) and lane 0 takes the decisions; a batch gives each
// scene a thread.
template <bool DIV>
__global__ void k_ctrl_jacobi(Dev d) {
    VFD_COUNT_LAUNCH(d);
    if (d.nscenes == 1) {
        if (threadIdx.x >= 32u) return;
        SceneDev& S = d.scenes[0];
        const bool act = (DIV ? S.div.active : S.pres.active) != 0u;
        const double sum = act ? fold_acc_warp(d, 0, 0, threadIdx.x) : 0.0;
        if (threadIdx.x == 0) {
            const bool again = act && jacobi_control<DIV>(S, sum);
            set_condition(d, DIV ? kLoopDiv : kLoopPres, (again && !aborted_p(d)) ? 1u : 0u);
        }
        return;
    }
    __shared__ uint32_t any;
    if (threadIdx.x == 0) any = 0;
    __syncthreads();
    for (uint32_t s = threadIdx.x; s < d.nscenes; s += blockDim.x) {
        SceneDev& S = d.scenes[s];
        if (!(DIV ? S.div.active : S.pres.active)) continue;
        if (jacobi_control<DIV>(S, fold_acc(d, s, 0))) atomicOr(&any, 1u);
    }
    __syncthreads();
    if (d.nscenes > 1)
        build_work_list(d, DIV ? kLoopDiv : kLoopPres,
                        [&](uint32_t sc) { return (DIV ? d.scenes[sc].div.active : d.scenes[sc].pres.active) != 0u; });
    if (threadIdx.x == 0) set_condition(d, DIV ? kLoopDiv : kLoopPres, aborted_p(d) ? 0u : any);
}

// K7 ComputePressureAccelerationAndFactorKernel (:555-602) + K8 ClearAccelerationKernel (:24-37).
template <uint32_t G, bool REL>
__global__ void __launch_bounds__(kMaxBlock) k_div_finish(Dev d) {
    VFD_COUNT_LAUNCH(d);
    GROUP_PROLOGUE(G)
    const SceneDev& S = d.scenes[scene_of(d, p)];
    if (S.enableDiv) {
        const Nbr nb = neighbors(d, p);
        const float3 a = pressure_accel<true, G, REL>(d, grp, p, S, nb);
        if (grp.lane == 0) {
            d.AP[p] = f4(a, 0.0f);
            const float4 v = d.V[p];
            d.V[p] = f4(f3(v) + S.dt * a, v.w);
            d.ALPHA[p] *= S.dt;
        }
    }
    if (grp.lane == 0) d.A[p] = make_float4(S.g[0], S.g[1], S.g[2], 0.0f);
}

// ---------------------------------------------------------------------------
// Surface tension (DFSPHImplementation.cu:810-839).
// K9: ComputeSurfaceTensionClassificationKernel (DFSPHKernels.cu:881-958); the
// Monte-Carlo samples are split over the group's lanes.
template <uint32_t G, bool REL>
__global__ void __launch_bounds__(kMaxBlock) k_st_classify(Dev d) {
    VFD_COUNT_LAUNCH(d);
    GROUP_PROLOGUE(G)
    const SceneDev& S = d.scenes[scene_of(d, p)];
    if (!S.enableST) return;
    const Nbr nb = neighbors(d, p);
    const float4 xi = d.X[p];
    if (nb.count == 0) {
        if (grp.lane == 0) d.STN[p] = make_float4(0.f, 0.f, 0.f, 1.0f / S.h);
        return;
    }
    float3 com = make_float3(0.f, 0.f, 0.f);
    for (uint32_t j = grp.lane; j < nb.count; j += G) com += pair_r<REL>(d, d.X[nb[j]], xi);
    com = grp.sum(com);
    com = make_float3(com.x / S.h, com.y / S.h, com.z / S.h);
    const float input = sqrtf(dot3(com, com)) / (float)nb.count;
    float3 nsum = make_float3(0.f, 0.f, 0.f);
    float curv = 0.0f;
    if ((float)nb.count <= S.slope * input + S.constant + 0.0f) {
        const uint32_t samples = S.stSamples;
        const uint32_t s0 = d.PID[p] * samples / 3u * 3u;
        const float ratio = S.nbrRadius / S.r;
        const float lim = ratio * ratio * S.h2;
        uint32_t count = 0;
        for (uint32_t k = grp.lane; k < samples; k += G) {
            const uint32_t i3 = s0 + 3u * k;
            const float3 pt = S.h * make_float3(__ldg(d.halton + i3 % kHaltonCount),
                                                __ldg(d.halton + (i3 + 1u) % kHaltonCount),
                                                __ldg(d.halton + (i3 + 2u) % kHaltonCount));
            bool covered = false;
            for (uint32_t j = 0; j < nb.count; j++) {
                const float3 v = pt - pair_r<REL>(d, d.X[nb[j]], xi);
                if (dot3(v, v) <= lim) { covered = true; break; }
            }
            if (!covered) { nsum += pt; count++; }
        }
        nsum = grp.sum(nsum);
        count = grp.sum(count);
        if (count > 0) {
            if (dot3(nsum, nsum) > 0.0f) nsum = normalize3(nsum);
            curv = 1.0f / S.h * -2.0f * sqrtf(1.0f - S.nbrRadius * S.nbrRadius / (S.r * S.r)) *
                   cosf(acosf(1.0f - 2.0f * ((float)count / (float)samples)) + S.mcFactor);
        } else {
            nsum = make_float3(0.f, 0.f, 0.f);
        }
    }
    if (grp.lane == 0) d.STN[p] = f4(nsum, curv);
}

__device__ __forceinline__ bool nonzero3(float4 a) { return a.x != 0.0f || a.y != 0.0f || a.z != 0.0f; }

// K10: ComputeSurfaceTensionNormalsAndCurvatureKernel (:960-1006).
template <uint32_t G, bool REL>
__global__ void __launch_bounds__(kMaxBlock) k_st_smooth(Dev d) {
    VFD_COUNT_LAUNCH(d);
    GROUP_PROLOGUE(G)
    const SceneDev& S = d.scenes[scene_of(d, p)];
    if (!S.enableST) return;
    const float4 ni = d.STN[p];
    if (!nonzero3(ni)) return;
    const Nbr nb = neighbors(d, p);
    const float4 xi = d.X[p];
    float3 nc = make_float3(0.f, 0.f, 0.f);
    float cc = 0.0f, cf = 0.0f;
    for_neighbors<G, false>(grp, nb, p, [&](uint32_t q, float, uint32_t, bool ok) {
        const float4 nj = d.STN[q];
        const float3 dx = pair_r<REL>(d, d.X[q], xi);
        if (ok && nonzero3(nj)) {
            const float num = 1.0f - __fdividef(fast_sqrt(dot3(dx, dx)), S.h);
            nc += f3(nj) * num;
            cc += nj.w * num;
            cf += num;
        }
    });
    nc = grp.sum(nc);
    cc = grp.sum(cc);
    cf = grp.sum(cf);
    if (grp.lane != 0) return;
    if (dot3(nc, nc) > 0.0f) nc = normalize3(nc);
    const float sf = S.smoothing;
    float3 ns = (1.0f - sf) * f3(ni) + sf * nc;
    if (dot3(ns, ns) > 0.0f) ns = normalize3(ns);
    d.STNS[p] = f4(ns, ((1.0f - sf) * ni.w + sf * cc) / (1.0f - sf + sf * cf));
}

// K11: ComputeSurfaceTensionBlendingKernel (:1008-1046), pass `pass` of SurfaceTensionSmoothPassCount.
__global__ void __launch_bounds__(kBlock) k_st_blend(Dev d, uint32_t pass) {
    VFD_COUNT_LAUNCH(d);
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= d.n || aborted_p(d)) return;
    const SceneDev& S = d.scenes[scene_of(d, p)];
    if (!S.enableST || pass >= S.stPasses) return;
    if (nonzero3(d.STN[p])) {
        const float4 ns = d.STNS[p];
        float fc = ns.w;
        if (S.temporal) fc = 0.05f * fc + 0.95f * d.DK[p];
        const float3 force = f3(ns) * S.st * fc;
        const float4 a = d.A[p];
        d.A[p] = f4(f3(a) - S.massInv * force, a.w);
        d.DK[p] = fc;
    } else {
        d.DK[p] = S.temporal ? 0.95f * d.DK[p] : 0.0f;
    }
}

// ---------------------------------------------------------------------------
// Viscosity (Weiler 2018 implicit, block-Jacobi PCG), DFSPHImplementation.cu:577-808.
struct Mat3 {
    float3 r0, r1, r2;
};
__device__ __forceinline__ float3 mul(const Mat3& m, float3 v) {
    return make_float3(dot3(m.r0, v), dot3(m.r1, v), dot3(m.r2, v));
}
__device__ __forceinline__ void add_outer(Mat3& m, float c, float3 a, float3 b) {  // m += c a b^T
    m.r0 += (c * a.x) * b;
    m.r1 += (c * a.y) * b;
    m.r2 += (c * a.z) * b;
}
__device__ __forceinline__ Mat3 load_mat(const float4* M, size_t stride, uint32_t p) {
    Mat3 m;
    m.r0 = f3(M[p]);
    m.r1 = f3(M[stride + p]);
    m.r2 = f3(M[2 * stride + p]);
    return m;
}
__device__ __forceinline__ void store_mat(float4* M, size_t stride, uint32_t p, const Mat3& m) {
    M[p] = f4(m.r0, 0.f);
    M[stride + p] = f4(m.r1, 0.f);
    M[2 * stride + p] = f4(m.r2, 0.f);
}
__device__ __forceinline__ Mat3 inverse3(const Mat3& a) {  // cofactors / determinant
    const float c00 = a.r1.y * a.r2.z - a.r1.z * a.r2.y;
    const float c01 = a.r1.z * a.r2.x - a.r1.x * a.r2.z;
    const float c02 = a.r1.x * a.r2.y - a.r1.y * a.r2.x;
    const float det = a.r0.x * c00 + a.r0.y * c01 + a.r0.z * c02;
    const float id = 1.0f / det;
    Mat3 r;
    r.r0 = make_float3(c00 * id, (a.r0.z * a.r2.y - a.r0.y * a.r2.z) * id, (a.r0.y * a.r1.z - a.r0.z * a.r1.y) * id);
    r.r1 = make_float3(c01 * id, (a.r0.x * a.r2.z - a.r0.z * a.r2.x) * id, (a.r0.z * a.r1.x - a.r0.x * a.r1.z) * id);
    r.r2 = make_float3(c02 * id, (a.r0.y * a.r2.x - a.r0.x * a.r2.y) * id, (a.r0.x * a.r1.y - a.r0.y * a.r1.x) * id);
    return r;
}

// K12 ComputeViscosityPreconditionerKernel (:604-684) + K13 ComputeViscosityGradientKernel
// (:686-756, whose boundary term dots a zero vector: b = v) + the boundary matrix BV of
// the SpMV's boundary term (:793-839): BV p_i = sum_k c_k (p_i . d_k) gradW_k.
// CG.w and CP.w hold m / rho (read by the SpMV's neighbours) from here on.
template <uint32_t G, bool REL>
__global__ void __launch_bounds__(kMaxBlock) k_visc_precond(Dev d) {
    VFD_COUNT_LAUNCH(d);
    GROUP_PROLOGUE(G)
    const SceneDev& S = d.scenes[scene_of(d, p)];
    if (!S.enableVisc) return;
    const Nbr nb = neighbors(d, p);
    const float4 xi4 = d.X[p];
    const float3 xi = f3(xi4);  // own frame of the boundary samples
    const float eps2 = 0.01f * S.h2;
    const float cmu = 10.0f * S.dynVisc;
    Mat3 m = {make_float3(0.f, 0.f, 0.f), make_float3(0.f, 0.f, 0.f), make_float3(0.f, 0.f, 0.f)};
    for_neighbors<G, true>(grp, nb, p, [&](uint32_t q, float gs, uint32_t, bool ok) {
        const float3 r = pair_r<REL>(d, xi4, d.X[q]);
        const float rho = d.RHO[q];
        if (!ok) return;
        const float3 g = gs * r;
        const float c = __fdividef(cmu * __fdividef(S.mass, rho), dot3(r, r) + eps2);
        add_outer(m, c, r, g);
    });
    m.r0 = grp.sum(m.r0);
    m.r1 = grp.sum(m.r1);
    m.r2 = grp.sum(m.r2);
    if (grp.lane != 0) return;
    Mat3 bv = {make_float3(0.f, 0.f, 0.f), make_float3(0.f, 0.f, 0.f), make_float3(0.f, 0.f, 0.f)};
    bool hasBV = false;
    if (S.dynBVisc != 0.0f && (nb.flags & kHasBoundary)) {
        for (uint32_t b = 0; b < S.bodyCount; b++) {
            const float4 xb4 = d.XB[(size_t)b * d.stride + p];
            if (!(xb4.w > 0.0f)) continue;
            const float3 xb = f3(xb4);
            float3 normal = -(xi - xb);
            const float nl = sqrtf(dot3(normal, normal));
            if (!(nl > 0.0001f)) continue;
            normal = make_float3(normal.x / nl, normal.y / nl, normal.z / nl);
            float3 t1, t2;
            orthogonal_vectors(normal, t1, t2);
            const float td = S.tangDist;
            const float3 pos[4] = {xb - t1 * td, xb + t1 * td, xb - t2 * td, xb + t2 * td};
            const float vol = 0.25f * xb4.w;
            const float3 d1 = xi - pos[0];
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const float3 dk = xi - pos[k];
                const float3 gk = kernel_grad(d, dk);
                const float c = 10.0f * S.dynBVisc * vol / (dot3(dk, dk) + eps2);
                add_outer(m, c, d1, gk);  // positionDirection1 in all four terms (:674-677)
                add_outer(bv, c, gk, dk);
            }
            hasBV = true;
        }
    }
    const float rho = d.RHO[p];
    const float f = S.dt / rho;
    Mat3 a;
    a.r0 = make_float3(1.0f - f * m.r0.x, -f * m.r0.y, -f * m.r0.z);
    a.r1 = make_float3(-f * m.r1.x, 1.0f - f * m.r1.y, -f * m.r1.z);
    a.r2 = make_float3(-f * m.r2.x, -f * m.r2.y, 1.0f - f * m.r2.z);
    store_mat(d.MINV, d.stride, p, inverse3(a));
    if (hasBV) {
        store_mat(d.BVM, d.stride, p, bv);
        d.NCNT[p] = nb.flags | kHasBoundaryVisc;
    } else if (nb.flags & kHasBoundaryVisc) {
        d.NCNT[p] = nb.flags & ~kHasBoundaryVisc;
    }
    const float4 v = d.V[p];
    d.CB[p] = v;
    d.CG[p] = f4(f3(v) + f3(d.DV[p]), S.mass / rho);
}

// ComputeMatrixVecProdFunctionKernel (:758-842): (A x)_i with vec[q].w = m / rho_q; lane 0.
// NS: gradW / r from the table, as in pressure_accel.
template <uint32_t G, bool REL, bool NS = false>
__device__ __forceinline__ float3 visc_matvec(const Dev& d, const Group<G>& grp, uint32_t p, const SceneDev& S,
                                              const float4* vec, float3 vi) {
    const Nbr nb = neighbors(d, p);
    const float4 xi = d.X[p];
    const float eps2 = 0.01f * S.h2;
    const float cmu = 10.0f * S.dynVisc;
    float3 acc = make_float3(0.f, 0.f, 0.f);
    for_neighbors<G, !NS>(grp, nb, p, [&](uint32_t q, float gsStream, uint32_t, bool ok) {
        const float3 r = pair_r<REL>(d, xi, d.X[q]);
        const float4 vq = vec[q];
        const float r2 = dot3(r, r);
        const float gs = NS ? grad_factor(d, r) : gsStream;
        const float3 t = (__fdividef(cmu * vq.w * dot3(vi - f3(vq), r), r2 + eps2) * gs) * r;
        if (ok) acc += t;
    });
    acc = grp.sum(acc);
    if (nb.flags & kHasBoundaryVisc) acc += mul(load_mat(d.BVM, d.stride, p), vi);
    return vi - (S.dt / d.RHO[p]) * acc;
}

// Initial residual r = b - A g and the norms |b|^2, |r|^2 (:627-669).
template <uint32_t G, bool REL>
__global__ void __launch_bounds__(kMaxBlock) k_visc_setup(Dev d) {
    VFD_COUNT_LAUNCH(d);
    const Group<G> grp;
    const uint32_t p = grp.p;
    const bool inRange = p < d.n && !aborted_p(d);
    const uint32_t sid = inRange ? scene_of(d, p) : 0u;
    const SceneDev& S = d.scenes[sid];
    const bool valid = inRange && S.enableVisc;
    float bb = 0.0f, rr = 0.0f;
    if (valid) {
        const float4 g4 = d.CG[p];
        const float3 ag = visc_matvec<G, REL>(d, grp, p, S, d.CG, f3(g4));
        if (grp.lane == 0) {
            const float3 b = f3(d.CB[p]);
            const float3 r = b - ag;
            d.CR[p] = f4(r, 0.0f);
            bb = dot_term(b, b);
            rr = dot_term(r, r);
        }
    }
    const float v[2] = {bb, rr};
    const int slot[2] = {0, 1};
    scene_accumulate<2, G>(d, sid, valid && grp.lane == 0, v, slot);
}

// Early outs of SolveViscosity (:646-675). The solver error sqrt(|r|^2 / |b|^2) is
// formed on the host from cgRR and cgRhs when the statistics are read, so that no
// controller spends an FP64 division and square root on it per iteration.
__device__ __forceinline__ void cg_start(const Dev& d, SceneDev& S, bool on, double rhs, double rr) {
    S.cgIt = 0;
    S.cgActive = 0;
    S.cgUpdateP = 0;
    S.cgZeroG = 0;
    S.cgDone = 1;
    S.cgRhs = 0.0;
    S.cgRR = 0.0;
    if (!on || aborted_p(d)) return;
    S.cgRhs = rhs;
    S.cgRR = rr;
    if (rhs == 0.0) {
        S.cgZeroG = 1;
        return;
    }
    const double e = (double)S.maxErrV;
    S.cgThr = fmax(e * e * 0.0001 * rhs, (double)FLT_MIN);
    if (rr < S.cgThr) return;
    S.cgDone = 0;
}

__global__ void k_ctrl_cg0(Dev d) {
    VFD_COUNT_LAUNCH(d);
    if (d.nscenes == 1) {
        if (threadIdx.x >= 32u) return;
        SceneDev& S = d.scenes[0];
        const bool on = S.enableVisc != 0;
        double rhs = 0.0, rr = 0.0;
        if (on) {
            rhs = fold_acc_warp(d, 0, 0, threadIdx.x);
            rr = fold_acc_warp(d, 0, 1, threadIdx.x);
        }
        if (threadIdx.x == 0) cg_start(d, S, on, rhs, rr);
        return;
    }
    for (uint32_t s = threadIdx.x; s < d.nscenes; s += blockDim.x) {
        SceneDev& S = d.scenes[s];
        const bool on = S.enableVisc != 0;
        const double rhs = on ? fold_acc(d, s, 0) : 0.0;
        const double rr = on ? fold_acc(d, s, 1) : 0.0;
        cg_start(d, S, on, rhs, rr);
    }
}

// p = M^-1 r (with p.w = m / rho) and |r . p| (:677-691).
__global__ void __launch_bounds__(kBlock) k_cg_p0(Dev d) {
    VFD_COUNT_LAUNCH(d);
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    const bool inRange = p < d.n && !aborted_p(d);
    const uint32_t sid = inRange ? scene_of(d, p) : 0u;
    const SceneDev& S = d.scenes[sid];
    const bool valid = inRange && S.enableVisc && !S.cgDone;
    float rz = 0.0f;
    if (valid) {
        const float3 r = f3(d.CR[p]);
        const float3 z = mul(load_mat(d.MINV, d.stride, p), r);
        d.CP[p] = f4(z, d.CG[p].w);
        rz = dot_term(r, z);
    }
    const float v[1] = {rz};
    const int slot[1] = {0};
    scene_accumulate<1>(d, sid, valid, v, slot);
}

__device__ __forceinline__ bool cg_first(const Dev& d, SceneDev& S, double rz) {
    S.cgAbsNew = fabs(rz);
    const bool run = S.cgIt >= S.minIterV && S.cgIt < S.maxIterV && !aborted_p(d);
    S.cgActive = run ? 1u : 0u;
    return run;
}

__global__ void k_ctrl_cg1(Dev d) {
    VFD_COUNT_LAUNCH(d);
    if (d.nscenes == 1) {
        if (threadIdx.x >= 32u) return;
        SceneDev& S = d.scenes[0];
        const bool on = S.enableVisc && !S.cgDone;
        const double rz = on ? fold_acc_warp(d, 0, 0, threadIdx.x) : 0.0;
        if (threadIdx.x == 0) set_condition(d, kLoopCG, (on && cg_first(d, S, rz)) ? 1u : 0u);
        return;
    }
    __shared__ uint32_t any;
    if (threadIdx.x == 0) any = 0;
    __syncthreads();
    for (uint32_t s = threadIdx.x; s < d.nscenes; s += blockDim.x) {
        SceneDev& S = d.scenes[s];
        if (!S.enableVisc || S.cgDone) continue;
        if (cg_first(d, S, fold_acc(d, s, 0))) atomicOr(&any, 1u);
    }
    __syncthreads();
    if (d.nscenes > 1) build_work_list(d, kLoopCG, [&](uint32_t sc) { return d.scenes[sc].cgActive != 0u; });
    if (threadIdx.x == 0) set_condition(d, kLoopCG, any);
}

// Loop body 1: Ap and p . Ap (:695-720).
template <uint32_t G, bool REL, bool NS = false>
__global__ void __launch_bounds__(kMaxBlock) k_cg_spmv(Dev d) {
    VFD_COUNT_LAUNCH(d);
    const Group<G> grp;
    const uint32_t p = grp.p;
    const bool inRange = p < d.n && !aborted_p(d);
    const uint32_t sid = inRange ? scene_of(d, p) : 0u;
    const SceneDev& S = d.scenes[sid];
    const bool valid = inRange && S.cgActive;
    float pap = 0.0f;
    if (valid) {
        const float3 pv = f3(d.CP[p]);
        const float3 ap = visc_matvec<G, REL, NS>(d, grp, p, S, d.CP, pv);
        if (grp.lane == 0) {
            d.CAP[p] = f4(ap, 0.0f);
            pap = dot_term(pv, ap);
        }
    }
    const float v[1] = {pap};
    const int slot[1] = {0};
    scene_accumulate<1, G>(d, sid, valid && grp.lane == 0, v, slot);
}

// Loop body 1 of a batch.
template <uint32_t G, bool REL>
__global__ void __launch_bounds__(kMaxBlock) k_cg_spmv_b(Dev d) {
    VFD_COUNT_LAUNCH(d);
    if (aborted_p(d)) return;
    BATCH_LOOP(kLoopCG, G) {
        const uint32_t vp = base_ + threadIdx.x / G;
        const bool in = vp < total_;
        uint32_t sid = 0;
        const uint32_t p = in ? work_slot(d, kLoopCG, vp, sid) : 0u;
        float pap = 0.0f;
        if (in) {
            const Group<G> grp(p);
            const float3 pv = f3(d.CP[p]);
            const float3 ap = visc_matvec<G, REL>(d, grp, p, d.scenes[sid], d.CP, pv);
            if (grp.lane == 0) {
                d.CAP[p] = f4(ap, 0.0f);
                pap = dot_term(pv, ap);
            }
        }
        const float v[1] = {pap};
        const int slot[1] = {0};
        scene_accumulate_core<1, G>(d, chunk_scene(d, kLoopCG, base_, per_, total_), sid, in && threadIdx.x % G == 0u,
                                 v, slot);
    }
}

// alpha = |r . z| / (p . Ap) (:714-720).
__global__ void k_ctrl_cg_alpha(Dev d) {
    VFD_COUNT_LAUNCH(d);
    if (d.nscenes == 1) {
        if (threadIdx.x >= 32u) return;
        SceneDev& S = d.scenes[0];
        if (!S.cgActive) return;
        const double pap = fold_acc_warp(d, 0, 0, threadIdx.x);
        if (threadIdx.x == 0) S.cgAlpha = (float)(S.cgAbsNew / pap);
        return;
    }
    for (uint32_t s = threadIdx.x; s < d.nscenes; s += blockDim.x) {
        SceneDev& S = d.scenes[s];
        if (!S.cgActive) continue;
        S.cgAlpha = (float)(S.cgAbsNew / fold_acc(d, s, 0));
    }
}

// Loop body 2: g += alpha p, r -= alpha Ap, |r|^2, z = M^-1 r, r . z (:722-784).
__device__ __forceinline__ void cg_update_item(const Dev& d, uint32_t p, const SceneDev& S, float& rr, float& rz,
                                               float alpha) {
    const float3 pv = f3(d.CP[p]);
    const float4 g4 = d.CG[p];
    const float3 g = f3(g4) + pv * alpha;
    const float3 r = f3(d.CR[p]) - f3(d.CAP[p]) * alpha;
    d.CG[p] = f4(g, g4.w);
    d.CR[p] = f4(r, 0.0f);
    const float3 z = mul(load_mat(d.MINV, d.stride, p), r);
    d.CZ[p] = f4(z, 0.0f);
    rr = dot_term(r, r);
    rz = dot_term(r, z);
}

// FOLD (a single scene on a small grid): every block forms alpha itself from the SpMV's
// p . Ap buckets, folded by its first warp as k_ctrl_cg_alpha folds them (the same bits),
// instead of a one-block launch between the two passes; k_ctrl_cg zeroes the buckets. On
// tens of thousands of blocks the bucket reads cost more than the launch.
template <bool FOLD>
__global__ void __launch_bounds__(kBlock) k_cg_update(Dev d) {
    VFD_COUNT_LAUNCH(d);
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    const bool inRange = p < d.n && !aborted_p(d);
    const uint32_t sid = inRange ? scene_of(d, p) : 0u;
    const SceneDev& S = d.scenes[sid];
    float alpha = S.cgAlpha;
    if (FOLD) {
        __shared__ float alphaBlock;
        if (threadIdx.x < 32u) {
            const double* q = acc_bucket(d, 0, 0, threadIdx.x);
            double v = __ldcg(q);
#pragma unroll
            for (int o = 16; o >= 1; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if (threadIdx.x == 0) {
                const SceneDev& S0 = d.scenes[0];
                alphaBlock = S0.cgActive ? (float)(S0.cgAbsNew / v) : 0.0f;
                if (blockIdx.x == 0 && S0.cgActive) d.scenes[0].cgAlpha = alphaBlock;
            }
        }
        __syncthreads();
        alpha = alphaBlock;
    }
    const bool valid = inRange && S.cgActive;
    float rr = 0.0f, rz = 0.0f;
    if (valid) cg_update_item(d, p, S, rr, rz, alpha);
    const float v[2] = {rr, rz};
    const int slot[2] = {1, 2};
    scene_accumulate<2>(d, sid, valid, v, slot);
}

__global__ void __launch_bounds__(kBlock) k_cg_update_b(Dev d) {
    VFD_COUNT_LAUNCH(d);
    if (aborted_p(d)) return;
    BATCH_LOOP(kLoopCG, 1u) {
        const uint32_t vp = base_ + threadIdx.x;
        const bool in = vp < total_;
        uint32_t sid = 0;
        const uint32_t p = in ? work_slot(d, kLoopCG, vp, sid) : 0u;
        float rr = 0.0f, rz = 0.0f;
        if (in) cg_update_item(d, p, d.scenes[sid], rr, rz, d.scenes[sid].cgAlpha);
        const float v[2] = {rr, rz};
        const int slot[2] = {1, 2};
        scene_accumulate_core<2>(d, chunk_scene(d, kLoopCG, base_, per_, total_), sid, in, v, slot);
    }
}

// Loop control: break on |r|^2 < threshold, else beta and the next iteration (:754-805).
__device__ __forceinline__ bool cg_control(const Dev& d, SceneDev& S, double rr, double rz) {
    S.cgRR = rr;
    if (rr < S.cgThr) {
        S.cgActive = 0;
        S.cgDone = 1;
        return false;
    }
    const double absOld = S.cgAbsNew;
    S.cgAbsNew = fabs(rz);
    S.cgBeta = (float)(S.cgAbsNew / absOld);
    S.cgIt++;
    S.cgUpdateP = 1;
    const bool again = S.cgIt >= S.minIterV && S.cgIt < S.maxIterV && !aborted_p(d);
    if (!again) S.flags |= 0x4u;
    S.cgActive = again ? 1u : 0u;
    return again;
}

__global__ void k_ctrl_cg(Dev d) {
    VFD_COUNT_LAUNCH(d);
    if (d.nscenes == 1) {
        if (threadIdx.x >= 32u) return;
        *acc_bucket(d, 0, 0, threadIdx.x) = 0.0;  // p . Ap, read by every block of a folding update
        SceneDev& S = d.scenes[0];
        const bool act = S.cgActive != 0u;
        double rr = 0.0, rz = 0.0;
        if (act) {
            rr = fold_acc_warp(d, 0, 1, threadIdx.x);
            rz = fold_acc_warp(d, 0, 2, threadIdx.x);
        }
        if (threadIdx.x == 0) {
            S.cgUpdateP = 0;
            set_condition(d, kLoopCG, (act && cg_control(d, S, rr, rz)) ? 1u : 0u);
        }
        return;
    }
    __shared__ uint32_t any;
    if (threadIdx.x == 0) any = 0;
    __syncthreads();
    for (uint32_t s = threadIdx.x; s < d.nscenes; s += blockDim.x) {
        SceneDev& S = d.scenes[s];
        S.cgUpdateP = 0;
        if (!S.cgActive) continue;
        const double rr = fold_acc(d, s, 1), rz = fold_acc(d, s, 2);
        if (cg_control(d, S, rr, rz)) atomicOr(&any, 1u);
    }
    __syncthreads();
    if (d.nscenes > 1) build_work_list(d, kLoopCG, [&](uint32_t sc) { return d.scenes[sc].cgActive != 0u; });
    if (threadIdx.x == 0) set_condition(d, kLoopCG, any);
}

// Loop body 3: p = beta p + z (:786-802), p.w = m / rho kept.
__global__ void __launch_bounds__(kBlock) k_cg_p(Dev d) {
    VFD_COUNT_LAUNCH(d);
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= d.n || aborted_p(d)) return;
    const SceneDev& S = d.scenes[scene_of(d, p)];
    if (!S.cgUpdateP) return;
    const float4 pv = d.CP[p];
    d.CP[p] = f4(f3(pv) * S.cgBeta + f3(d.CZ[p]), pv.w);
}

// Loop body 3 of a batch: the scenes going on to another iteration.
__global__ void __launch_bounds__(kBlock) k_cg_p_b(Dev d) {
    VFD_COUNT_LAUNCH(d);
    if (aborted_p(d)) return;
    BATCH_LOOP(kLoopCG, 1u) {
        const uint32_t vp = base_ + threadIdx.x;
        if (vp >= total_) continue;
        uint32_t sid;
        const uint32_t p = work_slot(d, kLoopCG, vp, sid);
        const float4 pv = d.CP[p];
        d.CP[p] = f4(f3(pv) * d.scenes[sid].cgBeta + f3(d.CZ[p]), pv.w);
    }
}

// K15 ApplyViscosityForceKernel (:844-862) + T1, the CFL maximum of |v + a dt|^2
// (ComputeMaxVelocityMagnitude, DFSPHImplementation.cu:430-441).
__global__ void __launch_bounds__(kBlock) k_visc_finish(Dev d) {
    VFD_COUNT_LAUNCH(d);
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = p < d.n && !aborted_p(d);
    const uint32_t sid = valid ? scene_of(d, p) : 0u;
    float m = 0.0f;
    if (valid) {
        const SceneDev& S = d.scenes[sid];
        const float3 v = f3(d.V[p]);
        float3 a = f3(d.A[p]);
        if (S.enableVisc) {
            const float3 g = S.cgZeroG ? make_float3(0.f, 0.f, 0.f) : f3(d.CG[p]);
            a += 1.0f / S.dt * (g - v);
            d.A[p] = f4(a, 0.0f);
            d.DV[p] = f4(g - v, 0.0f);
        }
        const float3 w = v + a * S.dt;
        m = dot3(w, w);
    }
    scene_max_float(d, sid, valid, m);
}

// ComputeTimeStepSize (DFSPHImplementation.cu:395-428) + the frame clock (:148-167).
__global__ void k_ctrl_dt(Dev d) {
    VFD_COUNT_LAUNCH(d);
    for (uint32_t s = threadIdx.x; s < d.nscenes; s += blockDim.x) {
        SceneDev& S = d.scenes[s];
        if (aborted_p(d)) continue;
        float mv = fmaxf(0.1f, __uint_as_float(fold_max(d, s, 0)));
        if (mv < 1.0e-9f) mv = 1.0e-9f;
        S.maxV2 = mv;
        float dt = 0.4f * (S.diam / sqrtf(mv));
        dt = fminf(dt, S.maxDt);
        dt = fmaxf(dt, S.minDt);
        S.dt = dt;
        S.dt2 = dt * dt;
        S.dtInv = 1.0f / dt;
        S.dt2Inv = 1.0f / S.dt2;
        S.stSamplesUsed = S.stSamples;
        S.stSamples = S.csdFix > 0 ? (uint32_t)S.csdFix : (uint32_t)(int)((float)S.csd * dt);
        S.frameTime += dt;
    }
}

// K16 ComputeVelocityKernel (:39-52).
__global__ void __launch_bounds__(kBlock) k_velocity(Dev d) {
    VFD_COUNT_LAUNCH(d);
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= d.n || aborted_p(d)) return;
    const SceneDev& S = d.scenes[scene_of(d, p)];
    const float4 v = d.V[p];
    d.V[p] = f4(f3(v) + S.dt * f3(d.A[p]), v.w);
}

// K17 ComputeDensityAdvectionKernel (:233-278).
template <uint32_t G, bool REL>
__global__ void __launch_bounds__(kMaxBlock) k_pres_init(Dev d) {
    VFD_COUNT_LAUNCH(d);
    GROUP_PROLOGUE(G)
    const SceneDev& S = d.scenes[scene_of(d, p)];
    const Nbr nb = neighbors(d, p);
    const float delta = velocity_divergence<G, REL>(d, grp, p, S, nb, d.X[p], f3(d.V[p]));
    if (grp.lane != 0) return;
    const float rhoAdv = d.RHO[p] / S.rho0 + S.dt * delta;
    d.RHOADV[p] = rhoAdv;
    const float alpha = d.ALPHA[p] * S.dt2Inv;
    d.ALPHA[p] = alpha;
    const float k = -fminf(1.0f - rhoAdv, 0.0f) * alpha;
    d.KAPPA[p] = k;
    set_kappa(d, p, k);
}

// K20 ComputePressureAccelerationAndVelocityKernel (:434-481) + K21 ComputePositionKernel (:54-67);
// positions go to XN so that the neighbours' positions read here stay unchanged.
template <uint32_t G, bool REL>
__global__ void __launch_bounds__(kMaxBlock) k_pres_finish(Dev d) {
    VFD_COUNT_LAUNCH(d);
    GROUP_PROLOGUE(G)
    const SceneDev& S = d.scenes[scene_of(d, p)];
    const Nbr nb = neighbors(d, p);
    const float3 a = pressure_accel<false, G, REL>(d, grp, p, S, nb);
    if (grp.lane != 0) return;
    d.AP[p] = f4(a, 0.0f);
    const float3 v = f3(d.V[p]) + S.dt * a;
    d.V[p] = f4(v, 0.0f);
    const float4 x4 = d.X[p];
    float3 x = f3(x4) + S.dt * v;
    if (!(isfinite(x.x) && isfinite(x.y) && isfinite(x.z))) atomicOr(d.status, 0x10u);
    if (d.cellRel) {  // back into [0, h) of a (possibly new) anchor cell
        const float L = d.radius;
        int3 A = anchor_of(x4.w);
        const float fx = floorf(x.x / L), fy = floorf(x.y / L), fz = floorf(x.z / L);
        if (isfinite(x.x) && isfinite(x.y) && isfinite(x.z)) {
            A = make_int3(A.x + (int)fx, A.y + (int)fy, A.z + (int)fz);
            x = make_float3(x.x - fx * L, x.y - fy * L, x.z - fz * L);
            if (abs(A.x) > 511 || abs(A.y) > 511 || abs(A.z) > 511) atomicOr(d.status, 0x40u);
        }
        d.XN[p] = f4(x, anchor_pack(A));
    } else {
        d.XN[p] = f4(x, 0.0f);
    }
}

// End of step: frame clock and iteration counter (DFSPHImplementation.cu:148-169);
// status[7] counts the steps completed since the host last looked.
__global__ void k_ctrl_end(Dev d) {
    VFD_COUNT_LAUNCH(d);
    if (threadIdx.x == 0 && !aborted_p(d)) d.status[7]++;
    for (uint32_t s = threadIdx.x; s < d.nscenes; s += blockDim.x) {
        SceneDev& S = d.scenes[s];
        if (aborted_p(d)) continue;
        S.frameDue = 0;
        if (S.frameIndex < S.frameCount && S.frameTime >= S.frameLength) {
            S.frameDue = 1;
            S.frameTime = 0.0f;
            S.frameIndex++;
        }
        S.iteration++;
        S.maxNbr = fold_max(d, s, 1);
        atomicOr(d.status, S.flags);
    }
}

// ---------------------------------------------------------------------------
// The solver-loop passes as cell-tile kernels (dfsph_tiles.cuh). Each Op states one
// pass's pair term and epilogue; the tile loop walks the neighbours (shared-memory halo
// and masks, or the row for kRowPath particles) and sums the terms over the group.

// K5 DivergenceSolveIterationKernel's force part / K18 (:388-432, :342-386): pressure
// acceleration a_p = -V sum_j (k_i + k_j) gradW_ij - k_i GB_i (kappa in X.w, or staged
// with cell-relative positions).
template <bool DIV, bool REL>
struct PressureAccelOp {
    static constexpr bool kField = REL;
    static constexpr bool kReduce = false;
    static constexpr int kSlot = 0;
    struct Own {
        float4 xi;
        float ki, V;
    };
    using Acc = float3;
    __device__ static bool active(const SceneDev& S) { return (DIV ? S.div.active : S.pres.active) != 0u; }
    __device__ static float4 field(const Dev& d, uint32_t q) {
        return make_float4((DIV ? d.KAPPAV : d.KAPPA)[q], 0.f, 0.f, 0.f);
    }
    __device__ static void load(const Dev& d, uint32_t p, const SceneDev& S, Own& o) {
        o.xi = d.X[p];
        o.ki = (DIV ? d.KAPPAV : d.KAPPA)[p];
        o.V = S.volume;
    }
    __device__ static void pair(const Dev& d, const Own& o, float4 xq, float4 fq, Acc& a) {
        const float sum = o.ki + (REL ? fq.x : xq.w);
        const float3 r = pair_r<REL>(d, o.xi, xq);
        const float gs = grad_factor(d, r);
        if (fabsf(sum) > kEps) a += (sum * (-o.V * gs)) * r;
    }
    __device__ static float finish(const Dev& d, uint32_t p, const SceneDev&, const Own& o, Acc a, uint32_t ncnt) {
        if (fabsf(o.ki) > kEps && (ncnt & kHasBoundary)) a += o.ki * (-f3(d.GB[p]));
        d.AP[p] = f4(a, 0.0f);
        return 0.0f;
    }
};

// K6 DivergenceSolveIterationKernel (:531-553) / K19 PressureSolveIterationKernel
// (:317-340), each with ComputeDensityPressureForce (:280-315): the density change of
// the pressure accelerations, the clamped residual, the kappa update, and the residual
// into the FP64-accurate sum.
template <bool DIV, bool REL>
struct JacobiOp {
    static constexpr bool kField = true;
    static constexpr bool kReduce = true;
    static constexpr int kSlot = 0;
    struct Own {
        float4 xi;
        float3 ai;
    };
    using Acc = float;
    __device__ static bool active(const SceneDev& S) { return (DIV ? S.div.active : S.pres.active) != 0u; }
    __device__ static float4 field(const Dev& d, uint32_t q) { return d.AP[q]; }
    __device__ static void load(const Dev& d, uint32_t p, const SceneDev&, Own& o) {
        o.xi = d.X[p];
        o.ai = f3(d.AP[p]);
    }
    __device__ static void pair(const Dev& d, const Own& o, float4 xq, float4 aq, Acc& f) {
        const float3 r = pair_r<REL>(d, o.xi, xq);
        const float gs = grad_factor(d, r);
        f += dot3(o.ai - f3(aq), gs * r);
    }
    __device__ static float finish(const Dev& d, uint32_t p, const SceneDev& S, const Own& o, Acc f, uint32_t ncnt) {
        f *= S.volume;
        if (ncnt & kHasBoundary) f += dot3(o.ai, f3(d.GB[p]));
        float r;
        if (DIV) {
            f *= S.dt;
            r = (ncnt & kCountMask) < 20u ? 0.0f : fminf(-d.RHOADV[p] - f, 0.0f);
            const float k = d.KAPPAV[p] - r * d.ALPHA[p];
            d.KAPPAV[p] = k;
            set_kappa(d, p, k);
        } else {
            f *= S.dt2;
            r = fminf(1.0f - d.RHOADV[p] - f, 0.0f);
            const float k = d.KAPPA[p] - r * d.ALPHA[p];
            d.KAPPA[p] = k;
            set_kappa(d, p, k);
        }
        d.RES[p] = r;
        return r;
    }
};

// ComputeMatrixVecProdFunctionKernel (:758-842) on the CG direction p (p.w = m / rho) and
// the p . Ap term of the step length (:695-720).
template <bool REL>
struct SpmvOp {
    static constexpr bool kField = true;
    static constexpr bool kReduce = true;
    static constexpr int kSlot = 0;
    struct Own {
        float4 xi;
        float3 vi;
        float cmu, eps2;
    };
    using Acc = float3;
    __device__ static bool active(const SceneDev& S) { return S.cgActive != 0u; }
    __device__ static float4 field(const Dev& d, uint32_t q) { return d.CP[q]; }
    __device__ static void load(const Dev& d, uint32_t p, const SceneDev& S, Own& o) {
        o.xi = d.X[p];
        o.vi = f3(d.CP[p]);
        o.cmu = 10.0f * S.dynVisc;
        o.eps2 = 0.01f * S.h2;
    }
    __device__ static void pair(const Dev& d, const Own& o, float4 xq, float4 vq, Acc& acc) {
        const float3 r = pair_r<REL>(d, o.xi, xq);
        const float r2 = dot3(r, r);
        const float gs = grad_factor_r2(d, r2);
        acc += (__fdividef(o.cmu * vq.w * dot3(o.vi - f3(vq), r), r2 + o.eps2) * gs) * r;
    }
    __device__ static float finish(const Dev& d, uint32_t p, const SceneDev& S, const Own& o, Acc acc, uint32_t ncnt) {
        if (ncnt & kHasBoundaryVisc) acc += mul(load_mat(d.BVM, d.stride, p), o.vi);
        const float3 ap = o.vi - (S.dt / d.RHO[p]) * acc;
        d.CAP[p] = f4(ap, 0.0f);
        return dot_term(o.vi, ap);
    }
};

// The tile kernels, one name per pass for profilers.
template <bool DIV, uint32_t L, uint32_t G, bool REL>
__global__ void __launch_bounds__(kTileBlock) k_pressure_accel_tile(Dev d) {
    VFD_COUNT_LAUNCH(d);
    tile_pass<PressureAccelOp<DIV, REL>, L, G, REL>(d);
}
template <bool DIV, uint32_t L, uint32_t G, bool REL>
__global__ void __launch_bounds__(kTileBlock) k_jacobi_iter_tile(Dev d) {
    VFD_COUNT_LAUNCH(d);
    tile_pass<JacobiOp<DIV, REL>, L, G, REL>(d);
}
template <uint32_t L, uint32_t G, bool REL>
__global__ void __launch_bounds__(kTileBlock) k_cg_spmv_tile(Dev d) {
    VFD_COUNT_LAUNCH(d);
    tile_pass<SpmvOp<REL>, L, G, REL>(d);
}

// ---------------------------------------------------------------- tile launches
// Blocks of a cell-tile pass stride over the tiles; the grid is one block per resident
// slot of the GPU (occupancy of the instantiation with its shared memory), found once by
// prepare_tile_kernels before any capture (it also raises the shared-memory limit).
template <void (*K)(Dev), size_t SMEM>
int& tile_resident() {
    static int resident = 0;
    return resident;
}
template <void (*K)(Dev), size_t SMEM>
cudaError_t prepare_tile() {
    int& r = tile_resident<K, SMEM>();
    if (r > 0) return cudaSuccess;
    // the limit covers dynamic + static shared memory; raise it to what this kernel asks
    cudaError_t e = cudaFuncSetAttribute(K, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM);
    int n = 0;
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, K, kTileBlock, SMEM);
    r = n > 0 ? n : 1;
    return e;
}
template <void (*K)(Dev), size_t SMEM>
void launch_tile(const Dev& d, cudaStream_t s, const char* name) {
    const uint32_t sms = d.batchBlocks / (2048u / kBlock);
    const int r = tile_resident<K, SMEM>();
    VFD_LAUNCH(name, s, K<<<sms * (uint32_t)(r > 0 ? r : 1), kTileBlock, SMEM, s>>>(d));
}
template <class Op, uint32_t L>
constexpr size_t tile_smem() { return (Op::kField ? 2u : 1u) * TileShape<L>::CAP * sizeof(float4); }

// The instantiations of one pass: tile size 2^L (L = 3: 2x2x2 cells, 4: 4x2x2), lanes per
// particle G (4, 8, 16), position storage mode. FN(L, G, REL) names the kernel, OP(REL)
// its Op; ACT(L, G, REL) is applied to each (kernel, shared memory) pair.
#define VFD_TILE_VARIANTS(ACT, FN, OP)                                                          \
    ACT(FN(3, 4, false), OP(false), 3) ACT(FN(3, 8, false), OP(false), 3)                       \
    ACT(FN(3, 16, false), OP(false), 3) ACT(FN(4, 4, false), OP(false), 4)                      \
    ACT(FN(4, 8, false), OP(false), 4) ACT(FN(4, 16, false), OP(false), 4)                      \
    ACT(FN(3, 4, true), OP(true), 3) ACT(FN(3, 8, true), OP(true), 3)                           \
    ACT(FN(3, 16, true), OP(true), 3) ACT(FN(4, 4, true), OP(true), 4)                          \
    ACT(FN(4, 8, true), OP(true), 4) ACT(FN(4, 16, true), OP(true), 4)
#define VFD_TILE_PREPARE(K, OPT, L) \
    if (e == cudaSuccess) e = prepare_tile<K, tile_smem<OPT, L>()>();

#define FN_PACC_D(L, G, R) k_pressure_accel_tile<true, L, G, R>
#define FN_PACC_P(L, G, R) k_pressure_accel_tile<false, L, G, R>
#define FN_JAC_D(L, G, R) k_jacobi_iter_tile<true, L, G, R>
#define FN_JAC_P(L, G, R) k_jacobi_iter_tile<false, L, G, R>
#define FN_SPMV(L, G, R) k_cg_spmv_tile<L, G, R>
#define OP_PACC_D(R) PressureAccelOp<true, R>
#define OP_PACC_P(R) PressureAccelOp<false, R>
#define OP_JAC_D(R) JacobiOp<true, R>
#define OP_JAC_P(R) JacobiOp<false, R>
#define OP_SPMV(R) SpmvOp<R>

cudaError_t prepare_tile_kernels() {
    cudaError_t e = cudaSuccess;
    VFD_TILE_VARIANTS(VFD_TILE_PREPARE, FN_PACC_D, OP_PACC_D)
    VFD_TILE_VARIANTS(VFD_TILE_PREPARE, FN_PACC_P, OP_PACC_P)
    VFD_TILE_VARIANTS(VFD_TILE_PREPARE, FN_JAC_D, OP_JAC_D)
    VFD_TILE_VARIANTS(VFD_TILE_PREPARE, FN_JAC_P, OP_JAC_P)
    VFD_TILE_VARIANTS(VFD_TILE_PREPARE, FN_SPMV, OP_SPMV)
    return e;
}

// Dispatch on (tile size, lanes, storage mode) of one pass.
#define VFD_TILE_DISPATCH(name, lanesId, FN, OP)                                               \
    do {                                                                                      \
        const uint32_t G_ = d.lanes[lanesId] == 4 ? 4u : d.lanes[lanesId] == 16 ? 16u : 8u;   \
        const bool l4_ = d.tiles[lanesId] == 4u;                                              \
        if (d.cellRel) {                                                                      \
            if (l4_) {                                                                        \
                if (G_ == 4u) launch_tile<FN(4, 4, true), tile_smem<OP(true), 4>()>(d, s, name);   \
                else if (G_ == 16u) launch_tile<FN(4, 16, true), tile_smem<OP(true), 4>()>(d, s, name); \
                else launch_tile<FN(4, 8, true), tile_smem<OP(true), 4>()>(d, s, name);        \
            } else {                                                                          \
                if (G_ == 4u) launch_tile<FN(3, 4, true), tile_smem<OP(true), 3>()>(d, s, name);   \
                else if (G_ == 16u) launch_tile<FN(3, 16, true), tile_smem<OP(true), 3>()>(d, s, name); \
                else launch_tile<FN(3, 8, true), tile_smem<OP(true), 3>()>(d, s, name);        \
            }                                                                                 \
        } else {                                                                              \
            if (l4_) {                                                                        \
                if (G_ == 4u) launch_tile<FN(4, 4, false), tile_smem<OP(false), 4>()>(d, s, name); \
                else if (G_ == 16u) launch_tile<FN(4, 16, false), tile_smem<OP(false), 4>()>(d, s, name); \
                else launch_tile<FN(4, 8, false), tile_smem<OP(false), 4>()>(d, s, name);      \
            } else {                                                                          \
                if (G_ == 4u) launch_tile<FN(3, 4, false), tile_smem<OP(false), 3>()>(d, s, name); \
                else if (G_ == 16u) launch_tile<FN(3, 16, false), tile_smem<OP(false), 3>()>(d, s, name); \
                else launch_tile<FN(3, 8, false), tile_smem<OP(false), 3>()>(d, s, name);      \
            }                                                                                 \
        }                                                                                     \
    } while (0)


// ---------------------------------------------------------------- launchers
// The instantiation for the position storage mode (K and its _R variant).
#define VFD_LAUNCH_MODE(LAUNCHER, name, id, K) \
    do {                                       \
        if (d.cellRel) LAUNCHER(name, id, K##_R); \
        else LAUNCHER(name, id, K);           \
    } while (0)
#define K_DENSITY(G) k_density_factor<G, false>
#define K_DENSITY_R(G) k_density_factor<G, true>
#define K_DENSITY_DIV(G) k_density_factor<G, false, true>
#define K_DENSITY_DIV_R(G) k_density_factor<G, true, true>
#define K_PACCEL_D(G) k_pressure_accel<true, G, false>
#define K_PACCEL_D_R(G) k_pressure_accel<true, G, true>
#define K_PACCEL_P(G) k_pressure_accel<false, G, false>
#define K_PACCEL_P_R(G) k_pressure_accel<false, G, true>
#define K_JACOBI_D(G) k_jacobi_iter<true, G, false>
#define K_JACOBI_D_R(G) k_jacobi_iter<true, G, true>
#define K_JACOBI_P(G) k_jacobi_iter<false, G, false>
#define K_JACOBI_P_R(G) k_jacobi_iter<false, G, true>
#define K_DIV_FINISH(G) k_div_finish<G, false>
#define K_DIV_FINISH_R(G) k_div_finish<G, true>
#define K_ST_CLASSIFY(G) k_st_classify<G, false>
#define K_ST_CLASSIFY_R(G) k_st_classify<G, true>
#define K_ST_SMOOTH(G) k_st_smooth<G, false>
#define K_ST_SMOOTH_R(G) k_st_smooth<G, true>
#define K_VISC_PRECOND(G) k_visc_precond<G, false>
#define K_VISC_PRECOND_R(G) k_visc_precond<G, true>
#define K_VISC_SETUP(G) k_visc_setup<G, false>
#define K_VISC_SETUP_R(G) k_visc_setup<G, true>
#define K_SPMV(G) k_cg_spmv<G, false>
#define K_SPMV_R(G) k_cg_spmv<G, true>
#define K_SPMV_NS(G) k_cg_spmv<G, false, true>
#define K_SPMV_NS_R(G) k_cg_spmv<G, true, true>
#define K_PACCEL_D_NS(G) k_pressure_accel<true, G, false, true>
#define K_PACCEL_D_NS_R(G) k_pressure_accel<true, G, true, true>
#define K_PACCEL_P_NS(G) k_pressure_accel<false, G, false, true>
#define K_PACCEL_P_NS_R(G) k_pressure_accel<false, G, true, true>
#define K_JACOBI_D_NS(G) k_jacobi_iter<true, G, false, true>
#define K_JACOBI_D_NS_R(G) k_jacobi_iter<true, G, true, true>
#define K_JACOBI_P_NS(G) k_jacobi_iter<false, G, false, true>
#define K_JACOBI_P_NS_R(G) k_jacobi_iter<false, G, true, true>
#define K_PRES_INIT(G) k_pres_init<G, false>
#define K_PRES_INIT_R(G) k_pres_init<G, true>
#define K_PRES_FINISH(G) k_pres_finish<G, false>
#define K_PRES_FINISH_R(G) k_pres_finish<G, true>

void launch_density(const Dev& d, cudaStream_t s) { VFD_LAUNCH_MODE(VFD_LAUNCH_LANES, "k_density_factor", kTDensity, K_DENSITY); }
// K2 + K3 + K4 in one pass, then the divergence loop's start.
void launch_density_div_init(const Dev& d, cudaStream_t s) {
    VFD_LAUNCH_MODE(VFD_LAUNCH_LANES, "k_density_factor", kTDensity, K_DENSITY_DIV);
    VFD_LAUNCH("k_ctrl_jacobi_init", s, k_ctrl_jacobi_init<true><<<1, 256, 0, s>>>(d));
}
#define K_PACCEL_DB(G) k_pressure_accel_b<true, G, false>
#define K_PACCEL_DB_R(G) k_pressure_accel_b<true, G, true>
#define K_PACCEL_PB(G) k_pressure_accel_b<false, G, false>
#define K_PACCEL_PB_R(G) k_pressure_accel_b<false, G, true>
#define K_JACOBI_DB(G) k_jacobi_iter_b<true, G, false>
#define K_JACOBI_DB_R(G) k_jacobi_iter_b<true, G, true>
#define K_JACOBI_PB(G) k_jacobi_iter_b<false, G, false>
#define K_JACOBI_PB_R(G) k_jacobi_iter_b<false, G, true>
#define K_SPMV_B(G) k_cg_spmv_b<G, false>
#define K_SPMV_B_R(G) k_cg_spmv_b<G, true>

// Whether a solver-loop pass runs on cell tiles (vfd_set_tiles / the autotuner) rather
// than the neighbour rows; the adjoint's CG always walks rows (Dev::rowLoops).
inline bool tiled(const Dev& d, int id) { return d.tiles[id] >= kTileMinLog2 && d.compactRows && !d.rowLoops; }
// Single-scene CG updates on at most this many blocks form alpha themselves (k_cg_update<true>).
constexpr uint32_t kFoldAlphaBlocks = 1024u;
// Single-scene row pass without the per-pair gradient stream (tiles[id] == kRowsNoStream).
inline bool no_stream(const Dev& d, int id) { return d.tiles[id] == kRowsNoStream && d.nscenes == 1; }

// Row path: batches run the solver-loop kernels over their work lists (the scenes still
// iterating) with a fixed grid; a single scene keeps one group per particle. Tile path:
// single scenes and batches alike (tiles of scenes that stopped iterating are skipped).
void launch_div_iter(const Dev& d, cudaStream_t s) {
    if (tiled(d, kTPAccel)) VFD_TILE_DISPATCH("k_pressure_accel", kTPAccel, FN_PACC_D, OP_PACC_D);
    else if (d.nscenes > 1) VFD_LAUNCH_MODE(VFD_LAUNCH_LANES_BATCH, "k_pressure_accel", kTPAccel, K_PACCEL_DB);
    else if (no_stream(d, kTPAccel)) VFD_LAUNCH_MODE(VFD_LAUNCH_LANES, "k_pressure_accel", kTPAccel, K_PACCEL_D_NS);
    else VFD_LAUNCH_MODE(VFD_LAUNCH_LANES, "k_pressure_accel", kTPAccel, K_PACCEL_D);
    if (tiled(d, kTJacobi)) VFD_TILE_DISPATCH("k_jacobi_iter", kTJacobi, FN_JAC_D, OP_JAC_D);
    else if (d.nscenes > 1) VFD_LAUNCH_MODE(VFD_LAUNCH_LANES_BATCH, "k_jacobi_iter", kTJacobi, K_JACOBI_DB);
    else if (no_stream(d, kTJacobi)) VFD_LAUNCH_MODE(VFD_LAUNCH_LANES, "k_jacobi_iter", kTJacobi, K_JACOBI_D_NS);
    else VFD_LAUNCH_MODE(VFD_LAUNCH_LANES, "k_jacobi_iter", kTJacobi, K_JACOBI_D);
    VFD_LAUNCH("k_ctrl_jacobi", s, k_ctrl_jacobi<true><<<1, 256, 0, s>>>(d));
}
void launch_div_finish(const Dev& d, cudaStream_t s) { VFD_LAUNCH_MODE(VFD_LAUNCH_LANES, "k_div_finish", kTDivFinish, K_DIV_FINISH); }
void launch_surface_tension(const Dev& d, uint32_t maxPasses, cudaStream_t s) {
    VFD_LAUNCH_MODE(VFD_LAUNCH_LANES, "k_st_classify", kTStClassify, K_ST_CLASSIFY);
    VFD_LAUNCH_MODE(VFD_LAUNCH_LANES, "k_st_smooth", kTStSmooth, K_ST_SMOOTH);
    for (uint32_t pass = 0; pass < maxPasses; pass++)
        VFD_LAUNCH("k_st_blend", s, k_st_blend<<<blocks_for(d.n), kBlock, 0, s>>>(d, pass));
}
void launch_visc_init(const Dev& d, cudaStream_t s) {
    VFD_LAUNCH_MODE(VFD_LAUNCH_LANES, "k_visc_precond", kTViscPrecond, K_VISC_PRECOND);
    VFD_LAUNCH_MODE(VFD_LAUNCH_LANES, "k_visc_setup", kTViscSetup, K_VISC_SETUP);
    VFD_LAUNCH("k_ctrl_cg0", s, k_ctrl_cg0<<<1, 256, 0, s>>>(d));
    VFD_LAUNCH("k_cg_p0", s, k_cg_p0<<<blocks_for(d.n), kBlock, 0, s>>>(d));
    VFD_LAUNCH("k_ctrl_cg1", s, k_ctrl_cg1<<<1, 256, 0, s>>>(d));
}
void launch_cg_iter(const Dev& d, cudaStream_t s) {
    if (tiled(d, kTSpmv)) VFD_TILE_DISPATCH("k_cg_spmv", kTSpmv, FN_SPMV, OP_SPMV);
    else if (d.nscenes > 1) VFD_LAUNCH_MODE(VFD_LAUNCH_LANES_BATCH, "k_cg_spmv", kTSpmv, K_SPMV_B);
    else if (no_stream(d, kTSpmv)) VFD_LAUNCH_MODE(VFD_LAUNCH_LANES, "k_cg_spmv", kTSpmv, K_SPMV_NS);
    else VFD_LAUNCH_MODE(VFD_LAUNCH_LANES, "k_cg_spmv", kTSpmv, K_SPMV);
    if (d.nscenes > 1) {
        VFD_LAUNCH("k_ctrl_cg_alpha", s, k_ctrl_cg_alpha<<<1, 256, 0, s>>>(d));
        VFD_LAUNCH("k_cg_update", s, k_cg_update_b<<<d.batchBlocks, kBlock, 0, s>>>(d));
        VFD_LAUNCH("k_ctrl_cg", s, k_ctrl_cg<<<1, 256, 0, s>>>(d));
        VFD_LAUNCH("k_cg_p", s, k_cg_p_b<<<d.batchBlocks, kBlock, 0, s>>>(d));
        return;
    }
    // a small grid forms alpha in the update's blocks (k_cg_update<true>): one launch fewer
    if (blocks_for(d.n) <= kFoldAlphaBlocks) {
        VFD_LAUNCH("k_cg_update", s, k_cg_update<true><<<blocks_for(d.n), kBlock, 0, s>>>(d));
    } else {
        VFD_LAUNCH("k_ctrl_cg_alpha", s, k_ctrl_cg_alpha<<<1, 256, 0, s>>>(d));
        VFD_LAUNCH("k_cg_update", s, k_cg_update<false><<<blocks_for(d.n), kBlock, 0, s>>>(d));
    }
    VFD_LAUNCH("k_ctrl_cg", s, k_ctrl_cg<<<1, 256, 0, s>>>(d));
    VFD_LAUNCH("k_cg_p", s, k_cg_p<<<blocks_for(d.n), kBlock, 0, s>>>(d));
}
void launch_visc_finish_dt(const Dev& d, cudaStream_t s) {
    VFD_LAUNCH("k_visc_finish", s, k_visc_finish<<<blocks_for(d.n), kBlock, 0, s>>>(d));
    VFD_LAUNCH("k_ctrl_dt", s, k_ctrl_dt<<<1, 256, 0, s>>>(d));
    VFD_LAUNCH("k_velocity", s, k_velocity<<<blocks_for(d.n), kBlock, 0, s>>>(d));
}
void launch_pres_init(const Dev& d, cudaStream_t s) {
    VFD_LAUNCH_MODE(VFD_LAUNCH_LANES, "k_pres_init", kTPresInit, K_PRES_INIT);
    VFD_LAUNCH("k_ctrl_jacobi_init", s, k_ctrl_jacobi_init<false><<<1, 256, 0, s>>>(d));
}
void launch_pres_iter(const Dev& d, cudaStream_t s) {
    if (tiled(d, kTPAccel)) VFD_TILE_DISPATCH("k_pressure_accel", kTPAccel, FN_PACC_P, OP_PACC_P);
    else if (d.nscenes > 1) VFD_LAUNCH_MODE(VFD_LAUNCH_LANES_BATCH, "k_pressure_accel", kTPAccel, K_PACCEL_PB);
    else if (no_stream(d, kTPAccel)) VFD_LAUNCH_MODE(VFD_LAUNCH_LANES, "k_pressure_accel", kTPAccel, K_PACCEL_P_NS);
    else VFD_LAUNCH_MODE(VFD_LAUNCH_LANES, "k_pressure_accel", kTPAccel, K_PACCEL_P);
    if (tiled(d, kTJacobi)) VFD_TILE_DISPATCH("k_jacobi_iter", kTJacobi, FN_JAC_P, OP_JAC_P);
    else if (d.nscenes > 1) VFD_LAUNCH_MODE(VFD_LAUNCH_LANES_BATCH, "k_jacobi_iter", kTJacobi, K_JACOBI_PB);
    else if (no_stream(d, kTJacobi)) VFD_LAUNCH_MODE(VFD_LAUNCH_LANES, "k_jacobi_iter", kTJacobi, K_JACOBI_P_NS);
    else VFD_LAUNCH_MODE(VFD_LAUNCH_LANES, "k_jacobi_iter", kTJacobi, K_JACOBI_P);
    VFD_LAUNCH("k_ctrl_jacobi", s, k_ctrl_jacobi<false><<<1, 256, 0, s>>>(d));
}
void launch_pres_finish(const Dev& d, cudaStream_t s) {
    VFD_LAUNCH_MODE(VFD_LAUNCH_LANES, "k_pres_finish", kTPresFinish, K_PRES_FINISH);
    VFD_LAUNCH("k_ctrl_end", s, k_ctrl_end<<<1, 256, 0, s>>>(d));
}

}  // namespace vfd
