// Reverse-mode derivative (adjoint) of the DFSPH step: the gradient of a function
// of the final positions and velocities after `steps` OnUpdate steps with respect
// to the initial positions, the initial velocities, Viscosity and BoundaryViscosity.
//
// The reference has no derivative of its step. The forward computation
// differentiated here is the step of DFSPHImplementation::OnUpdate
// (Simulation/DFSPH/DFSPHImplementation.cu:63-170) exactly as dfsph_physics.cu runs
// it. Per step, with neighbour sets N(i), the solver iteration counts and the
// clamp/skip decisions of the step frozen:
//   density    rho_i = rho0 (V W0 + V sum_j W_ij + sum_b Vb W(pd_b))
//              alpha_i = 1 / (sum_j |V gradW_ij|^2 + |V sum_j gradW_ij + GB_i|^2)
//   operators  D_i(w) = V sum_j (w_i - w_j).gradW_ij + w_i.GB_i          (K4, K6, K17, K19)
//              P_i(k) = -V sum_j (k_i + k_j) gradW_ij - k_i GB_i         (K5, K7, K18, K20)
//   divergence rho_adv = max(D(v0), 0); k0 = rho_adv alpha / dt_o;
//              k <- k + m_k (alpha / dt_o) (rho_adv + dt_o D(P(k)))      (unrolled, m_k = clamp active)
//              v1 = v0 + dt_o P(k)
//   viscosity  A(x, rho) g = v1 (Weiler 2018), solved by CG; through the implicit
//              function theorem the adjoint solves A lambda = g_bar with the same CG
//              (A is symmetric) and differentiates A g = v1 for x, rho, the two
//              viscosities and dt_o
//   CFL        dt_n = 0.4 d / sqrt(max_i |g_i + dt_o gravity|^2)   (through the argmax)
//   velocity   v2 = v1 + dt_n (gravity + (g - v1) / dt_o)
//   pressure   rho_adv = rho / rho0 + dt_n D(v2); k0 = max(rho_adv - 1, 0) alpha / dt_n^2;
//              k <- k - m_k (alpha / dt_n^2) (1 - rho_adv - dt_n^2 D(P(k)))
//              v3 = v2 + dt_n P(k); x' = x + dt_n v3
// D and P are transposes of each other up to sign (P = -D^T), so the adjoint of
// every linear solve step is again a pass of the same two operators. Their
// dependence on positions goes through gradW(x_i - x_j), whose derivative is the
// kernel Hessian H = gs I + gs'/|r| r r^T of the analytic cubic spline (the
// reference's midpoint table lookup is piecewise constant in |r|; its values are
// used wherever the forward uses them). Boundary samples: x - xb = pd n with
// pd = max(phi0 + r/2, 2r) and Vb = phi1 of the volume map; phi0, phi1 are
// differentiated through the shape-function gradients, the normal n is held
// fixed (exact on planar walls). The push-out of particles inside a wall moves
// them by a constant 0.1 r along n (identity Jacobian) and zeroes their velocity.
//
// Memory: states are checkpointed every `checkpoint_every` steps during the
// forward run (whose last segment is recorded as it runs); the backward pass re-runs
// each other segment from its checkpoint, recording per step the neighbour rows, four
// velocity fields and the Jacobi iterates, and then walks the segment's steps in
// reverse. Each backward step is one launch of a graph built once: its kernels read the
// step's arrays, time steps, iteration counts and decisions from the tape slot a device
// counter names, and its Jacobi loops and the adjoint CG are conditional WHILE nodes.
// Limits: one scene, surface tension off; neighbour sets must be symmetric, so a
// particle at the 70-neighbour cap is rejected.
#include <cuda_runtime.h>

#include <cfloat>
#include <cmath>
#include <cstring>
#include <memory>
#include <vector>

#include "dfsph_map.cuh"
#include "dfsph_sim.h"

namespace vfd {

namespace {

constexpr uint32_t kAG = 8;  // lanes per particle of the adjoint neighbour loops

// One recorded step: written by the tape kernels at the tape points of the step
// (TapePoint), so that one recording graph serves every step: the slot of the current
// step is steps[*cur], advanced by the step's last tape point.
struct TapeStep {
    float4 *Xpre, *V0, *V1, *G, *V2;
    uint32_t *PID, *NCNT, *NBR;
    float *RAD, *RAP;
    float *KD, *RD, *KP, *RP;   // kappa^0..cap, res^0..cap-1 (stride floats each) of each solve
    uint32_t capD, capP;
    // written on the device
    SceneDev pre;               // scene state at the start of the step
    uint32_t kd, kp, overflow, zeroG, maxNbr, aborted;
    float dto, dtn, maxV2;
};
struct TapeSet {
    TapeStep* steps;
    uint32_t* cur;
    uint32_t count;
};

// Cotangent arrays of the backward pass (slot order unless stated).
struct AdjDev {
    float4 *XBAR, *VBAR;      // x and v of the point of the step being differentiated
    float4 *ABAR, *AK;        // pressure-acceleration cotangent, recomputed acceleration
    float4 *GBAR, *GSUM;      // viscosity-solution cotangent; (sum gradW + GB, S bar)
    float4* BD;               // [3][body][stride]: (n, Vb), (grad pd, pd), (grad Vb, -)
    float *KBAR, *U, *RABAR, *APBAR, *DBAR, *RHOBAR, *ALBAR;
    float2* KU;               // (kappa^k, U) of the Jacobi iteration being differentiated
    float4 *LAM, *LAM2;       // the last two adjoint viscosity solutions (initial guesses of the next)
    uint32_t* ACNT;           // [0] adjoint CG iterations, [1] their maximum per solve, [2] solves,
                              // [3] solutions held in LAM / LAM2 (0..2)
    uint32_t* STOP;           // 1 where the boundary zeroed the velocity
    double* SC;               // [0] dt_o bar, [1] dt_n bar, [2] Viscosity bar, [3] BoundaryViscosity bar
    uint32_t* CLAIM;          // [0] largest recomputed CFL |w|^2 (bits), [1] argmax claimed
    float4 *XBO, *VBO;        // x and v cotangents in original particle order
    TapeSet* ts;              // the recorded steps; BW[0] is the slot of the step being differentiated
    uint32_t* BW;             // [0] that slot, [1] Jacobi iterations of the current solve left to differentiate
    unsigned long long hLoop[2];  // conditional handles of the pressure [0] and divergence [1] Jacobi
                                  // loops of the backward graph (0: launched from the host)
    float tolScale;               // the adjoint viscosity solves' tolerance relative to the forward's
};

// The recorded step being differentiated.
__device__ __forceinline__ const TapeStep& bstep(const AdjDev& a) { return a.ts->steps[a.BW[0]]; }

// Jacobi loop control of the backward pass: a solve's recorded iterations are
// differentiated last to first, BW[1] counting those left; in a graph the loop's
// conditional handle follows it (loop_start from one thread of the pass before the loop,
// k_adj_loop_next at the end of each iteration).
template <bool DIV>
__device__ __forceinline__ void loop_start(const AdjDev& a, const TapeStep& T) {
    const uint32_t left = DIV ? T.kd : T.kp;
    a.BW[1] = left;
    if (a.hLoop[DIV]) cudaGraphSetConditional((cudaGraphConditionalHandle)a.hLoop[DIV], left > 0u ? 1u : 0u);
}

// The reference's cubic spline (Kernel/DFSPHKernels.h:86-131) and its derivatives.
struct Spline {
    float h, K;
    __device__ explicit Spline(float radius) : h(radius), K(8.0f / (3.14159265358979f * radius * radius * radius)) {}
    __device__ float w(float s) const {
        const float q = s / h;
        if (q <= 0.5f) return K * (6.0f * q * q * q - 6.0f * q * q + 1.0f);
        if (q <= 1.0f) {
            const float f = 1.0f - q;
            return 2.0f * K * f * f * f;
        }
        return 0.0f;
    }
    // W'(s) and W''(s).
    __device__ void d12(float s, float& w1, float& w2) const {
        const float q = s / h;
        if (q <= 0.5f) {
            w1 = K * (18.0f * q * q - 12.0f * q) / h;
            w2 = K * (36.0f * q - 12.0f) / (h * h);
        } else if (q <= 1.0f) {
            const float f = 1.0f - q;
            w1 = -6.0f * K * f * f / h;
            w2 = 12.0f * K * f / (h * h);
        } else {
            w1 = w2 = 0.0f;
        }
    }
    // gs = W'(s) / s and gq = gs'(s) / s: gradW(r) = gs r, d gradW / dr = gs I + gq r r^T.
    __device__ void hess(float s, float& gs, float& gq) const {
        const float q = s / h;
        if (q <= 0.5f) {
            gs = K * (18.0f * q - 12.0f) / (h * h);
            gq = 18.0f * K / (h * h * h * s);
        } else if (q <= 1.0f) {
            const float f = 1.0f - q;
            gs = -6.0f * K * f * f / (h * s);
            const float w2 = 12.0f * K * f / (h * h);
            gq = (w2 - gs) / (s * s);
        } else {
            gs = gq = 0.0f;
        }
    }
};

__device__ __forceinline__ float3 hmul(float gs, float gq, float3 r, float3 w) { return gs * w + (gq * dot3(r, w)) * r; }

struct Row {
    const uint32_t* nbr;
    uint32_t count, flags;
};
__device__ __forceinline__ Row row_of(const Dev& d, uint32_t p) {
    const uint32_t w = d.NCNT[p];
    return Row{d.NBR + (size_t)p * kRow, w & kCountMask, w};
}
// Row entry j: the neighbour slot; its gradW / r (the forward's table value) is
// grad_factor of the same pair vector, computed by the caller.
__device__ __forceinline__ uint32_t row_entry(const Row& rw, uint32_t j) { return __ldg(rw.nbr + j); }

__device__ __forceinline__ float4 bd(const AdjDev& a, const Dev& d, uint32_t k, uint32_t b, uint32_t p) {
    return a.BD[((size_t)k * d.maxBodies + b) * d.stride + p];
}

// J_GB^T y: GB_i = sum_b Vb W'(pd) n, so d(GB . y)/dx = sum_b (n . y)(W'(pd) grad Vb + Vb W''(pd) grad pd).
__device__ float3 jgb_t(const Dev& d, const AdjDev& a, const Spline& sp, uint32_t nb, uint32_t p, float3 y) {
    float3 out = make_float3(0.f, 0.f, 0.f);
    for (uint32_t b = 0; b < nb; b++) {
        const float4 b0 = bd(a, d, 0, b, p);
        if (!(b0.w > 0.0f)) continue;
        const float4 b1 = bd(a, d, 1, b, p), b2 = bd(a, d, 2, b, p);
        float w1, w2;
        sp.d12(b1.w, w1, w2);
        const float ny = dot3(f3(b0), y);
        out += ny * (w1 * f3(b2) + (b0.w * w2) * f3(b1));
    }
    return out;
}

// Adds the FP32 terms v of the block into dst (one atomic per block): each warp sums as
// an FP32 pair (warp_sum_pair), the warps' pairs likewise, widened to FP64 once; every
// thread of the block must call it.
__device__ void block_add(double* dst, float term) {
    __shared__ float2 part[32];
    const float2 v = warp_sum_pair(term, 1);
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) part[warp] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        float hi = 0.0f, lo = 0.0f;
        for (uint32_t w = 0; w < (blockDim.x + 31u) / 32u; w++) pair_add(hi, lo, part[w].x, part[w].y);
        const double t = pair_value(make_float2(hi, lo));
        if (t != 0.0) atomicAdd(dst, t);
    }
}

__device__ __forceinline__ double dot3d(float3 a, float3 b) {
    return (double)a.x * b.x + (double)a.y * b.y + (double)a.z * b.z;
}

#define ADJ_GROUP                                          \
    const Group<kAG> grp;                                  \
    const uint32_t p = grp.p;                              \
    const bool live = p < d.n;                             \
    const uint32_t pp = live ? p : 0u;                     \
    (void)pp;

// ---------------------------------------------------------------- boundary data
// The boundary kernel's decisions (k_boundary, ComputeVolumeAndBoundaryKernel
// DFSPHKernels.cu:69-150) replayed on the positions before it ran, keeping what the
// adjoint needs: per body (n, Vb), (grad pd, pd), (grad Vb), and the velocity reset.
__device__ void bdata_item(const Dev& d, const AdjDev& a, const SceneDev& S, uint32_t p, float3 x) {
    uint32_t stop = 0;
    for (uint32_t b = 0; b < S.bodyCount; b++) {
        const BodyDev& m = d.bodies[S.bodyBegin + b];
        const MapSample s = map_lookup<true>(m, x);
        const float dist = s.inside ? s.phi0 : FLT_MAX;
        float4 b0 = make_float4(0.f, 0.f, 0.f, 0.f), b1 = b0, b2 = b0;
        if (dist > 0.0f && dist < S.h) {
            const float volume = s.phi1;
            if (volume > 0.0f && volume != FLT_MAX) {
                const float nl = sqrtf(dot3(s.grad0, s.grad0));
                if (nl > 1.0e-9f) {
                    const float3 n = make_float3(s.grad0.x / nl, s.grad0.y / nl, s.grad0.z / nl);
                    const float raw = dist + 0.5f * S.r;
                    const float pd = fmaxf(raw, S.diam);
                    b0 = f4(n, volume);
                    b1 = f4(raw > S.diam ? s.grad0 : make_float3(0.f, 0.f, 0.f), pd);
                    b2 = f4(s.grad1, 0.0f);
                }
            }
        } else if (dist <= 0.0f) {
            const float nl = sqrtf(dot3(s.grad0, s.grad0));
            if (nl > 1.0e-5f) {
                const float3 n = make_float3(s.grad0.x / nl, s.grad0.y / nl, s.grad0.z / nl);
                x += fminf(S.diam - dist, 0.1f * S.r) * n;
                stop = 1;
            }
        }
        a.BD[((size_t)0 * d.maxBodies + b) * d.stride + p] = b0;
        a.BD[((size_t)1 * d.maxBodies + b) * d.stride + p] = b1;
        a.BD[((size_t)2 * d.maxBodies + b) * d.stride + p] = b2;
    }
    a.STOP[p] = stop;
}

// ---------------------------------------------------------------- Jacobi passes
// The kappa iterate a Jacobi pass of the recorded step works on: with U the iteration
// being differentiated (BW[1] - 1), else the solve's last iterate; and the scale c of
// the pass (dt_o for the divergence solve, dt_n^2 for the pressure solve).
template <bool HAS_U, bool DIV>
__device__ __forceinline__ const float* jacobi_kappa(const Dev& d, const AdjDev& a, const TapeStep& T) {
    const uint32_t k = HAS_U ? a.BW[1] - 1u : (DIV ? T.kd : T.kp);
    return (DIV ? T.KD : T.KP) + (size_t)k * d.stride;
}
template <bool DIV>
__device__ __forceinline__ float jacobi_scale(const TapeStep& T) { return DIV ? T.dto : T.dtn * T.dtn; }

// The output of a solve, for particle p with its recomputed acceleration ap, and the
// cotangent arrays of the solve's iterations set up; returns its term of the dt bar sum.
//   pressure (K20 + K21): x' = x + dt_n v3, v3 = v2 + dt_n a_p: v3 bar, dt_n bar;
//                         ABAR = dt_n v3 bar;
//   divergence (K7):      v1 = v0 + dt_o a_d: dt_o bar; ABAR = dt_o v1 bar.
template <bool DIV>
__device__ __forceinline__ float solve_output(const AdjDev& a, const TapeStep& T, uint32_t p, float3 ap) {
    float term;
    if (DIV) {
        const float3 vb = f3(a.VBAR[p]);
        term = dot3(ap, vb);
        a.ABAR[p] = f4(T.dto * vb, 0.f);
    } else {
        const float dtn = T.dtn;
        const float3 v3 = f3(T.V2[p]) + dtn * ap;
        const float3 xb = f3(a.XBAR[p]);
        const float3 vb = f3(a.VBAR[p]) + dtn * xb;
        term = dot3(v3, xb) + dot3(ap, vb);
        a.VBAR[p] = f4(vb, 0.f);
        a.ABAR[p] = f4(dtn * vb, 0.f);
    }
    a.KBAR[p] = 0.f;
    a.RABAR[p] = 0.f;
    a.APBAR[p] = 0.f;
    return term;
}

// AK = P(kap) as the forward computes it (masks |k_i + k_j| > eps, |k_i| > eps);
// with U: ABAR = c D^T(U) = c (V sum_j (u_i + u_j) gradW_ij + u_i GB_i). Without U (the
// solve's last iterate) it also takes the solve's output (solve_output).
template <bool HAS_U, bool DIV>
__global__ void __launch_bounds__(kBlock) k_adj_jac_a(Dev d, AdjDev a) {
    ADJ_GROUP
    const TapeStep& T = bstep(a);
    const float* __restrict__ kap = jacobi_kappa<HAS_U, DIV>(d, a, T);
    const float c = jacobi_scale<DIV>(T);
    const SceneDev& S = d.scenes[0];
    const float V = S.volume;
    float3 acc = make_float3(0.f, 0.f, 0.f), ab = acc;
    Row rw{};
    float ki = 0.f, ui = 0.f;
    float3 xi = acc;
    if (live) {
        rw = row_of(d, p);
        if (HAS_U) {
            const float2 kui = a.KU[p];
            ki = kui.x;
            ui = kui.y;
        } else {
            ki = kap[p];
        }
        xi = f3(d.X[p]);
        for (uint32_t j = grp.lane; j < rw.count; j += kAG) {
            const uint32_t q = row_entry(rw, j);
            const float3 r = xi - f3(d.X[q]);
            const float gs = grad_factor(d, r);
            float kq, uq = 0.f;
            if (HAS_U) {
                const float2 kuq = a.KU[q];
                kq = kuq.x;
                uq = kuq.y;
            } else {
                kq = kap[q];
            }
            const float sum = ki + kq;
            if (fabsf(sum) > kEps) acc += (sum * (-V * gs)) * r;
            if (HAS_U) ab += ((ui + uq) * (V * gs)) * r;
        }
    }
    acc = grp.sum(acc);
    if (HAS_U) ab = grp.sum(ab);
    float term = 0.0f;
    if (live && grp.lane == 0) {
        const float3 gb = f3(d.GB[p]);
        if (fabsf(ki) > kEps && (rw.flags & kHasBoundary)) acc += ki * (-gb);
        // .w: U and kappa, for the neighbours' gathers in k_adj_jac_b
        a.AK[p] = f4(acc, ui);
        if (HAS_U) a.ABAR[p] = f4(c * (ab + ui * gb), ki);
        else term = solve_output<DIV>(a, T, p, acc);
    }
    if (!HAS_U) block_add(a.SC + (DIV ? 0 : 1), term);
}

// KBAR += P^T(ABAR) (masked like P); XBAR += XP(kap, ABAR) + c XD(AK, U), where
// XP(k, ab)_i = -V sum_j e_ij (k_i + k_j) H_ij (ab_i - ab_j) - k_i J_GB^T ab_i and
// XD(w, u)_i = V sum_j H_ij (w_i - w_j)(u_i + u_j) + u_i J_GB^T w_i.
template <bool HAS_U, bool DIV>
__global__ void __launch_bounds__(kBlock) k_adj_jac_b(Dev d, AdjDev a) {
    ADJ_GROUP
    const TapeStep& T = bstep(a);
    if (!HAS_U && blockIdx.x == 0 && threadIdx.x == 0) loop_start<DIV>(a, T);  // the solve's iterations next
    const float* __restrict__ kap = jacobi_kappa<HAS_U, DIV>(d, a, T);
    const float c = jacobi_scale<DIV>(T);
    const SceneDev& S = d.scenes[0];
    const Spline sp(d.radius);
    const float V = S.volume;
    float kb = 0.f;
    float3 xp = make_float3(0.f, 0.f, 0.f), xd = xp;
    Row rw{};
    float ki = 0.f, ui = 0.f;
    float3 xi = xp, abi = xp, aki = xp;
    if (live) {
        rw = row_of(d, p);
        ki = kap[p];
        xi = f3(d.X[p]);
        abi = f3(a.ABAR[p]);
        if (HAS_U) {
            const float4 ak4 = a.AK[p];
            ui = ak4.w;
            aki = f3(ak4);
        }
        for (uint32_t j = grp.lane; j < rw.count; j += kAG) {
            const uint32_t q = row_entry(rw, j);
            const float3 r = xi - f3(d.X[q]);
            const float gsT = grad_factor(d, r);
            const float s = sqrtf(dot3(r, r));
            float gs, gq;
            sp.hess(s, gs, gq);
            const float4 abq = a.ABAR[q];  // (a bar, kappa) of the neighbour
            const float kq = HAS_U ? abq.w : kap[q];
            const float3 dab = abi - f3(abq);
            if (fabsf(ki + kq) > kEps) {
                kb += -V * gsT * dot3(r, dab);
                xp += (-V * (ki + kq)) * hmul(gs, gq, r, dab);
            }
            if (HAS_U) {
                const float4 akq = a.AK[q];  // (a^k, U) of the neighbour
                xd += (V * (ui + akq.w)) * hmul(gs, gq, r, aki - f3(akq));
            }
        }
    }
    kb = grp.sum(kb);
    xp = grp.sum(xp);
    if (HAS_U) xd = grp.sum(xd);
    if (!live || grp.lane != 0) return;
    if (rw.flags & kHasBoundary) {
        if (fabsf(ki) > kEps) {
            kb += -dot3(f3(d.GB[p]), abi);
            xp += -ki * jgb_t(d, a, sp, S.bodyCount, p, abi);
        }
        if (HAS_U) xd += ui * jgb_t(d, a, sp, S.bodyCount, p, aki);
    }
    a.KBAR[p] += kb;
    a.XBAR[p] = f4(f3(a.XBAR[p]) + xp + c * xd, 0.0f);
}

// VBAR += D^T(DBAR); XBAR += XD(w, DBAR); with DT also SC[1] += sum RABAR_i D_i(w).
template <bool DT>
__global__ void __launch_bounds__(kBlock) k_adj_div_b(Dev d, AdjDev a) {
    ADJ_GROUP
    const TapeStep& T = bstep(a);
    const float4* __restrict__ w = DT ? T.V2 : T.V0;  // v2 for the pressure solve's D, v0 for the divergence solve's
    const SceneDev& S = d.scenes[0];
    const Spline sp(d.radius);
    const float V = S.volume;
    float3 vb = make_float3(0.f, 0.f, 0.f), xd = vb, wi = vb, xi = vb;
    float di = 0.f, dv = 0.f;
    Row rw{};
    if (live) {
        rw = row_of(d, p);
        xi = f3(d.X[p]);
        wi = f3(w[p]);
        di = a.DBAR[p];
        for (uint32_t j = grp.lane; j < rw.count; j += kAG) {
            const uint32_t q = row_entry(rw, j);
            const float3 r = xi - f3(d.X[q]);
            const float gsT = grad_factor(d, r);
            const float s = sqrtf(dot3(r, r));
            float gs, gq;
            sp.hess(s, gs, gq);
            const float dq = a.DBAR[q];
            const float3 dw = wi - f3(w[q]);
            vb += ((di + dq) * (V * gsT)) * r;
            xd += (V * (di + dq)) * hmul(gs, gq, r, dw);
            if (DT) dv += gsT * dot3(dw, r);
        }
    }
    vb = grp.sum(vb);
    xd = grp.sum(xd);
    if (DT) dv = grp.sum(dv);
    float acc = 0.0f;
    if (live && grp.lane == 0) {
        if (rw.flags & kHasBoundary) {
            const float3 gb = f3(d.GB[p]);
            vb += di * gb;
            xd += di * jgb_t(d, a, sp, S.bodyCount, p, wi);
            dv = V * dv + dot3(wi, gb);
        } else {
            dv = V * dv;
        }
        a.VBAR[p] = f4(f3(a.VBAR[p]) + vb, 0.0f);
        a.XBAR[p] = f4(f3(a.XBAR[p]) + xd, 0.0f);
        if (DT) acc = a.RABAR[p] * dv;
    }
    if (DT) block_add(a.SC + 1, acc);
}

// ---------------------------------------------------------------- density and factor
// GSUM = (G_i, S bar_i) with G_i = V sum_j gradW_ij + GB_i and S bar = -alpha_bar alpha^2.
__global__ void __launch_bounds__(kBlock) k_adj_gsum(Dev d, AdjDev a) {
    ADJ_GROUP
    const SceneDev& S = d.scenes[0];
    const float V = S.volume;
    float3 g = make_float3(0.f, 0.f, 0.f);
    float g2 = 0.0f;
    Row rw{};
    if (live) {
        rw = row_of(d, p);
        const float3 xi = f3(d.X[p]);
        for (uint32_t j = grp.lane; j < rw.count; j += kAG) {
            const uint32_t q = row_entry(rw, j);
            const float3 rq = xi - f3(d.X[q]);
            const float gsT = grad_factor(d, rq);
            const float3 gj = (V * gsT) * rq;
            g += gj;
            g2 += dot3(gj, gj);
        }
    }
    g = grp.sum(g);
    g2 = grp.sum(g2);
    if (!live || grp.lane != 0) return;
    if (rw.flags & kHasBoundary) g += f3(d.GB[p]);
    g2 += dot3(g, g);
    const float al = d.ALPHA[p];
    const float sbar = g2 > kEps ? -a.ALBAR[p] * al * al : 0.0f;
    a.GSUM[p] = f4(g, sbar);
}

// XBAR += rho0 V sum_j gradW_ij (rb_i + rb_j) + rb_i rho0 sum_b (W(pd) grad Vb + Vb W'(pd) grad pd)
//       + 2 V^2 sum_j (sb_i + sb_j) H_ij gradW_ij + V sum_j H_ij (Gb_i - Gb_j) + J_GB^T Gb_i,
// with Gb = 2 sb G.
__global__ void __launch_bounds__(kBlock) k_adj_density(Dev d, AdjDev a) {
    ADJ_GROUP
    const SceneDev& S = d.scenes[0];
    const Spline sp(d.radius);
    const float V = S.volume;
    float3 acc = make_float3(0.f, 0.f, 0.f);
    Row rw{};
    float rbi = 0.f, sbi = 0.f;
    float3 gbi = acc;
    if (live) {
        rw = row_of(d, p);
        const float3 xi = f3(d.X[p]);
        rbi = a.RHOBAR[p];
        const float4 gi = a.GSUM[p];
        sbi = gi.w;
        gbi = (2.0f * gi.w) * f3(gi);
        for (uint32_t j = grp.lane; j < rw.count; j += kAG) {
            const uint32_t q = __ldg(rw.nbr + j);
            const float3 r = xi - f3(d.X[q]);
            const float s = sqrtf(dot3(r, r));
            float gs, gq;
            sp.hess(s, gs, gq);
            const float4 gj = a.GSUM[q];
            const float3 gw = gs * r;
            acc += (S.rho0 * V * (rbi + a.RHOBAR[q])) * gw;
            acc += (2.0f * V * V * (sbi + gj.w)) * hmul(gs, gq, r, gw);
            acc += V * hmul(gs, gq, r, gbi - (2.0f * gj.w) * f3(gj));
        }
    }
    acc = grp.sum(acc);
    if (!live || grp.lane != 0) return;
    if (rw.flags & kHasBoundary) {
        for (uint32_t b = 0; b < S.bodyCount; b++) {
            const float4 b0 = bd(a, d, 0, b, p);
            if (!(b0.w > 0.0f)) continue;
            const float4 b1 = bd(a, d, 1, b, p), b2 = bd(a, d, 2, b, p);
            float w1, w2;
            sp.d12(b1.w, w1, w2);
            acc += (rbi * S.rho0) * (sp.w(b1.w) * f3(b2) + (b0.w * w1) * f3(b1));
        }
        acc += jgb_t(d, a, sp, S.bodyCount, p, gbi);
    }
    // the step's input cotangents, back in original order (the boundary's velocity reset)
    const uint32_t o = bstep(a).PID[p];
    a.XBO[o] = f4(f3(a.XBAR[p]) + acc, 0.0f);
    a.VBO[o] = a.STOP[p] ? make_float4(0.f, 0.f, 0.f, 0.f) : a.VBAR[p];
}

// ---------------------------------------------------------------- viscosity
// lambda = d.CG solves A lambda = g_bar. With lt_i = (dt / rho_i) lambda_i and
// Q_i = sum_j T_ij + B_i g_i (A g = g - (dt / rho) Q):
//   XBAR += R(r, g_ij, cmu m (lt_i / rho_j - lt_j / rho_i)) over j, plus the boundary terms,
//   RHOBAR += -lt_i . Q_i / rho_i + sum_j (cmu m / rho_i^2)(g_ij . r) phi (lt_j . r),
//   SC[0] += lambda_i . Q_i / rho_i, SC[2] += rho0 lt_i . dQ_i/d mu, SC[3] += rho0 lt_i . dQ_i/d mu_b,
// where T_ij = cmu (m / rho_j)(g_ij . r) phi(|r|) r, phi = gs / (|r|^2 + eps2) and
// R(r, g, w) = phi ((r . w) g + (g . r) w) + (g . r)(r . w)(phi' / |r|) r.
// Also: v1 bar += lambda, this step's lambda kept for the next solves' initial guesses,
// and the solve's iterations counted.
__global__ void __launch_bounds__(kBlock) k_adj_visc(Dev d, AdjDev a) {
    const TapeStep& T = bstep(a);
    if (T.zeroG) return;  // g = 0 in the forward step: no solve to differentiate
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        const SceneDev& S0 = d.scenes[0];
        const uint32_t it = S0.cgIt;
        a.ACNT[0] += it;
        a.ACNT[1] = max(a.ACNT[1], it);
        a.ACNT[2] += 1u;
        if (!S0.cgZeroG) a.ACNT[3] = min(a.ACNT[3] + 1u, 2u);
    }
    if (d.scenes[0].cgZeroG) return;  // lambda = 0
    const float4* __restrict__ G = T.G;
    const float dt = T.dto;
    ADJ_GROUP
    const SceneDev& S = d.scenes[0];
    const Spline sp(d.radius);
    const float eps2 = 0.01f * S.h2;
    const float cmu = 10.0f * S.dynVisc;
    const float m = S.mass;
    float3 xacc = make_float3(0.f, 0.f, 0.f), q1 = xacc, qf = xacc;
    float racc = 0.f;
    Row rw{};
    float rhoi = 1.f;
    float3 xi = xacc, gi = xacc, lti = xacc, li = xacc;
    if (live) {
        rw = row_of(d, p);
        xi = f3(d.X[p]);
        gi = f3(G[p]);
        rhoi = d.RHO[p];
        li = f3(d.CG[p]);
        lti = (dt / rhoi) * li;
        for (uint32_t j = grp.lane; j < rw.count; j += kAG) {
            const uint32_t q = row_entry(rw, j);
            const float3 r = xi - f3(d.X[q]);
            const float gsT = grad_factor(d, r);
            const float s2 = dot3(r, r);
            const float s = sqrtf(s2);
            float gs, gq;
            sp.hess(s, gs, gq);
            const float rhoq = d.RHO[q];
            const float3 ltq = (dt / rhoq) * f3(d.CG[q]);
            const float3 g = gi - f3(G[q]);
            const float gr = dot3(g, r);
            const float den = s2 + eps2;
            const float phiT = gsT / den;
            // values (table gradient, as the forward)
            const float3 t1 = (10.0f * (m / rhoq) * gr * phiT) * r;
            q1 += t1;
            qf += S.dynVisc * t1;
            racc += (cmu * m / (rhoi * rhoi)) * gr * phiT * dot3(ltq, r);
            // position derivative (analytic spline)
            const float phi = gs / den;
            const float phis = gq / den - 2.0f * gs / (den * den);
            const float3 w = (cmu * m) * ((1.0f / rhoq) * lti - (1.0f / rhoi) * ltq);
            const float rw_ = dot3(r, w);
            xacc += phi * (rw_ * g + gr * w) + (gr * rw_ * phis) * r;
        }
    }
    xacc = grp.sum(xacc);
    q1 = grp.sum(q1);
    qf = grp.sum(qf);
    racc = grp.sum(racc);
    float s0 = 0.0f, s2v = 0.0f, s3v = 0.0f;
    if (live && grp.lane == 0) {
        float3 b1 = make_float3(0.f, 0.f, 0.f);  // B g per unit dynamic boundary viscosity
        if (S.dynBVisc != 0.0f && (rw.flags & kHasBoundary)) {
            for (uint32_t b = 0; b < S.bodyCount; b++) {
                const float4 b0 = bd(a, d, 0, b, p);
                if (!(b0.w > 0.0f)) continue;
                const float4 bp = bd(a, d, 1, b, p), bv = bd(a, d, 2, b, p);
                const float3 n = f3(b0);
                const float pd = bp.w;
                float3 t1, t2;
                orthogonal_vectors(-n, t1, t2);
                const float td = S.tangDist;
                const float3 off[4] = {-td * t1, td * t1, -td * t2, td * t2};
                const float c1 = 10.0f * 0.25f * b0.w;  // per unit dynamic boundary viscosity
                float dpd = 0.0f, dvb = 0.0f;
                for (int k = 0; k < 4; k++) {
                    const float3 dk = pd * n - off[k];
                    const float s2 = dot3(dk, dk);
                    const float s = sqrtf(s2);
                    const float den = s2 + eps2;
                    const float3 gk = kernel_grad(d, dk);
                    const float dg = dot3(dk, gi), dl = dot3(dk, lti);
                    // value: c (d . g) gradW(d)
                    b1 += (c1 * dg / den) * gk;
                    dvb += S.dynBVisc * c1 * dg / den * dot3(gk, lti);
                    float gs, gq;
                    sp.hess(s, gs, gq);
                    const float C = S.dynBVisc * c1;
                    const float beta = C * gs / den;
                    const float betas = C * (gq / den - 2.0f * gs / (den * den));
                    dpd += betas * dot3(dk, n) * dg * dl + beta * (dot3(n, gi) * dl + dg * dot3(n, lti));
                }
                xacc += dpd * f3(bp) + (dvb / b0.w) * f3(bv);
            }
        }
        const float3 Q = qf + S.dynBVisc * b1;
        racc += -dot3(lti, Q) / rhoi;
        a.XBAR[p] = f4(f3(a.XBAR[p]) + xacc, 0.0f);
        a.RHOBAR[p] += racc;
        a.VBAR[p] = f4(f3(a.VBAR[p]) + li, 0.f);
        a.LAM2[p] = a.LAM[p];
        a.LAM[p] = f4(li, 0.f);
        s0 = dot3(li, Q) / rhoi;
        s2v = S.rho0 * dot3(lti, q1);
        s3v = S.rho0 * dot3(lti, b1);
    }
    block_add(a.SC + 0, s0);
    block_add(a.SC + 2, s2v);
    block_add(a.SC + 3, s3v);
}

// ---------------------------------------------------------------- element-wise steps

// One Jacobi update k <- k - r alpha', r = min(c0 - rho_adv - f, 0) (c0 = 0 divergence,
// 1 pressure; r = 0 where skipped): U = [r < 0] alpha' k_bar; rho_adv bar += U,
// alpha' bar += -r k_bar; f = scale * D(P(k)) gives SC[slot] += fdt * U f.
template <bool DIV>
__global__ void k_adj_u(Dev d, AdjDev a) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    const TapeStep& T = bstep(a);
    const uint32_t k = a.BW[1] - 1u;
    const float* res = (DIV ? T.RD : T.RP) + (size_t)k * d.stride;
    const float* rhoadv = DIV ? T.RAD : T.RAP;
    const float* kap = (DIV ? T.KD : T.KP) + (size_t)k * d.stride;
    const float alphaScale = DIV ? 1.0f / T.dto : 1.0f / (T.dtn * T.dtn);
    const float fdt = DIV ? 1.0f / T.dto : 2.0f / T.dtn;
    float acc = 0.0f;
    if (p < d.n) {
        const float r = res[p];
        const float kb = a.KBAR[p];
        const float u = r < 0.0f ? d.ALPHA[p] * alphaScale * kb : 0.0f;
        a.U[p] = u;
        a.KU[p] = make_float2(kap[p], u);
        a.RABAR[p] += u;
        a.APBAR[p] += -r * kb;
        if (u != 0.0f) {
            const float f = (DIV ? 0.0f : 1.0f) - rhoadv[p] - r;
            acc = fdt * u * f;
        }
    }
    block_add(a.SC + (DIV ? 0 : 1), acc);
}

// Pressure solve start (K17): k0 = max(rho_adv - 1, 0) alpha'', rho_adv = rho / rho0 + dt_n D(v2),
// alpha'' = alpha / dt_n^2.
__global__ void k_adj_pres_init(Dev d, AdjDev a) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    const TapeStep& T = bstep(a);
    const float* rhoadv = T.RAP;
    const float dtn = T.dtn;
    float acc = 0.0f;
    if (p < d.n) {
        const SceneDev& S = d.scenes[0];
        const float ra = rhoadv[p];
        const float al = d.ALPHA[p];
        const float a2 = al / (dtn * dtn);
        const float kb = a.KBAR[p];
        const float rab = a.RABAR[p] + (ra > 1.0f ? a2 * kb : 0.0f);
        const float apb = a.APBAR[p] + fmaxf(ra - 1.0f, 0.0f) * kb;
        a.RABAR[p] = rab;
        a.RHOBAR[p] += rab / S.rho0;
        a.DBAR[p] = dtn * rab;
        a.ALBAR[p] += apb / (dtn * dtn);
        acc = -2.0f * apb * al / (dtn * dtn * dtn);
    }
    block_add(a.SC + 1, acc);
}

// Divergence solve start (K4): k0 = rho_adv alpha', rho_adv = [n >= 20] max(D(v0), 0),
// alpha' = alpha / dt_o.
__global__ void k_adj_div_init(Dev d, AdjDev a) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    const TapeStep& T = bstep(a);
    const float* rhoadv = T.RAD;
    const float dto = T.dto;
    float acc = 0.0f;
    if (p < d.n) {
        const float ra = rhoadv[p];
        const float al = d.ALPHA[p];
        const float kb = a.KBAR[p];
        const float rab = a.RABAR[p] + al / dto * kb;
        const float apb = a.APBAR[p] + ra * kb;
        const bool counted = (d.NCNT[p] & kCountMask) >= 20u;
        a.DBAR[p] = (counted && ra > 0.0f) ? rab : 0.0f;
        a.ALBAR[p] += apb / dto;
        acc = -apb * al / (dto * dto);
    }
    block_add(a.SC + 0, acc);
}

// Viscosity mode of the recorded step: 0 no viscosity, 1 viscosity, 2 viscosity with g = 0
// (the forward CG's right-hand side was zero).
__device__ __forceinline__ int visc_mode(const TapeStep& T, int visc) { return !visc ? 0 : (T.zeroG ? 2 : 1); }

// CFL (k_visc_finish + k_ctrl_dt): dt_n = 0.4 d / sqrt(|w*|^2) for the particle with the
// largest |w|^2 = |v1 + a dt_o|^2; d dt_n / d w = -dt_n w / |w|^2. k_adj_velocity finds
// the largest recomputed |w|^2, k_adj_cfl_visc gives its particle the derivative. Both do
// nothing when dt_n was not the CFL value (clamped to its bounds, or |w|^2 <= 0.1): the
// forward's own expression, evaluated again on the device, decides.
__device__ __forceinline__ bool cfl_active(const TapeStep& T) {
    return T.maxV2 > 0.1f && 0.4f * (T.pre.diam / sqrtf(T.maxV2)) == T.dtn;
}
// |w|^2 of particle p, rounded operation by operation (no contraction into fused
// multiply-adds), so that the kernel finding the maximum and the kernel matching it compute
// the same bits whatever the compiler does with their surroundings.
__device__ __forceinline__ float cfl_w2(const Dev& d, const float4* V1, const float4* G, uint32_t p, float dto,
                                        int mode, float3& w) {
    const SceneDev& S = d.scenes[0];
    const float3 v1 = f3(V1[p]);
    float3 acc = make_float3(S.g[0], S.g[1], S.g[2]);
    if (mode != 0) {
        const float3 g = mode == 1 ? f3(G[p]) : make_float3(0.f, 0.f, 0.f);
        const float inv = __fdiv_rn(1.0f, dto);
        acc.x = __fadd_rn(acc.x, __fmul_rn(inv, __fsub_rn(g.x, v1.x)));
        acc.y = __fadd_rn(acc.y, __fmul_rn(inv, __fsub_rn(g.y, v1.y)));
        acc.z = __fadd_rn(acc.z, __fmul_rn(inv, __fsub_rn(g.z, v1.z)));
    }
    w = make_float3(__fadd_rn(v1.x, __fmul_rn(acc.x, dto)), __fadd_rn(v1.y, __fmul_rn(acc.y, dto)),
                    __fadd_rn(v1.z, __fmul_rn(acc.z, dto)));
    return __fadd_rn(__fadd_rn(__fmul_rn(w.x, w.x), __fmul_rn(w.y, w.y)), __fmul_rn(w.z, w.z));
}

// v2 = v1 + dt_n a with a = gravity (+ (g - v1) / dt_o with viscosity; g = 0 when the CG
// right-hand side was zero).
__global__ void k_adj_velocity(Dev d, AdjDev a, int visc) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    const TapeStep& T = bstep(a);
    const float4* V1 = T.V1;
    const float4* G = T.G;
    const float dto = T.dto, dtn = T.dtn;
    const int mode = visc_mode(T, visc);
    float sn = 0.0f, so = 0.0f;
    if (p < d.n) {
        const SceneDev& S = d.scenes[0];
        const float3 grav = make_float3(S.g[0], S.g[1], S.g[2]);
        const float3 vb = f3(a.VBAR[p]);
        if (mode == 0) {
            sn = dot3(vb, grav);
            a.GBAR[p] = make_float4(0.f, 0.f, 0.f, 0.f);
        } else {
            const float3 v1 = f3(V1[p]);
            const float3 g = mode == 1 ? f3(G[p]) : make_float3(0.f, 0.f, 0.f);
            const float3 dg = g - v1;
            sn = dot3(vb, grav + (1.0f / dto) * dg);
            so = -(dtn / (dto * dto)) * dot3(vb, dg);
            a.GBAR[p] = mode == 1 ? f4((dtn / dto) * vb, 0.f) : make_float4(0.f, 0.f, 0.f, 0.f);
            a.VBAR[p] = f4((1.0f - dtn / dto) * vb, 0.f);
        }
        if (cfl_active(T)) {  // the largest recomputed |w|^2
            float3 w;
            atomicMax(a.CLAIM, __float_as_uint(cfl_w2(d, V1, G, p, dto, mode, w)));
        }
    }
    block_add(a.SC + 1, sn);
    block_add(a.SC + 0, so);
}

// Right-hand side and initial guess lambda_0 of the adjoint viscosity solve (mode:
// VFD_WARM_*). The forward CG solves A g = V from V + DV, so V = g_bar (0 when the forward
// step's right-hand side was zero: the CG then stops at once) and DV = lambda_0 - V. LAM
// holds the lambda of the step after this one, LAM2 the one after that (the forward CG of
// replayed steps reuses CG, so they are kept apart). Cold: lambda_0 = g_bar (DV = 0);
// previous: LAM; extrapolate: 2 LAM - LAM2, the linear extrapolation in time of the
// sequence of solutions, once two exist.
__device__ __forceinline__ void visc_start_item(const Dev& d, const AdjDev& a, const TapeStep& T, uint32_t p, int mode) {
    const bool zero = T.zeroG != 0u;
    d.V[p] = zero ? make_float4(0.f, 0.f, 0.f, 0.f) : a.GBAR[p];
    const uint32_t have = a.ACNT[3];
    if (zero || mode == 0 || have == 0) {
        d.DV[p] = make_float4(0.f, 0.f, 0.f, 0.f);
        return;
    }
    const float3 l1 = f3(a.LAM[p]);
    const float3 x0 = (mode == 2 && have >= 2) ? 2.0f * l1 - f3(a.LAM2[p]) : l1;
    d.DV[p] = f4(x0 - f3(a.GBAR[p]), 0.f);
}

// The CFL derivative for the particle with the largest recomputed |w|^2 (it claims it; ties
// go to one), then, with viscosity, the adjoint solve's start for every particle.
__global__ void k_adj_cfl_visc(Dev d, AdjDev a, int visc, int warm) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= d.n) return;
    const TapeStep& T = bstep(a);
    const int mode = visc_mode(T, visc);
    if (cfl_active(T)) {
        const float dtn = T.dtn, maxV2 = T.maxV2;
        float3 w;
        const float w2 = cfl_w2(d, T.V1, T.G, p, T.dto, mode, w);
        if (__float_as_uint(w2) == a.CLAIM[0] && atomicExch(a.CLAIM + 1, 1u) == 0u) {
            const SceneDev& S = d.scenes[0];
            const float3 grav = make_float3(S.g[0], S.g[1], S.g[2]);
            const float dtnb = (float)a.SC[1];
            const float3 wb = (-dtnb * dtn / maxV2) * w;
            atomicAdd(a.SC + 0, dot3d(wb, grav));
            if (mode == 1) a.GBAR[p] = f4(f3(a.GBAR[p]) + wb, 0.f);
            else if (mode == 0) a.VBAR[p] = f4(f3(a.VBAR[p]) + wb, 0.f);
        }
    }
    if (visc) visc_start_item(d, a, T, p, warm);
}

// dt_o of this step is dt_n of the step before; the next step to differentiate is the
// one before (the slot below).
__global__ void k_adj_carry(AdjDev a) {
    a.SC[1] = a.SC[0];
    a.SC[0] = 0.0;
    a.CLAIM[0] = 0u;
    a.CLAIM[1] = 0u;
    if (a.BW[0] > 0u) a.BW[0] -= 1u;
}

// The bank a backward segment reads and the slot of its first step (the segment's last).
__global__ void k_adj_set_slot(AdjDev a, TapeStep* steps, uint32_t slot) {
    a.ts->steps = steps;
    a.BW[0] = slot;
}

// The forward arrays of the recorded step: positions before the step, neighbour counts and
// rows, and the scene state at its start (the first block copies it word by word; the
// adjoint viscosity solve's tolerance is the forward's scaled by tolScale).
__global__ void k_adj_fetch(Dev d, AdjDev a) {
    const TapeStep& T = bstep(a);
    if (blockIdx.x == 0) {
        static_assert(sizeof(SceneDev) % 4 == 0, "SceneDev is copied in 32-bit words");
        const uint32_t* src = reinterpret_cast<const uint32_t*>(&T.pre);
        uint32_t* dst = reinterpret_cast<uint32_t*>(d.scenes);
        for (uint32_t w = threadIdx.x; w < sizeof(SceneDev) / 4; w += blockDim.x) dst[w] = src[w];
        __syncthreads();
        if (threadIdx.x == 0) d.scenes[0].maxErrV = T.pre.maxErrV * a.tolScale;
    }
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= d.n) return;
    const float4 x = T.Xpre[p];
    d.X[p] = x;
    d.NCNT[p] = T.NCNT[p];
    const uint4* rs = reinterpret_cast<const uint4*>(T.NBR + (size_t)p * kRow);
    uint4* rd = reinterpret_cast<uint4*>(d.NBR + (size_t)p * kRow);
#pragma unroll
    for (uint32_t k = 0; k < kRow / 4u; k++) rd[k] = rs[k];
    // the boundary data on the positions before the boundary kernel moves them (the scene
    // constants it reads are those of the step's start), and the step's output cotangents
    // in slot order
    bdata_item(d, a, T.pre, p, f3(x));
    const uint32_t o = T.PID[p];
    a.XBAR[p] = a.XBO[o];
    a.VBAR[p] = a.VBO[o];
    a.RHOBAR[p] = 0.f;
    a.ALBAR[p] = 0.f;
}

template <bool DIV>
__global__ void k_adj_loop_next(AdjDev a) {
    const uint32_t left = a.BW[1] - 1u;
    a.BW[1] = left;
    if (a.hLoop[DIV]) cudaGraphSetConditional((cudaGraphConditionalHandle)a.hLoop[DIV], left > 0u ? 1u : 0u);
}

// ---------------------------------------------------------------- tape points
__device__ __forceinline__ TapeStep& tape_step(const TapeSet* ts) { return ts->steps[*ts->cur]; }

__global__ void k_tape_begin(Dev d, const TapeSet* ts) {
    TapeStep& T = tape_step(ts);
    T.pre = d.scenes[0];
    T.kd = T.kp = T.overflow = 0u;
}

__global__ void k_tape_search(Dev d, const TapeSet* ts) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= d.n) return;
    TapeStep& T = tape_step(ts);
    T.Xpre[p] = d.X[p];
    T.PID[p] = d.PID[p];
    T.NCNT[p] = d.NCNT[p];
    const uint4* src = reinterpret_cast<const uint4*>(d.NBR + (size_t)p * kRow);
    uint4* dst = reinterpret_cast<uint4*>(T.NBR + (size_t)p * kRow);
#pragma unroll
    for (uint32_t k = 0; k < kRow / 4u; k++) dst[k] = src[k];
}

// which: 0 V -> V0, 1 V -> V1, 2 CG -> G, 3 V -> V2
__global__ void k_tape_vec(Dev d, const TapeSet* ts, int which) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= d.n) return;
    TapeStep& T = tape_step(ts);
    float4* dst = which == 0 ? T.V0 : which == 1 ? T.V1 : which == 2 ? T.G : T.V2;
    dst[p] = which == 2 ? d.CG[p] : d.V[p];
}

// Start of a solve: kappa^0 and rho_adv; after iteration k (the controller has counted
// it): res^k and kappa^(k+1).
template <bool DIV>
__global__ void k_tape_solve(Dev d, const TapeSet* ts, int start) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= d.n) return;
    TapeStep& T = tape_step(ts);
    const SceneDev& S = d.scenes[0];
    const float* kap = DIV ? d.KAPPAV : d.KAPPA;
    float* K = DIV ? T.KD : T.KP;
    float* R = DIV ? T.RD : T.RP;
    const uint32_t cap = DIV ? T.capD : T.capP;
    if (start) {
        K[p] = kap[p];
        (DIV ? T.RAD : T.RAP)[p] = d.RHOADV[p];
        return;
    }
    const uint32_t it = DIV ? S.div.it : S.pres.it;
    if (it == 0u || it > cap) {
        if (p == 0) T.overflow = 1u;
        return;
    }
    R[(size_t)(it - 1u) * d.stride + p] = d.RES[p];
    K[(size_t)it * d.stride + p] = kap[p];
    if (p == 0) {
        if (DIV) T.kd = it;
        else T.kp = it;
    }
}

__global__ void k_tape_end(Dev d, TapeSet* ts) {
    TapeStep& T = tape_step(ts);
    const SceneDev& S = d.scenes[0];
    T.dto = T.pre.dt;
    T.dtn = S.dt;
    T.maxV2 = S.maxV2;
    T.zeroG = S.enableVisc && S.cgZeroG ? 1u : 0u;
    T.maxNbr = S.maxNbr;
    T.aborted = d.status[1];
    *ts->cur += 1u;
}

}  // namespace

namespace host {
void tape_point(const Dev& d, const void* rec, int point, cudaStream_t st) {
    TapeSet* ts = const_cast<TapeSet*>(static_cast<const TapeSet*>(rec));
    const uint32_t g = blocks_for(d.n);
    switch (point) {
        case kTapeBegin: k_tape_begin<<<1, 1, 0, st>>>(d, ts); break;
        case kTapeSearch: k_tape_search<<<g, kBlock, 0, st>>>(d, ts); break;
        case kTapeBoundary: k_tape_vec<<<g, kBlock, 0, st>>>(d, ts, 0); break;
        case kTapeDivInit: k_tape_solve<true><<<g, kBlock, 0, st>>>(d, ts, 1); break;
        case kTapeDivIter: k_tape_solve<true><<<g, kBlock, 0, st>>>(d, ts, 0); break;
        case kTapeDivFinish: k_tape_vec<<<g, kBlock, 0, st>>>(d, ts, 1); break;
        case kTapeVisc: k_tape_vec<<<g, kBlock, 0, st>>>(d, ts, 2); break;
        case kTapeVelocity: k_tape_vec<<<g, kBlock, 0, st>>>(d, ts, 3); break;
        case kTapePresInit: k_tape_solve<false><<<g, kBlock, 0, st>>>(d, ts, 1); break;
        case kTapePresIter: k_tape_solve<false><<<g, kBlock, 0, st>>>(d, ts, 0); break;
        case kTapeEnd: k_tape_end<<<1, 1, 0, st>>>(d, ts); break;
        default: break;
    }
}
}  // namespace host

namespace {

struct Checkpoint {
    float4 *XN = nullptr, *V = nullptr, *DV = nullptr;
    float* DK = nullptr;
    uint32_t* PID = nullptr;
    std::vector<SceneDev> scenes;
    uint32_t status[16] = {};
    int cs = 0;
};

}  // namespace

// One segment's recorded steps: `every` device slots and host copies of them (the
// device-written fields after record_segment reads them back).
struct TapeBank {
    std::vector<TapeStep> host;
    TapeStep* dsteps = nullptr;
    uint32_t* dcur = nullptr;
};

// The settings a replaying copy of the simulation must share with it.
struct ShadowKey {
    vfd_desc desc{};
    uint8_t lanes[16] = {}, tiles[16] = {};
    uint16_t blocks[16] = {};
    uint32_t n = 0, graphs = 0, analytic = 0, cellCap = 0;
    bool operator==(const ShadowKey& o) const {
        return std::memcmp(&desc, &o.desc, sizeof(desc)) == 0 && std::memcmp(lanes, o.lanes, sizeof(lanes)) == 0 &&
               std::memcmp(tiles, o.tiles, sizeof(tiles)) == 0 && std::memcmp(blocks, o.blocks, sizeof(blocks)) == 0 &&
               n == o.n && graphs == o.graphs && analytic == o.analytic && cellCap == o.cellCap;
    }
};

struct AdjointState {
    uint32_t steps = 0, every = 0, n = 0, stride = 0;
    uint64_t generation = 0;
    std::vector<Checkpoint> ckpt;  // ckpt[k]: before step k * every; back(): after the last step
    // bank[0]: what the simulation itself records (the forward run's last segment, replays
    // without a shadow); bank[1]: what the shadow records while a backward pass reads the other
    TapeBank bank[2];
    TapeSet* bset = nullptr;       // the backward pass's tape set: the bank of the segment it walks
    // A copy of the simulation (its own buffers and stream; the volume maps borrowed) that
    // replays the segment before the one the backward pass walks, into the other bank.
    vfd_sim* shadow = nullptr;
    ShadowKey shadowKey{};
    cudaEvent_t bankRead[2] = {nullptr, nullptr};  // the backward pass has finished reading bank k
    bool lastRecorded = false;     // the forward run recorded its last segment
    uint32_t replayed = 0;         // steps re-run by the last backward pass
    std::vector<void*> allocs;
    AdjDev a{};
    ~AdjointState() {
        for (cudaEvent_t& e : bankRead)
            if (e) cudaEventDestroy(e);
        delete shadow;
        for (void* p : allocs) cudaFree(p);
    }
};

namespace {

using namespace vfd::host;

template <class T>
int aalloc(AdjointState* A, T** p, size_t count) {
    void* q = nullptr;
    const size_t bytes = std::max<size_t>(1, count) * sizeof(T);
    const cudaError_t e = cudaMalloc(&q, bytes);
    if (e != cudaSuccess) return fail(VFD_E_NOMEM, "adjoint: cudaMalloc(%zu bytes): %s", bytes, cudaGetErrorString(e));
    A->allocs.push_back(q);
    *p = (T*)q;
    return VFD_OK;
}

// Bytes of one tape slot (one recorded step), iterates sized by the scene's iteration caps.
size_t tape_step_bytes(vfd_sim* s) {
    const size_t st = s->stride;
    const vfd_desc& dd = s->scenes[0].desc;
    const uint32_t capD = s->anyDiv ? dd.MaxDivergenceSolverIterations : 0u, capP = dd.MaxPressureSolverIterations;
    return st * (5 * sizeof(float4) + (2 + kRow) * sizeof(uint32_t) + 2 * sizeof(float)) +
           st * sizeof(float) * (2 * (size_t)capD + 1 + 2 * (size_t)capP + 1);
}

// `every` tape slots.
int alloc_bank(vfd_sim* s, AdjointState* A, TapeBank& B) {
    const size_t st = s->stride;
    const vfd_desc& dd = s->scenes[0].desc;
    const uint32_t capD = s->anyDiv ? dd.MaxDivergenceSolverIterations : 0u, capP = dd.MaxPressureSolverIterations;
    B.host.assign(A->every, TapeStep{});
    for (auto& T : B.host) {
        TRY(aalloc(A, &T.Xpre, st));
        TRY(aalloc(A, &T.V0, st));
        TRY(aalloc(A, &T.V1, st));
        TRY(aalloc(A, &T.G, st));
        TRY(aalloc(A, &T.V2, st));
        TRY(aalloc(A, &T.PID, st));
        TRY(aalloc(A, &T.NCNT, st));
        TRY(aalloc(A, &T.NBR, st * kRow));
        TRY(aalloc(A, &T.RAD, st));
        TRY(aalloc(A, &T.RAP, st));
        TRY(aalloc(A, &T.KD, st * (capD + 1)));
        TRY(aalloc(A, &T.RD, st * std::max<uint32_t>(1u, capD)));
        TRY(aalloc(A, &T.KP, st * (capP + 1)));
        TRY(aalloc(A, &T.RP, st * std::max<uint32_t>(1u, capP)));
        T.capD = capD;
        T.capP = capP;
    }
    TRY(aalloc(A, &B.dsteps, A->every));
    TRY(aalloc(A, &B.dcur, 1));
    CK(cudaMemcpy(B.dsteps, B.host.data(), sizeof(TapeStep) * A->every, cudaMemcpyHostToDevice));
    return VFD_OK;
}

// The recording tape set of simulation `sim` (its recording graphs address it; it lives
// with the simulation's buffers, so it is made again after they are reallocated).
int recording_set(vfd_sim* sim, TapeSet*& rec) {
    if (!sim->adjTapeSet) {
        TapeSet* p = nullptr;
        TRY(dalloc(sim, &p, 1));
        sim->adjTapeSet = p;
    }
    rec = static_cast<TapeSet*>(sim->adjTapeSet);
    return VFD_OK;
}

// Bank 0.
int alloc_tape(vfd_sim* s, AdjointState* A) {
    size_t freeB = 0, totalB = 0;
    CK(cudaMemGetInfo(&freeB, &totalB));
    const size_t per = tape_step_bytes(s);
    if (per * A->every > freeB / 2)
        return fail(VFD_E_NOMEM, "adjoint: %zu bytes of tape for %u steps exceed half the free device memory; "
                                 "use a smaller checkpoint_every", per * A->every, A->every);
    return alloc_bank(s, A, A->bank[0]);
}

int save_checkpoint(vfd_sim* s, AdjointState* A, Checkpoint& c) {
    const size_t st = s->stride;
    if (!c.XN) {
        TRY(aalloc(A, &c.XN, st));
        TRY(aalloc(A, &c.V, st));
        TRY(aalloc(A, &c.DV, st));
        TRY(aalloc(A, &c.DK, st));
        TRY(aalloc(A, &c.PID, st));
    }
    const Dev& d = s->dev[s->cs];
    cudaStream_t st_ = s->stream;
    CK(cudaMemcpyAsync(c.XN, d.XN, sizeof(float4) * st, cudaMemcpyDeviceToDevice, st_));
    CK(cudaMemcpyAsync(c.V, d.Vc, sizeof(float4) * st, cudaMemcpyDeviceToDevice, st_));
    CK(cudaMemcpyAsync(c.DV, d.DVc, sizeof(float4) * st, cudaMemcpyDeviceToDevice, st_));
    CK(cudaMemcpyAsync(c.DK, d.DKc, sizeof(float) * st, cudaMemcpyDeviceToDevice, st_));
    CK(cudaMemcpyAsync(c.PID, d.PIDc, sizeof(uint32_t) * st, cudaMemcpyDeviceToDevice, st_));
    c.scenes.resize(s->hScenes.size());
    CK(cudaMemcpyAsync(c.scenes.data(), s->dScenes, sizeof(SceneDev) * c.scenes.size(), cudaMemcpyDeviceToHost, st_));
    CK(cudaMemcpyAsync(c.status, s->dStatus, sizeof(c.status), cudaMemcpyDeviceToHost, st_));
    CK(cudaStreamSynchronize(st_));
    c.cs = s->cs;
    return VFD_OK;
}

int restore_checkpoint(vfd_sim* s, const Checkpoint& c) {
    const size_t st = s->stride;
    s->cs = c.cs;
    const Dev& d = s->dev[s->cs];
    cudaStream_t st_ = s->stream;
    CK(cudaMemcpyAsync(d.XN, c.XN, sizeof(float4) * st, cudaMemcpyDeviceToDevice, st_));
    CK(cudaMemcpyAsync(d.Vc, c.V, sizeof(float4) * st, cudaMemcpyDeviceToDevice, st_));
    CK(cudaMemcpyAsync(d.DVc, c.DV, sizeof(float4) * st, cudaMemcpyDeviceToDevice, st_));
    CK(cudaMemcpyAsync(d.DKc, c.DK, sizeof(float) * st, cudaMemcpyDeviceToDevice, st_));
    CK(cudaMemcpyAsync(d.PIDc, c.PID, sizeof(uint32_t) * st, cudaMemcpyDeviceToDevice, st_));
    CK(cudaMemcpyAsync(s->dScenes, c.scenes.data(), sizeof(SceneDev) * c.scenes.size(), cudaMemcpyHostToDevice, st_));
    CK(cudaMemcpyAsync(s->dStatus, c.status, sizeof(c.status), cudaMemcpyHostToDevice, st_));
    CK(cudaStreamSynchronize(st_));
    s->hScenes = c.scenes;
    return VFD_OK;
}

// `count` steps of simulation `sim` from its current state, recorded into bank B's slots
// 0..count-1 through sim's recording tape set, as CUDA graphs (one per parity) unless
// graphs are off; then the slots' device-written fields are read back and checked. Runs
// on sim's stream.
int record_segment(vfd_sim* sim, AdjointState* A, TapeBank& B, uint32_t count) {
    cudaStream_t st = sim->stream;
    TapeSet* rec = nullptr;
    TRY(recording_set(sim, rec));
    const TapeSet ts{B.dsteps, B.dcur, A->every};
    CK(cudaMemcpyAsync(rec, &ts, sizeof(ts), cudaMemcpyHostToDevice, st));
    CK(cudaMemsetAsync(B.dcur, 0, sizeof(uint32_t), st));
    const bool graphs = sim->graphMode && !sim->graphFailed;
    for (uint32_t t = 0; t < count; t++) {
        if (graphs && !sim->adjRecExec[sim->cs])
            TRY(build_graph(sim, sim->cs, rec, &sim->adjRecGraph[sim->cs], &sim->adjRecExec[sim->cs]));
        if (graphs) CK(cudaGraphLaunch(sim->adjRecExec[sim->cs], st));
        else TRY(launch_eager(sim, rec));
        sim->cs = 1 - sim->cs;
    }
    std::vector<TapeStep> dev(count);
    CK(cudaMemcpyAsync(dev.data(), B.dsteps, sizeof(TapeStep) * count, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    CK(cudaGetLastError());
    CK(cudaMemsetAsync(sim->dStatus + 7, 0, sizeof(uint32_t), st));
    for (uint32_t t = 0; t < count; t++) {
        const TapeStep& T = dev[t];
        if (T.aborted) return fail(VFD_E_STATE, "adjoint: a recorded step aborted (grid capacity or non-finite position)");
        if (T.overflow) return fail(VFD_E_STATE, "adjoint: solver iterations exceeded the tape capacity");
        if (T.maxNbr >= kMaxNeighbors)
            return fail(VFD_E_CAPACITY, "adjoint: a particle reached the %u-neighbour cap (neighbour sets must be "
                                        "symmetric)", kMaxNeighbors);
        TapeStep& H = B.host[t];
        H.pre = T.pre;
        H.kd = T.kd;
        H.kp = T.kp;
        H.zeroG = T.zeroG;
        H.dto = T.dto;
        H.dtn = T.dtn;
        H.maxV2 = T.maxV2;
    }
    return VFD_OK;
}

ShadowKey shadow_key(const vfd_sim* s) {
    ShadowKey k;
    k.desc = s->scenes[0].desc;
    std::memcpy(k.lanes, s->lanes, sizeof(k.lanes));
    std::memcpy(k.tiles, s->tiles, sizeof(k.tiles));
    std::memcpy(k.blocks, s->blocks, sizeof(k.blocks));
    k.n = s->n;
    k.graphs = s->graphMode && !s->graphFailed ? 1u : 0u;
    k.analytic = s->analyticKernel ? 1u : 0u;
    k.cellCap = s->cellCap;
    return k;
}

// The shadow simulation and bank 1, made (or remade, when the simulation's settings
// changed) for a backward pass over more than one segment. Returns false, with nothing
// made, when the second bank does not fit in half the free device memory or the copy
// cannot be set up: the backward pass then replays on the simulation itself.
bool ensure_shadow(vfd_sim* s, AdjointState* A) {
    const ShadowKey key = shadow_key(s);
    if (A->shadow && A->shadowKey == key) return true;
    delete A->shadow;
    A->shadow = nullptr;
    if (A->bank[1].host.empty()) {
        size_t freeB = 0, totalB = 0;
        if (cudaMemGetInfo(&freeB, &totalB) != cudaSuccess || tape_step_bytes(s) * A->every > freeB / 2) return false;
        if (alloc_bank(s, A, A->bank[1]) != VFD_OK) return false;
    }
    for (cudaEvent_t& e : A->bankRead)
        if (!e && cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return false;
    vfd_sim* t = new (std::nothrow) vfd_sim();
    if (!t) return false;
    t->device = s->device;
    if (cudaStreamCreateWithFlags(&t->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete t;
        return false;
    }
    t->scenes = s->scenes;
    t->borrowedBodies = true;  // the volume maps stay the simulation's
    t->table = s->table;
    t->halton = s->halton;
    t->graphMode = key.graphs != 0u;
    t->analyticKernel = s->analyticKernel;
    t->reserve = s->reserve;
    t->cellCap = s->cellCap;  // the search grid the simulation grew to, so replays do not abort on it
    std::memcpy(t->lanes, s->lanes, sizeof(t->lanes));
    std::memcpy(t->tiles, s->tiles, sizeof(t->tiles));
    std::memcpy(t->blocks, s->blocks, sizeof(t->blocks));
    if (ensure_ready(t) != VFD_OK || t->n != s->n || t->stride != s->stride) {
        delete t;
        cudaGetLastError();
        return false;
    }
    A->shadow = t;
    A->shadowKey = key;
    return true;
}

// ---------------------------------------------------------------- backward pass of one step
// The backward pass of recorded step BW[0] in stages, shared by the backward graph (one
// per simulation, launched once per step, its loops conditional nodes) and the host-driven
// path (loops counted on the host). Every kernel reads what it needs of the step (arrays,
// time steps, iteration counts, decisions) from its tape slot, so the same launches serve
// every step; a.hLoop / d.condHandle are the graph's conditional handles, or 0.
struct BwdLaunch {
    Dev d;
    AdjDev a;
    cudaStream_t st;
    uint32_t g1, gG;
    int visc, warm;
};

// Step inputs, boundary data, density and factor; the pressure solve's output (K20 + K21,
// v3 and x') and the start of its Jacobi iterations.
void bwd_head(const BwdLaunch& L, uint32_t* dStatus) {
    cudaMemsetAsync(dStatus, 0, 16 * sizeof(uint32_t), L.st);
    k_adj_fetch<<<L.g1, kBlock, 0, L.st>>>(L.d, L.a);
    launch_boundary(L.d, L.st);
    launch_density(L.d, L.st);
    k_adj_jac_a<false, false><<<L.gG, kBlock, 0, L.st>>>(L.d, L.a);
    k_adj_jac_b<false, false><<<L.gG, kBlock, 0, L.st>>>(L.d, L.a);
}

// One Jacobi iteration of a solve, differentiated (the last first).
template <bool DIV>
void bwd_jacobi(const BwdLaunch& L) {
    k_adj_u<DIV><<<L.g1, kBlock, 0, L.st>>>(L.d, L.a);
    k_adj_jac_a<true, DIV><<<L.gG, kBlock, 0, L.st>>>(L.d, L.a);
    k_adj_jac_b<true, DIV><<<L.gG, kBlock, 0, L.st>>>(L.d, L.a);
    k_adj_loop_next<DIV><<<1, 1, 0, L.st>>>(L.a);
}

// Pressure solve start (K17), K16 velocity update and the CFL time step; with viscosity the
// start of the adjoint solve A lambda = g_bar with the forward's CG.
void bwd_mid(const BwdLaunch& L) {
    k_adj_pres_init<<<L.g1, kBlock, 0, L.st>>>(L.d, L.a);
    k_adj_div_b<true><<<L.gG, kBlock, 0, L.st>>>(L.d, L.a);
    k_adj_velocity<<<L.g1, kBlock, 0, L.st>>>(L.d, L.a, L.visc);
    k_adj_cfl_visc<<<L.g1, kBlock, 0, L.st>>>(L.d, L.a, L.visc, L.warm);
    if (L.visc) launch_visc_init(L.d, L.st);
}

// After the adjoint viscosity solve: v1 bar += lambda, and the derivative of A g = v1.
void bwd_visc_tail(const BwdLaunch& L) {
    k_adj_visc<<<L.gG, kBlock, 0, L.st>>>(L.d, L.a);
}

// Divergence solve (K4-K7): its output v1 = v0 + dt_o a_d, then its iterations.
void bwd_div_head(const BwdLaunch& L) {
    k_adj_jac_a<false, true><<<L.gG, kBlock, 0, L.st>>>(L.d, L.a);
    k_adj_jac_b<false, true><<<L.gG, kBlock, 0, L.st>>>(L.d, L.a);
}
void bwd_div_tail(const BwdLaunch& L) {
    k_adj_div_init<<<L.g1, kBlock, 0, L.st>>>(L.d, L.a);
    k_adj_div_b<false><<<L.gG, kBlock, 0, L.st>>>(L.d, L.a);
}

// Density and factor (K2 + K3), the boundary's velocity reset and original order; the
// step before is next.
void bwd_end(const BwdLaunch& L) {
    k_adj_gsum<<<L.gG, kBlock, 0, L.st>>>(L.d, L.a);
    k_adj_density<<<L.gG, kBlock, 0, L.st>>>(L.d, L.a);
    k_adj_carry<<<1, 1, 0, L.st>>>(L.a);
}

BwdLaunch bwd_launch(vfd_sim* s, const AdjointState* A, cudaStream_t st) {
    BwdLaunch L{};
    L.d = s->dev[0];
    L.d.rowLoops = 1u;  // the recorded rows; the cell tables are not the recorded step's
    for (auto& h : L.d.condHandle) h = 0ull;
    L.a = A->a;
    L.a.hLoop[0] = L.a.hLoop[1] = 0ull;
    L.st = st;
    L.g1 = blocks_for(s->n);
    L.gG = blocks_for(s->n * kAG);
    L.visc = s->anyVisc ? 1 : 0;
    L.warm = s->adjWarm;
    L.a.tolScale = s->adjTol;
    return L;
}

// The backward pass of one step as a graph: the Jacobi loops and the adjoint CG as
// conditional WHILE nodes whose handles the loop-control kernels set.
int build_backward_graph(vfd_sim* s, AdjointState* A) {
    cudaGraph_t g;
    CK(cudaGraphCreate(&g, 0));
    const bool div = s->anyDiv, visc = s->anyVisc;
    cudaGraphConditionalHandle hP = 0, hD = 0, hC = 0;
    cudaError_t e = cudaGraphConditionalHandleCreate(&hP, g, 0, 0);
    if (e == cudaSuccess && div) e = cudaGraphConditionalHandleCreate(&hD, g, 0, 0);
    if (e == cudaSuccess && visc) e = cudaGraphConditionalHandleCreate(&hC, g, 0, 0);
    if (e != cudaSuccess) {
        cudaGraphDestroy(g);
        return fail(VFD_E_CUDA, "adjoint: cudaGraphConditionalHandleCreate: %s", cudaGetErrorString(e));
    }
    BwdLaunch L = bwd_launch(s, A, s->stream);
    L.a.hLoop[0] = (unsigned long long)hP;
    L.a.hLoop[1] = (unsigned long long)hD;
    L.d.condHandle[1] = (unsigned long long)hC;  // the CG loop's (set_condition of the forward's CG kernels)
    uint32_t* dStatus = s->dStatus;
    std::vector<cudaGraphNode_t> leaves;
    cudaStream_t cap = s->stream;
    e = add_segment(cap, g, leaves, [&](cudaStream_t st) {
        L.st = st;
        bwd_head(L, dStatus);
    });
    if (e == cudaSuccess) e = add_while(cap, g, hP, leaves, [&](cudaStream_t st) {
        L.st = st;
        bwd_jacobi<false>(L);
    });
    if (e == cudaSuccess) e = add_segment(cap, g, leaves, [&](cudaStream_t st) {
        L.st = st;
        bwd_mid(L);
    });
    if (e == cudaSuccess && visc) e = add_while(cap, g, hC, leaves, [&](cudaStream_t st) { launch_cg_iter(L.d, st); });
    if (e == cudaSuccess) e = add_segment(cap, g, leaves, [&](cudaStream_t st) {
        L.st = st;
        if (visc) bwd_visc_tail(L);
        if (div) bwd_div_head(L);
    });
    if (e == cudaSuccess && div) e = add_while(cap, g, hD, leaves, [&](cudaStream_t st) {
        L.st = st;
        bwd_jacobi<true>(L);
    });
    if (e == cudaSuccess) e = add_segment(cap, g, leaves, [&](cudaStream_t st) {
        L.st = st;
        if (div) bwd_div_tail(L);
        bwd_end(L);
    });
    cudaGraphExec_t exec = nullptr;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, g, 0);
    if (e != cudaSuccess) {
        cudaGetLastError();
        cudaGraphDestroy(g);
        return fail(VFD_E_CUDA, "adjoint: backward graph construction failed: %s", cudaGetErrorString(e));
    }
    s->adjBwdGraph = g;
    s->adjBwdExec = exec;
    return VFD_OK;
}

// Backward pass of recorded step t (tape slot t, which BW[0] holds) from the host: the
// loops run the recorded iteration counts, the CG reads its flag once per iteration.
// A->a.XBO / VBO hold the cotangents of the step's outputs on entry and of its inputs
// on return.
int backward_step_eager(vfd_sim* s, AdjointState* A, const TapeBank& B, uint32_t t) {
    const TapeStep& T = B.host[t];
    const BwdLaunch L = bwd_launch(s, A, s->stream);
    bwd_head(L, s->dStatus);
    for (uint32_t k = 0; k < T.kp; k++) bwd_jacobi<false>(L);
    bwd_mid(L);
    if (L.visc) {
        uint32_t more = 0;
        TRY(read_flag(s, 5, more));
        for (uint32_t guard = 0; more && guard < 100000u; guard++) {
            launch_cg_iter(L.d, L.st);
            TRY(read_flag(s, 5, more));
        }
        bwd_visc_tail(L);
    }
    if (s->anyDiv) {
        bwd_div_head(L);
        for (uint32_t k = 0; k < T.kd; k++) bwd_jacobi<true>(L);
        bwd_div_tail(L);
    }
    bwd_end(L);
    CK(cudaGetLastError());
    return VFD_OK;
}

// The backward pass of a segment of `count` steps recorded in bank B, the last first, on
// the simulation's stream (asynchronous with graphs).
int backward_segment(vfd_sim* s, AdjointState* A, const TapeBank& B, uint32_t count) {
    cudaStream_t st = s->stream;
    k_adj_set_slot<<<1, 1, 0, st>>>(A->a, B.dsteps, count - 1u);
    const bool graphs = s->graphMode && !s->graphFailed;
    if (graphs && !s->adjBwdExec) TRY(build_backward_graph(s, A));
    for (uint32_t t = count; t-- > 0;) {
        if (graphs) CK(cudaGraphLaunch(s->adjBwdExec, st));
        else TRY(backward_step_eager(s, A, B, t));
    }
    CK(cudaGetLastError());
    return VFD_OK;
}

int check_adjoint_scene(vfd_sim* s) {
    if (s->scenes.size() != 1) return fail(VFD_E_ARG, "adjoint: one scene per simulation");
    if (s->scenes[0].desc.EnableSurfaceTensionSolver) return fail(VFD_E_ARG, "adjoint: surface tension is not differentiated");
    if (s->cellRel) return fail(VFD_E_ARG, "adjoint: positions must be absolute (VFD_POSITIONS_ABSOLUTE)");
    if (s->scenes[0].emitted) return fail(VFD_E_ARG, "adjoint: emitted particles are not differentiated");
    return VFD_OK;
}

int alloc_cotangents(vfd_sim* s, AdjointState* A) {
    const size_t st = s->stride;
    AdjDev& a = A->a;
    TRY(aalloc(A, &a.XBAR, st));
    TRY(aalloc(A, &a.VBAR, st));
    TRY(aalloc(A, &a.ABAR, st));
    TRY(aalloc(A, &a.AK, st));
    TRY(aalloc(A, &a.GBAR, st));
    TRY(aalloc(A, &a.GSUM, st));
    TRY(aalloc(A, &a.BD, 3 * st * std::max<uint32_t>(1u, s->maxBodies)));
    TRY(aalloc(A, &a.KBAR, st));
    TRY(aalloc(A, &a.U, st));
    TRY(aalloc(A, &a.KU, st));
    TRY(aalloc(A, &a.LAM, st));
    TRY(aalloc(A, &a.LAM2, st));
    TRY(aalloc(A, &a.ACNT, 4));
    TRY(aalloc(A, &a.BW, 2));
    TRY(aalloc(A, &A->bset, 1));
    a.ts = A->bset;
    TRY(aalloc(A, &a.RABAR, st));
    TRY(aalloc(A, &a.APBAR, st));
    TRY(aalloc(A, &a.DBAR, st));
    TRY(aalloc(A, &a.RHOBAR, st));
    TRY(aalloc(A, &a.ALBAR, st));
    TRY(aalloc(A, &a.STOP, st));
    TRY(aalloc(A, &a.SC, 8));
    TRY(aalloc(A, &a.CLAIM, 2));
    TRY(aalloc(A, &a.XBO, st));
    TRY(aalloc(A, &a.VBO, st));
    return VFD_OK;
}

__global__ void k_adj_pack(float4* dst, const float* src, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = make_float4(src[3 * (size_t)i], src[3 * (size_t)i + 1], src[3 * (size_t)i + 2], 0.f);
}
__global__ void k_adj_unpack(float* dst, const float4* src, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 v = src[i];
    dst[3 * (size_t)i] = v.x;
    dst[3 * (size_t)i + 1] = v.y;
    dst[3 * (size_t)i + 2] = v.z;
}

}  // namespace

// The backward graph addresses the adjoint state's arrays: it goes with them.
void drop_backward_graph(vfd_sim* s) {
    if (s->adjBwdExec) cudaGraphExecDestroy(s->adjBwdExec);
    if (s->adjBwdGraph) cudaGraphDestroy(s->adjBwdGraph);
    s->adjBwdExec = nullptr;
    s->adjBwdGraph = nullptr;
}

void adjoint_release(vfd_sim* s) {
    drop_backward_graph(s);
    delete s->adjoint;
    s->adjoint = nullptr;
}

}  // namespace vfd

using namespace vfd;
using namespace vfd::host;

extern "C" {

int vfd_adjoint_forward(vfd_sim* s, uint32_t steps, uint32_t checkpoint_every, vfd_step_stats* stats) {
    if (!s) return fail(VFD_E_ARG, "null handle");
    if (s->fp64Mode) return fail(VFD_E_STATE, "the adjoint differentiates the FP32 step (VFD_PRECISION_FP32)");
    if (steps == 0 || checkpoint_every == 0) return fail(VFD_E_ARG, "adjoint: steps and checkpoint_every must be positive");
    TRY(check_adjoint_scene(s));
    TRY(ensure_ready(s));
    // the tape, checkpoints and cotangent arrays of the previous run are reused when the
    // layout matches (same particles, segment length and iteration caps)
    const uint32_t every = std::min(checkpoint_every, steps);
    const vfd_desc& dd = s->scenes[0].desc;
    const uint32_t capD = s->anyDiv ? dd.MaxDivergenceSolverIterations : 0u, capP = dd.MaxPressureSolverIterations;
    std::unique_ptr<AdjointState> A(s->adjoint);
    s->adjoint = nullptr;
    if (A && !(A->n == s->n && A->stride == s->stride && A->every == every && !A->bank[0].host.empty() &&
               A->bank[0].host[0].capD == capD && A->bank[0].host[0].capP == capP))
        A.reset();
    if (!A) {
        drop_backward_graph(s);
        A = std::make_unique<AdjointState>();
        A->every = every;
        A->n = s->n;
        A->stride = s->stride;
        TRY(alloc_tape(s, A.get()));
    }
    A->steps = steps;
    A->lastRecorded = false;
    const uint32_t segs = (steps + A->every - 1) / A->every;
    A->ckpt.resize(segs + 1);
    for (uint32_t k = 0; k < segs; k++) {
        TRY(save_checkpoint(s, A.get(), A->ckpt[k]));
        const uint32_t cnt = std::min(A->every, steps - k * A->every);
        if (k + 1 < segs) {
            TRY(run_steps(s, cnt, stats, true));
            continue;
        }
        // the last segment is recorded as it runs, so the backward pass starts on it
        // without a replay; a step the search had to abort (grid growth) falls back to a
        // plain run and a replay
        const int rc = record_segment(s, A.get(), A->bank[0], cnt);
        if (rc == VFD_OK) {
            A->lastRecorded = true;
            if (stats) {
                CK(cudaMemcpy(s->hScenes.data(), s->dScenes, sizeof(SceneDev) * s->hScenes.size(),
                              cudaMemcpyDeviceToHost));
                fill_stats(s->hScenes[0], stats);
            }
        } else if (rc == VFD_E_STATE) {
            TRY(restore_checkpoint(s, A->ckpt[k]));
            TRY(run_steps(s, cnt, stats, true));
        } else {
            return rc;
        }
    }
    TRY(save_checkpoint(s, A.get(), A->ckpt[segs]));
    A->generation = s->generation;
    s->adjoint = A.release();
    return VFD_OK;
}

int vfd_adjoint_backward(vfd_sim* s, const float* x_bar, const float* v_bar, float* x0_bar, float* v0_bar,
                         float* param_bar) {
    if (!s) return fail(VFD_E_ARG, "null handle");
    AdjointState* A = s->adjoint;
    if (!A) return fail(VFD_E_STATE, "adjoint: no recorded forward run (call vfd_adjoint_forward first)");
    if (A->generation != s->generation || A->n != s->n)
        return fail(VFD_E_STATE, "adjoint: the simulation was reset after the recorded forward run");
    if (!x_bar || !v_bar) return fail(VFD_E_ARG, "adjoint: null cotangent");
    const uint32_t n = s->n;
    cudaStream_t st = s->stream;
    if (!A->a.XBAR) TRY(alloc_cotangents(s, A));
    AdjDev& a = A->a;
    // cotangents of the final state, original order
    CK(cudaMemcpyAsync(s->dStage, x_bar, sizeof(float) * 3 * n, cudaMemcpyHostToDevice, st));
    k_adj_pack<<<blocks_for(n, 256), 256, 0, st>>>(a.XBO, s->dStage, n);
    CK(cudaMemcpyAsync(s->dStage, v_bar, sizeof(float) * 3 * n, cudaMemcpyHostToDevice, st));
    k_adj_pack<<<blocks_for(n, 256), 256, 0, st>>>(a.VBO, s->dStage, n);
    CK(cudaMemsetAsync(a.SC, 0, 8 * sizeof(double), st));
    CK(cudaMemsetAsync(a.CLAIM, 0, 2 * sizeof(uint32_t), st));
    CK(cudaMemsetAsync(a.ACNT, 0, 4 * sizeof(uint32_t), st));
    // The segments are walked from the last to the first. The last was recorded by the
    // forward run into bank 0 (else it is replayed now). With a shadow, the backward pass
    // of segment k (on the simulation's stream) runs while the shadow replays segment k - 1
    // into the other bank on its own stream; the shadow waits for the backward pass that
    // read that bank before overwriting it. Without one, each segment is replayed on the
    // simulation itself after the backward pass of the segment after it.
    const uint32_t segs = (uint32_t)A->ckpt.size() - 1;
    const bool overlap = segs > 1 && ensure_shadow(s, A);
    int rc = VFD_OK;
    A->replayed = 0;
    if (!A->lastRecorded) {
        const uint32_t cnt = A->steps - (segs - 1) * A->every;
        rc = restore_checkpoint(s, A->ckpt[segs - 1]);
        if (rc == VFD_OK) rc = record_segment(s, A, A->bank[0], cnt);
        A->replayed += cnt;
    }
    int b = 0;  // the bank holding segment k
    for (uint32_t k = segs; k-- > 0 && rc == VFD_OK;) {
        const uint32_t cnt = std::min(A->every, A->steps - k * A->every);
        rc = backward_segment(s, A, A->bank[b], cnt);
        if (rc != VFD_OK || k == 0) break;
        if (overlap) {
            CK(cudaEventRecord(A->bankRead[b], st));
            const int nb = 1 - b;
            vfd_sim* t = A->shadow;
            rc = restore_checkpoint(t, A->ckpt[k - 1]);
            if (rc == VFD_OK) {
                CK(cudaStreamWaitEvent(t->stream, A->bankRead[nb], 0));
                rc = record_segment(t, A, A->bank[nb], A->every);
            }
            b = nb;
        } else {
            rc = restore_checkpoint(s, A->ckpt[k - 1]);
            if (rc == VFD_OK) rc = record_segment(s, A, A->bank[0], A->every);
        }
        A->replayed += A->every;
    }
    // the tape now holds the first segment; leave the simulation where the forward run ended
    A->lastRecorded = false;
    const int rc2 = restore_checkpoint(s, A->ckpt[segs]);
    if (rc != VFD_OK) return rc;
    if (rc2 != VFD_OK) return rc2;
    if (x0_bar) {
        k_adj_unpack<<<blocks_for(n, 256), 256, 0, st>>>(s->dStage, a.XBO, n);
        CK(cudaMemcpyAsync(x0_bar, s->dStage, sizeof(float) * 3 * n, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
    }
    if (v0_bar) {
        k_adj_unpack<<<blocks_for(n, 256), 256, 0, st>>>(s->dStage, a.VBO, n);
        CK(cudaMemcpyAsync(v0_bar, s->dStage, sizeof(float) * 3 * n, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
    }
    if (param_bar) {
        double sc[8];
        CK(cudaMemcpyAsync(sc, a.SC, sizeof(sc), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        param_bar[0] = (float)sc[2];
        param_bar[1] = (float)sc[3];
    }
    CK(cudaGetLastError());
    return VFD_OK;
}

int vfd_adjoint_release(vfd_sim* s) {
    if (!s) return fail(VFD_E_ARG, "null handle");
    adjoint_release(s);
    return VFD_OK;
}

int vfd_adjoint_set_warm_start(vfd_sim* s, int32_t mode) {
    if (!s) return fail(VFD_E_ARG, "null handle");
    if (mode < VFD_WARM_COLD || mode > VFD_WARM_EXTRAPOLATE) return fail(VFD_E_ARG, "unknown warm-start mode %d", mode);
    if (mode != s->adjWarm) drop_backward_graph(s);  // the backward graph carries the mode
    s->adjWarm = mode;
    return VFD_OK;
}

int vfd_adjoint_set_tolerance(vfd_sim* s, float factor) {
    if (!s) return fail(VFD_E_ARG, "null handle");
    if (!(factor > 0.0f && factor <= 1.0f)) return fail(VFD_E_ARG, "adjoint tolerance factor must be in (0, 1]");
    if (factor != s->adjTol) drop_backward_graph(s);  // the backward graph carries it
    s->adjTol = factor;
    return VFD_OK;
}

int vfd_adjoint_get_stats(vfd_sim* s, vfd_adjoint_stats* out) {
    if (!s || !out) return fail(VFD_E_ARG, "null argument");
    *out = vfd_adjoint_stats{};
    const AdjointState* A = s->adjoint;
    if (!A) return fail(VFD_E_STATE, "adjoint: no recorded forward run (call vfd_adjoint_forward first)");
    out->Steps = A->steps;
    if (!A->a.ACNT) return VFD_OK;  // no backward pass yet
    uint32_t c[4];
    CK(cudaSetDevice(s->device));
    CK(cudaMemcpyAsync(c, A->a.ACNT, sizeof(c), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    out->ReplayedSteps = A->replayed;
    out->ViscositySolverIterations = c[0];
    out->MaxViscositySolverIterations = c[1];
    out->ViscositySolves = c[2];
    return VFD_OK;
}

}  // extern "C"
