"""FP64 CPU reference of the DFSPH step and of its derivative (test infrastructure).

Checks the GPU adjoint (vfd_adjoint_forward / vfd_adjoint_backward); the product
never imports it. It restates one OnUpdate step (Simulation/DFSPH/DFSPHImplementation.cu:63-170,
kernels DFSPHKernels.cu:24-862) in float64 numpy for one scene without surface
tension, and differentiates it in reverse mode by the same equations as the CUDA
adjoint:
  * the cubic spline is evaluated analytically (Kernel/DFSPHKernels.h:86-131) instead
    of through the reference's 10 000-entry midpoint table, whose lookup is piecewise
    constant in |r| and so has no useful derivative;
  * neighbour sets: every pair with 0 < |x_i - x_j|^2 < h^2 at the search positions;
  * boundary samples from the volume maps (SDFDeviceData.cuh:36-474, evaluated by the
    C++ oracle in FP64): x - xb = pd n, pd = max(phi0 + r/2, 2r), Vb = phi1, with the
    normal n held fixed under differentiation (exact on planar walls), push-out by a
    constant 0.1 r along n with the velocity zeroed (ComputeVolumeAndBoundaryKernel
    DFSPHKernels.cu:69-150);
  * divergence and pressure Jacobi solves (DFSPHImplementation.cu:443-575) with the
    reference's loop conditions, unrolled in the derivative;
  * the Weiler viscosity system A g = v (DFSPHImplementation.cu:577-808) solved exactly
    by a sparse direct solve (on large scenes by CG to a relative residual of 1e-13; A is
    symmetric), differentiated by the implicit function theorem;
  * the CFL step (DFSPHImplementation.cu:395-441) through its argmax particle.
The reference itself ships no derivative, so this module is pinned by its own
central differences in FP64 (tests/test_adjoint_ref.py).
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from . import oracle as O

EPS = 1.0e-5           # Core/Math/Math.h:6
FLT_MAX = float(np.finfo(np.float32).max)


# Above these sizes the all-pairs distance matrix and the direct solve give way to a k-d
# tree and CG (the same pair set and the same solution to rounding).
_ALL_PAIRS_MAX = 4096
_DIRECT_MAX = 30000


def _pairs(x, h):
    """(I, J) of every pair with 0 < |x_i - x_j|^2 < h^2, row-major order."""
    if len(x) <= _ALL_PAIRS_MAX:
        d2 = np.sum((x[:, None, :] - x[None, :, :]) ** 2, axis=2)
        return np.nonzero((d2 > 0) & (d2 < h * h))
    from scipy.spatial import cKDTree
    pr = cKDTree(x).query_pairs(h * (1.0 + 1e-9), output_type="ndarray")
    I = np.concatenate([pr[:, 0], pr[:, 1]])
    J = np.concatenate([pr[:, 1], pr[:, 0]])
    d2 = np.sum((x[I] - x[J]) ** 2, axis=1)
    keep = (d2 > 0) & (d2 < h * h)
    I, J = I[keep], J[keep]
    order = np.lexsort((J, I))
    return I[order], J[order]


def _solve_spd(A, b):
    """A x = b for the symmetric positive definite viscosity matrix."""
    if A.shape[0] <= _DIRECT_MAX:
        return spla.spsolve(A.tocsc(), b)
    A = A.tocsr()
    M = sp.diags(1.0 / A.diagonal())
    try:
        x, info = spla.cg(A, b, rtol=1e-13, atol=0.0, maxiter=10000, M=M)
    except TypeError:  # scipy < 1.12
        x, info = spla.cg(A, b, tol=1e-13, atol=0.0, maxiter=10000, M=M)
    if info != 0:
        raise RuntimeError(f"viscosity CG did not converge ({info})")
    return x


class Kernel:
    """Cubic spline of support h and its derivatives."""

    def __init__(self, h: float):
        self.h = h
        self.K = 8.0 / (np.pi * h ** 3)

    def w(self, s):
        q = s / self.h
        return np.where(q <= 0.5, self.K * (6 * q ** 3 - 6 * q ** 2 + 1),
                        np.where(q <= 1.0, 2 * self.K * np.clip(1 - q, 0, None) ** 3, 0.0))

    def w1(self, s):
        q = s / self.h
        return np.where(q <= 0.5, self.K * (18 * q * q - 12 * q) / self.h,
                        np.where(q <= 1.0, -6 * self.K * np.clip(1 - q, 0, None) ** 2 / self.h, 0.0))

    def w2(self, s):
        q = s / self.h
        return np.where(q <= 0.5, self.K * (36 * q - 12) / self.h ** 2,
                        np.where(q <= 1.0, 12 * self.K * np.clip(1 - q, 0, None) / self.h ** 2, 0.0))

    def gs(self, s):
        """W'(s) / s, so gradW(r) = gs r."""
        q = s / self.h
        ss = np.maximum(s, 1e-300)
        return np.where(q <= 0.5, self.K * (18 * q - 12) / self.h ** 2,
                        np.where(q <= 1.0, -6 * self.K * np.clip(1 - q, 0, None) ** 2 / (self.h * ss), 0.0))

    def gq(self, s):
        """gs'(s) / s, so d gradW / dr = gs I + gq r r^T."""
        q = s / self.h
        ss = np.maximum(s, 1e-300)
        return np.where(q <= 0.5, 18 * self.K / (self.h ** 3 * ss),
                        np.where(q <= 1.0, (self.w2(s) - self.gs(s)) / ss ** 2, 0.0))


def orthogonal_vectors(n):
    """Core/Math/Math.h:19-33 for rows of unit vectors."""
    v = np.tile(np.array([1.0, 0.0, 0.0]), (len(n), 1))
    flip = np.abs(n @ np.array([1.0, 0.0, 0.0])) > 0.999
    v[flip] = np.array([0.0, 1.0, 0.0])
    x = np.cross(n, v)
    y = np.cross(n, x)
    x /= np.linalg.norm(x, axis=1, keepdims=True)
    y /= np.linalg.norm(y, axis=1, keepdims=True)
    return x, y


def _dot(a, b):
    return np.sum(a * b, axis=-1)


class Params:
    def __init__(self, desc: dict):
        d = dict(O._abi.DEFAULTS)
        d.update(desc)
        self.r = float(d["ParticleRadius"])
        self.diam = 2 * self.r
        self.h = 4 * self.r
        self.rho0 = 1000.0
        self.V = 0.8 * self.diam ** 3
        self.m = self.V * self.rho0
        self.nu = float(d["Viscosity"])
        self.nub = float(d["BoundaryViscosity"])
        self.tang = float(d["TangentialDistanceFactor"]) * self.h
        self.g = np.array(d["Gravity"], np.float64)
        self.min_dt, self.max_dt, self.dt0 = float(d["MinTimeStepSize"]), float(d["MaxTimeStepSize"]), float(
            d["TimeStepSize"])
        self.div = bool(d["EnableDivergenceSolverError"])
        self.visc = bool(d["EnableViscositySolver"])
        self.it_d = (int(d["MinDivergenceSolverIterations"]), int(d["MaxDivergenceSolverIterations"]))
        self.it_p = (int(d["MinPressureSolverIterations"]), int(d["MaxPressureSolverIterations"]))
        self.err_d, self.err_p = float(d["MaxDivergenceSolverError"]), float(d["MaxPressureSolverError"])
        if d["EnableSurfaceTensionSolver"]:
            raise ValueError("surface tension is outside the differentiated step")


class Step:
    """One step: forward(x, v, dt_o) records what backward(...) needs."""

    def __init__(self, P: Params, maps: list):
        self.P, self.maps, self.k = P, maps, Kernel(P.h)

    # ---------------------------------------------------------------- operators
    def _sum(self, vals):
        n = self.n
        if vals.ndim == 1:
            return np.bincount(self.I, vals, n)
        return np.stack([np.bincount(self.I, vals[:, c], n) for c in range(vals.shape[1])], 1)

    def D(self, w):
        return self.P.V * self._sum(_dot(w[self.I] - w[self.J], self.gw)) + _dot(w, self.GB)

    def Pk(self, k):
        e = np.abs(k[self.I] + k[self.J]) > EPS
        a = -self.P.V * self._sum(((k[self.I] + k[self.J]) * e)[:, None] * self.gw)
        return a - (np.abs(k) > EPS)[:, None] * k[:, None] * self.GB

    def DT(self, u):
        return self.P.V * self._sum((u[self.I] + u[self.J])[:, None] * self.gw) + u[:, None] * self.GB

    def PT(self, k, ab):
        e = np.abs(k[self.I] + k[self.J]) > EPS
        out = -self.P.V * self._sum(e * _dot(self.gw, ab[self.I] - ab[self.J]))
        return out - (np.abs(k) > EPS) * _dot(self.GB, ab)

    def H(self, w):
        return self.gsv[:, None] * w + (self.gqv * _dot(self.r, w))[:, None] * self.r

    def JGB_T(self, y):
        out = np.zeros_like(y)
        for b in self.bd:
            m = b["valid"]
            if not m.any():
                continue
            c = _dot(b["n"], y)[:, None]
            out += m[:, None] * c * (self.k.w1(b["pd"])[:, None] * b["gvb"] +
                                     (b["vb"] * self.k.w2(b["pd"]))[:, None] * b["gpd"])
        return out

    def XD(self, w, u):
        return self.P.V * self._sum((u[self.I] + u[self.J])[:, None] * self.H(w[self.I] - w[self.J])) + \
            u[:, None] * self.JGB_T(w)

    def XP(self, k, ab):
        e = np.abs(k[self.I] + k[self.J]) > EPS
        out = -self.P.V * self._sum(((k[self.I] + k[self.J]) * e)[:, None] * self.H(ab[self.I] - ab[self.J]))
        return out - ((np.abs(k) > EPS) * k)[:, None] * self.JGB_T(ab)

    # ---------------------------------------------------------------- forward
    def _boundary(self, x):
        P, n = self.P, len(x)
        x = x.copy()
        stop = np.zeros(n, bool)
        self.bd = []
        for vm in self.maps:
            phi0, g0 = O.map_interpolate_d(vm, 0, x)
            phi1, g1 = O.map_interpolate_d(vm, 1, x)
            inside = phi0 != FLT_MAX
            dist = np.where(inside, phi0, np.inf)
            nl = np.linalg.norm(g0, axis=1)
            nhat = g0 / np.maximum(nl, 1e-300)[:, None]
            valid = (dist > 0) & (dist < P.h) & (phi1 > 0) & (phi1 != FLT_MAX) & (nl > 1e-9)
            raw = np.where(valid, dist + 0.5 * P.r, 0.0)
            pd = np.maximum(raw, P.diam)
            self.bd.append(dict(valid=valid, n=np.where(valid[:, None], nhat, 0.0), vb=np.where(valid, phi1, 0.0),
                                pd=np.where(valid, pd, 1.0),
                                gpd=np.where((valid & (raw > P.diam))[:, None], g0, 0.0),
                                gvb=np.where(valid[:, None], g1, 0.0)))
            push = (dist <= 0) & (nl > 1e-5)
            delta = np.minimum(P.diam - dist, 0.1 * P.r)
            x[push] += delta[push, None] * nhat[push]
            stop |= push
        return x, stop

    def forward(self, x_in, v_in, dt_o):
        P, k = self.P, self.k
        n = self.n = len(x_in)
        # neighbour search on the positions before the boundary kernel
        I, J = _pairs(x_in, P.h)
        self.I, self.J = I, J
        self.cnt = np.bincount(I, minlength=n)
        if self.cnt.max() >= 70:
            raise ValueError("a particle reached the 70-neighbour cap")
        x, stop = self._boundary(x_in)
        self.stop = stop
        v0 = np.where(stop[:, None], 0.0, v_in)
        self.x, self.v0, self.dto = x, v0, dt_o
        r = x[I] - x[J]
        s = np.linalg.norm(r, axis=1)
        self.r, self.s = r, s
        self.gsv, self.gqv = k.gs(s), k.gq(s)
        gw = self.gsv[:, None] * r
        self.gw = gw
        GB = np.zeros((n, 3))
        rhob = np.zeros(n)
        for b in self.bd:
            GB += (b["vb"] * k.w1(b["pd"]))[:, None] * b["n"]
            rhob += b["vb"] * k.w(b["pd"])
        self.GB = GB
        rho = P.rho0 * (P.V * k.w(0.0) + P.V * self._sum(k.w(s)) + rhob)
        G = P.V * self._sum(gw) + GB
        S = P.V * P.V * self._sum(_dot(gw, gw)) + _dot(G, G)
        alpha = np.where(S > EPS, 1.0 / np.where(S > EPS, S, 1.0), 0.0)
        self.rho, self.G, self.S, self.alpha = rho, G, S, alpha
        mc = self.cnt >= 20
        self.mc = mc
        # divergence solve
        self.kd, self.rd = [], []
        if P.div:
            ra = np.where(mc, np.maximum(self.D(v0), 0.0), 0.0)
            a1 = alpha / dt_o
            kap = ra * a1
            self.kd.append(kap)
            eta = (1.0 / dt_o) * P.err_d * 1e-4 * P.rho0
            it, mn, mx = 0, *P.it_d
            active = ((0.0 > eta) or 0 < mn) and 0 < mx
            while active:
                f = dt_o * self.D(self.Pk(kap))
                res = np.where(mc, np.minimum(-ra - f, 0.0), 0.0)
                kap = kap - res * a1
                self.rd.append(res)
                self.kd.append(kap)
                err = -P.rho0 * res.sum() / n
                it += 1
                active = (err > eta or it < mn) and it < mx
            self.ra_d = ra
            v1 = v0 + dt_o * self.Pk(kap)
        else:
            v1 = v0.copy()
        self.v1 = v1
        # viscosity
        self.zeroG = False
        if P.visc:
            b = v1
            if not np.any(b != 0):
                g = np.zeros_like(b)
                self.zeroG = True
            else:
                A = self._visc_matrix(dt_o)
                g = _solve_spd(A, b.reshape(-1)).reshape(n, 3)
            self.gv = g
            acc = P.g[None, :] + (g - v1) / dt_o
        else:
            acc = np.tile(P.g, (n, 1))
        self.acc = acc
        w = v1 + acc * dt_o
        m2 = _dot(w, w)
        mv_raw = m2.max()
        mv = max(0.1, mv_raw, 1e-9)
        dt_raw = 0.4 * (P.diam / np.sqrt(mv))
        dt_n = max(min(dt_raw, P.max_dt), P.min_dt)
        self.cfl = (mv_raw > 0.1) and dt_n == dt_raw
        self.imax, self.w, self.mv, self.dtn = int(np.argmax(m2)), w, mv, dt_n
        v2 = v1 + dt_n * acc
        self.v2 = v2
        # pressure solve
        ra = rho / P.rho0 + dt_n * self.D(v2)
        a2 = alpha / dt_n ** 2
        kap = np.maximum(ra - 1.0, 0.0) * a2
        self.kp, self.rp = [kap], []
        eta = P.err_p * 1e-4 * P.rho0
        it, mn, mx = 0, *P.it_p
        active = ((0.0 > eta) or 0 < mn) and 0 < mx
        while active:
            f = dt_n * dt_n * self.D(self.Pk(kap))
            res = np.minimum(1.0 - ra - f, 0.0)
            kap = kap - res * a2
            self.rp.append(res)
            self.kp.append(kap)
            err = -P.rho0 * res.sum() / n
            it += 1
            active = (err > eta or it < mn) and it < mx
        self.ra_p = ra
        v3 = v2 + dt_n * self.Pk(kap)
        self.v3 = v3
        return x + dt_n * v3, v3, dt_n

    def _pair_visc(self):
        P = self.P
        eps2 = 0.01 * P.h * P.h
        return 10.0 * P.nu * P.rho0, eps2

    def _bvisc_terms(self):
        """Per body and tangent sample k: d_k = pd n - off_k."""
        P = self.P
        out = []
        for b in self.bd:
            t1, t2 = orthogonal_vectors(-np.where(b["valid"][:, None], b["n"], np.array([0.0, 0.0, 1.0])))
            offs = [-P.tang * t1, P.tang * t1, -P.tang * t2, P.tang * t2]
            out.append((b, [b["pd"][:, None] * b["n"] - o for o in offs]))
        return out

    def _visc_matrix(self, dt):
        P, n, I, J = self.P, self.n, self.I, self.J
        cmu, eps2 = self._pair_visc()
        c = cmu * (P.m / self.rho[J]) * self.gsv / (self.s ** 2 + eps2)
        rr = self.r[:, :, None] * self.r[:, None, :] * c[:, None, None]  # c r r^T per pair
        blocks_i, blocks_j, vals = [], [], []
        # F_i(g) = sum_j c (r r^T)(g_i - g_j)
        for a in range(3):
            for bb in range(3):
                blocks_i += [3 * I + a, 3 * I + a]
                blocks_j += [3 * I + bb, 3 * J + bb]
                vals += [rr[:, a, bb], -rr[:, a, bb]]
        if P.nub != 0.0:
            cb = 10.0 * P.nub * P.rho0
            eps2b = 0.01 * P.h * P.h
            for b, ds in self._bvisc_terms():
                m = b["valid"]
                for dk in ds:
                    s = np.linalg.norm(dk, axis=1)
                    c = m * cb * 0.25 * b["vb"] * self.k.gs(s) / (s ** 2 + eps2b)
                    dd = dk[:, :, None] * dk[:, None, :] * c[:, None, None]
                    ii = np.arange(n)
                    for a in range(3):
                        for bb in range(3):
                            blocks_i.append(3 * ii + a)
                            blocks_j.append(3 * ii + bb)
                            vals.append(dd[:, a, bb])
        M = sp.coo_matrix((np.concatenate(vals), (np.concatenate(blocks_i), np.concatenate(blocks_j))),
                          shape=(3 * n, 3 * n)).tocsr()
        Dr = sp.diags(np.repeat(dt / self.rho, 3))
        return sp.identity(3 * n, format="csr") - Dr @ M

    # ---------------------------------------------------------------- backward
    def backward(self, xb, vb, dtnb):
        """Cotangents of (x', v3, dt_n) -> those of (x_in, v_in, dt_o), Viscosity, BoundaryViscosity."""
        P, k, n, I, J = self.P, self.k, self.n, self.I, self.J
        dto, dtn = self.dto, self.dtn
        X = xb.copy()
        rhob = np.zeros(n)
        alb = np.zeros(n)
        dtob = 0.0
        nub = nubb = 0.0
        # x' = x + dt_n v3, v3 = v2 + dt_n a_p
        ap = self.Pk(self.kp[-1])
        dtnb += _dot(self.v3, xb).sum()
        vb3 = vb + dtn * xb
        dtnb += _dot(ap, vb3).sum()
        ab = dtn * vb3
        kb = self.PT(self.kp[-1], ab)
        X += self.XP(self.kp[-1], ab)
        vbar = vb3.copy()
        a2 = self.alpha / dtn ** 2
        rab = np.zeros(n)
        apb = np.zeros(n)
        for it in range(len(self.rp) - 1, -1, -1):
            res = self.rp[it]
            u = np.where(res < 0, a2 * kb, 0.0)
            rab += u
            apb += -res * kb
            f = 1.0 - self.ra_p - res
            dtnb += (2.0 / dtn) * np.sum(np.where(u != 0, u * f, 0.0))
            ak = self.Pk(self.kp[it])
            ab = dtn * dtn * self.DT(u)
            kb = kb + self.PT(self.kp[it], ab)
            X += dtn * dtn * self.XD(ak, u) + self.XP(self.kp[it], ab)
        ra = self.ra_p
        rab += np.where(ra > 1.0, a2 * kb, 0.0)
        apb += np.maximum(ra - 1.0, 0.0) * kb
        rhob += rab / P.rho0
        db = dtn * rab
        alb += apb / dtn ** 2
        dtnb += -2.0 * np.sum(apb * self.alpha) / dtn ** 3
        dtnb += np.sum(rab * self.D(self.v2))
        vbar += self.DT(db)
        X += self.XD(self.v2, db)
        # v2 = v1 + dt_n a
        gbar = np.zeros((n, 3))
        if P.visc:
            g = self.gv
            dtnb += np.sum(_dot(vbar, P.g[None, :] + (g - self.v1) / dto))
            dtob += -(dtn / dto ** 2) * np.sum(_dot(vbar, g - self.v1))
            if not self.zeroG:
                gbar = (dtn / dto) * vbar
            vbar = (1.0 - dtn / dto) * vbar
        else:
            dtnb += np.sum(_dot(vbar, P.g[None, :]))
        # CFL
        if self.cfl:
            i = self.imax
            wb = (-dtnb * dtn / self.mv) * self.w[i]
            dtob += float(wb @ P.g)
            if P.visc and not self.zeroG:
                gbar[i] += wb
            elif not P.visc:
                vbar[i] += wb
        # viscosity: A lambda = g_bar
        if P.visc and not self.zeroG:
            A = self._visc_matrix(dto)
            lam = _solve_spd(A.T, gbar.reshape(-1)).reshape(n, 3)
            vbar += lam
            X_, rho_, dtob_, nub, nubb = self._visc_derivative(lam, dto)
            X += X_
            rhob += rho_
            dtob += dtob_
        # divergence solve
        if P.div:
            ad = self.Pk(self.kd[-1])
            dtob += np.sum(_dot(ad, vbar))
            ab = dto * vbar
            kb = self.PT(self.kd[-1], ab)
            X += self.XP(self.kd[-1], ab)
            a1 = self.alpha / dto
            rab = np.zeros(n)
            apb = np.zeros(n)
            for it in range(len(self.rd) - 1, -1, -1):
                res = self.rd[it]
                u = np.where(res < 0, a1 * kb, 0.0)
                rab += u
                apb += -res * kb
                f = -self.ra_d - res
                dtob += (1.0 / dto) * np.sum(np.where(u != 0, u * f, 0.0))
                ak = self.Pk(self.kd[it])
                ab = dto * self.DT(u)
                kb = kb + self.PT(self.kd[it], ab)
                X += dto * self.XD(ak, u) + self.XP(self.kd[it], ab)
            rab += a1 * kb
            apb += self.ra_d * kb
            db = np.where(self.mc & (self.ra_d > 0), rab, 0.0)
            alb += apb / dto
            dtob += -np.sum(apb * self.alpha) / dto ** 2
            vbar += self.DT(db)
            X += self.XD(self.v0, db)
        # density and factor
        sbar = np.where(self.S > EPS, -alb * self.alpha ** 2, 0.0)
        Gb = 2.0 * sbar[:, None] * self.G
        gwa = self.gw
        X += P.rho0 * P.V * self._sum((rhob[I] + rhob[J])[:, None] * gwa)
        X += 2 * P.V * P.V * self._sum((sbar[I] + sbar[J])[:, None] * self.H(gwa))
        X += P.V * self._sum(self.H(Gb[I] - Gb[J]))
        for b in self.bd:
            X += b["valid"][:, None] * (rhob * P.rho0)[:, None] * (
                k.w(b["pd"])[:, None] * b["gvb"] + (b["vb"] * k.w1(b["pd"]))[:, None] * b["gpd"])
        X += self.JGB_T(Gb)
        # boundary: push-out has identity Jacobian, stopped particles lose their velocity
        vbar = np.where(self.stop[:, None], 0.0, vbar)
        return X, vbar, dtob, nub, nubb

    def _visc_derivative(self, lam, dt):
        """lambda^T d(dt/rho Q)/d(x, rho, dt, nu, nu_b) at the solution g."""
        P, k, n, I, J = self.P, self.k, self.n, self.I, self.J
        cmu, eps2 = self._pair_visc()
        g = self.gv
        rho = self.rho
        lt = (dt / rho)[:, None] * lam
        r, s = self.r, self.s
        den = s ** 2 + eps2
        gs, gq = self.gsv, self.gqv
        gij = g[I] - g[J]
        gr = _dot(gij, r)
        phi = gs / den
        phis = gq / den - 2.0 * gs / den ** 2
        # values: T_ij = cmu (m / rho_j)(g_ij . r) phi r
        T1 = (10.0 * (P.m / rho[J]) * gr * phi)[:, None] * r
        q1 = self._sum(T1)
        Q = P.nu * P.rho0 * q1
        rhob = self._sum((cmu * P.m / rho[I] ** 2) * gr * phi * _dot(lt[J], r))
        w = (cmu * P.m) * (lt[I] / rho[J][:, None] - lt[J] / rho[I][:, None])
        rw = _dot(r, w)
        X = self._sum(phi[:, None] * (rw[:, None] * gij + gr[:, None] * w) + (gr * rw * phis)[:, None] * r)
        b1 = np.zeros((n, 3))
        if P.nub != 0.0:
            C0 = P.nub * P.rho0  # dynamic boundary viscosity; c1 carries the factor 10
            for b, ds in self._bvisc_terms():
                m = b["valid"]
                c1 = 10.0 * 0.25 * b["vb"]
                dpd = np.zeros(n)
                dvb = np.zeros(n)
                for dk in ds:
                    ss = np.linalg.norm(dk, axis=1)
                    den_b = ss ** 2 + eps2
                    gsb = k.gs(ss)
                    dg, dl = _dot(dk, g), _dot(dk, lt)
                    b1 += (m * c1 * dg * gsb / den_b)[:, None] * dk
                    dvb += m * C0 * c1 * dg * gsb / den_b * dl
                    beta = C0 * c1 * gsb / den_b
                    betas = C0 * c1 * (k.gq(ss) / den_b - 2.0 * gsb / den_b ** 2)
                    dpd += m * (betas * _dot(dk, b["n"]) * dg * dl +
                                beta * (_dot(b["n"], g) * dl + dg * _dot(b["n"], lt)))
                X += dpd[:, None] * b["gpd"] + np.where(m, dvb / np.where(m, b["vb"], 1.0), 0.0)[:, None] * b["gvb"]
            Q = Q + P.nub * P.rho0 * b1
        rhob += -_dot(lt, Q) / rho
        dtob = float(np.sum(_dot(lam, Q) / rho))
        nub = float(P.rho0 * np.sum(_dot(lt, q1)))
        nubb = float(P.rho0 * np.sum(_dot(lt, b1)))
        return X, rhob, dtob, nub, nubb


class Rollout:
    """`steps` steps from (x0, v0); loss gradients by reverse sweeps over the steps."""

    def __init__(self, desc: dict, maps: list):
        self.P = Params(desc)
        self.maps = maps

    def forward(self, x0, v0, steps: int):
        self.steps = []
        x, v, dt = np.asarray(x0, np.float64), np.asarray(v0, np.float64), self.P.dt0
        for _ in range(steps):
            st = Step(self.P, self.maps)
            x, v, dt = st.forward(x, v, dt)
            self.steps.append(st)
        return x, v

    def backward(self, xb, vb):
        xb, vb = np.asarray(xb, np.float64), np.asarray(vb, np.float64)
        dtb = 0.0
        nub = nubb = 0.0
        for st in reversed(self.steps):
            xb, vb, dtb, a, b = st.backward(xb, vb, dtb)
            nub += a
            nubb += b
        return xb, vb, np.array([nub, nubb])


def rollout_loss(desc: dict, maps: list, x0, v0, steps: int, target):
    """Mean squared distance of the final positions to `target`."""
    R = Rollout(desc, maps)
    x, _ = R.forward(x0, v0, steps)
    return float(np.mean(np.sum((x - target) ** 2, axis=1)))
