// lbfgs_lane.cuh — the bounded L-BFGS polish of lbfgs.cuh (lbfgs_refine,
// src/parametric.rs:1453-1535; argmin 0.11 LBFGS with memory 7 and the
// MINPACK Moré–Thuente line search), laid out across the lanes of a warp:
// lane l holds component (l & 7) of every parameter-space vector (iterate,
// gradient, direction, the seven curvature pairs), so the vector algebra is
// one FP64 operation per lane and a dot product is a three-step shuffle sum
// inside each group of eight lanes (the four groups hold identical copies).
// The curvature history is a shift register with the newest pair at index
// 0.  The two-loop recursion and the shift are not unrolled (the history
// then lives in local memory, cached in L1): the polish is bound by
// instruction fetch, and the unrolled loops were ~16 KB of its code per
// model.  The scalar line-search state is uniform across the warp.
//
// Arithmetic is that of lbfgs.cuh except the order of the terms of each dot
// product (a tree instead of a left-to-right sum) and 1 / (y.s) being kept
// with its pair instead of recomputed (the same value).
//
// Ctx supplies:
//   static constexpr int np;         problem dimension (<= 7)
//   double lo_j, hi_j;               this lane's box bounds (0 for j >= np)
//   void cost_grad(double xj, double& f, double& gj, bool want_grad);
//       cost at the clamped point whose component j is xj in lane j, and this
//       lane's component of the projected gradient (warp-collective)
//   int evals, iters;                work counters
#pragma once

#include <math.h>

#include "lbfgs.cuh"

namespace lcf {

__device__ __forceinline__ double dot8(double a, double b) {
    double v = a * b;
    v += __shfl_xor_sync(0xffffffffu, v, 4);
    v += __shfl_xor_sync(0xffffffffu, v, 2);
    v += __shfl_xor_sync(0xffffffffu, v, 1);
    return v;
}

template <class Ctx>
__device__ bool lane_linesearch(Ctx& c, double xj, double f0, double g0j, double dj, double& xoj, double& fo,
                                double& goj) {
    const double ftol = 1e-4, gtol = 0.9, xtol = 1e-10, xtrapf = 4.0, stpmin_g = 0.0, stpmax_g = INFINITY;
    double dginit = dot8(g0j, dj);
    if (dginit >= 0.0) return false;
    bool brackt = false, stage1 = true;
    int infoc = 1;
    double finit = f0, dgtest = ftol * dginit, width = stpmax_g - stpmin_g, width1 = 2.0 * width;
    double stx = 0.0, fx = finit, dgx = dginit, sty = 0.0, fy = finit, dgy = dginit, stp = 1.0;
    for (int iter = 0; iter < 100; iter++) {
        double stmin, stmax;
        if (brackt) { stmin = fmin(stx, sty); stmax = fmax(stx, sty); }
        else { stmin = stx; stmax = stp + xtrapf * (stp - stx); }
        stp = fmax(stp, stpmin_g);
        stp = fmin(stp, stpmax_g);
        if ((brackt && (stp <= stmin || stp >= stmax)) || infoc == 0 || (brackt && stmax - stmin <= xtol * stmax))
            stp = stx;
        xoj = xj + stp * dj;
        double f;
        c.cost_grad(xoj, f, goj, true);
        double dg = dot8(goj, dj);
        double ftest1 = finit + stp * dgtest;
        int info = 0;
        if ((brackt && (stp <= stmin || stp >= stmax)) || infoc == 0) info = 6;
        if (stp == stpmax_g && f <= ftest1 && dg <= dgtest) info = 5;
        if (stp == stpmin_g && (f > ftest1 || dg >= dgtest)) info = 4;
        if (brackt && stmax - stmin <= xtol * stmax) info = 2;
        if (f <= ftest1 && fabs(dg) <= gtol * (-dginit)) info = 1;
        if (info != 0) { fo = f; return true; }
        if (stage1 && f <= ftest1 && dg >= fmin(ftol, gtol) * dginit) stage1 = false;
        if (stage1 && f <= fx && f > ftest1) {
            double fm = f - stp * dgtest, fxm = fx - stx * dgtest, fym = fy - sty * dgtest;
            double dgm = dg - dgtest, dgxm = dgx - dgtest, dgym = dgy - dgtest;
            infoc = lb_cstep(stx, fxm, dgxm, sty, fym, dgym, stp, fm, dgm, brackt, stmin, stmax);
            fx = fxm + stx * dgtest; fy = fym + sty * dgtest;
            dgx = dgxm + dgtest; dgy = dgym + dgtest;
        } else {
            infoc = lb_cstep(stx, fx, dgx, sty, fy, dgy, stp, f, dg, brackt, stmin, stmax);
        }
        if (brackt) {
            if (fabs(sty - stx) >= 0.66 * width1) stp = stx + 0.5 * (sty - stx);
            width1 = width;
            width = fabs(sty - stx);
        }
    }
    double g_unused;
    c.cost_grad(xoj, fo, g_unused, false);
    return true;
}

// Polishes the parameter vector whose component j sits in lane j (pj);
// returns the polished cost, and updates pj when the polish improved the
// PSO cost.
template <class Ctx>
__device__ double lane_lbfgs_polish(Ctx& c, double& pj, double pso_cost) {
    constexpr int M = 7, MAXIT = 50;
    const double tol_grad = 1e-6, tol_cost = 2.220446049250313e-16;
    double xj = pj, gj, f;
    c.cost_grad(xj, f, gj, true);
    double best_xj = xj, best_f = INFINITY, prev_f = INFINITY;
    if (f < best_f) { best_f = f; best_xj = xj; }
    double S[M], Y[M], rho[M];
#pragma unroll
    for (int k = 0; k < M; k++) { S[k] = 0.0; Y[k] = 0.0; rho[k] = 0.0; }
    int cm = 0, it = 0;
    bool ok = true;
    auto converged = [&]() { return lb_sqrt(dot8(gj, gj)) < tol_grad || fabs(prev_f - f) < tol_cost; };
    bool stop = converged() || it >= MAXIT;
    while (!stop) {
        double gamma = cm > 0 ? lb_div(dot8(S[0], Y[0]), dot8(Y[0], Y[0])) : 1.0;
        // two-loop recursion: newest (index 0) to oldest, then back
        double q = gj, alpha[M];
#pragma unroll 1
        for (int k = 0; k < cm; k++) {
            alpha[k] = rho[k] * dot8(S[k], q);
            q -= Y[k] * alpha[k];
        }
        double r = q * gamma;
#pragma unroll 1
        for (int k = cm - 1; k >= 0; k--) {
            double beta = dot8(Y[k], r) * rho[k];
            r += S[k] * (alpha[k] - beta);
        }
        double dj = -r, xnj, gnj, fnew;
        if (!lane_linesearch(c, xj, f, gj, dj, xnj, fnew, gnj)) { ok = false; break; }
        double sj = xnj - xj, yj = gnj - gj;
#pragma unroll 1
        for (int k = M - 1; k > 0; k--) { S[k] = S[k - 1]; Y[k] = Y[k - 1]; rho[k] = rho[k - 1]; }
        S[0] = sj;
        Y[0] = yj;
        rho[0] = lb_div(1.0, dot8(yj, sj));
        cm = cm < M ? cm + 1 : M;
        xj = xnj;
        gj = gnj;
        prev_f = f;
        f = fnew;
        if (f < best_f) { best_f = f; best_xj = xj; }
        it++;
        stop = converged() || it >= MAXIT;
    }
    c.iters = it;
    if (!ok) return pso_cost;
    double clj = fmin(fmax(best_xj, c.lo_j), c.hi_j), fc, g_unused;
    c.cost_grad(clj, fc, g_unused, false);
    if (fc < pso_cost && isfinite(fc)) {
        pj = clj;
        return fc;
    }
    return pso_cost;
}

}  // namespace lcf
