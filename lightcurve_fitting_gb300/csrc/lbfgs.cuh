// lbfgs.cuh — bounded L-BFGS polish (lbfgs_refine, src/parametric.rs:1453-1535)
// on a cost/gradient supplier.  The reference calls argmin 0.11's LBFGS (memory
// 7, gradient tolerance 1e-6, cost tolerance machine epsilon, 50 iterations)
// with the MINPACK Moré–Thuente line search (ftol 1e-4, gtol 0.9, xtol 1e-10,
// initial step 1); both are restated here from the published algorithms, in
// FP64, identically in every lane of a warp.
//
// Ctx supplies:
//   int np;                     problem dimension
//   double lo[MAXP], hi[MAXP];  box of the bounded problem
//   void cost_grad(const double* x, double& f, double* g, bool want_grad);
//       cost of the clamped point and its projected gradient (warp-collective)
//   int evals, iters;           work counters (evaluations counted by cost_grad,
//                               iterations written by lbfgs_polish)
#pragma once

#include <math.h>

#include "lcf_internal.cuh"

namespace lcf {

// FP64 division and square root out of line: the IEEE-rounded results of
// the operators themselves, one copy of their instruction sequences instead
// of one per use.  The polish is bound by instruction fetch, and the line
// search's many divisions dominated its code.
#ifdef LCF_LB_INLINE_DIV
__device__ __forceinline__ double lb_div(double a, double b) { return a / b; }
__device__ __forceinline__ double lb_sqrt(double x) { return sqrt(x); }
#else
static __device__ __noinline__ double lb_div(double a, double b) { return a / b; }
static __device__ __noinline__ double lb_sqrt(double x) { return sqrt(x); }
#endif

// MINPACK cstep (Moré–Thuente), min/max with Rust's NaN-ignoring semantics;
// out of line (one copy shared by every call site and model)
#ifndef LCF_CSTEP_ATTR
#define LCF_CSTEP_ATTR static __device__ __noinline__
#endif
LCF_CSTEP_ATTR int lb_cstep(double& stx, double& fx, double& dx, double& sty, double& fy, double& dy, double& stp, double fp,
                        double dp, bool& brackt, double stpmin, double stpmax) {
    if ((brackt && (stp <= fmin(stx, sty) || stp >= fmax(stx, sty))) || dx * (stp - stx) >= 0.0 || stpmax < stpmin)
        return 0;
    int info;
    bool bound;
    double sgnd = dp * lb_div(dx, fabs(dx));
    double stpf, stpc, stpq, theta, s, gamma, p, q, r;
    if (fp > fx) {
        info = 1; bound = true;
        theta = lb_div(3.0 * (fx - fp), stp - stx) + dx + dp;
        s = fmax(fmax(fabs(theta), fabs(dx)), fabs(dp));
        gamma = s * lb_sqrt(lb_div(theta, s) * lb_div(theta, s) - lb_div(dx, s) * lb_div(dp, s));
        if (stp < stx) gamma = -gamma;
        p = (gamma - dx) + theta;
        q = ((gamma - dx) + gamma) + dp;
        r = lb_div(p, q);
        stpc = stx + r * (stp - stx);
        stpq = stx + (lb_div(dx, lb_div(fx - fp, stp - stx) + dx) / 2.0) * (stp - stx);
        stpf = fabs(stpc - stx) < fabs(stpq - stx) ? stpc : stpc + (stpq - stpc) / 2.0;
        brackt = true;
    } else if (sgnd < 0.0) {
        info = 2; bound = false;
        theta = lb_div(3.0 * (fx - fp), stp - stx) + dx + dp;
        s = fmax(fmax(fabs(theta), fabs(dx)), fabs(dp));
        gamma = s * lb_sqrt(lb_div(theta, s) * lb_div(theta, s) - lb_div(dx, s) * lb_div(dp, s));
        if (stp > stx) gamma = -gamma;
        p = (gamma - dp) + theta;
        q = ((gamma - dp) + gamma) + dx;
        r = lb_div(p, q);
        stpc = stp + r * (stx - stp);
        stpq = stp + lb_div(dp, dp - dx) * (stx - stp);
        stpf = fabs(stpc - stp) > fabs(stpq - stp) ? stpc : stpq;
        brackt = true;
    } else if (fabs(dp) < fabs(dx)) {
        info = 3; bound = true;
        theta = lb_div(3.0 * (fx - fp), stp - stx) + dx + dp;
        s = fmax(fmax(fabs(theta), fabs(dx)), fabs(dp));
        gamma = s * lb_sqrt(fmax(0.0, lb_div(theta, s) * lb_div(theta, s) - lb_div(dx, s) * lb_div(dp, s)));
        if (stp > stx) gamma = -gamma;
        p = (gamma - dp) + theta;
        q = (gamma + (dx - dp)) + gamma;
        r = lb_div(p, q);
        if (r < 0.0 && gamma != 0.0) stpc = stp + r * (stx - stp);
        else if (stp > stx) stpc = stpmax;
        else stpc = stpmin;
        stpq = stp + lb_div(dp, dp - dx) * (stx - stp);
        if (brackt) stpf = fabs(stp - stpc) < fabs(stp - stpq) ? stpc : stpq;
        else stpf = fabs(stp - stpc) > fabs(stp - stpq) ? stpc : stpq;
    } else {
        info = 4; bound = false;
        if (brackt) {
            theta = lb_div(3.0 * (fp - fy), sty - stp) + dy + dp;
            s = fmax(fmax(fabs(theta), fabs(dy)), fabs(dp));
            gamma = s * lb_sqrt(lb_div(theta, s) * lb_div(theta, s) - lb_div(dy, s) * lb_div(dp, s));
            if (stp > sty) gamma = -gamma;
            p = (gamma - dp) + theta;
            q = ((gamma - dp) + gamma) + dy;
            r = lb_div(p, q);
            stpc = stp + r * (sty - stp);
            stpf = stpc;
        } else {
            stpf = stp > stx ? stpmax : stpmin;
        }
    }
    if (fp > fx) {
        sty = stp; fy = fp; dy = dp;
    } else {
        if (sgnd < 0.0) { sty = stx; fy = fx; dy = dx; }
        stx = stp; fx = fp; dx = dp;
    }
    stpf = fmin(stpmax, stpf);
    stpf = fmax(stpmin, stpf);
    stp = stpf;
    if (brackt && bound) {
        if (sty > stx) stp = fmin(stx + 0.66 * (sty - stx), stp);
        else stp = fmax(stx + 0.66 * (sty - stx), stp);
    }
    return info;
}

__device__ __forceinline__ double dotn(const double* a, const double* b, int n) {
    double s = 0.0;
    for (int i = 0; i < n; i++) s += a[i] * b[i];
    return s;
}

// Moré–Thuente line search; false = not a descent direction (argmin error)
template <class Ctx>
__device__ bool lb_linesearch(Ctx& c, const double* x, double f0, const double* g0, const double* d, double* xo,
                              double& fo, double* go) {
    const int n = c.np;
    const double ftol = 1e-4, gtol = 0.9, xtol = 1e-10, xtrapf = 4.0, stpmin_g = 0.0, stpmax_g = INFINITY;
    double dginit = dotn(g0, d, n);
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
        for (int i = 0; i < n; i++) xo[i] = x[i] + stp * d[i];
        double f;
        c.cost_grad(xo, f, go, true);
        double dg = dotn(go, d, n);
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
    double g_unused[MAXP];
    c.cost_grad(xo, fo, g_unused, false);
    return true;
}

// lbfgs_refine, src/parametric.rs:1453-1497: returns the polished cost and
// writes the parameters when the polish improved the PSO result.
template <class Ctx>
__device__ double lbfgs_polish(Ctx& c, double* params, double pso_cost) {
    const int n = c.np, M = 7, MAXIT = 50;
    const double tol_grad = 1e-6, tol_cost = 2.220446049250313e-16;
    double x[MAXP], g[MAXP], f;
    for (int i = 0; i < n; i++) x[i] = params[i];
    c.cost_grad(x, f, g, true);
    double best_x[MAXP], best_f = INFINITY, prev_f = INFINITY;
    if (f < best_f) { best_f = f; for (int i = 0; i < n; i++) best_x[i] = x[i]; }
    double S[M][MAXP], Y[M][MAXP];
    int cm = 0, head = 0;  // ring buffer: oldest at head
    int it = 0;
    bool ok = true;
    auto converged = [&]() { return sqrt(dotn(g, g, n)) < tol_grad || fabs(prev_f - f) < tol_cost; };
    bool stop = converged() || it >= MAXIT;
    while (!stop) {
        double gamma = 1.0;
        if (cm > 0) {
            int last = (head + cm - 1) % M;
            gamma = dotn(S[last], Y[last], n) / dotn(Y[last], Y[last], n);
        }
        double q[MAXP], alpha[M], rho[M];
        for (int k = 0; k < n; k++) q[k] = g[k];
        for (int i = 0; i < cm; i++) {
            int idx = (head + cm - 1 - i) % M;
            double rt = 1.0 / dotn(Y[idx], S[idx], n);
            alpha[i] = rt * dotn(S[idx], q, n);
            for (int k = 0; k < n; k++) q[k] -= Y[idx][k] * alpha[i];
            rho[i] = rt;
        }
        double r[MAXP];
        for (int k = 0; k < n; k++) r[k] = q[k] * gamma;
        for (int i = 0; i < cm; i++) {
            int idx = (head + i) % M;
            double beta = dotn(Y[idx], r, n) * rho[cm - i - 1];
            for (int k = 0; k < n; k++) r[k] += S[idx][k] * (alpha[cm - i - 1] - beta);
        }
        double dvec[MAXP], xn[MAXP], gn[MAXP], fnew;
        for (int k = 0; k < n; k++) dvec[k] = -r[k];
        // the line search returns the cost and gradient of its accepted point
        // (argmin re-evaluates the gradient there: the same deterministic value)
        if (!lb_linesearch(c, x, f, g, dvec, xn, fnew, gn)) { ok = false; break; }
        int slot;
        if (cm < M) { slot = (head + cm) % M; cm++; }
        else { slot = head; head = (head + 1) % M; }
        for (int k = 0; k < n; k++) { S[slot][k] = xn[k] - x[k]; Y[slot][k] = gn[k] - g[k]; x[k] = xn[k]; g[k] = gn[k]; }
        prev_f = f;
        f = fnew;
        if (f < best_f) { best_f = f; for (int i = 0; i < n; i++) best_x[i] = x[i]; }
        it++;
        stop = converged() || it >= MAXIT;
    }
    c.iters = it;
    if (!ok) return pso_cost;
    double cl[MAXP], fc, gdummy[MAXP];
    for (int i = 0; i < n; i++) cl[i] = fmin(fmax(best_x[i], c.lo[i]), c.hi[i]);
    c.cost_grad(cl, fc, gdummy, false);
    if (fc < pso_cost && isfinite(fc)) {
        for (int i = 0; i < n; i++) params[i] = cl[i];
        return fc;
    }
    return pso_cost;
}

}  // namespace lcf
