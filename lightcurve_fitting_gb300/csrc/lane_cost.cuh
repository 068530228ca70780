// lane_cost.cuh — PsoCost::cost_from_slice and PsoCost::gradient
// (src/parametric.rs:1303-1446) of one parameter vector over a band, laid
// out across the lanes of a warp: component j of the vector in lane j, the
// observations split over the lanes, double-float observation terms with the
// FP64 term wherever an exponent or the prediction could leave FP32's range.
// Used by the swarms' accurate re-check of near-tied comparisons (pso.cu);
// the L-BFGS polish evaluates per group of eight lanes (lbfgs_group.cuh)
// with the same observation terms.
#pragma once

#include <cuda_runtime.h>

#include "lcf_internal.cuh"
#include "models_f32.cuh"
#include "models_f64.cuh"
#include "models_ff.cuh"

#ifndef FULL
#define FULL 0xffffffffu
#endif

namespace lcf {

// a.b over lanes j = lane & 7 (xor 4, 2, 1 sums; the four groups of eight
// lanes hold identical copies in the warp-wide uses)
__device__ __forceinline__ double dot8(double a, double b) {
    double v = a * b;
    v += __shfl_xor_sync(0xffffffffu, v, 4);
    v += __shfl_xor_sync(0xffffffffu, v, 2);
    v += __shfl_xor_sync(0xffffffffu, v, 1);
    return v;
}

__device__ __forceinline__ double warp_sum_d(double v) {
    for (int k = 16; k; k >>= 1) v += __shfl_xor_sync(FULL, v, k);
    return v;
}
__device__ __forceinline__ float warp_sum_f(float v) {
    for (int k = 16; k; k >>= 1) v += __shfl_xor_sync(FULL, v, k);
    return v;
}
__device__ __forceinline__ int warp_or(int v) { return __any_sync(FULL, v) ? 1 : 0; }

// Sums 8 per-lane values over the warp by recursive halving: 4 + 2 + 1
// exchanges halve the values each lane carries, two more finish the sum.
// Lane l returns the warp total of v[(l >> 2) & 7].
__device__ __forceinline__ double reduce_scatter8(const double* v) {
    const int lane = threadIdx.x & 31;
    const bool b4 = lane & 16, b3 = lane & 8, b2 = lane & 4;
    double a[4], b[2];
#pragma unroll
    for (int i = 0; i < 4; i++) {
        double keep = b4 ? v[4 + i] : v[i], give = b4 ? v[i] : v[4 + i];
        a[i] = keep + __shfl_xor_sync(FULL, give, 16);
    }
#pragma unroll
    for (int i = 0; i < 2; i++) {
        double keep = b3 ? a[2 + i] : a[i], give = b3 ? a[i] : a[2 + i];
        b[i] = keep + __shfl_xor_sync(FULL, give, 8);
    }
    double c = (b2 ? b[1] : b[0]) + __shfl_xor_sync(FULL, b2 ? b[0] : b[1], 4);
    c += __shfl_xor_sync(FULL, c, 2);
    c += __shfl_xor_sync(FULL, c, 1);
    return c;
}

// One observation's term of PsoCost::cost_from_slice and PsoCost::gradient
// (src/parametric.rs:1303-1446) in FP64: adds to the negative log-likelihood
// and to the gradient partials.  One FP64 reciprocal per observation stands
// in for a division per term (the FP64 pipe bounds the polish).
template <int MODEL>
__device__ __forceinline__ void lb_obs_term(const Model64& mod, double t, double var, double flux, uint8_t up,
                                            double uf, double se2, bool want_grad, double& nll, double* gl,
                                            int& nonfinite) {
    constexpr int np = n_params_of(MODEL), se = se_idx_of(MODEL);
    double mg[MAXP];
    double pr = mod.eval(t, want_grad ? mg : nullptr);
    if (!isfinite(pr)) { nonfinite = 1; return; }
    double tv = var + se2;
    if (up) {
        double isv = 1.0 / sqrt(tv);
        double z = (uf - pr) * isv;
        double ratio;
        nll -= upper_cost_ratio(z, want_grad, ratio);
        if (want_grad) {
            double ri = ratio * isv;
#pragma unroll
            for (int k = 0; k < np; k++) gl[k] += ri * mg[k];
            gl[se] += ratio * z * se2 * (isv * isv);
        }
    } else {
        double dd = pr - flux;
        double itv = 1.0 / tv;
        nll += dd * dd * itv + log(tv);
        if (want_grad) {
            double sc = 2.0 * dd * itv;
#pragma unroll
            for (int k = 0; k < np; k++) gl[k] += sc * mg[k];
            gl[se] += (-dd * dd * itv * itv + itv) * (2.0 * se2);
        }
    }
}

#ifndef LCF_FALLBACK_ATTR
#define LCF_FALLBACK_ATTR __device__ __forceinline__
#endif
// Cost and projected gradient of the bounded problem (BoundedPsoCost,
// src/parametric.rs:1500-1535) for the lane-distributed polish: the full
// parameter vector is gathered from lanes 0..np-1, the lanes split the
// observations, and each lane keeps its own component of the gradient.
// FP64 throughout: PsoCost::cost_from_slice (population prior, Villar
// constraint) and PsoCost::gradient (neither), as in the reference.  The
// polish runs in the reference's arithmetic because its acceptance tests
// (descent direction, sufficient decrease, curvature) compare differences of
// near-equal costs and gradients near the optimum.
template <int MODEL>
struct LaneLb {
    static constexpr int np = n_params_of(MODEL);
    const double *t, *flux, *var, *uf;
    const uint8_t* up;
    const float4* fa;   // the band's observations as double-float pairs
    const float2* fb;
    double t_first, t_last;
    int n;
    double nd, inv_nd;
    double lo_j, hi_j;
    int evals, iters, fp64_evals;
    bool with_prior;  // add the population prior (PsoCost with priors)

    // the observation terms in FP64 (lb_obs_term), this lane's share
    template <int M>
    LCF_FALLBACK_ATTR int fp64_terms(const double* q, const double* ep, const double* rp, double se2, bool want_grad,
                                     double& nll, double* gl) const {
        int nonfinite = 0;
        Model64 mod;
        mod.init_pre(M, q, ep, rp);
        for (int i = (int)(threadIdx.x & 31); i < n; i += 32)
            lb_obs_term<M>(mod, t[i], var[i], flux[i], up[i], uf[i], se2, want_grad, nll, gl, nonfinite);
        return nonfinite;
    }

#ifdef LCF_LB_INLINE
    __device__ void cost_grad(double xj, double& fo, double& gj, bool want_grad) {
#else
    // out of line: one copy of the observation loop per model instead of one
    // per call site keeps the polish's hot code in the instruction cache
    __device__ __noinline__ void cost_grad(double xj, double& fo, double& gj, bool want_grad) {
#endif
        evals++;
        const int lane = threadIdx.x & 31, j = lane & 7;
        // lane j forms e^(+-p_j) of its own component in double-float; the
        // full vectors are gathered by shuffles
        const double qj = fmin(fmax(xj, lo_j), hi_j);
        const ff qjf = ff_from(qj);
        const ff ejf = ff_exp(qjf), rjf = ff_exp(ff_neg(qjf));
        double q[MAXP];
        ff ef[MAXP], rf[MAXP];
#pragma unroll
        for (int k = 0; k < MAXP; k++) {
            q[k] = k < np ? __shfl_sync(FULL, qj, k) : 0.0;
            ef[k] = k < np ? shfl_ff(ejf, k) : ffm(1.0f, 0.0f);
            rf[k] = k < np ? shfl_ff(rjf, k) : ffm(1.0f, 0.0f);
        }
        constexpr int se = se_idx_of(MODEL);
        const ff se2f = ff_sqr(ef[se]);  // sigma_extra = exp(p[se]), squared
        bool constrained = false;
        double f = 0.0;
        if (MODEL == VILLAR) {
            // Villar constraint of PsoCost (src/parametric.rs:1305-1318):
            // beta = p1, gamma = e^p2, tr = e^p4, tf = e^p5
            const ff beta = ff_from(q[1]), gamma = ef[2], itr = rf[4], tf = ef[5];
            const ff one = ffm(1.0f, 0.0f);
            ff c1 = ff_sub(ff_mul(gamma, beta), one);
            ff c2 = ff_sub(ff_mul(ff_exp(ff_neg(ff_mul(gamma, itr))), ff_sub(ff_mul(tf, itr), one)), one);
            ff c3 = ff_add(ff_sub(ff_mul(beta, tf), one), ff_mul(beta, gamma));
            ff cc = ff_add(ff_add(c1.hi > 0.0f ? c1 : ffm(0.0f, 0.0f), c2.hi > 0.0f ? c2 : ffm(0.0f, 0.0f)),
                           c3.hi > 0.0f ? c3 : ffm(0.0f, 0.0f));
            if (cc.hi > 0.0f) { f = 1e12 + 10000.0 * ff_to(cc); constrained = true; }
        }
        // population prior, one component per lane (PsoCost::cost_from_slice)
        const double zj = j < np ? (qj - c_pop_c[MODEL][j]) * c_pop_iw[MODEL][j] : 0.0;
        const double prior = with_prior ? dot8(0.5 * zj, zj) : 0.0;
        int nonfinite = 0;
        double nsum, gs = 0.0;
        // the observation terms in double-float (the FP64 pipe is 1/64 of
        // FP32 here) unless an exponent or the prediction could leave FP32's
        // range over the band's span, or an upper limit's gradient ratio does
        // (the same decision in every lane)
        const double t0 = q[t0_idx_of(MODEL)];
        bool in_ff = ff_range_ok<MODEL>(q, rf, t_first - t0, t_last - t0);
        if (in_ff) {
            FfModel<MODEL> fm;
            fm.init(q, ef, rf);
            ff nf = ffm(0.0f, 0.0f), gf[MAXP];
#pragma unroll
            for (int k = 0; k < MAXP; k++) gf[k] = ffm(0.0f, 0.0f);
            int redo = 0;
            for (int i = lane; i < n; i += 32)
                ff_obs_term<MODEL>(fm, fa[i], fb[i], se2f, want_grad, nf, gf, nonfinite, redo);
            in_ff = !warp_or(redo);
            if (in_ff) {
                nonfinite = warp_or(nonfinite);
                if (want_grad) {
                    // reduce-scatter of the 8 sums: lane l ends with sum (l >> 2) & 7
                    const ff v[8] = {nf, gf[0], gf[1], gf[2], gf[3], gf[4], gf[5], gf[6]};
                    const double tot = ff_to(reduce_scatter8_ff(v));
                    nsum = __shfl_sync(FULL, tot, 0);
                    gs = __shfl_sync(FULL, tot, (4 * (1 + j)) & 31);
                } else {
                    nsum = ff_to(warp_sum_ff(nf));
                }
            }
        }
        if (!in_ff) {
            fp64_evals++;
            double ep[MAXP], rp[MAXP];
#pragma unroll
            for (int k = 0; k < MAXP; k++) { ep[k] = ff_to(ef[k]); rp[k] = ff_to(rf[k]); }
            const double se2 = ep[se] * ep[se];
            double nll = 0.0, gl[MAXP];
#pragma unroll
            for (int k = 0; k < MAXP; k++) gl[k] = 0.0;
            nonfinite = fp64_terms<MODEL>(q, ep, rp, se2, want_grad, nll, gl);
            nonfinite = warp_or(nonfinite);
            if (want_grad) {
                double v[8] = {nll, gl[0], gl[1], gl[2], gl[3], gl[4], gl[5], gl[6]};
                double tot = reduce_scatter8(v);
                nsum = __shfl_sync(FULL, tot, 0);
                gs = __shfl_sync(FULL, tot, (4 * (1 + j)) & 31);
            } else {
                nsum = warp_sum_d(nll);
            }
        }
        if (!constrained) f = nonfinite ? BIG_COST : (nsum + prior * inv_nd) * inv_nd;
        fo = f;
        if (!want_grad) return;
        gj = (nonfinite || j >= np) ? 0.0 : gs * inv_nd;
        if ((xj <= lo_j && gj > 0.0) || (xj >= hi_j && gj < 0.0)) gj = 0.0;
    }
};


}  // namespace lcf
