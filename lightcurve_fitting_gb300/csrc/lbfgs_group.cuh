// lbfgs_group.cuh — the restart reduction and bounded L-BFGS polish of
// pso_fit_single_model (src/parametric.rs:1864-1972; lbfgs_refine,
// :1453-1535: argmin 0.11 LBFGS with memory 7, gradient tolerance 1e-6, cost
// tolerance machine epsilon, 50 iterations, and the MINPACK Moré–Thuente
// line search with ftol 1e-4, gtol 0.9, xtol 1e-10, initial step 1), with
// four polishes per warp.
//
// The bands of the metric's workload hold ~45 observations.  Spread over a
// whole warp, one cost evaluation left most lanes one observation, and the
// work per evaluation that does not scale with the band (the parameters'
// exponentials and gathers, the reductions, the line search's scalar FP64
// arithmetic, which every lane repeated) dominated the polish.  Here each
// group of eight lanes runs its own polish: lane j of a group holds
// component j of every parameter-space vector, and the group's lanes split
// its band's observations (j, j + 8, ...).  One warp instruction of the
// vector algebra or of the line search now serves four polishes.
//
// The polish is written as a state machine whose one suspension point is the
// cost evaluation.  Each round every group evaluates its pending point (the
// warp's lanes together: the same model, each group its own band), then
// advances its own state: the accurate re-check of near-tied restarts, one
// Moré–Thuente step, the L-BFGS update and two-loop direction, or the final
// clamped evaluation.  A group whose polish has ended takes the next band
// from the model's queue; bands are queued longest first, so the groups of a
// warp hold bands of similar length and their observation loops end
// together.
//
// On a batch that fills the grid the polish is bound by instruction fetch
// (its double-float terms and FP64 line search are long code; measured on
// GB300, more resident warps at different points of it made it slower).  The
// warps of a block then run a round in step: a block barrier before and
// after the evaluation, so that they fetch the same code.  A smaller batch is
// bound by the latency of its polishes, which the barriers would lengthen.  The group's scalar state and the per-lane
// vectors live in shared memory, leaving the registers to the evaluation.
//
// Arithmetic: the reference's algorithm in FP64 (lbfgs.cuh restates it for
// one thread).  The dot products are sums over the eight lanes by xor 4, 2, 1
// exchanges; the curvature pairs sit in a ring of seven (newest first in the
// two-loop recursion); the observation terms are double-float (ff.cuh,
// models_ff.cuh) with the FP64 term wherever an exponent or the prediction
// could leave FP32's range, summed per lane and then by a reduce-scatter
// over the group's eight lanes.
#pragma once

#include <math.h>

#include "lane_cost.cuh"
#include "lbfgs.cuh"

#ifndef FULL
#define FULL 0xffffffffu
#endif

namespace lcf {

// A group's scalar state (its band, the restart reduction, the polish and
// the line search, its work counters), in shared memory: the group's eight
// lanes write the same values and read them back by broadcast.  Kept out of
// the registers, it leaves them to the cost evaluation, which is bound by
// latency and so by the warps resident per SM.
struct LbGroupState {
    double best_c, acc0, acc1, acc2;
    double f, prev_f, best_f;
    double dginit, dgtest, finit, width, width1, stx, fx, dgx, sty, fy, dgy, stp, stmin, stmax;
    double t_first, t_last, inv_nd;
    unsigned long long c_pol, c_it, c_ev, c_obs, c_fp64;
    int64_t off;
    int n, b, acc_mask, nc, best_r, cm, head, it, evals, fp64_evals, infoc, ls_iter;
    bool brackt, stage1;
};

// Per warp, in shared memory: the curvature pairs, 1 / (y.s) and the
// two-loop coefficients, [ring slot][lane], and the four groups' states.
struct LbWarpShared {
    double S[7][32], Y[7][32], rho[7][32], alpha[7][32];
    double V[7][32];  // per lane: x, g, search direction, trial point and gradient, best point, swarm point
    LbGroupState st[4];
};

// a.b over the eight lanes of this lane's group (mask gm)
__device__ __forceinline__ double gdot(double a, double b, unsigned gm) {
    double v = a * b;
    v += __shfl_xor_sync(gm, v, 4);
    v += __shfl_xor_sync(gm, v, 2);
    v += __shfl_xor_sync(gm, v, 1);
    return v;
}

__device__ __forceinline__ ff shfl_xor_ff_m(ff v, int m, unsigned gm) {
    return ffm(__shfl_xor_sync(gm, v.hi, m), __shfl_xor_sync(gm, v.lo, m));
}

// Reduce-scatter of eight per-lane values over a group of eight lanes
// (4 + 2 + 1 exchanges): lane j returns the group's total of v[j].
__device__ __forceinline__ ff group_rs8_ff(const ff* v, unsigned gm) {
    const int lane = threadIdx.x & 31;
    const bool b2 = lane & 4, b1 = lane & 2, b0 = lane & 1;
    ff a[4], b[2];
#pragma unroll
    for (int i = 0; i < 4; i++) a[i] = ff_add(b2 ? v[4 + i] : v[i], shfl_xor_ff_m(b2 ? v[i] : v[4 + i], 4, gm));
#pragma unroll
    for (int i = 0; i < 2; i++) b[i] = ff_add(b1 ? a[2 + i] : a[i], shfl_xor_ff_m(b1 ? a[i] : a[2 + i], 2, gm));
    return ff_add(b0 ? b[1] : b[0], shfl_xor_ff_m(b0 ? b[0] : b[1], 1, gm));
}
__device__ __forceinline__ double group_rs8(const double* v, unsigned gm) {
    const int lane = threadIdx.x & 31;
    const bool b2 = lane & 4, b1 = lane & 2, b0 = lane & 1;
    double a[4], b[2];
#pragma unroll
    for (int i = 0; i < 4; i++) a[i] = (b2 ? v[4 + i] : v[i]) + __shfl_xor_sync(gm, b2 ? v[i] : v[4 + i], 4);
#pragma unroll
    for (int i = 0; i < 2; i++) b[i] = (b1 ? a[2 + i] : a[i]) + __shfl_xor_sync(gm, b1 ? a[i] : a[2 + i], 2);
    return (b0 ? b[1] : b[0]) + __shfl_xor_sync(gm, b0 ? b[0] : b[1], 1);
}

// A group's band: where its observations start, their count (0 for a group
// without a polish), the time span, 1 / n and this lane's box bounds.
struct GroupBand {
    int64_t off;
    int n;
    double t_first, t_last, inv_nd, lo_j, hi_j;
};

// The observation terms in FP64 (lb_obs_term) for the FP32-range fallback:
// this lane's share of the group's band, v = {nll, gradient partials}.
template <int MODEL, int G>
__device__ __noinline__ int group_fp64_terms(const double* t, const double* flux, const double* var, const double* uf,
                                             const uint8_t* up, int n, const double* q, const double* ep,
                                             const double* rp, double se2, bool want_grad, double* v) {
    int nonfinite = 0;
    Model64 mod;
    mod.init_pre(MODEL, q, ep, rp);
    double nll = 0.0, gl[MAXP];
#pragma unroll
    for (int k = 0; k < MAXP; k++) gl[k] = 0.0;
    for (int i = (int)(threadIdx.x & (G - 1)); i < n; i += G)
        lb_obs_term<MODEL>(mod, t[i], var[i], flux[i], up[i], uf[i], se2, want_grad, nll, gl, nonfinite);
    v[0] = nll;
#pragma unroll
    for (int k = 0; k < MAXP; k++) v[1 + k] = gl[k];
    return nonfinite;
}

// Cost and projected gradient of the bounded problem (BoundedPsoCost,
// src/parametric.rs:1500-1535) at the point whose component j is xj in lane
// j of each group: PsoCost::cost_from_slice with the population prior and
// the Villar constraint, and PsoCost::gradient.  G lanes a group (8, or 32:
// the whole warp, whose four sets of eight lanes hold the same vectors).
// Warp-collective (every lane calls it; a group with B.n == 0 evaluates
// nothing of use).  Returns 1 when the group's terms ran in FP64.
template <int MODEL, int G>
__device__ __forceinline__ int group_cost_grad(const DeviceBatch& d, const GroupBand& B, double xj, bool want_grad,
                                               double& fo, double& gj) {
    constexpr int np = n_params_of(MODEL), se = se_idx_of(MODEL);
    const int lane = threadIdx.x & 31, j = lane & 7, g0 = lane & (32 - G);
    const unsigned gm = G == 32 ? FULL : 0xffu << g0;
    // lane j forms e^(+-p_j) of its own component in double-float; the group's
    // vectors are gathered by shuffles
    const double qj = fmin(fmax(xj, B.lo_j), B.hi_j);
    const ff qjf = ff_from(qj);
    const ff ejf = ff_exp(qjf), rjf = ff_exp(ff_neg(qjf));
    double q[MAXP];
    ff ef[MAXP], rf[MAXP];
#pragma unroll
    for (int k = 0; k < MAXP; k++) {
        q[k] = k < np ? __shfl_sync(FULL, qj, g0 + k) : 0.0;
        ef[k] = k < np ? shfl_ff(ejf, g0 + k) : ffm(1.0f, 0.0f);
        rf[k] = k < np ? shfl_ff(rjf, g0 + k) : ffm(1.0f, 0.0f);
    }
    const ff se2f = ff_sqr(ef[se]);  // sigma_extra = exp(p[se]), squared
    bool constrained = false;
    double f = 0.0;
    if (MODEL == VILLAR) {
        // Villar constraint of PsoCost (src/parametric.rs:1305-1318):
        // beta = p1, gamma = e^p2, tr = e^p4, tf = e^p5
        const ff beta = ff_from(q[1]), gamma = ef[2], itr = rf[4], tf = ef[5];
        const ff one = ffm(1.0f, 0.0f), zero = ffm(0.0f, 0.0f);
        const ff c1 = ff_sub(ff_mul(gamma, beta), one);
        const ff c2 = ff_sub(ff_mul(ff_exp(ff_neg(ff_mul(gamma, itr))), ff_sub(ff_mul(tf, itr), one)), one);
        const ff c3 = ff_add(ff_sub(ff_mul(beta, tf), one), ff_mul(beta, gamma));
        const ff cc = ff_add(ff_add(c1.hi > 0.0f ? c1 : zero, c2.hi > 0.0f ? c2 : zero), c3.hi > 0.0f ? c3 : zero);
        if (cc.hi > 0.0f) {
            f = 1e12 + 10000.0 * ff_to(cc);
            constrained = true;
        }
    }
    // population prior, one component per lane
    const double zj = j < np ? (qj - c_pop_c[MODEL][j]) * c_pop_iw[MODEL][j] : 0.0;
    const double prior = gdot(0.5 * zj, zj, FULL);
    int nonfinite = 0, fp64 = 0;
    double nsum = 0.0, gs = 0.0;
    // double-float terms unless an exponent or the prediction could leave
    // FP32's range over the band's span, or an upper limit's gradient ratio
    // does (a group-uniform decision)
    const double t0 = q[t0_idx_of(MODEL)];
    bool in_ff = B.n == 0 || ff_range_ok<MODEL>(q, rf, B.t_first - t0, B.t_last - t0);
    if (in_ff) {
        FfModel<MODEL> fm;
        fm.init(q, ef, rf);
        ff nf = ffm(0.0f, 0.0f), gf[MAXP];
#pragma unroll
        for (int k = 0; k < MAXP; k++) gf[k] = ffm(0.0f, 0.0f);
        int redo = 0;
        const float4* fa = d.ffa + B.off;
        const float2* fb = d.ffb + B.off;
        for (int i = lane & (G - 1); i < B.n; i += G)
            ff_obs_term<MODEL>(fm, fa[i], fb[i], se2f, want_grad, nf, gf, nonfinite, redo);
        in_ff = __ballot_sync(gm, redo) == 0u;
        if (in_ff) {
            nonfinite = __ballot_sync(gm, nonfinite) != 0u;
            const ff v[8] = {nf, gf[0], gf[1], gf[2], gf[3], gf[4], gf[5], gf[6]};
            if (G == 32) {  // lane l: the warp's total of v[(l >> 2) & 7]
                const double tot = ff_to(reduce_scatter8_ff(v));
                nsum = __shfl_sync(FULL, tot, 0);
                gs = __shfl_sync(FULL, tot, (4 * (1 + j)) & 31);
            } else {  // lane j: the group's total of v[j]
                const double tot = ff_to(group_rs8_ff(v, gm));
                nsum = __shfl_sync(gm, tot, g0);
                gs = __shfl_sync(gm, tot, g0 + ((j + 1) & 7));
            }
        }
    }
    if (!in_ff) {
        fp64 = 1;
        double ep[MAXP], rp[MAXP], v[8];
#pragma unroll
        for (int k = 0; k < MAXP; k++) {
            ep[k] = ff_to(ef[k]);
            rp[k] = ff_to(rf[k]);
        }
        const double se2 = ep[se] * ep[se];
        const int64_t o = B.off;
        const int nf64 = group_fp64_terms<MODEL, G>(d.t64 + o, d.f64 + o, d.var64 + o, d.uf64 + o, d.up + o, B.n, q,
                                                    ep, rp, se2, want_grad, v);
        nonfinite = __ballot_sync(gm, nf64) != 0u;
        if (G == 32) {
            const double tot = reduce_scatter8(v);
            nsum = __shfl_sync(FULL, tot, 0);
            gs = __shfl_sync(FULL, tot, (4 * (1 + j)) & 31);
        } else {
            const double tot = group_rs8(v, gm);
            nsum = __shfl_sync(gm, tot, g0);
            gs = __shfl_sync(gm, tot, g0 + ((j + 1) & 7));
        }
    }
    if (!constrained) f = nonfinite ? BIG_COST : (nsum + prior * B.inv_nd) * B.inv_nd;
    fo = f;
    gj = (nonfinite || j >= np) ? 0.0 : gs * B.inv_nd;
    if ((xj <= B.lo_j && gj > 0.0) || (xj >= B.hi_j && gj < 0.0)) gj = 0.0;
    return fp64;
}

// Two swarm result costs closer than the FP32 estimate's error (3e-5 of the
// reference value; the special values 1e99, +inf and the Villar constraint's
// 1e12 + 1e4 c compare as they are).
__device__ __forceinline__ bool swarm_cost_tie(double a, double ref) {
    if (!(fabs(ref) < 1e11) || !(fabs(a) < 1e11)) return a == ref;
    return fabs(a - ref) <= 3e-5 * fabs(ref);
}

// A polish's phases: the point a group evaluates next, and what it does with
// the result.
enum LbPhase : int {
    LB_FETCH = 0,  // take a band from the queue
    LB_ACC,        // accurate cost of a restart's swarm result (no gradient)
    LB_START,      // cost and gradient at the chosen restart's parameters
    LB_LS,         // a line-search trial point (with gradient)
    LB_TAIL,       // the line search's 100 steps ran out: cost at its last point
    LB_FINAL,      // cost at the clamped best point
    LB_DONE        // the queue is empty
};

// Polishes the queued bands of MODEL with G lanes a band (8: four bands a
// warp; 32: one): d.polish_order[i] for the indices i in [lo, hi) that this
// warp's groups take from the queue counter `next`.  `lockstep` (uniform
// over the grid): the block's warps run each round in step.
// Out of line: the two instantiations of a model (8 and 32 lanes a band)
// then take their registers separately.
#ifndef LCF_LB_QUEUE_ATTR
#define LCF_LB_QUEUE_ATTR __noinline__
#endif
template <int MODEL, int G>
__device__ LCF_LB_QUEUE_ATTR void polish_queue(const DeviceBatch& d, LbWarpShared& sh, int lo, int hi, int* next,
                                               bool lockstep) {
    constexpr int np = n_params_of(MODEL), t0i = t0_idx_of(MODEL), M = 7, MAXIT = 50;
    const double ftol = 1e-4, gtol = 0.9, xtol = 1e-10, xtrapf = 4.0, stpmin = 0.0, stpmax = INFINITY;
    const double tol_grad = 1e-6, tol_cost = 2.220446049250313e-16;
    const int lane = threadIdx.x & 31, j = lane & 7, gl = lane & (G - 1), g0 = lane & (32 - G);
    const unsigned gm = G == 32 ? FULL : 0xffu << g0;

    int phase = LB_FETCH;
    // this lane's components: box bounds, the swarm's parameter, the point
    // evaluated next, the iterate, its gradient, the search direction, the
    // trial point and its gradient, the best point
    double lo_j = 0.0, hi_j = 0.0, xe = 0.0;
    double &x = sh.V[0][lane], &g = sh.V[1][lane], &dv = sh.V[2][lane], &xo = sh.V[3][lane], &go = sh.V[4][lane],
           &bx = sh.V[5][lane], &pj = sh.V[6][lane];
    x = g = dv = xo = go = bx = pj = 0.0;
    // the group's scalars
    LbGroupState& st = sh.st[lane / G];
    int& b = st.b;
    // the restart reduction
    double &best_c = st.best_c, &acc0 = st.acc0, &acc1 = st.acc1, &acc2 = st.acc2;
    int &acc_mask = st.acc_mask, &nc = st.nc, &best_r = st.best_r;
    // the polish
    double &f = st.f, &prev_f = st.prev_f, &best_f = st.best_f;
    int &cm = st.cm, &head = st.head, &it = st.it, &evals = st.evals, &fp64_evals = st.fp64_evals;
    // the line search
    double &dginit = st.dginit, &dgtest = st.dgtest, &finit = st.finit, &width = st.width, &width1 = st.width1;
    double &stx = st.stx, &fx = st.fx, &dgx = st.dgx, &sty = st.sty, &fy = st.fy, &dgy = st.dgy;
    double &stp = st.stp, &stmin = st.stmin, &stmax = st.stmax;
    int &infoc = st.infoc, &ls_iter = st.ls_iter;
    bool &brackt = st.brackt, &stage1 = st.stage1;
    b = 0;
    st.n = 0;
    st.off = 0;
    st.t_first = st.t_last = 0.0;
    st.inv_nd = 1.0;
    best_c = acc0 = acc1 = acc2 = INFINITY;
    acc_mask = nc = 0;
    best_r = -1;
    f = 0.0;
    prev_f = best_f = INFINITY;
    cm = it = evals = fp64_evals = 0;
    head = M - 1;
    dginit = dgtest = finit = width = width1 = stx = fx = dgx = sty = fy = dgy = stp = stmin = stmax = 0.0;
    infoc = 1;
    ls_iter = 0;
    brackt = false;
    stage1 = true;
    st.c_pol = st.c_it = st.c_ev = st.c_obs = st.c_fp64 = 0;

    auto restarts = [&]() { return d.pso_res + (size_t)(b * 8 + MODEL) * 3; };
    auto finish = [&](double cost) {
        ModelFit& F = d.fits[b * 8 + MODEL];
        if (gl == 0) F.cost = cost;
        if (gl < MAXP) F.params[gl] = gl < np ? pj : NAN;
        phase = LB_FETCH;
    };
    auto converged = [&]() { return lb_sqrt(gdot(g, g, gm)) < tol_grad || fabs(prev_f - f) < tol_cost; };

    while (true) {
        // groups without a polish take bands until one needs polishing
        while (phase == LB_FETCH) {
            int i = 0;
            if (gl == 0) i = lo + atomicAdd(next, 1);
            i = __shfl_sync(gm, i, g0);
            if (i >= hi) {
                phase = LB_DONE;
                st.n = 0;
                break;
            }
            b = d.polish_order[i];
            const BandStats bs = d.stats[b];
            if (!bs.valid) continue;
            const PsoResult* R = restarts();
            if (R[0].iters < 0) continue;  // this model was not fitted for this band
            best_c = INFINITY;
            best_r = -1;
            for (int r = 0; r < 3; r++)
                if (R[r].iters >= 0 && R[r].cost < best_c) { best_c = R[r].cost; best_r = r; }
            pj = (best_r >= 0 && j < np) ? pso_param(R[best_r], j) : 0.0;
            if (MODEL == METZGER || best_r < 0) {  // MetzgerKN keeps its swarm result
                finish(best_c);
                continue;
            }
            st.off = bs.off;
            st.n = bs.n;
            st.t_first = bs.t_first;
            st.t_last = bs.t_last;
            st.inv_nd = 1.0 / (double)max(bs.n, 1);
            lo_j = j < np ? c_lo[MODEL][j] : 0.0;
            hi_j = j < np ? c_hi[MODEL][j] : 0.0;
            const double t0_lo = fmax(bs.t_first - 30.0, c_lo[MODEL][t0i]);
            const double t0_hi = fmin(bs.t_peak + 10.0, c_hi[MODEL][t0i]);
            if (j == t0i && t0_lo < t0_hi) { lo_j = t0_lo; hi_j = t0_hi; }
            // the restarts' swarms report FP32 estimates of their best costs:
            // the chosen restart's cost, and the choice among restarts within
            // the estimates' error of it, are settled on accurate costs (the
            // first strict minimum, as the reference's restart loop)
            acc_mask = 0;
            for (int r = 0; r < 3; r++)
                if (R[r].iters >= 0 && (r == best_r || swarm_cost_tie(R[r].cost, best_c))) acc_mask |= 1 << r;
            nc = __popc(acc_mask);
            acc0 = acc1 = acc2 = INFINITY;
            evals = 0;
            fp64_evals = 0;
            it = 0;
            xe = j < np ? pso_param(R[__ffs(acc_mask) - 1], j) : 0.0;
            phase = LB_ACC;
        }
        // in step, the block's warps evaluate together (see the header): a
        // barrier before and after the evaluation
        const bool active = phase != LB_DONE;
        if (lockstep ? !__syncthreads_or(active) : !__any_sync(FULL, active)) break;
        if constexpr (MODEL == METZGER) continue;  // never polished (every group is done)
        const bool want_grad = phase == LB_START || phase == LB_LS;
        GroupBand B;
        B.off = st.off;
        B.n = active ? st.n : 0;
        B.t_first = st.t_first;
        B.t_last = st.t_last;
        B.inv_nd = st.inv_nd;
        B.lo_j = lo_j;
        B.hi_j = hi_j;
        double fe = 0.0, ge = 0.0;
        int used64 = 0;
        if (__any_sync(FULL, active)) used64 = group_cost_grad<MODEL, G>(d, B, xe, want_grad, fe, ge);
        if (lockstep) __syncthreads();
        if (!active) continue;
        fp64_evals += used64;
        // the transition of this group's phase; the steps shared by several
        // phases (accepting a line-search point, a new direction, the next
        // trial point, the end of the polish) run once each, below the switch
        bool do_accept = false, do_begin = false, do_trial = false, do_end = false;
        double fnew = 0.0, end_cost = 0.0;
        switch (phase) {
            case LB_ACC: {
                const int r = __ffs(acc_mask) - 1;
                if (r == 0) acc0 = fe;
                else if (r == 1) acc1 = fe;
                else acc2 = fe;
                acc_mask &= acc_mask - 1;
                const PsoResult* R = restarts();
                if (acc_mask) {
                    xe = j < np ? pso_param(R[__ffs(acc_mask) - 1], j) : 0.0;
                    break;
                }
                if (nc > 1) {
                    best_r = -1;
                    best_c = INFINITY;
                    if (acc0 < best_c) { best_c = acc0; best_r = 0; }
                    if (acc1 < best_c) { best_c = acc1; best_r = 1; }
                    if (acc2 < best_c) { best_c = acc2; best_r = 2; }
                    if (best_r < 0) best_r = 0;
                    pj = j < np ? pso_param(R[best_r], j) : 0.0;
                } else {
                    best_c = best_r == 0 ? acc0 : best_r == 1 ? acc1 : acc2;
                }
                x = pj;
                xe = x;
                phase = LB_START;
                break;
            }
            case LB_START:
                evals++;
                f = fe;
                g = ge;
                best_f = INFINITY;
                prev_f = INFINITY;
                bx = x;
                if (f < best_f) { best_f = f; bx = x; }
                cm = 0;
                head = M - 1;
                if (converged() || it >= MAXIT) {
                    xe = fmin(fmax(bx, lo_j), hi_j);
                    phase = LB_FINAL;
                } else {
                    do_begin = true;
                }
                break;
            case LB_LS: {
                evals++;
                const double fl = fe;
                go = ge;
                const double dg = gdot(go, dv, gm);
                const double ftest1 = finit + stp * dgtest;
                int info = 0;
                if ((brackt && (stp <= stmin || stp >= stmax)) || infoc == 0) info = 6;
                if (stp == stpmax && fl <= ftest1 && dg <= dgtest) info = 5;
                if (stp == stpmin && (fl > ftest1 || dg >= dgtest)) info = 4;
                if (brackt && stmax - stmin <= xtol * stmax) info = 2;
                if (fl <= ftest1 && fabs(dg) <= gtol * (-dginit)) info = 1;
                if (info != 0) {
                    fnew = fl;
                    do_accept = true;
                    break;
                }
                if (stage1 && fl <= ftest1 && dg >= fmin(ftol, gtol) * dginit) stage1 = false;
                const bool modified = stage1 && fl <= fx && fl > ftest1;
                // cstep on the modified function psi (MINPACK) or on f itself
                double fxa = fx, fya = fy, dgxa = dgx, dgya = dgy, fpa = fl, dpa = dg;
                if (modified) {
                    fpa = fl - stp * dgtest;
                    fxa = fx - stx * dgtest;
                    fya = fy - sty * dgtest;
                    dpa = dg - dgtest;
                    dgxa = dgx - dgtest;
                    dgya = dgy - dgtest;
                }
                infoc = lb_cstep(stx, fxa, dgxa, sty, fya, dgya, stp, fpa, dpa, brackt, stmin, stmax);
                if (modified) {
                    fx = fxa + stx * dgtest;
                    fy = fya + sty * dgtest;
                    dgx = dgxa + dgtest;
                    dgy = dgya + dgtest;
                } else {
                    fx = fxa;
                    fy = fya;
                    dgx = dgxa;
                    dgy = dgya;
                }
                if (brackt) {
                    if (fabs(sty - stx) >= 0.66 * width1) stp = stx + 0.5 * (sty - stx);
                    width1 = width;
                    width = fabs(sty - stx);
                }
                if (++ls_iter == 100) {
                    xe = xo;  // argmin evaluates the last trial point once more
                    phase = LB_TAIL;
                } else {
                    do_trial = true;
                }
                break;
            }
            case LB_TAIL:
                evals++;
                fnew = fe;  // with the last trial's gradient
                do_accept = true;
                break;
            case LB_FINAL:
                evals++;
                end_cost = best_c;
                if (fe < best_c && isfinite(fe)) {
                    pj = xe;
                    end_cost = fe;
                }
                do_end = true;
                break;
            default: break;
        }
        if (do_accept) {  // the line search accepted (xo, fnew, go)
            const double sj = xo - x, yj = go - g;
            head = head == M - 1 ? 0 : head + 1;
            sh.S[head][lane] = sj;
            sh.Y[head][lane] = yj;
            sh.rho[head][lane] = lb_div(1.0, gdot(yj, sj, gm));
            cm = cm < M ? cm + 1 : M;
            x = xo;
            g = go;
            prev_f = f;
            f = fnew;
            if (f < best_f) { best_f = f; bx = x; }
            it++;
            if (converged() || it >= MAXIT) {
                xe = fmin(fmax(bx, lo_j), hi_j);
                phase = LB_FINAL;
            } else {
                do_begin = true;
            }
        }
        if (do_begin) {  // an L-BFGS iteration: two-loop direction, line search start
            double gamma = 1.0;
            if (cm > 0) {
                const double sn = sh.S[head][lane], yn = sh.Y[head][lane];
                gamma = lb_div(gdot(sn, yn, gm), gdot(yn, yn, gm));
            }
            double q = g;
            int s = head;
#pragma unroll 1
            for (int k = 0; k < cm; k++) {
                const double a = sh.rho[s][lane] * gdot(sh.S[s][lane], q, gm);
                sh.alpha[s][lane] = a;
                q -= sh.Y[s][lane] * a;
                s = s == 0 ? M - 1 : s - 1;
            }
            double r = q * gamma;
#pragma unroll 1
            for (int k = cm - 1; k >= 0; k--) {
                s = s == M - 1 ? 0 : s + 1;
                const double beta = gdot(sh.Y[s][lane], r, gm) * sh.rho[s][lane];
                r += sh.S[s][lane] * (sh.alpha[s][lane] - beta);
            }
            dv = -r;
            dginit = gdot(g, dv, gm);
            if (dginit >= 0.0) {  // not a descent direction: argmin stops with an error
                end_cost = best_c;
                do_end = true;
            } else {
                brackt = false;
                stage1 = true;
                infoc = 1;
                finit = f;
                dgtest = ftol * dginit;
                width = stpmax - stpmin;
                width1 = 2.0 * width;
                stx = 0.0; fx = finit; dgx = dginit;
                sty = 0.0; fy = finit; dgy = dginit;
                stp = 1.0;
                ls_iter = 0;
                phase = LB_LS;
                do_trial = true;
            }
        }
        if (do_trial) {  // the top of a line-search step: its trial point
            if (brackt) {
                stmin = fmin(stx, sty);
                stmax = fmax(stx, sty);
            } else {
                stmin = stx;
                stmax = stp + xtrapf * (stp - stx);
            }
            stp = fmax(stp, stpmin);
            stp = fmin(stp, stpmax);
            if ((brackt && (stp <= stmin || stp >= stmax)) || infoc == 0 || (brackt && stmax - stmin <= xtol * stmax))
                stp = stx;
            xo = x + stp * dv;
            xe = xo;
        }
        if (do_end) {
            st.c_pol++;
            st.c_it += (unsigned long long)it;
            st.c_ev += (unsigned long long)evals;
            st.c_obs += (unsigned long long)evals * (unsigned long long)st.n;
            st.c_fp64 += (unsigned long long)fp64_evals * (unsigned long long)st.n;
            finish(end_cost);
        }
    }
    // the work counters, summed over the warp's groups
    unsigned long long c_pol = st.c_pol, c_it = st.c_it, c_ev = st.c_ev, c_obs = st.c_obs, c_fp64 = st.c_fp64;
#pragma unroll
    for (int m = G; m < 32; m <<= 1) {
        c_pol += __shfl_xor_sync(FULL, c_pol, m);
        c_it += __shfl_xor_sync(FULL, c_it, m);
        c_ev += __shfl_xor_sync(FULL, c_ev, m);
        c_obs += __shfl_xor_sync(FULL, c_obs, m);
        c_fp64 += __shfl_xor_sync(FULL, c_fp64, m);
    }
    if (lane == 0 && c_pol) {
        atomicAdd(&d.ctr->lb_polishes, c_pol);
        atomicAdd(&d.ctr->lb_iters, c_it);
        atomicAdd(&d.ctr->lb_evals, c_ev);
        atomicAdd(&d.ctr->lb_obs_evals, c_obs);
        atomicAdd(&d.ctr->lb_obs_evals_by_model[MODEL], c_obs);
        if (c_fp64) atomicAdd(&d.ctr->lb_fp64_obs_evals_by_model[MODEL], c_fp64);
    }
}

}  // namespace lcf
