// polish.cu — restart reduction, bounded L-BFGS polish and BIC model
// selection (pso_fit_single_model / pso_model_select, src/parametric.rs:
// 1864-2066), and the SVI uncertainty kernel (svi_fit, :2215-2454).
//
// L-BFGS: one warp per (band, model).  Cost and gradient are accumulated by
// the lanes over the band's observations in FP32 (Kahan for the cost) and
// reduced across the warp; the quasi-Newton algebra (two-loop recursion,
// memory 7) and the Moré–Thuente line search run in FP64, identically in
// every lane, following the argmin 0.11 algorithm the reference calls
// (restated from the published method, as in the test oracle).
//
// SVI: one warp per band.  Per step the four reparameterised samples
// theta = mu + sigma * eps are evaluated with the lanes over observations;
// the adjoint of the log-likelihood with respect to each prediction is
// propagated through the model's analytic gradient and reduced across the
// warp.  The noise eps is regenerated from the reference's SmallRng(42)
// stream (a table indexed by step, sample and parameter) instead of being
// stored.  Adam runs in FP64 with one variational parameter per lane.
#include <cuda_runtime.h>

#include "grads_f32.cuh"
#include "lbfgs_lane.cuh"
#include "lcf_internal.cuh"
#include "models_f32.cuh"
#include "metzger_dual.cuh"
#include "models_f64.cuh"

namespace lcf {

#define FULL 0xffffffffu

__device__ __forceinline__ double warp_sum_d(double v) {
    for (int k = 16; k; k >>= 1) v += __shfl_xor_sync(FULL, v, k);
    return v;
}
__device__ __forceinline__ float warp_sum_f(float v) {
    for (int k = 16; k; k >>= 1) v += __shfl_xor_sync(FULL, v, k);
    return v;
}
__device__ __forceinline__ int warp_or(int v) { return __any_sync(FULL, v) ? 1 : 0; }

// Warp-wide negative log-likelihood of a parameter vector (cost of PsoCost
// without the Villar constraint and prior): lanes over observations.
__device__ double warp_nll(int m, const double* pd, const float4* obs, int n, double nd, double prior) {
    float se = (float)exp(pd[se_idx_of(m)]);
    float se2 = se * se;
    Nll acc;
    acc.reset();
    int lane = threadIdx.x & 31;
    for (int i = lane; i < n; i += 32) {
        float4 o = obs[i];
        int st = ST_OK;
        float pr;
        switch (m) {
            case BAZIN: { BazinF e; e.init64(pd); pr = e.eval(o.x, o.y, st); break; }
            case VILLAR: { VillarF e; e.init64(pd); pr = e.eval(o.x, o.y, st); break; }
            case TDE: { TdeF e; e.init64(pd); pr = e.eval(o.x, o.y, st); break; }
            case ARNETT: { ArnettF e; e.init64(pd); pr = e.eval(o.x, o.y, st); break; }
            case MAGNETAR: { MagnetarF e; e.init64(pd); pr = e.eval(o.x, o.y, st); break; }
            case SHOCK: { ShockF e; e.init64(pd); pr = e.eval(o.x, o.y, st); break; }
            default: { AfterglowF e; e.init64(pd); pr = e.eval(o.x, o.y, st); break; }
        }
        acc.obs(o, pr, st, se2);
    }
    // combine the lanes
    double s = warp_sum_d((double)acc.s - (double)acc.c);
    int nf = warp_or(acc.nonfinite), inf = warp_or(acc.inf);
    float big = acc.big;
    for (int k = 16; k; k >>= 1) {
        float o = __shfl_xor_sync(FULL, big, k);
        float mx = fmaxf(big, o);
        big = (mx == -INFINITY) ? -INFINITY : mx + log1pf(expf(-fabsf(big - o)));
    }
    if (nf) return BIG_COST;
    if (inf) return INFINITY;
    if (big > -INFINITY) {
        if (big > LN_DBL_MAX) return INFINITY;
        s += exp((double)big);
    }
    return (s + prior / nd) / nd;
}

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
    int n;
    double nd;
    double lo_j, hi_j;
    int evals, iters;

    __device__ void cost_grad(double xj, double& fo, double& gj, bool want_grad) {
        evals++;
        const int lane = threadIdx.x & 31, j = lane & 7;
        const double qj = fmin(fmax(xj, lo_j), hi_j);
        double q[MAXP];
#pragma unroll
        for (int k = 0; k < MAXP; k++) q[k] = k < np ? __shfl_sync(FULL, qj, k) : 0.0;
        constexpr int se = se_idx_of(MODEL);
        const double se2 = exp(2.0 * q[se]);
        bool constrained = false;
        double f = 0.0;
        if (MODEL == VILLAR) {
            double beta = q[1], gamma = exp(q[2]), tr = exp(q[4]), tf = exp(q[5]);
            double c1 = fmax(gamma * beta - 1.0, 0.0);
            double c2 = fmax(exp(-gamma / tr) * (tf / tr - 1.0) - 1.0, 0.0);
            double c3 = fmax(beta * tf - 1.0 + beta * gamma, 0.0);
            double cc = c1 + c2 + c3;
            if (cc > 0.0) { f = 1e12 + 10000.0 * cc; constrained = true; }
        }
        double nll = 0.0, gl[MAXP];
#pragma unroll
        for (int k = 0; k < MAXP; k++) gl[k] = 0.0;
        int nonfinite = 0;
        Model64 mod;
        mod.init(MODEL, q);
        for (int i = lane; i < n; i += 32) {
            double mg[MAXP];
            double pr = mod.eval(t[i], want_grad ? mg : nullptr);
            if (!isfinite(pr)) { nonfinite = 1; continue; }
            double tv = var[i] + se2;
            if (up[i]) {
                double sv = sqrt(tv);
                double z = (uf[i] - pr) / sv;
                nll -= log_normal_cdf_f64(z);
                if (want_grad) {
                    double phi = exp(-0.5 * z * z) / sqrt(2.0 * 3.14159265358979323846);
                    double cdf = 0.5 * (1.0 + erf_approx_f64(z / 1.41421356237309504880));
                    double ratio = phi / fmax(cdf, 1e-300);
#pragma unroll
                    for (int k = 0; k < np; k++) gl[k] += ratio * mg[k] / sv;
                    gl[se] += ratio * z * se2 / tv;
                }
            } else {
                double dd = pr - flux[i];
                nll += dd * dd / tv + log(tv);
                if (want_grad) {
                    double sc = 2.0 * dd / tv;
#pragma unroll
                    for (int k = 0; k < np; k++) gl[k] += sc * mg[k];
                    gl[se] += (-dd * dd / (tv * tv) + 1.0 / tv) * (2.0 * se2);
                }
            }
        }
        nonfinite = warp_or(nonfinite);
        if (!constrained) {
            if (nonfinite) f = BIG_COST;
            else {
                double prior = 0.0;
#pragma unroll
                for (int k = 0; k < np; k++) {
                    double w = c_pop_w[MODEL][k];
                    if (w > 0.0) {
                        double z = (q[k] - c_pop_c[MODEL][k]) / w;
                        prior += 0.5 * z * z;
                    }
                }
                f = (warp_sum_d(nll) + prior / nd) / nd;
            }
        }
        fo = f;
        if (!want_grad) return;
        double gs = 0.0;
#pragma unroll
        for (int k = 0; k < np; k++) {
            double gk = warp_sum_d(gl[k]);
            if (k == j) gs = gk;
        }
        gj = (nonfinite || j >= np) ? 0.0 : gs / nd;
        if ((xj <= lo_j && gj > 0.0) || (xj >= hi_j && gj < 0.0)) gj = 0.0;
    }
};

// Best of the three restarts of (band, MODEL), then the polish.
template <int MODEL>
__device__ void polish_band(const DeviceBatch& d, int b) {
    const BandStats bs = d.stats[b];
    if (!bs.valid) return;
    const PsoResult* R = d.pso_res + (size_t)(b * 8 + MODEL) * 3;
    if (R[0].iters < 0) return;  // this model was not fitted for this band
    double best_c = INFINITY;
    int best_r = -1;
    for (int r = 0; r < 3; r++)
        if (R[r].iters >= 0 && R[r].cost < best_c) { best_c = R[r].cost; best_r = r; }
    constexpr int np = n_params_of(MODEL);
    const int lane = threadIdx.x & 31, j = lane & 7;
    double pj = (best_r >= 0 && j < np) ? (double)R[best_r].params[j] : 0.0;
    double cost = best_c;
    if (MODEL != METZGER && best_r >= 0) {
        LaneLb<MODEL> c;
        c.t = d.t64 + bs.off;
        c.flux = d.f64 + bs.off;
        c.var = d.var64 + bs.off;
        c.uf = d.uf64 + bs.off;
        c.up = d.up + bs.off;
        c.n = bs.n;
        c.nd = (double)max(bs.n, 1);
        c.evals = 0;
        c.iters = 0;
        c.lo_j = j < np ? c_lo[MODEL][j] : 0.0;
        c.hi_j = j < np ? c_hi[MODEL][j] : 0.0;
        constexpr int t0i = t0_idx_of(MODEL);
        double t0_lo = fmax(bs.t_first - 30.0, c_lo[MODEL][t0i]);
        double t0_hi = fmin(bs.t_peak + 10.0, c_hi[MODEL][t0i]);
        if (j == t0i && t0_lo < t0_hi) { c.lo_j = t0_lo; c.hi_j = t0_hi; }
        cost = lane_lbfgs_polish(c, pj, best_c);
        if (lane == 0) {
            atomicAdd(&d.ctr->lb_polishes, 1ull);
            atomicAdd(&d.ctr->lb_iters, (unsigned long long)c.iters);
            atomicAdd(&d.ctr->lb_evals, (unsigned long long)c.evals);
            atomicAdd(&d.ctr->lb_obs_evals, (unsigned long long)c.evals * (unsigned long long)bs.n);
        }
    }
    ModelFit& F = d.fits[b * 8 + MODEL];
    if (lane == 0) F.cost = cost;
    if (lane < MAXP) F.params[lane] = lane < np ? pj : NAN;
}

// One warp per (band, model), model-major: consecutive warps (and so the
// warps resident on an SM) polish the same model, whose code then stays in
// the instruction cache.
__global__ void __launch_bounds__(128) lbfgs_kernel(DeviceBatch d, int model_mask) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (warp >= d.n_bands * 8) return;
    const int m = warp / d.n_bands, b = warp - m * d.n_bands;
    if (!((model_mask >> m) & 1)) return;
    switch (m) {
        case BAZIN: polish_band<BAZIN>(d, b); break;
        case VILLAR: polish_band<VILLAR>(d, b); break;
        case TDE: polish_band<TDE>(d, b); break;
        case ARNETT: polish_band<ARNETT>(d, b); break;
        case MAGNETAR: polish_band<MAGNETAR>(d, b); break;
        case SHOCK: polish_band<SHOCK>(d, b); break;
        case AFTERGLOW: polish_band<AFTERGLOW>(d, b); break;
        default: polish_band<METZGER>(d, b); break;
    }
}

void launch_lbfgs(const DeviceBatch& d, int model_mask, cudaStream_t s) {
    if (d.n_bands == 0) return;
    int block = 128;
    int64_t threads = (int64_t)d.n_bands * 8 * 32;
    lbfgs_kernel<<<(int)((threads + block - 1) / block), block, 0, s>>>(d, model_mask);
}

// ---------------------------------------------------------------------------
// BIC model selection (pso_model_select, src/parametric.rs:2016-2065), one
// thread per band.  mode 0: full selection over the fitted models;
// mode 1: Bazin gate of fit_all_models == false (cost < 2 -> stop).
// ---------------------------------------------------------------------------
__global__ void select_kernel(DeviceBatch d, int fit_all, int forced) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= d.n_bands) return;
    BandStats bs = d.stats[b];
    BandOut& o = d.out[b];
    o.model = -1;
    for (int m = 0; m < 8; m++) o.per_chi2[m] = NAN;
    if (!bs.valid) return;
    double nn = (double)max(bs.n, 1), ln_n = log(nn);
    int best = -1;
    double best_bic = INFINITY, best_cost = INFINITY;
    for (int k = 0; k < 8; k++) {
        int m = forced >= 0 ? (k == 0 ? forced : -1) : c_select_order[k];
        if (m < 0) break;
        const PsoResult* R = d.pso_res + (size_t)(b * 8 + m) * 3;
        if (R[0].iters < 0) continue;
        double c = d.fits[b * 8 + m].cost;
        o.per_chi2[m] = isfinite(c) ? c : NAN;
        double bic = 2.0 * c * nn + (double)n_params_of(m) * ln_n;
        if (best < 0) { best = m; best_bic = bic; best_cost = c; }
        else if (bic < best_bic) { best = m; best_bic = bic; best_cost = c; }
    }
    o.model = best;
    o.pso_cost = best_cost;
    for (int j = 0; j < MAXP; j++) o.pso_params[j] = best >= 0 ? d.fits[b * 8 + best].params[j] : NAN;
}

void launch_select(const DeviceBatch& d, int fit_all, int forced, cudaStream_t s) {
    if (d.n_bands == 0) return;
    select_kernel<<<(d.n_bands + 127) / 128, 128, 0, s>>>(d, fit_all, forced);
}

// ---------------------------------------------------------------------------
// SVI, one warp per band
// ---------------------------------------------------------------------------
__global__ void svi_kernel(DeviceBatch d) {
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (warp >= d.n_bands) return;
    const int b = warp;
    const BandStats bs = d.stats[b];
    BandOut& o = d.out[b];
    if (!bs.valid || o.model < 0) return;
    const int m = o.model, np = n_params_of(m), se = se_idx_of(m), n = bs.n;
    const float4* obs = d.obs + bs.off;
    double init[MAXP];
    for (int j = 0; j < np; j++) init[j] = o.pso_params[j];
    // lane i < 2 np owns variational parameter i (mu_j, then log sigma_j)
    double vp = 0.0, am = 0.0, av = 0.0;
    bool frozen = false;
    if (lane < np) vp = init[lane];
    else if (lane < 2 * np) vp = -1.0;
    const float* eps_tab = d.svi_eps + (size_t)(np - 5) * SVI_STEPS * SVI_SAMPLES * 7;
    double pc[MAXP], pw2[MAXP];
    for (int j = 0; j < np; j++) {
        pc[j] = j == se ? c_pri_c[m][j] : init[j];
        double w = c_pri_w[m][j];
        pw2[j] = w * w;
    }
    const double ln_2pie = 2.8378770664093453;  // ln(2 pi e)
    double b1t = 1.0, b2t = 1.0;
    double ema = -INFINITY, best_ema = -INFINITY, final_elbo = -INFINITY;
    int no_imp = 0, steps = 0;
    // MetzgerKN: per step, lanes 0..3 sweep samples 0..3 (value + 4 derivatives per observation)
    float* mscr = d.scratch_svi + 20 * bs.off;
    struct ObsTimes {
        const float4* o;
        __device__ float operator()(int j) const { return o[j].x + o[j].y; }
    } otimes{obs};
    for (int step = 0; step < SVI_STEPS; step++) {
        steps = step + 1;
        double mu[MAXP], sg[MAXP];
        for (int j = 0; j < np; j++) {
            mu[j] = __shfl_sync(FULL, vp, j);
            sg[j] = exp(__shfl_sync(FULL, vp, np + j));
        }
        double gmu[MAXP], gls[MAXP];
        for (int j = 0; j < np; j++) { gmu[j] = 0.0; gls[j] = 0.0; }
        double elbo_sum = 0.0;
        int huge_any = 0;
        if (m == METZGER) {
            if (lane < SVI_SAMPLES) {
                const float* ep = eps_tab + ((size_t)step * SVI_SAMPLES + lane) * 7;
                float pv[MAXP];
                for (int j = 0; j < np; j++) pv[j] = (float)(mu[j] + sg[j] * (double)ep[j]);
                metzger_dual_sweep(pv, (float)bs.t_last, otimes, n, mscr + (size_t)lane * 5 * n);
            }
            __syncwarp();
        }
        for (int k = 0; k < SVI_SAMPLES; k++) {
            const float* ep = eps_tab + ((size_t)step * SVI_SAMPLES + k) * 7;
            double th[MAXP], eps[MAXP];
            float pf[MAXP];
            for (int j = 0; j < np; j++) {
                eps[j] = (double)ep[j];
                th[j] = mu[j] + sg[j] * eps[j];
                pf[j] = (float)th[j];
            }
            float sx = expf(pf[se]);
            float sx2 = sx * sx;
            float dll[MAXP];
            for (int j = 0; j < MAXP; j++) dll[j] = 0.0f;
            Nll ll;
            ll.reset();
            int huge = 0;
            bool skip_sample = false;
            if (m == METZGER) {
                // predictions and derivatives of the normalised model, then the
                // reference's peak rescale (src/parametric.rs:2303-2323)
                const float* ms = mscr + (size_t)k * 5 * n;
                float mx = -INFINITY;
                for (int i = lane; i < n; i += 32)
                    if (obs[i].w >= 0.0f) mx = fmaxf(mx, ms[i * 5]);
                for (int kk = 16; kk; kk >>= 1) mx = fmaxf(mx, __shfl_xor_sync(FULL, mx, kk));
                float scl = 1.0f;
                if (mx > 1e-10f && isfinite(mx)) {
                    float raw = 1.0f / mx;
                    scl = fminf(fmaxf(raw, 0.1f), 10.0f);
                    if (fabsf(raw - scl) / raw > 0.5f) skip_sample = true;
                }
                if (!skip_sample) {
                    for (int i = lane; i < n; i += 32) {
                        float4 ob = obs[i];
                        float pr = ms[i * 5] * scl;
                        float gb[MAXP];
                        for (int j = 0; j < 4; j++) gb[j] = ms[i * 5 + 1 + j] * scl;
                        gb[4] = 0.0f;
                        float tv = fabsf(ob.w) + sx2;
                        float stv = sqrtf(tv);
                        if (ob.w < 0.0f) {
                            float z = (ob.z - pr) / stv;
                            ll.add(log_normal_cdf_f(z));
                            bool hg;
                            float ratio = upper_ratio_f32(z, hg);
                            if (hg) huge = 1;
                            for (int j = 0; j < 4; j++) if (isfinite(gb[j])) dll[j] += -ratio / stv * gb[j];
                            dll[se] += ratio * (-(ob.z - pr) * sx2 / (stv * tv));
                        } else {
                            float res = ob.z - pr;
                            float it = 1.0f / tv;
                            float r2 = res * res;
                            ll.add(-0.5f * (r2 * it + logf(6.283185307179586f * tv)));
                            for (int j = 0; j < 4; j++) if (isfinite(gb[j])) dll[j] += res * it * gb[j];
                            dll[se] += (r2 * it * it - it) * sx2;
                        }
                    }
                }
            } else {
                for (int i = lane; i < n; i += 32) {
                    float4 ob = obs[i];
                    float gb[MAXP];
                    int st;
                    float pr = model_grad_f32(m, pf, ob.x, ob.y, gb, st);
                    if (st == ST_NONFINITE || !isfinite(pr)) continue;
                    float tv = fabsf(ob.w) + sx2;
                    float stv = sqrtf(tv);
                    if (ob.w < 0.0f) {
                        float z = (ob.z - pr) / stv;
                        ll.add(log_normal_cdf_f(z));
                        bool hg;
                        float ratio = upper_ratio_f32(z, hg);
                        if (hg) huge = 1;
                        float dpred = -ratio / stv;
                        for (int j = 0; j < np; j++)
                            if (j != se && isfinite(gb[j])) dll[j] += dpred * gb[j];
                        dll[se] += ratio * (-(ob.z - pr) * sx2 / (stv * tv));
                    } else {
                        float res = ob.z - pr;
                        float it = 1.0f / tv;
                        float r2 = res * res;
                        ll.add(-0.5f * (r2 * it + logf(6.283185307179586f * tv)));
                        for (int j = 0; j < np; j++)
                            if (j != se && isfinite(gb[j])) dll[j] += res * it * gb[j];
                        dll[se] += (r2 * it * it - it) * sx2;
                    }
                }
            }
            if (__any_sync(FULL, skip_sample)) continue;
            if (warp_or(huge)) huge_any = 1;
            double lls = warp_sum_d((double)ll.s - (double)ll.c);
            double lp = 0.0;
            for (int j = 0; j < np; j++) {
                double dlj = (double)warp_sum_f(dll[j]);
                double dd = th[j] - pc[j];
                lp += -0.5 * dd * dd / pw2[j];
                double df = dlj + (-dd / pw2[j]);
                gmu[j] += df;
                gls[j] += df * sg[j] * eps[j];
            }
            elbo_sum += lls + lp;
        }
        const double ns = (double)SVI_SAMPLES;
        double ent = 0.0;
        for (int j = 0; j < np; j++) ent += __shfl_sync(FULL, vp, np + j);
        ent += 0.5 * (double)np * ln_2pie;
        final_elbo = elbo_sum / ns + ent;
        // Adam, lane i owns variational parameter i
        double gi = 0.0;
        for (int j = 0; j < np; j++) {
            if (lane == j) gi = -(gmu[j] / ns);
            if (lane == np + j) gi = -(gls[j] / ns + 1.0);
        }
        b1t *= 0.9;
        b2t *= 0.999;
        if (huge_any) frozen = true;  // the reference's v overflows to +inf: updates stop
        if (lane < 2 * np && isfinite(gi) && !frozen) {
            am = 0.9 * am + (1.0 - 0.9) * gi;
            av = 0.999 * av + (1.0 - 0.999) * gi * gi;
            double mh = am / (1.0 - b1t), vh = av / (1.0 - b2t);
            vp -= SVI_LR * mh / (sqrt(vh) + 1e-8);
        }
        if (lane >= np && lane < 2 * np) vp = fmin(fmax(vp, -6.0), 2.0);
        if (step >= 200) {
            if (ema == -INFINITY) ema = final_elbo;
            else ema = 0.1 * final_elbo + 0.9 * ema;
            bool imp = ema - best_ema > 0.01 * fmax(fabs(best_ema), 1e-10);
            if (imp) { best_ema = ema; no_imp = 0; }
            else if (++no_imp >= 50) break;
        }
    }
    const double ln4 = 1.3862943611198906;
    double out_v = lane < np ? vp : vp + ln4;
    if (lane < np) o.mu[lane] = out_v;
    else if (lane < 2 * np) o.log_sigma[lane - np] = out_v;
    if (lane >= np && lane < MAXP) o.mu[lane] = NAN;
    if (lane == 0) {
        for (int j = np; j < MAXP; j++) o.log_sigma[j] = NAN;
        o.elbo = final_elbo;
        o.svi_steps = steps;
    }
}

void launch_svi(const DeviceBatch& d, cudaStream_t s) {
    if (d.n_bands == 0) return;
    int block = 128;
    int64_t threads = (int64_t)d.n_bands * 32;
    svi_kernel<<<(int)((threads + block - 1) / block), block, 0, s>>>(d);
}

}  // namespace lcf
