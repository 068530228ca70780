// plain.cu — the plain FP64 GPU form of the fit: the straightforward CUDA
// rendering of fit_parametric's model selection and SVI
// (src/parametric.rs:1646-1757, 1864-2066, 2215-2454) that the fused kernels
// are measured against.  It computes the same quantities with none of the
// fused design:
//   * FP64 everywhere, the model formulas written out per observation
//     (eval_model_f64 / model_grad_f64, nothing hoisted per parameter vector);
//   * observations read from global memory (no shared-memory staging);
//   * PSO: one block per swarm (band, restart), one thread per particle,
//     synchronous global best (the particles of an iteration all move with
//     the previous iteration's best, as the reference's own GPU loop does,
//     src/gpu_cuda.rs:368-567);
//   * one launch per model per stage (PSO, L-BFGS, SVI), no CUDA graph, no
//     task queue;
//   * L-BFGS and SVI: one warp per band, lanes over observations, with the
//     reference's analytic per-observation gradients (MetzgerKN: forward
//     differences with step 1e-5, as metzger_kn_grad_batch_into :843-860).
// It covers PSO model selection (8 models x 3 restarts), the L-BFGS polish,
// BIC selection and SVI; the profile t0 search, the refinements, the
// magnitude chi2 and MultiBazin are not part of it.
#include <cuda_runtime.h>

#include "lbfgs.cuh"
#include "lcf_internal.cuh"
#include "models_f32.cuh"
#include "models_f64.cuh"

namespace lcf {

#define FULL 0xffffffffu

namespace {

__device__ __forceinline__ double warp_sum(double v) {
    for (int k = 16; k; k >>= 1) v += __shfl_xor_sync(FULL, v, k);
    return v;
}

struct BandView {
    const double *t, *f, *var, *uf;
    const uint8_t* up;
    int n;
};

__device__ __forceinline__ BandView band_view(const DeviceBatch& d, const BandStats& bs) {
    BandView v;
    v.t = d.t64 + bs.off;
    v.f = d.f64 + bs.off;
    v.var = d.var64 + bs.off;
    v.uf = d.uf64 + bs.off;
    v.up = d.up + bs.off;
    v.n = bs.n;
    return v;
}

__device__ __forceinline__ double villar_constraint(const double* p) {
    double beta = p[1], gamma = exp(p[2]), tr = exp(p[4]), tf = exp(p[5]);
    double c1 = fmax(gamma * beta - 1.0, 0.0);
    double c2 = fmax(exp(-gamma / tr) * (tf / tr - 1.0) - 1.0, 0.0);
    double c3 = fmax(beta * tf - 1.0 + beta * gamma, 0.0);
    return c1 + c2 + c3;
}

// MetzgerKN predictions of one parameter vector into pred[0..n), with the
// reference's peak rescale of the PSO cost (src/parametric.rs:1317-1330).
__device__ void metzger_pred_rescaled(const double* p, const BandView& b, double* pred) {
    metzger_f64(p, b.t, b.n, pred);
    double mx = -INFINITY;
    for (int i = 0; i < b.n; i++)
        if (!b.up[i]) mx = fmax(mx, pred[i]);
    if (mx > 1e-10 && isfinite(mx)) {
        double s = fmin(fmax(1.0 / mx, 0.1), 10.0);
        for (int i = 0; i < b.n; i++) pred[i] *= s;
    }
}

// PsoCost::cost_from_slice (src/parametric.rs:1303-1370) by one thread.
__device__ double thread_cost(int m, const double* p, const BandView& b, bool prior, double* mscr) {
    if (m == VILLAR) {
        double c = villar_constraint(p);
        if (c > 0.0) return 1e12 + 10000.0 * c;
    }
    if (m == METZGER) metzger_pred_rescaled(p, b, mscr);
    double se = exp(p[se_idx_of(m)]);
    double se2 = se * se;
    double nn = (double)max(b.n, 1);
    double nll = 0.0;
    for (int i = 0; i < b.n; i++) {
        double pr = m == METZGER ? mscr[i] : eval_model_f64(m, p, b.t[i]);
        if (!isfinite(pr)) return BIG_COST;
        double tv = b.var[i] + se2;
        if (b.up[i]) {
            nll -= log_normal_cdf_f64((b.uf[i] - pr) / sqrt(tv));
        } else {
            double dd = pr - b.f[i];
            nll += dd * dd / tv + log(tv);
        }
    }
    if (prior) {
        double nlp = 0.0;
        for (int j = 0; j < n_params_of(m); j++) {
            double w = c_pop_w[m][j];
            if (w > 0.0) {
                double z = (p[j] - c_pop_c[m][j]) / w;
                nlp += 0.5 * z * z;
            }
        }
        nll += nlp / nn;
    }
    return nll / nn;
}

// Box of pso_fit_single_model with its data-informed t0 bounds
// (src/parametric.rs:1881-1909).
__device__ void model_box(int m, const BandStats& bs, double* lo, double* hi) {
    for (int j = 0; j < MAXP; j++) { lo[j] = c_lo[m][j]; hi[j] = c_hi[m][j]; }
    int t0i = t0_idx_of(m);
    double t0_lo = fmax(bs.t_first - 30.0, lo[t0i]);
    double t0_hi = fmin(bs.t_peak + 10.0, hi[t0i]);
    if (t0_lo < t0_hi) { lo[t0i] = t0_lo; hi[t0i] = t0_hi; }
}

}  // namespace

// ---------------------------------------------------------------------------
// PSO: block = one swarm (band, restart), thread = particle.  Random numbers:
// the reference's SmallRng streams of seeds 42 / 137 / 271, at the positions
// the sequential loop would draw them for (iteration, particle, dimension).
// gate: skip bands whose polished Bazin cost is below 2 (BAZIN_GOOD_ENOUGH,
// src/parametric.rs:1862) — the fit_all_models = false path.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(32) plain_pso_kernel(DeviceBatch d, int m, int gate, double* mscr_base) {
    const int b = blockIdx.x / 3, r = blockIdx.x % 3, p = threadIdx.x;
    const BandStats bs = d.stats[b];
    if (!bs.valid) return;
    if (gate && !(d.fits[b * 8 + BAZIN].cost >= 2.0)) return;  // left "not fitted" (iters = -1)
    const BandView bv = band_view(d, bs);
    const bool live = p < NP;
    double* mscr = mscr_base + (size_t)bs.off * 96 + (size_t)(r * 32 + p) * bs.n;
    const int D = n_params_of(m), t0i = t0_idx_of(m);
    double lo[MAXP], hi[MAXP], vmax[MAXP];
    model_box(m, bs, lo, hi);
    for (int j = 0; j < D; j++) vmax[j] = 0.5 * (hi[j] - lo[j]);
    const float* dr = d.draws + (size_t)r * DRAWS_PER_SEED;
    const bool seeded = r > 0;
    double x[MAXP], v[MAXP], pb[MAXP];
    for (int j = 0; j < MAXP; j++) { x[j] = 0.0; v[j] = 0.0; }
    int base;
    if (seeded) {
        if (p == 0) {
            // seed particle of pso_fit_single_model, src/parametric.rs:1924-1964
            for (int j = 0; j < D; j++) {
                x[j] = fmin(fmax(c_pop_c[m][j], lo[j]), hi[j]);
                v[j] = vmax[j] * 0.2 * (2.0 * (double)dr[j] - 1.0);
            }
            double t0s = r == 1 ? bs.t_peak - 5.0 : bs.t_first - 15.0;
            x[t0i] = fmin(fmax(t0s, lo[t0i]), hi[t0i]);
        } else if (live) {
            int o = D + 2 * D * (p - 1);
            for (int j = 0; j < D; j++) {
                x[j] = lo[j] + (double)dr[o + j] * (hi[j] - lo[j]);
                v[j] = vmax[j] * 0.2 * (2.0 * (double)dr[o + D + j] - 1.0);
            }
        }
        base = 2 * D * NP - D;
    } else {
        if (live) {
            int o = 2 * D * p;
            for (int j = 0; j < D; j++) {
                x[j] = lo[j] + (double)dr[o + 2 * j] * (hi[j] - lo[j]);
                v[j] = vmax[j] * 0.2 * (2.0 * (double)dr[o + 2 * j + 1] - 1.0);
            }
        }
        base = 2 * D * NP;
    }
    for (int j = 0; j < MAXP; j++) pb[j] = x[j];
    double c = live ? thread_cost(m, x, bv, true, mscr) : INFINITY;
    double pbc = c;
    __shared__ double s_cost[32];
    __shared__ double s_g[MAXP];
    __shared__ double s_gc;
    __shared__ int s_q;
    s_cost[p] = c;
    __syncthreads();
    if (p == 0) {
        double gc = INFINITY;
        int q = -1;
        for (int k = 0; k < NP; k++)
            if (s_cost[k] < gc) { gc = s_cost[k]; q = k; }
        s_gc = gc;
        s_q = q;
    }
    __syncthreads();
    {
        int q = s_q;
        if (p == q)
            for (int j = 0; j < MAXP; j++) s_g[j] = x[j];
        if (q < 0 && p == 0)
            for (int j = 0; j < MAXP; j++) s_g[j] = 0.0;
    }
    __syncthreads();
    int stall = 0, it = 0, evals = live ? 1 : 0;
    double prev = s_gc;
    for (; it < MAX_ITERS; it++) {
        const double w = 0.9 - (0.9 - 0.4) * (double)it / (double)MAX_ITERS;
        if (live) {
            const float* rr = dr + base + it * 2 * D * NP + 2 * D * p;
            for (int j = 0; j < D; j++) {
                double r1 = (double)rr[2 * j], r2 = (double)rr[2 * j + 1];
                double vv = w * v[j] + 1.5 * r1 * (pb[j] - x[j]) + 1.5 * r2 * (s_g[j] - x[j]);
                vv = fmin(fmax(vv, -vmax[j]), vmax[j]);
                double nx = x[j] + vv;
                if (nx <= lo[j]) { x[j] = lo[j]; v[j] = 0.0; }
                else if (nx >= hi[j]) { x[j] = hi[j]; v[j] = 0.0; }
                else { x[j] = nx; v[j] = vv; }
            }
            c = thread_cost(m, x, bv, true, mscr);
            evals++;
            if (c < pbc) {
                pbc = c;
                for (int j = 0; j < D; j++) pb[j] = x[j];
            }
        }
        __syncthreads();  // every thread has read s_g
        s_cost[p] = live ? c : INFINITY;
        __syncthreads();
        if (p == 0) {
            double gc = s_gc;
            int q = -1;
            for (int k = 0; k < NP; k++)
                if (s_cost[k] < gc) { gc = s_cost[k]; q = k; }
            s_gc = gc;
            s_q = q;
        }
        __syncthreads();
        int q = s_q;
        if (p == q)
            for (int j = 0; j < D; j++) s_g[j] = x[j];
        __syncthreads();
        double gc = s_gc;
        if (prev - gc > 0.01 * fmax(fabs(prev), 1e-10)) {
            stall = 0;
            prev = gc;
        } else if (++stall >= STALL_ITERS) {
            it++;
            break;
        }
    }
    int tot = evals;
    for (int k = 16; k; k >>= 1) tot += __shfl_xor_sync(FULL, tot, k);
    if (p == 0) {
        PsoResult& R = d.pso_res[(size_t)(b * 8 + m) * 3 + r];
        R.cost = s_gc;
        R.iters = it;
        R.evals = tot;
        for (int j = 0; j < MB_MAXP; j++) R.params[j] = j < D ? (float)s_g[j] : 0.0f;
        atomicAdd(&d.ctr->particle_obs_evals, (unsigned long long)tot * (unsigned long long)bs.n);
    }
}

// ---------------------------------------------------------------------------
// L-BFGS: one warp per band, lanes over observations, FP64 per-observation
// formulas (eval_model_f64 / model_grad_f64).
// ---------------------------------------------------------------------------
struct PlainLb {
    BandView b;
    int m, np;
    double nd;
    double lo[MAXP], hi[MAXP];
    int evals, iters;

    // BoundedPsoCost (src/parametric.rs:1500-1535): cost with prior and the
    // Villar constraint, gradient without either, projected at the box.
    __device__ void cost_grad(const double* x, double& f, double* g, bool want_grad) {
        evals++;
        double q[MAXP];
        for (int j = 0; j < MAXP; j++) q[j] = j < np ? fmin(fmax(x[j], lo[j]), hi[j]) : 0.0;
        const int lane = threadIdx.x & 31, se = se_idx_of(m);
        const double sx = exp(q[se]), se2 = sx * sx;
        bool constrained = false;
        if (m == VILLAR) {
            double cc = villar_constraint(q);
            if (cc > 0.0) { f = 1e12 + 10000.0 * cc; constrained = true; }
        }
        double nll = 0.0, gl[MAXP];
        for (int j = 0; j < MAXP; j++) gl[j] = 0.0;
        int nonfinite = 0;
        for (int i = lane; i < b.n; i += 32) {
            double pr = eval_model_f64(m, q, b.t[i]);
            if (!isfinite(pr)) { nonfinite = 1; continue; }
            double mg[MAXP];
            if (want_grad) model_grad_f64(m, q, b.t[i], mg);
            double tv = b.var[i] + se2;
            if (b.up[i]) {
                double sv = sqrt(tv);
                double z = (b.uf[i] - pr) / sv;
                nll -= log_normal_cdf_f64(z);
                if (want_grad) {
                    double phi = exp(-0.5 * z * z) / sqrt(2.0 * 3.14159265358979323846);
                    double cdf = 0.5 * (1.0 + erf_approx_f64(z / 1.41421356237309504880));
                    double ratio = phi / fmax(cdf, 1e-300);
                    for (int j = 0; j < np; j++) gl[j] += ratio * mg[j] / sv;
                    gl[se] += ratio * z * se2 / tv;
                }
            } else {
                double dd = pr - b.f[i];
                nll += dd * dd / tv + log(tv);
                if (want_grad) {
                    double sc = 2.0 * dd / tv;
                    for (int j = 0; j < np; j++) gl[j] += sc * mg[j];
                    gl[se] += (-dd * dd / (tv * tv) + 1.0 / tv) * (2.0 * se2);
                }
            }
        }
        nonfinite = __any_sync(FULL, nonfinite) ? 1 : 0;
        double nsum = warp_sum(nll);
        if (!constrained) {
            if (nonfinite) f = BIG_COST;
            else {
                double prior = 0.0;
                for (int j = 0; j < np; j++) {
                    double w = c_pop_w[m][j];
                    if (w > 0.0) {
                        double z = (q[j] - c_pop_c[m][j]) / w;
                        prior += 0.5 * z * z;
                    }
                }
                f = (nsum + prior / nd) / nd;
            }
        }
        if (!want_grad) return;
        for (int j = 0; j < np; j++) {
            double gj = warp_sum(gl[j]);
            g[j] = nonfinite ? 0.0 : gj / nd;
        }
        for (int j = 0; j < np; j++)
            if ((x[j] <= lo[j] && g[j] > 0.0) || (x[j] >= hi[j] && g[j] < 0.0)) g[j] = 0.0;
    }
};

__global__ void plain_lbfgs_kernel(DeviceBatch d, int m) {
    const int b = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (b >= d.n_bands) return;
    const BandStats bs = d.stats[b];
    if (!bs.valid) return;
    const PsoResult* R = d.pso_res + (size_t)(b * 8 + m) * 3;
    if (R[0].iters < 0) return;
    double best_c = INFINITY;
    int best_r = -1;
    for (int r = 0; r < 3; r++)
        if (R[r].iters >= 0 && R[r].cost < best_c) { best_c = R[r].cost; best_r = r; }
    const int np = n_params_of(m);
    double params[MAXP];
    for (int j = 0; j < MAXP; j++) params[j] = (best_r >= 0 && j < np) ? (double)R[best_r].params[j] : 0.0;
    double cost = best_c;
    if (m != METZGER && best_r >= 0) {
        PlainLb c;
        c.b = band_view(d, bs);
        c.m = m;
        c.np = np;
        c.nd = (double)max(bs.n, 1);
        c.evals = 0;
        c.iters = 0;
        model_box(m, bs, c.lo, c.hi);
        cost = lbfgs_polish(c, params, best_c);
        if ((threadIdx.x & 31) == 0) {
            atomicAdd(&d.ctr->lb_polishes, 1ull);
            atomicAdd(&d.ctr->lb_iters, (unsigned long long)c.iters);
            atomicAdd(&d.ctr->lb_evals, (unsigned long long)c.evals);
            atomicAdd(&d.ctr->lb_obs_evals, (unsigned long long)c.evals * (unsigned long long)bs.n);
        }
    }
    if ((threadIdx.x & 31) == 0) {
        ModelFit& F = d.fits[b * 8 + m];
        F.cost = cost;
        for (int j = 0; j < MAXP; j++) F.params[j] = j < np ? params[j] : NAN;
    }
}

// ---------------------------------------------------------------------------
// SVI (svi_fit, src/parametric.rs:2215-2454): one warp per band whose
// selected model is m; lanes over observations; FP64 with the reference's
// analytic gradient; Adam with one lane per variational parameter.
// MetzgerKN: lanes 0..19 run the 4 samples x (value + 4 forward-difference
// sweeps) into the band's scratch rows.
// ---------------------------------------------------------------------------
__global__ void plain_svi_kernel(DeviceBatch d, int m, double* mscr_base) {
    const int lane = threadIdx.x & 31;
    const int b = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (b >= d.n_bands) return;
    const BandStats bs = d.stats[b];
    BandOut& o = d.out[b];
    if (!bs.valid || o.model != m) return;
    const BandView bv = band_view(d, bs);
    const int np = n_params_of(m), se = se_idx_of(m), n = bs.n;
    double* mscr = mscr_base + (size_t)bs.off * 96;
    double init[MAXP];
    for (int j = 0; j < np; j++) init[j] = o.pso_params[j];
    double vp = 0.0, am = 0.0, av = 0.0;
    if (lane < np) vp = init[lane];
    else if (lane < 2 * np) vp = -1.0;
    const double* eps_tab = d.svi_eps + (size_t)(np - 5) * SVI_STEPS * SVI_SAMPLES * 7;
    double pc[MAXP], pw2[MAXP];
    for (int j = 0; j < np; j++) {
        pc[j] = j == se ? c_pri_c[m][j] : init[j];
        double w = c_pri_w[m][j];
        pw2[j] = w * w;
    }
    const double PI = 3.14159265358979323846;
    double ema = -INFINITY, best_ema = -INFINITY, final_elbo = -INFINITY;
    int no_imp = 0, steps = 0, at = 0;
    for (int step = 0; step < SVI_STEPS; step++) {
        steps = step + 1;
        double mu[MAXP], sg[MAXP];
        for (int j = 0; j < np; j++) {
            mu[j] = __shfl_sync(FULL, vp, j);
            sg[j] = exp(__shfl_sync(FULL, vp, np + j));
        }
        if (m == METZGER) {
            if (lane < SVI_SAMPLES * 5) {
                int k = lane / 5, q = lane % 5;
                const double* ep = eps_tab + ((size_t)step * SVI_SAMPLES + k) * 7;
                double th[MAXP];
                for (int j = 0; j < np; j++) th[j] = mu[j] + sg[j] * ep[j];
                if (q > 0) th[q - 1] += 1e-5;
                metzger_f64(th, bv.t, n, mscr + (size_t)lane * n);
            }
            __syncwarp();
        }
        double gmu[MAXP], gls[MAXP];
        for (int j = 0; j < np; j++) { gmu[j] = 0.0; gls[j] = 0.0; }
        double elbo_sum = 0.0;
        for (int k = 0; k < SVI_SAMPLES; k++) {
            const double* ep = eps_tab + ((size_t)step * SVI_SAMPLES + k) * 7;
            double th[MAXP], eps[MAXP];
            for (int j = 0; j < np; j++) {
                eps[j] = ep[j];
                th[j] = mu[j] + sg[j] * eps[j];
            }
            double sx = exp(th[se]), sx2 = sx * sx;
            double scl = 1.0;
            bool skip = false;
            const double* mk = mscr + (size_t)k * 5 * n;
            if (m == METZGER) {
                double mx = -INFINITY;
                for (int i = lane; i < n; i += 32)
                    if (!bv.up[i]) mx = fmax(mx, mk[i]);
                for (int kk = 16; kk; kk >>= 1) mx = fmax(mx, __shfl_xor_sync(FULL, mx, kk));
                if (mx > 1e-10 && isfinite(mx)) {
                    double raw = 1.0 / mx;
                    scl = fmin(fmax(raw, 0.1), 10.0);
                    if (fabs(raw - scl) / raw > 0.5) skip = true;
                }
            }
            if (skip) continue;
            double ll = 0.0, dll[MAXP];
            for (int j = 0; j < MAXP; j++) dll[j] = 0.0;
            for (int i = lane; i < n; i += 32) {
                double pr, gb[MAXP];
                if (m == METZGER) {
                    pr = mk[i] * scl;
                    for (int j = 0; j < 4; j++) gb[j] = (mk[(size_t)(j + 1) * n + i] - mk[i]) / 1e-5 * scl;
                    gb[4] = 0.0;
                } else {
                    pr = eval_model_f64(m, th, bv.t[i]);
                }
                if (!isfinite(pr)) continue;
                if (m != METZGER) model_grad_f64(m, th, bv.t[i], gb);
                double tv = bv.var[i] + sx2, st = sqrt(tv);
                if (bv.up[i]) {
                    double z = (bv.uf[i] - pr) / st;
                    ll += log_normal_cdf_f64(z);
                    double phi = exp(-0.5 * z * z) / sqrt(2.0 * PI);
                    double cdf = fmax(0.5 * (1.0 + erf_approx_f64(z * 0.70710678118654752440)), 1e-300);
                    double dpred = -phi / (cdf * st);
                    for (int j = 0; j < np; j++)
                        if (j != se && isfinite(gb[j])) dll[j] += dpred * gb[j];
                    dll[se] += (phi / cdf) * (-(bv.uf[i] - pr) * sx2 / (st * tv));
                } else {
                    double res = bv.f[i] - pr, it = 1.0 / tv, r2 = res * res;
                    ll += -0.5 * (r2 * it + log(2.0 * PI * tv));
                    for (int j = 0; j < np; j++)
                        if (j != se && isfinite(gb[j])) dll[j] += res * it * gb[j];
                    dll[se] += (r2 * it * it - it) * sx2;
                }
            }
            double lls = warp_sum(ll), lp = 0.0;
            for (int j = 0; j < np; j++) {
                double dlj = warp_sum(dll[j]);
                double dd = th[j] - pc[j];
                lp += -0.5 * dd * dd / pw2[j];
                double df = dlj - dd / pw2[j];
                gmu[j] += df;
                gls[j] += df * sg[j] * eps[j];
            }
            elbo_sum += lls + lp;
        }
        const double ns = (double)SVI_SAMPLES;
        double ent = 0.0;
        for (int j = 0; j < np; j++) ent += __shfl_sync(FULL, vp, np + j);
        ent += 0.5 * (double)np * log(2.0 * PI * 2.71828182845904523536);
        final_elbo = elbo_sum / ns + ent;
        double gi = 0.0;
        for (int j = 0; j < np; j++) {
            if (lane == j) gi = -(gmu[j] / ns);
            if (lane == np + j) gi = -(gls[j] / ns + 1.0);
        }
        at++;
        double bc1 = 1.0 - pow(0.9, (double)at), bc2 = 1.0 - pow(0.999, (double)at);
        if (lane < 2 * np && isfinite(gi)) {
            am = 0.9 * am + 0.1 * gi;
            av = 0.999 * av + 0.001 * gi * gi;
            vp -= SVI_LR * (am / bc1) / (sqrt(av / bc2) + 1e-8);
        }
        if (lane >= np && lane < 2 * np) vp = fmin(fmax(vp, -6.0), 2.0);
        if (step >= 200) {
            if (ema == -INFINITY) ema = final_elbo;
            else ema = 0.1 * final_elbo + 0.9 * ema;
            if (ema - best_ema > 0.01 * fmax(fabs(best_ema), 1e-10)) { best_ema = ema; no_imp = 0; }
            else if (++no_imp >= 50) break;
        }
        __syncwarp();  // MetzgerKN scratch rows are rewritten next step
    }
    const double ln4 = 1.3862943611198906;
    if (lane < np) o.mu[lane] = vp;
    else if (lane < 2 * np) o.log_sigma[lane - np] = vp + ln4;
    if (lane >= np && lane < MAXP) o.mu[lane] = NAN;
    if (lane == 0) {
        for (int j = np; j < MAXP; j++) o.log_sigma[j] = NAN;
        o.elbo = final_elbo;
        o.svi_steps = steps;
        o.mag_chi2 = NAN;
    }
}

void launch_plain_pso(const DeviceBatch& d, int m, int gate, double* mscr, cudaStream_t s) {
    if (d.n_bands == 0) return;
    plain_pso_kernel<<<d.n_bands * 3, 32, 0, s>>>(d, m, gate, mscr);
}

void launch_plain_lbfgs(const DeviceBatch& d, int m, cudaStream_t s) {
    if (d.n_bands == 0) return;
    int64_t threads = (int64_t)d.n_bands * 32;
    plain_lbfgs_kernel<<<(int)((threads + 127) / 128), 128, 0, s>>>(d, m);
}

void launch_plain_svi(const DeviceBatch& d, int m, double* mscr, cudaStream_t s) {
    if (d.n_bands == 0) return;
    int64_t threads = (int64_t)d.n_bands * 32;
    plain_svi_kernel<<<(int)((threads + 127) / 128), 128, 0, s>>>(d, m, mscr);
}

}  // namespace lcf
