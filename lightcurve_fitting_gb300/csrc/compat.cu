// compat.cu — the reference's CUDA FFI, with the names and signatures its Rust
// host binds (src/gpu_cuda.rs:17-164) and the semantics of the kernels behind
// them (cuda/models.cu, cuda/svi.cu), so that an unmodified `GpuContext`
// links against liblcf_gb300.so.  FP64 throughout, device pointers, the
// legacy default stream, void return (errors surface through
// cudaGetLastError, as in the reference).  `grid` and `block` are accepted
// and ignored: the launch shapes are this library's.
//
//   launch_{bazin,...,metzger_kn}      model evaluation at draws x times
//   launch_batch_pso_cost             swarm cost of (source, particle) rows
//   launch_batch_pso_cost_multi_bazin the same for MultiBazin, K per source
//   launch_batch_svi_fit              the reference GPU's SVI, one source each
//
// The reference runs one thread per (source, particle) row, or one warp per
// source with lane 0 doing the bookkeeping; here a warp takes each row or
// source, its lanes split the observations, and the FP64 sums are reduced
// across the warp (the same terms, summed in a different order).
#include <cuda_runtime.h>

#include "lcf_internal.cuh"
#include "lane_cost.cuh"
#include "models_f64.cuh"

namespace {

// ---------------------------------------------------------------------------
// Model evaluation (cuda/models.cu:590-617)
// ---------------------------------------------------------------------------
__global__ void eval_draws_kernel(int m, const double* p, const double* t, double* o, int nd, int nt, int np) {
    int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)nd * nt) return;
    int dd = (int)(idx / nt), ti = (int)(idx % nt);
    o[idx] = lcf::eval_model_f64(m, p + (int64_t)dd * np, t[ti]);
}

// MetzgerKN over the whole (unsorted) times array of one draw, as the
// reference's metzger_kn_eval (cuda/models.cu:146-260): one ODE over the
// draw's largest phase, normalised by its peak.
__global__ void metzger_draws_kernel(const double* p, const double* t, double* o, int nd, int nt, int np,
                                     double* tmp) {
    int dd = blockIdx.x * blockDim.x + threadIdx.x;
    if (dd >= nd) return;
    // sort the times by insertion into tmp (stable), evaluate, scatter back
    double* ts = tmp + (int64_t)dd * 2 * nt;
    double* ys = ts + nt;
    for (int i = 0; i < nt; i++) {
        double v = t[i];
        int j = i;
        while (j > 0 && ts[j - 1] > v) { ts[j] = ts[j - 1]; j--; }
        ts[j] = v;
    }
    lcf::metzger_f64(p + (int64_t)dd * np, ts, nt, ys);
    for (int i = 0; i < nt; i++) {
        // position of t[i] in the sorted array (first match of equal times)
        int lo = 0, hi = nt;
        while (lo < hi) {
            int mid = (lo + hi) / 2;
            if (ts[mid] < t[i]) lo = mid + 1; else hi = mid;
        }
        o[(int64_t)dd * nt + i] = ys[lo];
    }
}

void eval_draws(int m, const double* p, const double* t, double* o, int nd, int nt, int np) {
    int64_t total = (int64_t)nd * nt;
    if (total <= 0) return;
    eval_draws_kernel<<<(int)((total + 255) / 256), 256>>>(m, p, t, o, nd, nt, np);
}

// The reference GPU kernels' model value at one time: the analytic models as
// the CPU path, MetzgerKN by its per-observation ODE (cuda/models_device.h:
// 458-470).
__device__ __forceinline__ double gpu_model_at(int m, const double* p, double t) {
    return m == 7 ? lcf::metzger_at_obs_f64(p, t) : lcf::eval_model_f64(m, p, t);
}

// One observation's term of the reference GPU cost (cuda/models.cu:546-581):
// (pred - y)^2 / v + ln v for a detection, -ln Phi((u - pred) / sqrt v) for
// an upper limit, with v = obs_var + sigma_extra^2.  No 1/2, no prior, no
// Villar constraint, no MetzgerKN peak rescale: those belong to the CPU
// path's PsoCost, not to this kernel.
__device__ __forceinline__ double gpu_obs_term(double pred, double y, double var, int up, double uf, double se2) {
    const double tv = var + se2;
    if (up) return -lcf::log_normal_cdf_f64((uf - pred) / sqrt(tv));
    const double d = pred - y;
    return d * d / tv + log(tv);
}

// ---------------------------------------------------------------------------
// batch_pso_cost (cuda/models.cu:516-584): costs[s * n_part + k] = sum of the
// terms / n for positions[s][k][n_params], sigma_extra the last parameter;
// 1e99 for an empty source or a non-finite prediction.  One warp per row.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) pso_cost_kernel(const double* all_t, const double* all_f,
                                                       const double* all_var, const int* all_up, const double* all_uf,
                                                       const int* offs, const double* pos, double* costs, int n_src,
                                                       int n_part, int np, int model) {
    const int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (row >= (int64_t)n_src * n_part) return;
    const int s = (int)(row / n_part);
    const int o0 = offs[s], o1 = offs[s + 1];
    if (o1 - o0 <= 0) {
        if (lane == 0) costs[row] = 1e99;
        return;
    }
    double p[lcf::MAXP];
#pragma unroll
    for (int j = 0; j < lcf::MAXP; j++) p[j] = j < np ? pos[row * np + j] : 0.0;
    const double sx = exp(pos[row * np + np - 1]);
    const double se2 = sx * sx;
    double nll = 0.0;
    int bad = 0;
    for (int i = o0 + lane; i < o1; i += 32) {
        const double pred = gpu_model_at(model, p, all_t[i]);
        if (!isfinite(pred)) {
            bad = 1;
            break;
        }
        nll += gpu_obs_term(pred, all_f[i], all_var[i], all_up[i], all_uf[i], se2);
    }
    bad = lcf::warp_or(bad);
    nll = lcf::warp_sum_d(nll);
    if (lane == 0) costs[row] = bad ? 1e99 : nll / (double)(o1 - o0);
}

// ---------------------------------------------------------------------------
// batch_pso_cost_multi_bazin (cuda/models.cu:295-362): sum of K Bazin
// components (log A, t0, log tau_rise, log tau_fall each) plus the shared
// baseline B and log sigma_extra; K = source_k[s], rows padded to n_params.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) pso_cost_mb_kernel(const double* all_t, const double* all_f,
                                                          const double* all_var, const int* all_up,
                                                          const double* all_uf, const int* offs, const double* pos,
                                                          double* costs, const int* source_k, int n_src, int n_part,
                                                          int np) {
    const int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (row >= (int64_t)n_src * n_part) return;
    const int s = (int)(row / n_part);
    const int o0 = offs[s], o1 = offs[s + 1];
    if (o1 - o0 <= 0) {
        if (lane == 0) costs[row] = 1e99;
        return;
    }
    const int k = source_k[s];
    const double* p = pos + row * np;
    const double sx = exp(p[4 * k + 1]);
    const double se2 = sx * sx;
    const double b = p[4 * k];
    double nll = 0.0;
    int bad = 0;
    for (int i = o0 + lane; i < o1; i += 32) {
        const double t = all_t[i];
        double sum = 0.0;
        for (int c = 0; c < k; c++) {
            const double* q = p + 4 * c;
            const double dt = t - q[1];
            sum += exp(q[0]) * exp(-dt / exp(q[3])) * (1.0 / (1.0 + exp(-(dt / exp(q[2])))));
        }
        const double pred = sum + b;
        if (!isfinite(pred)) {
            bad = 1;
            break;
        }
        nll += gpu_obs_term(pred, all_f[i], all_var[i], all_up[i], all_uf[i], se2);
    }
    bad = lcf::warp_or(bad);
    nll = lcf::warp_sum_d(nll);
    if (lane == 0) costs[row] = bad ? 1e99 : nll / (double)(o1 - o0);
}

// ---------------------------------------------------------------------------
// batch_svi_fit (cuda/svi.cu:48-330): the reference GPU's SVI of one source
// per warp.  Its semantics, which differ from the CPU path's svi_fit:
//   * noise from xorshift64 seeded 42 + source * 123456789, uniforms
//     (x & (2^53 - 1)) / (2^53 - 1), Box-Muller per parameter (u1 then u2);
//   * prior centres and widths from the caller's arrays;
//   * MetzgerKN by its per-observation ODE, with forward differences
//     h = max(1e-5, 1e-5 |theta_j|) for its gradient;
//   * early stop after >= 50 steps once the ELBO's EMA(0.1) has not improved
//     by 1 % for 20 steps;
//   * log sigma clamped to [-6, 2] and reported without the CPU path's
//     ln 4 inflation; rows padded with 0 up to max_params; an empty source
//     gets elbo -1e99 and nothing else.
// Every lane steps the same generator state, so the draws need no broadcast;
// the lanes split the observations and the sums are reduced across the warp
// by a butterfly, which leaves the same total in every lane.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double xs_uniform(unsigned long long& x) {
    x ^= x << 13;
    x ^= x >> 7;
    x ^= x << 17;
    return (double)(x & 0x1FFFFFFFFFFFFFULL) / (double)0x1FFFFFFFFFFFFFULL;
}

__global__ void __launch_bounds__(128) svi_fit_kernel(const double* all_t, const double* all_f, const double* all_var,
                                                      const int* all_up, const double* all_uf, const int* offs,
                                                      const double* pso_params, const int* model_ids,
                                                      const int* n_params_arr, const int* se_idx_arr,
                                                      const double* prior_c, const double* prior_w, double* out_mu,
                                                      double* out_ls, double* out_elbo, int n_src, int max_params,
                                                      int n_steps, int n_samples, double lr) {
    const int s = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (s >= n_src) return;
    const int o0 = offs[s], o1 = offs[s + 1];
    if (o1 - o0 <= 0) {
        if (lane == 0) out_elbo[s] = -1e99;
        return;
    }
    constexpr int MP = lcf::MAXP;
    const int model = model_ids[s], np = min(n_params_arr[s], MP), se = se_idx_arr[s];
    const int64_t base = (int64_t)s * max_params;
    double mu[MP], ls[MP], pc[MP], pw2[MP], am[2 * MP], av[2 * MP];
    for (int j = 0; j < MP; j++) {
        mu[j] = j < np ? pso_params[base + j] : 0.0;
        ls[j] = -1.0;
        pc[j] = j < np ? prior_c[base + j] : 0.0;
        const double w = j < np ? prior_w[base + j] : 1.0;
        pw2[j] = w * w;
        am[j] = av[j] = am[MP + j] = av[MP + j] = 0.0;
    }
    unsigned long long rng = 42ULL + (unsigned long long)s * 123456789ULL;
    const double PI = 3.14159265358979323846;
    double final_elbo = -1e300, ema = -1e300, best = -1e300;
    int stall = 0, t_adam = 0;
    for (int step = 0; step < n_steps; step++) {
        double sg[MP], gmu[MP], gls[MP];
        for (int j = 0; j < MP; j++) {
            sg[j] = exp(ls[j]);
            gmu[j] = gls[j] = 0.0;
        }
        double elbo_sum = 0.0;
        for (int smp = 0; smp < n_samples; smp++) {
            double th[MP], eps[MP];
            for (int j = 0; j < MP; j++) {
                if (j < np) {
                    const double u1 = fmax(xs_uniform(rng), 1e-10);
                    const double u2 = xs_uniform(rng);
                    eps[j] = sqrt(-2.0 * log(u1)) * cos(2.0 * PI * u2);
                    th[j] = mu[j] + sg[j] * eps[j];
                } else {
                    eps[j] = th[j] = 0.0;
                }
            }
            const double sx = exp(th[se]);
            const double se2 = sx * sx;
            double ll = 0.0, dll[MP];
            for (int j = 0; j < MP; j++) dll[j] = 0.0;
            for (int i = o0 + lane; i < o1; i += 32) {
                const double t = all_t[i];
                const double pred = gpu_model_at(model, th, t);
                if (!isfinite(pred)) continue;
                double g[MP];
                if (model != 7) {
                    lcf::model_grad_f64(model, th, t, g);
                } else {
                    double tp[MP];
                    for (int k = 0; k < MP; k++) tp[k] = th[k];
                    for (int j = 0; j < np; j++) {
                        if (j == se) {
                            g[j] = 0.0;
                            continue;
                        }
                        const double h = fmax(1e-5, 1e-5 * fabs(th[j]));
                        tp[j] = th[j] + h;
                        const double pp = lcf::metzger_at_obs_f64(tp, t);
                        tp[j] = th[j];
                        g[j] = isfinite(pp) ? (pp - pred) / h : 0.0;
                    }
                    g[se] = 0.0;
                }
                const double tv = all_var[i] + se2;
                const double st = sqrt(tv);
                const double it = 1.0 / tv;
                if (all_up[i]) {
                    const double z = (all_uf[i] - pred) / st;
                    ll += lcf::log_normal_cdf_f64(z);
                    const double phi = exp(-0.5 * z * z) / sqrt(2.0 * PI);
                    const double cdf = fmax(0.5 * (1.0 + lcf::erf_approx_f64(z * 0.70710678118654752440)), 1e-300);
                    const double dpred = -phi / (cdf * st);
                    for (int j = 0; j < np; j++)
                        if (j != se && isfinite(g[j])) dll[j] += dpred * g[j];
                    dll[se] += (phi / cdf) * (-(all_uf[i] - pred) * se2 / (st * tv));
                } else {
                    const double r = all_f[i] - pred;
                    const double r2 = r * r;
                    ll += -0.5 * (r2 * it + log(2.0 * PI * tv));
                    for (int j = 0; j < np; j++)
                        if (j != se && isfinite(g[j])) dll[j] += r * it * g[j];
                    dll[se] += (r2 * it * it - it) * se2;
                }
            }
            ll = lcf::warp_sum_d(ll);
            double lp = 0.0;
            for (int j = 0; j < np; j++) {
                const double dj = lcf::warp_sum_d(dll[j]);
                const double d = th[j] - pc[j];
                lp += -0.5 * d * d / pw2[j];
                const double df = dj + (-d / pw2[j]);
                gmu[j] += df;
                gls[j] += df * sg[j] * eps[j];
            }
            elbo_sum += ll + lp;
        }
        const double ns = (double)n_samples;
        double ent = 0.0;
        for (int j = 0; j < np; j++) {
            gmu[j] /= ns;
            gls[j] /= ns;
            ent += ls[j];
        }
        ent += 0.5 * (double)np * log(2.0 * PI * 2.71828182845904523536);
        final_elbo = elbo_sum / ns + ent;
        t_adam++;
        const double bc1 = 1.0 - pow(0.9, (double)t_adam), bc2 = 1.0 - pow(0.999, (double)t_adam);
        for (int j = 0; j < np; j++) {
            const double g_mu = -gmu[j];
            if (isfinite(g_mu)) {
                am[j] = 0.9 * am[j] + 0.1 * g_mu;
                av[j] = 0.999 * av[j] + 0.001 * g_mu * g_mu;
                mu[j] -= lr * (am[j] / bc1) / (sqrt(av[j] / bc2) + 1e-8);
            }
            const double g_ls = -(gls[j] + 1.0);
            if (isfinite(g_ls)) {
                am[MP + j] = 0.9 * am[MP + j] + 0.1 * g_ls;
                av[MP + j] = 0.999 * av[MP + j] + 0.001 * g_ls * g_ls;
                ls[j] -= lr * (am[MP + j] / bc1) / (sqrt(av[MP + j] / bc2) + 1e-8);
            }
        }
        for (int j = 0; j < np; j++) ls[j] = fmax(-6.0, fmin(2.0, ls[j]));
        if (step >= 50) {
            ema = ema < -1e290 ? final_elbo : 0.1 * final_elbo + 0.9 * ema;
            if (ema - best > 0.01 * fmax(fabs(best), 1e-10)) {
                best = ema;
                stall = 0;
            } else if (++stall >= 20) {
                break;
            }
        }
    }
    if (lane == 0) {
        for (int j = 0; j < max_params; j++) {
            out_mu[base + j] = j < np ? mu[j] : 0.0;
            out_ls[base + j] = j < np ? fmax(-6.0, fmin(2.0, ls[j])) : 0.0;
        }
        out_elbo[s] = final_elbo;
    }
}

}  // namespace

extern "C" {
void launch_bazin(const double* p, const double* t, double* o, int nd, int nt, int np, int, int) { eval_draws(0, p, t, o, nd, nt, np); }
void launch_villar(const double* p, const double* t, double* o, int nd, int nt, int np, int, int) { eval_draws(1, p, t, o, nd, nt, np); }
void launch_tde(const double* p, const double* t, double* o, int nd, int nt, int np, int, int) { eval_draws(2, p, t, o, nd, nt, np); }
void launch_arnett(const double* p, const double* t, double* o, int nd, int nt, int np, int, int) { eval_draws(3, p, t, o, nd, nt, np); }
void launch_magnetar(const double* p, const double* t, double* o, int nd, int nt, int np, int, int) { eval_draws(4, p, t, o, nd, nt, np); }
void launch_shock_cooling(const double* p, const double* t, double* o, int nd, int nt, int np, int, int) { eval_draws(5, p, t, o, nd, nt, np); }
void launch_afterglow(const double* p, const double* t, double* o, int nd, int nt, int np, int, int) { eval_draws(6, p, t, o, nd, nt, np); }
void launch_metzger_kn(const double* p, const double* t, double* o, int nd, int nt, int np, int, int) {
    if (nd <= 0 || nt <= 0) return;
    double* tmp = nullptr;
    if (cudaMalloc(&tmp, (size_t)nd * 2 * nt * sizeof(double)) != cudaSuccess) return;
    metzger_draws_kernel<<<(nd + 63) / 64, 64>>>(p, t, o, nd, nt, np, tmp);
    cudaFree(tmp);
}

void launch_batch_pso_cost(const double* all_times, const double* all_flux, const double* all_obs_var,
                           const int* all_is_upper, const double* all_upper_flux, const int* source_offsets,
                           const double* positions, double* costs, int n_sources, int n_particles, int n_params,
                           int model_id, int, int) {
    const int64_t rows = (int64_t)n_sources * n_particles;
    if (rows <= 0 || n_params < 1 || n_params > lcf::MAXP || model_id < 0 || model_id > 7) return;
    pso_cost_kernel<<<(int)((rows * 32 + 255) / 256), 256>>>(all_times, all_flux, all_obs_var, all_is_upper,
                                                             all_upper_flux, source_offsets, positions, costs,
                                                             n_sources, n_particles, n_params, model_id);
}

void launch_batch_pso_cost_multi_bazin(const double* all_times, const double* all_flux, const double* all_obs_var,
                                       const int* all_is_upper, const double* all_upper_flux,
                                       const int* source_offsets, const double* positions, double* costs,
                                       const int* source_k, int n_sources, int n_particles, int n_params, int, int) {
    const int64_t rows = (int64_t)n_sources * n_particles;
    if (rows <= 0 || n_params < 6) return;
    pso_cost_mb_kernel<<<(int)((rows * 32 + 255) / 256), 256>>>(all_times, all_flux, all_obs_var, all_is_upper,
                                                                all_upper_flux, source_offsets, positions, costs,
                                                                source_k, n_sources, n_particles, n_params);
}

void launch_batch_svi_fit(const double* all_times, const double* all_flux, const double* all_obs_var,
                          const int* all_is_upper, const double* all_upper_flux, const int* source_offsets,
                          const double* pso_params, const int* model_ids, const int* n_params_arr,
                          const int* se_idx_arr, const double* prior_centers, const double* prior_widths,
                          double* out_mu, double* out_log_sigma, double* out_elbo, int n_sources, int max_params,
                          int n_steps, int n_samples, double lr, int, int) {
    if (n_sources <= 0 || max_params < 1) return;
    const int64_t threads = (int64_t)n_sources * 32;
    svi_fit_kernel<<<(int)((threads + 127) / 128), 128>>>(all_times, all_flux, all_obs_var, all_is_upper,
                                                          all_upper_flux, source_offsets, pso_params, model_ids,
                                                          n_params_arr, se_idx_arr, prior_centers, prior_widths,
                                                          out_mu, out_log_sigma, out_elbo, n_sources, max_params,
                                                          n_steps, n_samples, lr);
}
}
