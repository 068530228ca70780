// polish.cu — restart reduction, bounded L-BFGS polish and BIC model
// selection (pso_fit_single_model / pso_model_select, src/parametric.rs:
// 1864-2066), and the SVI uncertainty kernel (svi_fit, :2215-2454).
//
// L-BFGS: four polishes per warp, eight lanes each (lbfgs_group.cuh): the
// lanes of a group split its band's observations (double-float terms, FP64
// where FP32's range would not hold them); the quasi-Newton algebra (two-loop
// recursion, memory 7) and the Moré–Thuente line search run in FP64,
// following the argmin 0.11 algorithm the reference calls (restated from the
// published method, as in the test oracle).
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
#include "lane_cost.cuh"
#include "lbfgs_group.cuh"
#include "lcf_internal.cuh"
#include "models_f32.cuh"
#include "metzger_dual.cuh"
#include "models_f64.cuh"
#include "models_ff.cuh"

namespace lcf {

#define FULL 0xffffffffu

// The polish (lbfgs_group.cuh): a persistent grid whose warps drain the
// models' queues in turn, four polishes per warp.  Two blocks of 8 warps per
// SM (128 registers a thread), each block's warps in step: measured on
// GB300 at 10k sources, 415 ms against 435 ms for four blocks of 4 warps,
// 491 ms for one block of 16, and 486 ms for 16 warps not in step.
#ifndef LCF_LB_MINB
#define LCF_LB_MINB 2
#endif
#ifndef LCF_LB_BLOCK
#define LCF_LB_BLOCK 256
#endif
// Each model's queue in two parts: its first n_long bands (the longest) with
// a warp a band, the rest with eight lanes a band.
template <int MODEL>
__device__ __forceinline__ void polish_model(const DeviceBatch& d, LbWarpShared& w, int n_long, bool lockstep) {
    polish_queue<MODEL, 32>(d, w, 0, n_long, &d.ctr->lb_next_long[MODEL], lockstep);
    polish_queue<MODEL, 8>(d, w, n_long, d.n_bands, &d.ctr->lb_next[MODEL], lockstep);
}

// `stagger`: block k starts at model 8k / gridDim.x and takes the models in
// turn from there, and the warps of a block do not run in step: a batch with
// fewer bands than the grid has polish slots runs the eight models' queues
// at once.  Otherwise every block takes the models in order, its warps in
// step, and the warps of an SM share one model's code.
__global__ void __launch_bounds__(LCF_LB_BLOCK, LCF_LB_MINB)
    lbfgs_kernel(DeviceBatch d, int model_mask, int stagger, int n_long) {
    extern __shared__ LbWarpShared lb_sh[];
    LbWarpShared& w = lb_sh[threadIdx.x >> 5];
    const int start = stagger ? (int)((8ll * blockIdx.x) / gridDim.x) : 0;
    const bool lockstep = !stagger;
    for (int k = 0; k < 8; k++) {
        const int m = (start + k) & 7;
        if (!((model_mask >> m) & 1)) continue;
        switch (m) {
            case BAZIN: polish_model<BAZIN>(d, w, n_long, lockstep); break;
            case VILLAR: polish_model<VILLAR>(d, w, n_long, lockstep); break;
            case TDE: polish_model<TDE>(d, w, n_long, lockstep); break;
            case ARNETT: polish_model<ARNETT>(d, w, n_long, lockstep); break;
            case MAGNETAR: polish_model<MAGNETAR>(d, w, n_long, lockstep); break;
            case SHOCK: polish_model<SHOCK>(d, w, n_long, lockstep); break;
            case AFTERGLOW: polish_model<AFTERGLOW>(d, w, n_long, lockstep); break;
            default: polish_model<METZGER>(d, w, n_long, lockstep); break;
        }
    }
}

constexpr size_t LB_SMEM = (LCF_LB_BLOCK / 32) * sizeof(LbWarpShared);

int lbfgs_grid(int num_sms) {
    int n = 0;
    if (cudaFuncSetAttribute(lbfgs_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)LB_SMEM) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, lbfgs_kernel, LCF_LB_BLOCK, LB_SMEM) != cudaSuccess || n < 1)
        n = 1;
    return num_sms * n;
}

void launch_lbfgs(const DeviceBatch& d, int model_mask, cudaStream_t s) {
    if (d.n_bands == 0) return;
    // a warp a band for the bands of LB_LONG_OBS observations or more (the
    // polish of a long band on eight lanes would set the kernel's tail).  The
    // split depends on the band alone, not on the batch: a band's summation
    // order, and so its fit, is the same in any batch.
    const int64_t warps = (int64_t)d.lb_grid * (LCF_LB_BLOCK / 32);
    lbfgs_kernel<<<d.lb_grid, LCF_LB_BLOCK, LB_SMEM, s>>>(d, model_mask, (int64_t)d.n_bands < 4 * warps ? 1 : 0,
                                                          d.lb_n_long);
}

// The polish queue's band order: longest first (counting sort on 256 keys,
// 8 observations a key), so that the groups of a warp take bands of similar
// length.  The order inside a key is not fixed; no result depends on it.
__device__ __forceinline__ int polish_key(const DeviceBatch& d, int b) { return 255 - min(d.stats[b].n >> 3, 255); }
// the long bands (a warp a band) are then exactly the first lb_n_long
static_assert(LB_LONG_OBS % 8 == 0 && LB_LONG_OBS / 8 <= 255, "LB_LONG_OBS must fall on a key boundary");
__global__ void polish_hist_kernel(DeviceBatch d) {
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < d.n_bands; b += gridDim.x * blockDim.x)
        atomicAdd(&d.ctr->polish_hist[polish_key(d, b)], 1);
}
__global__ void polish_scan_kernel(DeviceBatch d) {  // one block of 256 threads
    __shared__ int sh[256];
    const int i = threadIdx.x;
    const int v = d.ctr->polish_hist[i];
    sh[i] = v;
    __syncthreads();
    for (int off = 1; off < 256; off <<= 1) {
        const int a = i >= off ? sh[i - off] : 0;
        __syncthreads();
        sh[i] += a;
        __syncthreads();
    }
    d.ctr->polish_hist[i] = sh[i] - v;
}
__global__ void polish_scatter_kernel(DeviceBatch d) {
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < d.n_bands; b += gridDim.x * blockDim.x)
        d.polish_order[atomicAdd(&d.ctr->polish_hist[polish_key(d, b)], 1)] = b;
}
void launch_polish_order(const DeviceBatch& d, cudaStream_t s) {
    if (d.n_bands == 0) return;
    int grid = (d.n_bands + 255) / 256;
    grid = grid < 1024 ? grid : 1024;
    polish_hist_kernel<<<grid, 256, 0, s>>>(d);
    polish_scan_kernel<<<1, 256, 0, s>>>(d);
    polish_scatter_kernel<<<grid, 256, 0, s>>>(d);
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
// FP64 peaks for the polish's roofline.  probe_obs_kernel streams the polish's
// own observation term (lb_obs_term: value, gradient and cost of one
// observation, FP64) over a synthetic band held in L1, lanes over
// observations, with none of the line search, reductions or divergence of a
// real polish; its rate is the ceiling of the polish's observation work on
// this GPU.  probe_dfma_kernel: independent DFMA chains (FP64 FLOP/s).
// ---------------------------------------------------------------------------
static __device__ __constant__ double c_probe_p[7][MAXP] = {
    {0.0, 0.0, 30.0, 1.0, 3.0, -3.0, 0.0},
    {0.0, 0.005, 2.3, 30.0, 1.0, 3.0, -3.0},
    {0.0, 0.0, 30.0, 1.0, 3.0, 1.67, -3.0},
    {0.0, 30.0, 2.3, 0.0, -3.0, 0.0, 0.0},
    {0.0, 30.0, 3.0, 2.3, -3.0, 0.0, 0.0},
    {0.0, 30.0, 0.5, 1.0, -3.0, 0.0, 0.0},
    {0.0, 30.0, 1.0, 0.8, 2.2, -3.0, 0.0}};

template <int MODEL>
__global__ void __launch_bounds__(256) probe_obs_kernel(const double* band, int nb, int reps, double* sink) {
    const int lane = threadIdx.x & 31;
    const double *t = band, *var = band + nb, *flux = band + 2 * nb, *uf = band + 3 * nb, *upd = band + 4 * nb;
    double nll = 0.0, gl[MAXP];
    for (int k = 0; k < MAXP; k++) gl[k] = 0.0;
    int nf = 0;
    for (int r = 0; r < reps; r++) {
        double q[MAXP];
        for (int k = 0; k < MAXP; k++) q[k] = c_probe_p[MODEL][k] + 1e-9 * (double)r;  // a new point per pass
        Model64 mod;
        mod.init(MODEL, q);
        const double se2 = exp(2.0 * q[se_idx_of(MODEL)]);
        for (int i = lane; i < nb; i += 32)
            lb_obs_term<MODEL>(mod, t[i], var[i], flux[i], upd[i] != 0.0, uf[i], se2, true, nll, gl, nf);
    }
    double s = nll + (double)nf;
    for (int k = 0; k < MAXP; k++) s += gl[k];
    sink[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// The same stream through the double-float term (ff_obs_term), the band as
// ff pairs.
template <int MODEL>
__global__ void __launch_bounds__(256) probe_ff_kernel(const float4* fa, const float2* fb, int nb, int reps,
                                                       double* sink) {
    const int lane = threadIdx.x & 31;
    ff nll = ffm(0.0f, 0.0f), gl[MAXP];
    for (int k = 0; k < MAXP; k++) gl[k] = ffm(0.0f, 0.0f);
    int nf = 0;
    for (int r = 0; r < reps; r++) {
        double q[MAXP];
        ff ef[MAXP], rf[MAXP];
        for (int k = 0; k < MAXP; k++) {
            q[k] = c_probe_p[MODEL][k] + 1e-9 * (double)r;
            ef[k] = ff_exp(ff_from(q[k]));
            rf[k] = ff_exp(ff_neg(ff_from(q[k])));
        }
        FfModel<MODEL> mod;
        mod.init(q, ef, rf);
        const ff se2 = ff_sqr(ef[se_idx_of(MODEL)]);
        int redo = 0;
        for (int i = lane; i < nb; i += 32) ff_obs_term<MODEL>(mod, fa[i], fb[i], se2, true, nll, gl, nf, redo);
    }
    double s = ff_to(nll) + (double)nf;
    for (int k = 0; k < MAXP; k++) s += ff_to(gl[k]);
    sink[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// Agreement of the ff and FP64 observation terms: one warp per parameter
// point (pts[w], MAXP doubles), lanes over the probe band; writes per point
// the FP64 sums, the ff sums and the sums of the terms' magnitudes of the
// cost (all observations) and of the MAXP gradient components (detections),
// 3 * (1 + MAXP) doubles, and whether the point stays in double-float.
template <int MODEL>
__global__ void ff_check_kernel(const double* band, const float4* fa, const float2* fb, int nb, const double* pts,
                                int n_pts, double* out) {
    const int w = blockIdx.x, lane = threadIdx.x & 31;
    if (w >= n_pts) return;
    const double *t = band, *var = band + nb, *flux = band + 2 * nb, *uf = band + 3 * nb, *upd = band + 4 * nb;
    double q[MAXP], ep[MAXP], rp[MAXP];
    for (int k = 0; k < MAXP; k++) {
        q[k] = pts[(size_t)w * MAXP + k];
        ep[k] = exp(q[k]);
        rp[k] = 1.0 / ep[k];
    }
    Model64 m64;
    m64.init_pre(MODEL, q, ep, rp);
    ff ef[MAXP], rf[MAXP];
    for (int k = 0; k < MAXP; k++) { ef[k] = ff_from(ep[k]); rf[k] = ff_from(rp[k]); }
    FfModel<MODEL> mff;
    mff.init(q, ef, rf);
    const double se2 = ep[se_idx_of(MODEL)] * ep[se_idx_of(MODEL)];
    const ff se2f = ff_from(se2);
    double v64[1 + MAXP], vff[1 + MAXP], mag[1 + MAXP];
    for (int k = 0; k <= MAXP; k++) v64[k] = vff[k] = mag[k] = 0.0;
    int nf64 = 0, nfff = 0, redo = 0;
    for (int i = lane; i < nb; i += 32) {
        double n1 = 0.0, g1[MAXP];
        ff n2 = ffm(0.0f, 0.0f), g2[MAXP];
        for (int k = 0; k < MAXP; k++) { g1[k] = 0.0; g2[k] = ffm(0.0f, 0.0f); }
        lb_obs_term<MODEL>(m64, t[i], var[i], flux[i], upd[i] != 0.0, uf[i], se2, true, n1, g1, nf64);
        ff_obs_term<MODEL>(mff, fa[i], fb[i], se2f, true, n2, g2, nfff, redo);
        v64[0] += n1; vff[0] += ff_to(n2); mag[0] += fabs(n1);
        // gradients of detections only: an upper limit's FP64 gradient ratio
        // carries the reference's cancellation (see ff_upper)
        if (upd[i] == 0.0)
            for (int k = 0; k < MAXP; k++) { v64[1 + k] += g1[k]; vff[1 + k] += ff_to(g2[k]); mag[1 + k] += fabs(g1[k]); }
    }
    for (int k = 0; k <= MAXP; k++) {
        v64[k] = warp_sum_d(v64[k]);
        vff[k] = warp_sum_d(vff[k]);
        mag[k] = warp_sum_d(mag[k]);
    }
    nf64 = warp_or(nf64);
    nfff = warp_or(nfff);
    redo = warp_or(redo);
    if (lane == 0) {
        double* o = out + (size_t)w * (3 * (1 + MAXP) + 2);
        for (int k = 0; k <= MAXP; k++) { o[k] = v64[k]; o[1 + MAXP + k] = vff[k]; o[2 * (1 + MAXP) + k] = mag[k]; }
        const double t0 = q[t0_idx_of(MODEL)];
        double tmin = t[0], tmax = t[0];
        for (int i = 1; i < nb; i++) { tmin = fmin(tmin, t[i]); tmax = fmax(tmax, t[i]); }
        o[3 * (1 + MAXP)] = (ff_range_ok<MODEL>(q, rf, tmin - t0, tmax - t0) && !redo) ? 1.0 : 0.0;
        o[3 * (1 + MAXP) + 1] = (double)(nf64 + 2 * nfff);
    }
}

__global__ void probe_dfma_kernel(double* out, int iters) {
    double a0 = threadIdx.x * 1e-3, a1 = a0 + 1.0, a2 = a0 + 2.0, a3 = a0 + 3.0;
    const double b = 1.0000001, c = 1e-9;
    for (int i = 0; i < iters; i++) {
        a0 = fma(a0, b, c); a1 = fma(a1, b, c); a2 = fma(a2, b, c); a3 = fma(a3, b, c);
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = a0 + a1 + a2 + a3;
}

int probe_fp64_peaks(int num_sms, double* out9) {
    // synthetic band: 64 observations over 100 days, a Bazin-like light curve,
    // 27 % of them upper limits (the workload's fraction)
    const int nb = 64;
    double h[5 * nb];
    for (int i = 0; i < nb; i++) {
        double t = 100.0 * i / (nb - 1), dt = t - 30.0;
        double f = exp(-dt / 20.0) / (1.0 + exp(-dt / 3.0));
        bool up = (i % 11) < 3;
        h[i] = t;
        h[nb + i] = 0.0025 + 1e-10;
        h[2 * nb + i] = f;
        h[3 * nb + i] = 0.15;
        h[4 * nb + i] = up ? 1.0 : 0.0;
    }
    const int blocks = num_sms * 8, threads = 256;
    double *band = nullptr, *sink = nullptr;
    if (cudaMalloc(&band, sizeof(h)) != cudaSuccess) return -1;
    if (cudaMalloc(&sink, (size_t)blocks * threads * sizeof(double)) != cudaSuccess) { cudaFree(band); return -1; }
    cudaMemcpy(band, h, sizeof(h), cudaMemcpyHostToDevice);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int reps = 16;
    for (int m = 0; m < 7; m++) {
        float best = 1e30f;
        for (int rep = 0; rep < 2; rep++) {
            cudaEventRecord(e0);
            switch (m) {
                case 0: probe_obs_kernel<0><<<blocks, threads>>>(band, nb, reps, sink); break;
                case 1: probe_obs_kernel<1><<<blocks, threads>>>(band, nb, reps, sink); break;
                case 2: probe_obs_kernel<2><<<blocks, threads>>>(band, nb, reps, sink); break;
                case 3: probe_obs_kernel<3><<<blocks, threads>>>(band, nb, reps, sink); break;
                case 4: probe_obs_kernel<4><<<blocks, threads>>>(band, nb, reps, sink); break;
                case 5: probe_obs_kernel<5><<<blocks, threads>>>(band, nb, reps, sink); break;
                default: probe_obs_kernel<6><<<blocks, threads>>>(band, nb, reps, sink); break;
            }
            cudaEventRecord(e1);
            cudaEventSynchronize(e1);
            float ms = 0.0f;
            cudaEventElapsedTime(&ms, e0, e1);
            best = ms < best ? ms : best;
        }
        double evals = (double)blocks * (threads / 32) * reps * nb;
        out9[m] = evals / (best * 1e-3);
    }
    out9[7] = 0.0;
    {
        const int iters = 4000;
        float best = 1e30f;
        for (int rep = 0; rep < 2; rep++) {
            cudaEventRecord(e0);
            probe_dfma_kernel<<<blocks, threads>>>(sink, iters);
            cudaEventRecord(e1);
            cudaEventSynchronize(e1);
            float ms = 0.0f;
            cudaEventElapsedTime(&ms, e0, e1);
            best = ms < best ? ms : best;
        }
        out9[8] = 2.0 * 4.0 * iters * (double)blocks * threads / (best * 1e-3) * 1e-12;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(band);
    cudaFree(sink);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

// Parameter points for ff_check_kernel: uniform inside the model's PSO box,
// t0 inside [-30, 60] (the probe band spans [0, 100]).
__global__ void ff_points_kernel(int model, int n_pts, double* pts) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_pts * MAXP) return;
    const int w = i / MAXP, k = i % MAXP;
    uint64_t h = 0x9E3779B97F4A7C15ull * (uint64_t)(model * 100003 + w * 17 + k + 1);
    h ^= h >> 31; h *= 0xBF58476D1CE4E5B9ull; h ^= h >> 27; h *= 0x94D049BB133111EBull; h ^= h >> 33;
    const double u = (double)(h >> 11) * (1.0 / 9007199254740992.0);
    double lo = c_lo[model][k], hi = c_hi[model][k];
    if (k == t0_idx_of(model)) { lo = -30.0; hi = 60.0; }
    pts[i] = k < n_params_of(model) ? lo + u * (hi - lo) : 0.0;
}

int probe_ff(int num_sms, double* out) {
    const int nb = 64, n_pts = 256, W = 3 * (1 + MAXP) + 2;
    double h[5 * nb];
    float4 ha[nb];
    float2 hb[nb];
    for (int i = 0; i < nb; i++) {
        double t = 100.0 * i / (nb - 1), dt = t - 30.0;
        double f = exp(-dt / 20.0) / (1.0 + exp(-dt / 3.0));
        bool up = (i % 11) < 3;
        double var = 0.0025 + 1e-10, uf = 0.15, y = up ? uf : f;
        h[i] = t; h[nb + i] = var; h[2 * nb + i] = f; h[3 * nb + i] = uf; h[4 * nb + i] = up ? 1.0 : 0.0;
        float th = (float)t, yh = (float)y, vh = (float)var, vl = (float)(var - (double)vh);
        ha[i] = make_float4(th, (float)(t - (double)th), yh, (float)(y - (double)yh));
        hb[i] = up ? make_float2(-vh, -vl) : make_float2(vh, vl);
    }
    const int blocks = num_sms * 8, threads = 256;
    double *band = nullptr, *sink = nullptr, *pts = nullptr, *res = nullptr;
    float4* fa = nullptr;
    float2* fb = nullptr;
    bool ok = cudaMalloc(&band, sizeof(h)) == cudaSuccess && cudaMalloc(&fa, sizeof(ha)) == cudaSuccess &&
              cudaMalloc(&fb, sizeof(hb)) == cudaSuccess &&
              cudaMalloc(&sink, (size_t)blocks * threads * sizeof(double)) == cudaSuccess &&
              cudaMalloc(&pts, (size_t)n_pts * MAXP * sizeof(double)) == cudaSuccess &&
              cudaMalloc(&res, (size_t)n_pts * W * sizeof(double)) == cudaSuccess;
    if (ok) {
        cudaMemcpy(band, h, sizeof(h), cudaMemcpyHostToDevice);
        cudaMemcpy(fa, ha, sizeof(ha), cudaMemcpyHostToDevice);
        cudaMemcpy(fb, hb, sizeof(hb), cudaMemcpyHostToDevice);
        cudaEvent_t e0, e1;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        const int reps = 16;
        double* hr = new double[(size_t)n_pts * W];
        out[77] = 0.0;
        for (int m = 0; m < 7; m++) {
            float best = 1e30f;
            for (int rep = 0; rep < 2; rep++) {
                cudaEventRecord(e0);
                switch (m) {
                    case 0: probe_ff_kernel<0><<<blocks, threads>>>(fa, fb, nb, reps, sink); break;
                    case 1: probe_ff_kernel<1><<<blocks, threads>>>(fa, fb, nb, reps, sink); break;
                    case 2: probe_ff_kernel<2><<<blocks, threads>>>(fa, fb, nb, reps, sink); break;
                    case 3: probe_ff_kernel<3><<<blocks, threads>>>(fa, fb, nb, reps, sink); break;
                    case 4: probe_ff_kernel<4><<<blocks, threads>>>(fa, fb, nb, reps, sink); break;
                    case 5: probe_ff_kernel<5><<<blocks, threads>>>(fa, fb, nb, reps, sink); break;
                    default: probe_ff_kernel<6><<<blocks, threads>>>(fa, fb, nb, reps, sink); break;
                }
                cudaEventRecord(e1);
                cudaEventSynchronize(e1);
                float ms = 0.0f;
                cudaEventElapsedTime(&ms, e0, e1);
                best = ms < best ? ms : best;
            }
            out[m] = (double)blocks * (threads / 32) * reps * nb / (best * 1e-3);
            ff_points_kernel<<<(n_pts * MAXP + 255) / 256, 256>>>(m, n_pts, pts);
            switch (m) {
                case 0: ff_check_kernel<0><<<n_pts, 32>>>(band, fa, fb, nb, pts, n_pts, res); break;
                case 1: ff_check_kernel<1><<<n_pts, 32>>>(band, fa, fb, nb, pts, n_pts, res); break;
                case 2: ff_check_kernel<2><<<n_pts, 32>>>(band, fa, fb, nb, pts, n_pts, res); break;
                case 3: ff_check_kernel<3><<<n_pts, 32>>>(band, fa, fb, nb, pts, n_pts, res); break;
                case 4: ff_check_kernel<4><<<n_pts, 32>>>(band, fa, fb, nb, pts, n_pts, res); break;
                case 5: ff_check_kernel<5><<<n_pts, 32>>>(band, fa, fb, nb, pts, n_pts, res); break;
                default: ff_check_kernel<6><<<n_pts, 32>>>(band, fa, fb, nb, pts, n_pts, res); break;
            }
            cudaMemcpy(hr, res, (size_t)n_pts * W * sizeof(double), cudaMemcpyDeviceToHost);
            double worst = 0.0;
            int in_range = 0;
            for (int c = 0; c <= MAXP; c++) out[14 + m * 8 + c] = 0.0;
            for (int w = 0; w < n_pts; w++) {
                const double* o = hr + (size_t)w * W;
                if (o[3 * (1 + MAXP)] == 0.0) continue;
                in_range++;
                if (o[3 * (1 + MAXP) + 1] != 0.0 && o[3 * (1 + MAXP) + 1] != 3.0) out[77] += 1.0;
                if (o[3 * (1 + MAXP) + 1] != 0.0) continue;
                // each component against the magnitude of its own terms,
                // floored at 1e-10 of the gradient's total (a component below
                // that, e.g. 1e-40 in FP64 against 0 in double-float, is
                // compared in absolute terms)
                double gsum = 0.0;
                for (int c = 1; c <= MAXP; c++) gsum += o[2 * (1 + MAXP) + c];
                for (int c = 0; c <= MAXP; c++) {
                    const double mg = c == 0 ? o[2 * (1 + MAXP)] : fmax(o[2 * (1 + MAXP) + c], 1e-10 * gsum);
                    if (!(mg > 0.0)) continue;
                    const double rel = fabs(o[1 + MAXP + c] - o[c]) / mg;
                    out[14 + m * 8 + c] = fmax(out[14 + m * 8 + c], rel);
                    worst = fmax(worst, rel);
                }
            }
            out[7 + m] = worst;
            out[70 + m] = (double)in_range;
        }
        delete[] hr;
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
    }
    cudaFree(band); cudaFree(fa); cudaFree(fb); cudaFree(sink); cudaFree(pts); cudaFree(res);
    return ok && cudaGetLastError() == cudaSuccess ? 0 : -1;
}


// ---------------------------------------------------------------------------
// SVI, one warp per band, templated on the band's selected model.  Lanes
// split the observations for the likelihood and its adjoint; the
// per-parameter bookkeeping (reparameterisation, prior, ELBO gradient) runs
// with component j in lane j, and Adam with variational parameter i (mu_i,
// then log sigma_i) in lane i.
// ---------------------------------------------------------------------------
// Sums 8 per-lane FP32 values over the warp (recursive halving, as
// reduce_scatter8): lane l returns the total of v[(l >> 2) & 7].
__device__ __forceinline__ float reduce_scatter8f(const float* v) {
    const int lane = threadIdx.x & 31;
    const bool b4 = lane & 16, b3 = lane & 8, b2 = lane & 4;
    float a[4], b[2];
#pragma unroll
    for (int i = 0; i < 4; i++) {
        float keep = b4 ? v[4 + i] : v[i], give = b4 ? v[i] : v[4 + i];
        a[i] = keep + __shfl_xor_sync(FULL, give, 16);
    }
#pragma unroll
    for (int i = 0; i < 2; i++) {
        float keep = b3 ? a[2 + i] : a[i], give = b3 ? a[i] : a[2 + i];
        b[i] = keep + __shfl_xor_sync(FULL, give, 8);
    }
    float c = (b2 ? b[1] : b[0]) + __shfl_xor_sync(FULL, b2 ? b[0] : b[1], 4);
    c += __shfl_xor_sync(FULL, c, 2);
    c += __shfl_xor_sync(FULL, c, 1);
    return c;
}

// FP64 value and gradient of an analytic model in the reference's own forms
// (eval_model / *_flux_grad, src/parametric.rs:199-538), out of line: the
// rare FP64 cases of svi_deferred_pass, kept apart so that the FP64 code's
// registers do not count against the pass or the SVI loop around it.
template <int M>
__device__ __noinline__ double svi_model64(const double* p64, double t, double* g64) {
    model_grad_f64(M, p64, t, g64);
    return eval_model_f64(M, p64, t);
}

// x * e^lr in FP64, for |x| in FP32's range and any lr: e^lr is split into
// 2^k * 2^f (0 <= f < 1), the FP32 mantissa x * 2^f is widened and its FP64
// exponent raised by k with integer arithmetic on the bits (no FP64
// multiply: a warp FP64 instruction costs 16 SM cycles on this part).  A
// result below FP64's normal range is 0 and one above it +-inf, as the
// reference's FP64 product gives (up to its subnormals).  Relative error
// ~1e-4 for |lr| ~ 700 (lr is an FP32 value), far inside what the terms it
// carries need: they reach Adam through their order of magnitude and sign.
__device__ __forceinline__ double scaled_exp(float x, float lr) {
    const float y = fminf(fmaxf(lr * 1.4426950408889634f, -3000.0f), 3000.0f);
    const float kf = floorf(y);
    const float m = x * exp2f(y - kf);
    if (m == 0.0f || !isfinite(m)) return (double)m;
    const long long bits = __double_as_longlong((double)m);
    const int e = (int)((bits >> 52) & 0x7ff) + (int)kf;
    if (e <= 0) return 0.0;
    if (e >= 2047) return m > 0.0f ? INFINITY : -INFINITY;
    return __longlong_as_double((bits & ~(0x7ffLL << 52)) | ((long long)e << 52));
}

struct SviDeferred {
    double dlx;   // lane l's share: the warp total of component l & 7
    int floored;  // a deferred upper limit hit the CDF floor (warp-uniform)
};

// The reference's gradient terms of the upper limits that upper_ratio_f32
// deferred: those whose quantised CDF 0.5 (1 + erf) holds fewer than 64 units
// of 2^-53 (src/parametric.rs:2336-2352: dpred = -phi / (cdf sigma) times each
// model-gradient component, and the sigma_extra term).
//  * Below the floor (the unit count k = rint(P * 2^53) is 0): cdf = 1e-300
//    and the ratio phi / 1e-300 = e^lr, lr = 690.78 - ln sqrt(2 pi) - z^2 / 2,
//    spans 0 .. ~1e285.  The terms are
//    carried at full magnitude into FP64 (scaled_exp) and reach the ELBO
//    gradient and Adam as in the reference, whose second moment overflows and
//    stops the components they touch.  The FP32 model gradient is exact to
//    FP32 rounding except where a component underflows FP32; a component that
//    is 0 in FP32 while the ratio could lift its FP64 value into range is
//    taken from the FP64 model gradient instead (analytic models; MetzgerKN
//    keeps its FP32 sweep's derivatives).
//  * Near the floor (1 <= k < 64): the ratio phi / (k 2^-54) is ~10 and the
//    terms are formed in FP32 as in the main loop, with k rounded from the
//    FP32 unit count.  Where that count lies within its own error of a
//    rounding boundary (k or k + 1?  0, the floor, or 1?) the observation is
//    evaluated in FP64 from the sample's FP64 parameters, as the reference
//    does, so that the unit count and with it the ratio are the reference's.
// Observations: bit r of xm = observation c0 + 32 r + lane, marked by the
// FP32 loop.  Out of line and called after that loop by the whole warp, so
// the hot loop holds none of this code's registers.
template <int M>
__device__ __noinline__ SviDeferred svi_deferred_pass(const float4* obs, const float* ms, float scl, int c0,
                                                      unsigned long long xm, double th_j, float sx2) {
    constexpr int np = n_params_of(M), se = se_idx_of(M);
    const int lane = threadIdx.x & 31;
    const float ln_ratio0 = 690.77552789821368f - 0.91893853320467274f;  // ln(1e300) - ln sqrt(2 pi)
    double p64[MAXP], dx[MAXP];
    float pf[MAXP];  // the sample's FP32 parameters, as the caller forms them
#pragma unroll
    for (int q = 0; q < MAXP; q++) {
        p64[q] = q < np ? __shfl_sync(FULL, th_j, q) : 0.0;
        pf[q] = (float)p64[q];
        dx[q] = 0.0;
    }
    int floored = 0;
    const int any = xm != 0;
    while (xm) {
        const int i = c0 + ((__ffsll((long long)xm) - 1) << 5) + lane;
        xm &= xm - 1;
        const float4 ob = obs[i];
        float gb[MAXP];
        float pr;
        if constexpr (M == METZGER) {
            pr = ms[i * 5] * scl;
            for (int q = 0; q < 4; q++) gb[q] = ms[i * 5 + 1 + q] * scl;
            gb[4] = 0.0f;
        } else {
            int st;
            pr = model_grad_f32(M, pf, ob.x, ob.y, gb, st);
        }
        const float tv = fabsf(ob.w) + sx2;
        const float stv = sqrtf(tv);
        const float z = (ob.z - pr) / stv;
        // the reference's unit count k: exact from the FP32 estimate unless
        // that lies within its error (~1e-5 relative) of a rounding boundary
        const float units = upper_units_f32(z);
        const float kr = rintf(units);
        const bool exact_k = fabsf(units - kr) < 0.5f - (1e-4f * units + 1e-4f);
        if (exact_k && kr >= 1.0f) {
            // 1 <= k < 64: the ratio phi / (k 2^-54) is ~10, inside FP32
            const float ratio = 0.39894228040143268f * expf(-0.5f * z * z) / (0.5f * kr * 1.1102230246251565e-16f);
#pragma unroll
            for (int q = 0; q < np; q++)
                if (q != se && isfinite(gb[q])) dx[q] += (double)(-ratio / stv * gb[q]);
            dx[se] += (double)(ratio * (-(ob.z - pr) * sx2 / (stv * tv)));
        } else if (exact_k) {
            floored = 1;
            const float lr = fmaf(-0.5f * z, z, ln_ratio0);
            bool rescue = false;
#pragma unroll
            for (int q = 0; q < np; q++) {
                if (q == se || !isfinite(gb[q])) continue;
                if (gb[q] != 0.0f) dx[q] += scaled_exp(-gb[q] / stv, lr);
                else if (M != METZGER && lr > 60.0f) rescue = true;  // ratio > 1e26: an FP32 underflow may matter
            }
            dx[se] += scaled_exp(-(ob.z - pr) * sx2 / (stv * tv), lr);
            if constexpr (M != METZGER) {
                if (rescue) {
                    double g64[MAXP];
                    svi_model64<M>(p64, (double)ob.x + (double)ob.y, g64);
                    const double sc = scaled_exp(-1.0f / stv, lr);
#pragma unroll
                    for (int q = 0; q < np; q++)
                        if (q != se && gb[q] == 0.0f && isfinite(g64[q])) dx[q] += sc * g64[q];
                }
            }
        } else {
            double g64[MAXP];
            double pd;
            if constexpr (M == METZGER) {
                pd = (double)pr;
                for (int q = 0; q < np; q++) g64[q] = (double)gb[q];
            } else {
                pd = svi_model64<M>(p64, (double)ob.x + (double)ob.y, g64);
            }
            if (!isfinite(pd)) continue;
            const double sx = exp(p64[se]);
            const double sxx = sx * sx;
            const double tvd = (double)fabsf(ob.w) + sxx;
            const double sd = sqrt(tvd);
            const double uf = (double)ob.z;
            const double zd = (uf - pd) / sd;
            const double phi = exp(-0.5 * zd * zd) * 0.39894228040143267794;
            const double raw = 0.5 * (1.0 + erf_approx_f64(zd * 0.70710678118654752440));
            const double cdf = fmax(raw, 1e-300);
            if (!(raw > 1e-300)) floored = 1;
            const double dpred = -phi / (cdf * sd);
#pragma unroll
            for (int q = 0; q < np; q++)
                if (q != se && isfinite(g64[q])) dx[q] += dpred * g64[q];
            dx[se] += (phi / cdf) * (-(uf - pd) * sxx / (sd * tvd));
        }
    }
    // warp totals: only the lanes that deferred something contribute (few),
    // so each of those lanes' components is broadcast and lane l keeps
    // component l & 7
    SviDeferred r;
    r.dlx = 0.0;
    unsigned act = __ballot_sync(FULL, any);
    while (act) {
        const int src = __ffs(act) - 1;
        act &= act - 1;
        double mine = 0.0;
#pragma unroll
        for (int q = 0; q < np; q++) {
            const double v = __shfl_sync(FULL, dx[q], src);
            if (q == (lane & 7)) mine = v;
        }
        r.dlx += mine;
    }
    r.floored = warp_or(floored);
    return r;
}

// One reparameterised sample's log-likelihood over the band and its
// gradient, the adjoint through the analytic model gradient (the body of an
// SVI step, src/parametric.rs:2280-2330).  pf = the sample's parameters in
// FP32, held by every lane; th_j = lane j's component in FP64 (j = lane & 7);
// ms = this sample's MetzgerKN sweep rows (value + 4 derivatives per
// observation), unused by the other models.  Returns false when the
// reference skips the sample (MetzgerKN peak rescale outside its clamp).
// Otherwise lls = the log-likelihood (every lane), dl_tot = lane l's FP32
// total d loglik / d theta_{(l >> 2) & 7} (reduce_scatter8f), dlx = lane l's
// FP64 part of d loglik / d theta_{l & 7} from the upper limits at or near the
// reference's CDF floor (svi_deferred_pass), floored = 1 when one of them was
// at the floor.  The observations are taken in chunks of 2048: the FP32 loop
// marks the deferred ones in a per-lane bitmask of its 32-observation rounds,
// and the out-of-line pass after the loop evaluates them (only in the samples
// that have any), so the FP32 loop carries none of that code's registers.
template <int M>
__device__ __forceinline__ bool svi_sample_loglik(const float4* obs, int n, const float* pf, double th_j,
                                                  const float* ms, double& lls, float& dl_tot, double& dlx,
                                                  int& floored) {
    constexpr int np = n_params_of(M), se = se_idx_of(M);
    constexpr int CHUNK = 64 * 32;
    const int lane = threadIdx.x & 31;
    float sx = expf(pf[se]);
    float sx2 = sx * sx;
    float dll[8];
#pragma unroll
    for (int q = 0; q < 8; q++) dll[q] = 0.0f;
    Nll ll;
    ll.reset();
    dlx = 0.0;
    floored = 0;
    float scl = 1.0f;
    if constexpr (M == METZGER) {
        // predictions and derivatives of the normalised model, then the
        // reference's peak rescale (src/parametric.rs:2303-2323)
        float mx = -INFINITY;
        for (int i = lane; i < n; i += 32)
            if (obs[i].w >= 0.0f) mx = fmaxf(mx, ms[i * 5]);
        for (int kk = 16; kk; kk >>= 1) mx = fmaxf(mx, __shfl_xor_sync(FULL, mx, kk));
        bool skip_sample = false;
        if (mx > 1e-10f && isfinite(mx)) {
            float raw = 1.0f / mx;
            scl = fminf(fmaxf(raw, 0.1f), 10.0f);
            if (fabsf(raw - scl) / raw > 0.5f) skip_sample = true;
        }
        if (skip_sample) return false;  // warp-uniform: mx and scl are the warp's
    }
    for (int c0 = 0; c0 < n; c0 += CHUNK) {
        const int c1 = min(n, c0 + CHUNK);
        unsigned long long xm = 0;  // rounds of this chunk with a deferred observation of this lane
        for (int i = c0 + lane; i < c1; i += 32) {
            float4 ob = obs[i];
            bool defer = false;
            if constexpr (M == METZGER) {
                float pr = ms[i * 5] * scl;
                float gb[4];
                for (int q = 0; q < 4; q++) gb[q] = ms[i * 5 + 1 + q] * scl;
                float tv = fabsf(ob.w) + sx2;
                float stv = sqrtf(tv);
                if (ob.w < 0.0f) {
                    float z = (ob.z - pr) / stv;
                    ll.add(log_normal_cdf_f(z));
                    float ratio = upper_ratio_f32(z, defer);
                    for (int q = 0; q < 4; q++) if (isfinite(gb[q])) dll[q] += -ratio / stv * gb[q];
                    dll[se] += ratio * (-(ob.z - pr) * sx2 / (stv * tv));
                } else {
                    float res = ob.z - pr;
                    float it = 1.0f / tv;
                    float r2 = res * res;
                    ll.add(-0.5f * (r2 * it + logf(6.283185307179586f * tv)));
                    for (int q = 0; q < 4; q++) if (isfinite(gb[q])) dll[q] += res * it * gb[q];
                    dll[se] += (r2 * it * it - it) * sx2;
                }
            } else {
                float gb[MAXP];
                int st;
                float pr = model_grad_f32(M, pf, ob.x, ob.y, gb, st);
                if (st == ST_NONFINITE || !isfinite(pr)) continue;
                float tv = fabsf(ob.w) + sx2;
                float stv = sqrtf(tv);
                if (ob.w < 0.0f) {
                    float z = (ob.z - pr) / stv;
                    ll.add(log_normal_cdf_f(z));
                    float ratio = upper_ratio_f32(z, defer);
                    float dpred = -ratio / stv;
#pragma unroll
                    for (int q = 0; q < np; q++)
                        if (q != se && isfinite(gb[q])) dll[q] += dpred * gb[q];
                    dll[se] += ratio * (-(ob.z - pr) * sx2 / (stv * tv));
                } else {
                    float res = ob.z - pr;
                    float it = 1.0f / tv;
                    float r2 = res * res;
                    ll.add(-0.5f * (r2 * it + logf(6.283185307179586f * tv)));
#pragma unroll
                    for (int q = 0; q < np; q++)
                        if (q != se && isfinite(gb[q])) dll[q] += res * it * gb[q];
                    dll[se] += (r2 * it * it - it) * sx2;
                }
            }
            if (defer) xm |= 1ull << ((i - c0) >> 5);
        }
        if (__any_sync(FULL, xm != 0)) {
            const SviDeferred r = svi_deferred_pass<M>(obs, ms, scl, c0, xm, th_j, sx2);
            dlx += r.dlx;
            floored |= r.floored;
        }
    }
    lls = warp_sum_d((double)ll.s - (double)ll.c);
    dl_tot = reduce_scatter8f(dll);
    return true;
}

template <int M>
__device__ void svi_band(const DeviceBatch& d, int b) {
    const int lane = threadIdx.x & 31, j = lane & 7;
    const BandStats bs = d.stats[b];
    BandOut& o = d.out[b];
    if (!bs.valid || o.model != M) return;
    constexpr int np = n_params_of(M), se = se_idx_of(M);
    const int n = bs.n;
    const float4* obs = d.obs + bs.off;
    const bool own = j < np;  // this lane's component is a model parameter
    // prior of component j: centre (the PSO value, or the fixed centre of
    // sigma_extra) and variance
    const double init_j = own ? o.pso_params[j] : 0.0;
    const double pc_j = own ? (j == se ? c_pri_c[M][j] : init_j) : 0.0;
    const double pw2_j = own ? c_pri_w[M][j] * c_pri_w[M][j] : 1.0;
    // 1 / variance, formed once: the FP64 divisions of the step are its
    // costliest instructions on this part (a few are left: sqrt, Adam's step)
    const double ipw2_j = own ? 1.0 / pw2_j : 0.0;
    // lane i < 2 np owns variational parameter i (mu_i, then log sigma_i)
    double vp = 0.0, am = 0.0, av = 0.0;
    if (lane < np) vp = o.pso_params[lane];
    else if (lane < 2 * np) vp = -1.0;
    const double* eps_tab = d.svi_eps + (size_t)(np - 5) * SVI_STEPS * SVI_SAMPLES * 7;
    const double ln_2pie = 2.8378770664093453;  // ln(2 pi e)
    double ema = -INFINITY, best_ema = -INFINITY, final_elbo = -INFINITY;
    int no_imp = 0, steps = 0;
    // MetzgerKN: per step, lanes 0..15 sweep samples 0..3 (value + 4 derivatives per observation)
    float* mscr = d.scratch_svi + 20 * bs.off;
    struct ObsTimes {
        const float4* o;
        __device__ float operator()(int q) const { return o[q].x + o[q].y; }
    } otimes{obs};
    for (int step = 0; step < SVI_STEPS; step++) {
        steps = step + 1;
        const double mu_j = __shfl_sync(FULL, vp, j);
        const double ls_j = __shfl_sync(FULL, vp, (np + j) & 31);
        // sigma = e^(log sigma) in double-float on the FP32 pipe (log sigma is
        // clamped to [-6, 2]; ~1e-14 relative): the FP64 exp was the step's
        // costliest remaining FP64 call
        const double sg_j = own ? ff_to(ff_exp(ff_from(ls_j))) : 0.0;
        if constexpr (M == METZGER) {
            double mu[MAXP], sg[MAXP];
#pragma unroll
            for (int q = 0; q < np; q++) { mu[q] = __shfl_sync(FULL, mu_j, q); sg[q] = __shfl_sync(FULL, sg_j, q); }
            // lane 4 s + k sweeps sample s with the tangent of parameter k
            // only (the four-tangent sweep's arithmetic, split over lanes)
            const int smp = lane >> 2, tan = lane & 3;
            bool mz_ok = false;
            float mz_lp = 0.0f, mz_lpd = 0.0f;
            if (lane < 4 * SVI_SAMPLES) {
                const double* ep = eps_tab + ((size_t)step * SVI_SAMPLES + smp) * 7;
                float pv[MAXP];
                for (int q = 0; q < np; q++) pv[q] = (float)(mu[q] + sg[q] * ep[q]);
                mz_ok = metzger_dual_raw<1>(pv, tan, (float)bs.t_last, otimes, n, mscr + (size_t)smp * 5 * n, mz_lp,
                                            &mz_lpd);
            }
            __syncwarp();
            // normalise by the peak (its tangent included): each lane its
            // tangent column, then the value column
            if (lane < 4 * SVI_SAMPLES) {
                float* ms = mscr + (size_t)smp * 5 * n;
                const float ip = 1.0f / mz_lp;
                for (int q = 0; q < n; q++) {
                    const float y = ms[q * 5] * ip;
                    ms[q * 5 + 1 + tan] = mz_ok ? (ms[q * 5 + 1 + tan] - y * mz_lpd) * ip : 0.0f;
                }
            }
            __syncwarp();
            if (lane < 4 * SVI_SAMPLES && tan == 0) {
                float* ms = mscr + (size_t)smp * 5 * n;
                const float ip = 1.0f / mz_lp;
                for (int q = 0; q < n; q++) ms[q * 5] = mz_ok ? ms[q * 5] * ip : 0.0f;
            }
            __syncwarp();
        }
        double gmu_j = 0.0, gls_j = 0.0, elbo_sum = 0.0;
        for (int k = 0; k < SVI_SAMPLES; k++) {
            const double* ep = eps_tab + ((size_t)step * SVI_SAMPLES + k) * 7;
            const double eps_j = own ? ep[j] : 0.0;
            const double th_j = mu_j + sg_j * eps_j;
            float pf[MAXP];
#pragma unroll
            for (int q = 0; q < MAXP; q++) pf[q] = q < np ? __shfl_sync(FULL, (float)th_j, q) : 0.0f;
            double lls, dlx;
            float dl_tot;
            int floored;
            if (!svi_sample_loglik<M>(obs, n, pf, th_j, mscr + (size_t)k * 5 * n, lls, dl_tot, dlx, floored))
                continue;
            // lane j: total d loglik / d theta_j (FP32 terms, plus the FP64
            // terms of deferred upper limits), then its prior and ELBO terms
            const double dl_j = (double)__shfl_sync(FULL, dl_tot, (4 * j) & 31) + dlx;
            double lp_j = 0.0;
            if (own) {
                const double dd = th_j - pc_j;
                const double dq = dd * ipw2_j;
                lp_j = -0.5 * dd * dq;
                const double df = dl_j - dq;
                gmu_j += df;
                gls_j += df * sg_j * eps_j;
            }
            const double lp = dot8(lp_j, 1.0);
            elbo_sum += lls + lp;
        }
        const double ns = (double)SVI_SAMPLES;
        const double ent = dot8(own ? ls_j : 0.0, 1.0) + 0.5 * (double)np * ln_2pie;
        final_elbo = elbo_sum / ns + ent;
        // Adam, lane i owns variational parameter i
        const double gmu_i = __shfl_sync(FULL, gmu_j, lane & 7);
        const double gls_i = __shfl_sync(FULL, gls_j, (lane - np) & 7);
        double gi = 0.0;
        if (lane < np) gi = -(gmu_i / ns);
        else if (lane < 2 * np) gi = -(gls_i / ns + 1.0);
        // a component hit by a floored upper limit's ~1e285 term overflows its
        // second moment to +inf and stops, as in the reference
        if (lane < 2 * np && isfinite(gi)) {
            am = 0.9 * am + (1.0 - 0.9) * gi;
            av = 0.999 * av + (1.0 - 0.999) * gi * gi;
            const double mh = am * d.svi_adam_bc[step], vh = av * d.svi_adam_bc[SVI_STEPS + step];
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
        __syncwarp();  // MetzgerKN scratch rows are rewritten next step
    }
    const double ln4 = 1.3862943611198906;
    double out_v = lane < np ? vp : vp + ln4;
    if (lane < np) o.mu[lane] = out_v;
    else if (lane < 2 * np) o.log_sigma[lane - np] = out_v;
    if (lane >= np && lane < MAXP) o.mu[lane] = NAN;
    if (lane == 0) {
        for (int q = np; q < MAXP; q++) o.log_sigma[q] = NAN;
        o.elbo = final_elbo;
        o.svi_steps = steps;
    }
}

// One warp per band, in band_order (grouped by selected model, so that the
// warps of a model run together and share its code).
#ifndef LCF_SVI_BLOCK
#define LCF_SVI_BLOCK 128
#endif
__global__ void __launch_bounds__(LCF_SVI_BLOCK) svi_kernel(DeviceBatch d) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (warp >= d.n_bands) return;
    const int b = d.band_order[warp];
    const int m = d.out[b].model;
    if (m < 0) return;
    switch (m) {
        case BAZIN: svi_band<BAZIN>(d, b); break;
        case VILLAR: svi_band<VILLAR>(d, b); break;
        case TDE: svi_band<TDE>(d, b); break;
        case ARNETT: svi_band<ARNETT>(d, b); break;
        case MAGNETAR: svi_band<MAGNETAR>(d, b); break;
        case SHOCK: svi_band<SHOCK>(d, b); break;
        case AFTERGLOW: svi_band<AFTERGLOW>(d, b); break;
        default: svi_band<METZGER>(d, b); break;
    }
}

void launch_svi(const DeviceBatch& d, cudaStream_t s) {
    if (d.n_bands == 0) return;
    int block = LCF_SVI_BLOCK;
    int64_t threads = (int64_t)d.n_bands * 32;
    svi_kernel<<<(int)((threads + block - 1) / block), block, 0, s>>>(d);
}

// ---------------------------------------------------------------------------
// ELBO gradient check (lcf_svi_elbo_grad): one SVI step's Monte-Carlo ELBO
// estimate and its gradient at caller-given variational parameters and
// standard-normal draws, through svi_sample_loglik and the prior and entropy
// terms of svi_band — the SVI kernel's step without Adam.  One warp per
// parameter point; `mscr` holds 5 n floats (one MetzgerKN sweep) per warp.
// ---------------------------------------------------------------------------
template <int M>
__device__ void svi_grad_point(const float4* obs, int n, float t_last, const double* init, const double* vpar,
                               const double* eps, int n_samples, double* elbo_out, double* grad_out, int* flags_out,
                               float* mscr) {
    constexpr int np = n_params_of(M), se = se_idx_of(M);
    const int lane = threadIdx.x & 31, j = lane & 7;
    const bool own = j < np;
    const double init_j = own ? init[j] : 0.0;
    const double pc_j = own ? (j == se ? c_pri_c[M][j] : init_j) : 0.0;
    const double pw2_j = own ? c_pri_w[M][j] * c_pri_w[M][j] : 1.0;
    const double mu_j = own ? vpar[j] : 0.0;
    const double ls_j = own ? vpar[np + j] : 0.0;
    const double sg_j = own ? exp(ls_j) : 0.0;
    const double ln_2pie = 2.8378770664093453;  // ln(2 pi e)
    struct ObsTimes {
        const float4* o;
        __device__ float operator()(int q) const { return o[q].x + o[q].y; }
    } otimes{obs};
    double gmu_j = 0.0, gls_j = 0.0, elbo_sum = 0.0;
    int floored_any = 0, skipped = 0;
    for (int k = 0; k < n_samples; k++) {
        const double eps_j = own ? eps[(size_t)k * np + j] : 0.0;
        const double th_j = mu_j + sg_j * eps_j;
        float pf[MAXP];
#pragma unroll
        for (int q = 0; q < MAXP; q++) pf[q] = q < np ? __shfl_sync(FULL, (float)th_j, q) : 0.0f;
        if constexpr (M == METZGER) {
            if (lane == 0) metzger_dual_sweep(pf, t_last, otimes, n, mscr);
            __syncwarp();
        }
        double lls, dlx;
        float dl_tot;
        int floored;
        const bool ok = svi_sample_loglik<M>(obs, n, pf, th_j, mscr, lls, dl_tot, dlx, floored);
        __syncwarp();  // the MetzgerKN rows are rewritten by the next sample
        if (!ok) {
            skipped = 1;
            continue;
        }
        if (floored) floored_any = 1;
        const double dl_j = (double)__shfl_sync(FULL, dl_tot, (4 * j) & 31) + dlx;
        double lp_j = 0.0;
        if (own) {
            const double dd = th_j - pc_j;
            lp_j = -0.5 * dd * dd / pw2_j;
            const double df = dl_j + (-dd / pw2_j);
            gmu_j += df;
            gls_j += df * sg_j * eps_j;
        }
        const double lp = dot8(lp_j, 1.0);
        elbo_sum += lls + lp;
    }
    const double ns = (double)n_samples;
    const double ent = dot8(own ? ls_j : 0.0, 1.0) + 0.5 * (double)np * ln_2pie;
    if (lane < np) {
        grad_out[lane] = gmu_j / ns;
        grad_out[np + lane] = gls_j / ns + 1.0;
    }
    if (lane == 0) {
        *elbo_out = elbo_sum / ns + ent;
        *flags_out = floored_any | (skipped << 1);
    }
}

__global__ void __launch_bounds__(128) svi_grad_kernel(int model, const float4* obs, int n, float t_last,
                                                       const double* init, const double* vpar, int n_points,
                                                       const double* eps, int n_samples, double* elbo, double* grad,
                                                       int* flags, float* scratch) {
    const int p = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (p >= n_points) return;
    const int np = n_params_of(model);
    const double* vp = vpar + (size_t)p * 2 * np;
    const double* ep = eps + (size_t)p * n_samples * np;
    double* g = grad + (size_t)p * 2 * np;
    float* ms = scratch + (size_t)p * 5 * n;
    switch (model) {
        case BAZIN: svi_grad_point<BAZIN>(obs, n, t_last, init, vp, ep, n_samples, elbo + p, g, flags + p, ms); break;
        case VILLAR: svi_grad_point<VILLAR>(obs, n, t_last, init, vp, ep, n_samples, elbo + p, g, flags + p, ms); break;
        case TDE: svi_grad_point<TDE>(obs, n, t_last, init, vp, ep, n_samples, elbo + p, g, flags + p, ms); break;
        case ARNETT: svi_grad_point<ARNETT>(obs, n, t_last, init, vp, ep, n_samples, elbo + p, g, flags + p, ms); break;
        case MAGNETAR:
            svi_grad_point<MAGNETAR>(obs, n, t_last, init, vp, ep, n_samples, elbo + p, g, flags + p, ms);
            break;
        case SHOCK: svi_grad_point<SHOCK>(obs, n, t_last, init, vp, ep, n_samples, elbo + p, g, flags + p, ms); break;
        case AFTERGLOW:
            svi_grad_point<AFTERGLOW>(obs, n, t_last, init, vp, ep, n_samples, elbo + p, g, flags + p, ms);
            break;
        default: svi_grad_point<METZGER>(obs, n, t_last, init, vp, ep, n_samples, elbo + p, g, flags + p, ms); break;
    }
}

void launch_svi_grad(int model, const float4* obs, int n, float t_last, const double* init, const double* vpar,
                     int n_points, const double* eps, int n_samples, double* elbo, double* grad, int* flags,
                     float* scratch, cudaStream_t s) {
    if (n_points <= 0) return;
    const int block = 128;
    const int64_t threads = (int64_t)n_points * 32;
    svi_grad_kernel<<<(int)((threads + block - 1) / block), block, 0, s>>>(model, obs, n, t_last, init, vpar, n_points,
                                                                         eps, n_samples, elbo, grad, flags, scratch);
}

}  // namespace lcf
