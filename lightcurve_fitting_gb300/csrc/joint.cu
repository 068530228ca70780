// joint.cu — the joint multi-band Villar fit (fit_parametric_multiband,
// src/parametric.rs:3815-4131) that fit_parametric uses for sources with two
// or more bands when fit_all_models is false (:3742-3761).
//
// One block per (source, restart): 200 particles (threads 0..199 of 224)
// search the 7 * n_bands joint space (the most populated band's Villar
// parameters, then per-band offsets) with the reference's PSO (200
// particles, 1500 iterations, stall 60; seeds 42 / 137 / 271, restart 1
// seeded).  The source's bands are staged in shared memory; positions,
// velocities, their pre-iteration copies and the personal bests live in
// shared memory, column-major (parameter j of particle p at [j * 200 + p]).
// The reference's asynchronous global best (each particle moves with the
// best after the particles before it) is reproduced by speculative rounds,
// as in the per-band swarm: the particles from `start` on move with the
// current best and are evaluated; the first one that improves the best is
// accepted with those before it, and the rest are recomputed.  Costs are
// FP32 evaluations of the reference's band-balanced cost (Villar constraint
// on every band, 1e99 for a non-finite prediction, population prior on the
// reference band and the relative priors of de Soto et al. on the offsets)
// with FP64 band sums.
//
// joint_pick_kernel then writes each band's Villar parameters (reference +
// offset) into the per-band outputs, after which the per-band SVI / Laplace,
// refinements, magnitude chi2 and MultiBazin stages run unchanged.
#include <cuda_runtime.h>

#include "lcf_internal.cuh"
#include "models_f32.cuh"

namespace lcf {

#define FULL 0xffffffffu

constexpr int JP = 200;          // particles (src/parametric.rs:3951-3956)
constexpr int J_MAXIT = 1500;
constexpr int J_STALL = 60;
constexpr int J_THREADS = 224;

// de Soto et al. relative priors of the offsets, src/parametric.rs:3771-3786
static __device__ __constant__ float c_rel_mean[7] = {-0.015f * 2.302585093f, -0.001f, -0.095f * 2.302585093f,
                                                      -1.181f, -0.195f * 2.302585093f, -0.323f * 2.302585093f,
                                                      -0.025f * 2.302585093f};
static __device__ __constant__ float c_rel_sigma[7] = {0.08f * 2.302585093f, 0.008f, 0.25f * 2.302585093f, 1.5f,
                                                       0.35f * 2.302585093f, 0.25f * 2.302585093f,
                                                       0.30f * 2.302585093f};

struct JointBands {
    int nb;                 // bands in rank order
    int n[J_MAX_BANDS];     // observations per band
    int off[J_MAX_BANDS];   // first observation in the staged records
    int n_total;
};

// The joint cost of one particle (column p of the position array xs).
__device__ double joint_cost(const JointBands& jb, const float4* obs, const float* xs, int p) {
    float ref[7];
#pragma unroll
    for (int j = 0; j < 7; j++) ref[j] = xs[j * JP + p];
    {
        float c = VillarF::constraint(ref);
        if (c > 0.0f) return 1e12 + 10000.0 * (double)c;
    }
    const double scale = (double)jb.n_total / (double)jb.nb;
    double balanced = 0.0;
    for (int b = 0; b < jb.nb; b++) {
        float bp[7];
#pragma unroll
        for (int j = 0; j < 7; j++) bp[j] = b == 0 ? ref[j] : ref[j] + xs[(7 * b + j) * JP + p];
        if (b > 0) {
            float c = VillarF::constraint(bp);
            if (c > 0.0f) return 1e12 + 10000.0 * (double)c;
        }
        const float se = expf(bp[6]);
        const float se2 = se * se;
        VillarF e;
        e.init(bp);
        Nll acc;
        acc.reset();
        const float4* o = obs + jb.off[b];
        for (int i = 0; i < jb.n[b]; i++) {
            float4 r = o[i];
            int st = ST_OK;
            float pr = e.eval(r.x, r.y, st);
            acc.obs(r, pr, st, se2);
        }
        if (acc.nonfinite) return BIG_COST;
        if (acc.inf) return INFINITY;
        double band_nll = (double)acc.s - (double)acc.c;
        if (acc.big > -INFINITY) {
            if (acc.big > LN_DBL_MAX) return INFINITY;
            band_nll += exp((double)acc.big);
        }
        if (jb.n[b] > 0) balanced += (band_nll / (double)jb.n[b]) * scale;
    }
    // population prior of the reference band, relative priors of the offsets
    float lp = 0.0f;
#pragma unroll
    for (int j = 0; j < 7; j++) {
        float w = (float)c_pop_w[VILLAR][j];
        if (w > 0.0f) {
            float z = (ref[j] - (float)c_pop_c[VILLAR][j]) / w;
            lp += 0.5f * z * z;
        }
    }
    for (int b = 1; b < jb.nb; b++)
#pragma unroll
        for (int j = 0; j < 7; j++) {
            float z = (xs[(7 * b + j) * JP + p] - c_rel_mean[j]) / c_rel_sigma[j];
            lp += 0.5f * z * z;
        }
    return (balanced + (double)lp) / (double)max(jb.n_total, 1);
}

// Block-wide first index q in [start, JP) with improve[q] (or -1).
__device__ int block_first(bool flag, int* s_warp) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned m = __ballot_sync(FULL, flag);
    if (lane == 0) s_warp[warp] = m ? warp * 32 + __ffs(m) - 1 : 0x7fffffff;
    __syncthreads();
    int q = 0x7fffffff;
    for (int w = 0; w < J_THREADS / 32; w++) q = min(q, s_warp[w]);
    __syncthreads();
    return q == 0x7fffffff ? -1 : q;
}

__global__ void __launch_bounds__(J_THREADS) joint_pso_kernel(DeviceBatch d) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int js = blockIdx.x / 3, restart = blockIdx.x % 3;
    const int src = d.joint_src[js];
    const int tid = threadIdx.x;
    const bool live = tid < JP;
    __shared__ JointBands jb;
    __shared__ double s_cost[J_THREADS];
    __shared__ int s_warp[J_THREADS / 32];
    __shared__ double s_gc;
    __shared__ int s_D;
    // ---- the source's valid bands in rank order
    if (tid == 0) {
        int nb = 0, tot = 0;
        for (int r = 0; r < J_MAX_BANDS; r++) {
            for (int b = d.src_off[src]; b < d.src_off[src + 1]; b++) {
                const BandStats& bs = d.stats[b];
                if (bs.valid && bs.rank == r) {
                    jb.n[nb] = bs.n;
                    jb.off[nb] = tot;
                    tot += bs.n;
                    nb++;
                }
            }
        }
        jb.nb = nb;
        jb.n_total = tot;
        s_D = 7 * nb;
    }
    __syncthreads();
    const int nb = jb.nb, D = s_D;
    if (nb == 0) return;
    float4* obs = reinterpret_cast<float4*>(smem_raw);
    float* xs = reinterpret_cast<float*>(obs + d.joint_max_obs);
    float* vs = xs + (size_t)D * JP;
    float* x0s = vs + (size_t)D * JP;
    float* v0s = x0s + (size_t)D * JP;
    float* pbs = v0s + (size_t)D * JP;
    float* gs = pbs + (size_t)D * JP;      // global best, D
    float* lo = gs + J_MAX_D;              // bounds, D each
    float* hi = lo + J_MAX_D;
    // stage the bands' records
    for (int r = 0; r < nb; r++) {
        int b_idx = -1;
        for (int b = d.src_off[src]; b < d.src_off[src + 1]; b++)
            if (d.stats[b].valid && d.stats[b].rank == r) b_idx = b;
        const BandStats bs = d.stats[b_idx];
        for (int i = tid; i < bs.n; i += J_THREADS) obs[jb.off[r] + i] = d.obs[bs.off + i];
    }
    // ---- bounds (src/parametric.rs:3860-3882): Villar box with the reference
    // band's data-informed t0 (no lo < hi check), offsets at +-3 sigma
    __shared__ float s_tpeak;
    if (tid < D) {
        int j = tid % 7;
        if (tid < 7) { lo[tid] = (float)c_lo[VILLAR][tid]; hi[tid] = (float)c_hi[VILLAR][tid]; }
        else { lo[tid] = -3.0f * c_rel_sigma[j]; hi[tid] = 3.0f * c_rel_sigma[j]; }
    }
    __syncthreads();
    if (tid == 0) {
        int b_ref = -1;
        for (int b = d.src_off[src]; b < d.src_off[src + 1]; b++)
            if (d.stats[b].valid && d.stats[b].rank == 0) b_ref = b;
        const BandStats bs = d.stats[b_ref];
        lo[3] = (float)fmax(bs.t_first - 30.0, c_lo[VILLAR][3]);
        hi[3] = (float)fmin(bs.t_peak + 10.0, c_hi[VILLAR][3]);
        s_tpeak = (float)bs.t_peak;
    }
    __syncthreads();
    const float t_peak = s_tpeak;
    const float* dr = d.joint_draws + (size_t)restart * d.joint_draws_per_seed;
    const bool seeded = restart == 1;
    // ---- initialisation (pso_minimize :1677-1692; seeded :1189-1210)
    if (live) {
        for (int j = 0; j < D; j++) {
            float vmax = 0.5f * (hi[j] - lo[j]);
            float x, v;
            if (seeded) {
                if (tid == 0) {
                    float c;
                    if (j < 7) c = (float)c_pop_c[VILLAR][j];
                    else c = c_rel_mean[j % 7];
                    if (j == 3) c = t_peak - 5.0f;
                    x = fminf(fmaxf(c, lo[j]), hi[j]);
                    v = vmax * 0.2f * (2.0f * dr[j] - 1.0f);
                } else {
                    int o = D + 2 * D * (tid - 1);
                    x = lo[j] + dr[o + j] * (hi[j] - lo[j]);
                    v = vmax * 0.2f * (2.0f * dr[o + D + j] - 1.0f);
                }
            } else {
                int o = 2 * D * tid;
                x = lo[j] + dr[o + 2 * j] * (hi[j] - lo[j]);
                v = vmax * 0.2f * (2.0f * dr[o + 2 * j + 1] - 1.0f);
            }
            xs[j * JP + tid] = x;
            vs[j * JP + tid] = v;
            pbs[j * JP + tid] = x;
        }
    }
    __syncthreads();
    double c = live ? joint_cost(jb, obs, xs, tid) : INFINITY;
    double pbc = c;
    int evals = live ? 1 : 0;
    // global best after the sequential initial loop: the first strict minimum
    s_cost[tid] = c;
    __syncthreads();
    if (tid == 0) {
        double gc = INFINITY;
        int q = -1;
        for (int k = 0; k < JP; k++)
            if (s_cost[k] < gc) { gc = s_cost[k]; q = k; }
        s_gc = gc;
        s_warp[0] = q;
    }
    __syncthreads();
    {
        const int q = s_warp[0];
        if (tid < D) gs[tid] = q >= 0 ? xs[tid * JP + q] : 0.0f;
    }
    __syncthreads();
    const int base = seeded ? 2 * D * JP - D : 2 * D * JP;
    int stall = 0, it = 0;
    double prev = s_gc;
    for (; it < J_MAXIT; it++) {
        const float w = (float)(0.9 - (0.9 - 0.4) * (double)it / (double)J_MAXIT);
        if (live)
            for (int j = 0; j < D; j++) { x0s[j * JP + tid] = xs[j * JP + tid]; v0s[j * JP + tid] = vs[j * JP + tid]; }
        __syncthreads();
        int start = 0;
        while (start < JP) {
            const bool active = live && tid >= start;
            if (active) {
                const float* r = dr + base + (size_t)it * 2 * D * JP + (size_t)2 * D * tid;
                for (int j = 0; j < D; j++) {
                    float vmax = 0.5f * (hi[j] - lo[j]);
                    float x0 = x0s[j * JP + tid], v0 = v0s[j * JP + tid];
                    float vv = w * v0 + 1.5f * r[2 * j] * (pbs[j * JP + tid] - x0) + 1.5f * r[2 * j + 1] * (gs[j] - x0);
                    vv = fminf(fmaxf(vv, -vmax), vmax);
                    float nx = x0 + vv;
                    if (nx <= lo[j]) { xs[j * JP + tid] = lo[j]; vs[j * JP + tid] = 0.0f; }
                    else if (nx >= hi[j]) { xs[j * JP + tid] = hi[j]; vs[j * JP + tid] = 0.0f; }
                    else { xs[j * JP + tid] = nx; vs[j * JP + tid] = vv; }
                }
                c = joint_cost(jb, obs, xs, tid);
                evals++;
            }
            const double gc = s_gc;
            int q = block_first(active && c < gc, s_warp);
            const int qe = q < 0 ? JP - 1 : q;
            if (live && tid >= start && tid <= qe && c < pbc) {
                pbc = c;
                for (int j = 0; j < D; j++) pbs[j * JP + tid] = xs[j * JP + tid];
            }
            if (q >= 0) {
                if (tid < D) gs[tid] = xs[tid * JP + q];
                if (tid == q) s_gc = c;
            }
            __syncthreads();
            start = qe + 1;
        }
        const double gc = s_gc;
        if (prev - gc > 0.01 * fmax(fabs(prev), 1e-10)) {
            stall = 0;
            prev = gc;
        } else if (++stall >= J_STALL) {
            it++;
            break;
        }
    }
    // ---- result
    int tot = evals;
    for (int k = 16; k; k >>= 1) tot += __shfl_xor_sync(FULL, tot, k);
    if ((tid & 31) == 0) s_warp[tid >> 5] = tot;
    __syncthreads();
    if (tid == 0) {
        int all = 0;
        for (int w = 0; w < J_THREADS / 32; w++) all += s_warp[w];
        JointResult& R = d.joint_res[(size_t)js * 3 + restart];
        R.cost = s_gc;
        R.iters = it;
        R.evals = all;
        atomicAdd(&d.ctr->particle_obs_evals, (unsigned long long)all * (unsigned long long)jb.n_total);
    }
    if (tid < J_MAX_D) d.joint_res[(size_t)js * 3 + restart].params[tid] = tid < D ? gs[tid] : 0.0f;
}

// Best of the three restarts; each band (rank k) gets reference + offset k.
__global__ void joint_pick_kernel(DeviceBatch d) {
    const int js = blockIdx.x * blockDim.x + threadIdx.x;
    if (js >= d.n_joint) return;
    const int src = d.joint_src[js];
    const JointResult* R = d.joint_res + (size_t)js * 3;
    double best = INFINITY;
    int br = -1;
    for (int r = 0; r < 3; r++)
        if (R[r].cost < best) { best = R[r].cost; br = r; }
    for (int b = d.src_off[src]; b < d.src_off[src + 1]; b++) {
        const BandStats bs = d.stats[b];
        BandOut& o = d.out[b];
        o.model = -1;
        for (int m = 0; m < 8; m++) o.per_chi2[m] = NAN;
        if (!bs.valid || br < 0) continue;  // no finite joint cost: not fitted
        const int k = bs.rank;
        o.model = VILLAR;
        o.pso_cost = best;
        o.per_chi2[VILLAR] = isfinite(best) ? best : NAN;
        for (int j = 0; j < MAXP; j++) {
            double ref = (double)R[br].params[j];
            o.pso_params[j] = j < 7 ? (k == 0 ? ref : ref + (double)R[br].params[7 * k + j]) : NAN;
        }
    }
}

size_t joint_smem_bytes(int max_obs, int max_d) {
    return (size_t)max_obs * sizeof(float4) + ((size_t)5 * max_d * JP + 3 * J_MAX_D) * sizeof(float);
}

int launch_joint(const DeviceBatch& d, cudaStream_t s) {
    if (d.n_joint == 0) return 0;
    size_t smem = joint_smem_bytes(d.joint_max_obs, d.joint_max_d);
    if (cudaFuncSetAttribute(joint_pso_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return -1;
    joint_pso_kernel<<<d.n_joint * 3, J_THREADS, smem, s>>>(d);
    joint_pick_kernel<<<(d.n_joint + 127) / 128, 128, 0, s>>>(d);
    return 0;
}

}  // namespace lcf
