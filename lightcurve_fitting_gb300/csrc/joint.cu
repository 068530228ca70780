// joint.cu — the joint multi-band Villar fit (fit_parametric_multiband,
// src/parametric.rs:3815-4131) that fit_parametric uses for sources with two
// or more bands when fit_all_models is false (:3742-3761).
//
// A persistent grid of blocks takes (source, restart) tasks: 200 particles
// (two threads each, threads 0..399 of 448) search the 7 * n_bands joint space (the most
// populated band's Villar parameters, then per-band offsets) with the
// reference's PSO (200 particles, 1500 iterations, stall 60; seeds 42 / 137 /
// 271, restart 1 seeded).  The source's bands are staged in shared memory;
// positions, velocities and personal bests are double-float pairs in the
// block's global slice, column-major (parameter j of particle p at
// [j * 200 + p]).
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

#include <algorithm>

#include "ff.cuh"
#include "lcf_internal.cuh"
#include "models_f32.cuh"

namespace lcf {

#define FULL 0xffffffffu

constexpr int JP = 200;          // particles (src/parametric.rs:3951-3956)
constexpr int J_MAXIT = 1500;
constexpr int J_STALL = 60;
constexpr int J_THREADS = 448;  // two threads per particle

// de Soto et al. relative priors of the offsets, src/parametric.rs:3771-3786
static __device__ __constant__ float c_rel_mean[7] = {-0.015f * 2.302585093f, -0.001f, -0.095f * 2.302585093f,
                                                      -1.181f, -0.195f * 2.302585093f, -0.323f * 2.302585093f,
                                                      -0.025f * 2.302585093f};
static __device__ __constant__ float c_rel_sigma[7] = {0.08f * 2.302585093f, 0.008f, 0.25f * 2.302585093f, 1.5f,
                                                       0.35f * 2.302585093f, 0.25f * 2.302585093f,
                                                       0.30f * 2.302585093f};

// the same in FP64 for the box and the seed particle (as the reference
// computes them)
static __device__ __constant__ double c_rel_mean64[7] = {-0.015 * 2.302585092994045684, -0.001,
                                                         -0.095 * 2.302585092994045684, -1.181,
                                                         -0.195 * 2.302585092994045684, -0.323 * 2.302585092994045684,
                                                         -0.025 * 2.302585092994045684};
static __device__ __constant__ double c_rel_sigma64[7] = {0.08 * 2.302585092994045684, 0.008,
                                                          0.25 * 2.302585092994045684, 1.5,
                                                          0.35 * 2.302585092994045684, 0.25 * 2.302585092994045684,
                                                          0.30 * 2.302585092994045684};

struct JointBands {
    int nb;                 // bands in rank order
    int n[J_MAX_BANDS];     // observations per band
    int off[J_MAX_BANDS];   // first observation in the staged records
    int n_total;
    // the band balancing (n_total / nb) / n[b] and 1 / max(n_total, 1),
    // formed once per task: the FP64 divisions of the reference's cost
    // (src/parametric.rs:3815-4131) become multiplications, which move the
    // cost by ~1e-16, far below its FP32 evaluation's ~1e-7
    double w[J_MAX_BANDS];
    double inv_total;
    ff wf[J_MAX_BANDS];     // the same as double-float pairs (the cost's sums run on the FP32 pipe)
    ff inv_total_f;
};

// The joint cost of one particle (column p of the position array xs),
// evaluated by the particle's two threads (h = 0, 1: observations h, h + 2,
// ...; pm = the pair's lane mask).  Each band's partial sums are combined
// before any decision, by a commutative sum, so both threads return the same
// cost.
__device__ double joint_cost(const JointBands& jb, const float4* obs, const float* xs, int p, int h, unsigned pm) {
    float ref[7];
#pragma unroll
    for (int j = 0; j < 7; j++) ref[j] = xs[j * JP + p];
    {
        float c = VillarF::constraint(ref);
        if (c > 0.0f) return 1e12 + 10000.0 * (double)c;
    }
    // the band sums as double-float pairs: ~1e-14 relative, far below the FP32
    // terms' own error, on the FP32 pipe instead of FP64's 1/64 rate; ff_add
    // is commutative, so both threads of the pair form the same cost
    ff balanced = ffm(0.0f, 0.0f);
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
        for (int i = h; i < jb.n[b]; i += 2) {
            float4 r = o[i];
            int st = ST_OK;
            float pr = e.eval(r.x, r.y, st);
            acc.obs(r, pr, st, se2);
        }
        const ff part = ff_add(ffm(acc.s, 0.0f), -acc.c);
        ff band_nll = ff_add(part, ffm(__shfl_xor_sync(pm, part.hi, 1), __shfl_xor_sync(pm, part.lo, 1)));
        const float ob = __shfl_xor_sync(pm, acc.big, 1);
        float big = acc.big;
        if (ob > -INFINITY) big = big > -INFINITY ? fmaxf(big, ob) + log1pf(expf(-fabsf(big - ob))) : ob;
        const int fl = acc.nonfinite | (acc.inf << 1);
        const int flags = fl | __shfl_xor_sync(pm, fl, 1);
        if (flags & 1) return BIG_COST;
        if (flags & 2) return INFINITY;
        if (big > -INFINITY) {
            if (big > LN_DBL_MAX) return INFINITY;
            band_nll = ff_add(band_nll, ff_from(exp((double)big)));
        }
        if (jb.n[b] > 0) balanced = ff_add(balanced, ff_mul(band_nll, jb.wf[b]));
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
    return ff_to(ff_mul(ff_add(balanced, lp), jb.inv_total_f));
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

// The persistent joint swarm: each block takes (source, restart) tasks from a
// device counter.  Positions, velocities and personal bests are double-float
// pairs, private to each particle's thread and kept in the block's slice of
// joint_state (L1/L2-resident, coalesced: parameter j of particle p at
// [j * 200 + p]), so that shared memory holds only the staged observations
// and up to four blocks share an SM.  They move with the reference's FP64
// draws and box:
// rounding only the joint swarm's positions to FP32 in the FP64
// restatement moves the joint cost of 29 of the reference's 30 real ZTF
// sources by more than 1e-4, 13 of them by more than 1 % (up to 72 %).  A
// trial move is evaluated in FP32 at its leading floats (xt) and dropped;
// the particles accepted in a round recompute the same move (same inputs,
// the global best not yet updated) and commit it, so the particles not yet
// accepted still hold their iteration-start state and no copy of it is kept.
__global__ void __launch_bounds__(J_THREADS) joint_pso_kernel(DeviceBatch d) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int tid = threadIdx.x;
    const int p = tid >> 1, h = tid & 1;       // particle, half
    const unsigned pm = 3u << (tid & 30);      // the particle's two lanes
    const bool live = p < JP;
    __shared__ JointBands jb;
    __shared__ int s_warp[J_THREADS / 32];
    __shared__ double s_gc;
    __shared__ int s_task;
    __shared__ ff s_lo[J_MAX_D], s_hi[J_MAX_D], s_vm[J_MAX_D], s_g[J_MAX_D];
    __shared__ double s_tpeak;
    const int DM = d.joint_max_d;
    float4* obs = reinterpret_cast<float4*>(smem_raw);
    // the block's slice of the swarm state: high and low halves of the
    // positions, velocities and personal bests, and the trial positions
    float* xh = d.joint_state + (size_t)blockIdx.x * JOINT_STATE_ARRAYS * DM * JP;
    float* xl = xh + (size_t)DM * JP;
    float* vh = xl + (size_t)DM * JP;
    float* vl = vh + (size_t)DM * JP;
    float* pbh = vl + (size_t)DM * JP;
    float* pl = pbh + (size_t)DM * JP;
    float* xt = pl + (size_t)DM * JP;
    const int n_tasks = 3 * d.n_joint;
    while (true) {
        __syncthreads();
        if (tid == 0) s_task = atomicAdd(&d.ctr->joint_head, 1);
        __syncthreads();
        const int task = s_task;
        if (task >= n_tasks) break;
        const int js = task / 3, restart = task % 3;
        const int src = d.joint_src[js];
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
            const double scale = (double)tot / (double)max(nb, 1);
            for (int b = 0; b < nb; b++) {
                jb.w[b] = jb.n[b] > 0 ? scale / (double)jb.n[b] : 0.0;
                jb.wf[b] = ff_from(jb.w[b]);
            }
            jb.inv_total = 1.0 / (double)max(tot, 1);
            jb.inv_total_f = ff_from(jb.inv_total);
        }
        __syncthreads();
        const int nb = jb.nb, D = 7 * nb;
        if (nb == 0) continue;
        // stage the bands' records
        for (int r = 0; r < nb; r++) {
            int b_idx = -1;
            for (int b = d.src_off[src]; b < d.src_off[src + 1]; b++)
                if (d.stats[b].valid && d.stats[b].rank == r) b_idx = b;
            const BandStats bs = d.stats[b_idx];
            for (int i = tid; i < bs.n; i += J_THREADS) obs[jb.off[r] + i] = d.obs[bs.off + i];
        }
        // ---- bounds in FP64 (src/parametric.rs:3860-3882): Villar box with the
        // reference band's data-informed t0 (no lo < hi check), offsets at
        // +-3 sigma of the relative priors; vmax = (hi - lo) / 2
        if (tid == 0) {
            int b_ref = -1;
            for (int b = d.src_off[src]; b < d.src_off[src + 1]; b++)
                if (d.stats[b].valid && d.stats[b].rank == 0) b_ref = b;
            const BandStats bs = d.stats[b_ref];
            s_tpeak = bs.t_peak;
            for (int j = 0; j < D; j++) {
                double lo, hi;
                if (j < 7) {
                    lo = c_lo[VILLAR][j];
                    hi = c_hi[VILLAR][j];
                    if (j == 3) {
                        lo = fmax(bs.t_first - 30.0, lo);
                        hi = fmin(bs.t_peak + 10.0, hi);
                    }
                } else {
                    lo = -3.0 * c_rel_sigma64[j % 7];
                    hi = 3.0 * c_rel_sigma64[j % 7];
                }
                s_lo[j] = ff_from(lo);
                s_hi[j] = ff_from(hi);
                s_vm[j] = ff_from(__dmul_rn(0.5, __dsub_rn(hi, lo)));
            }
        }
        __syncthreads();
        const double t_peak = s_tpeak;
        const double* dr = d.joint_draws64 + (size_t)restart * d.joint_init_per_seed;
        const float2* d15 = d.joint_draws15 + (size_t)restart * d.joint_draws_per_seed;
        const bool seeded = restart == 1;
        // ---- initialisation (pso_minimize :1677-1692; seeded :1189-1210) in
        // FP64 without contractions; the seed particle (:3884-3895) is the
        // population prior centre with t0 = t_peak - 5 and the relative
        // priors' means, clamped to the box
        if (live) {
            for (int j = h; j < D; j += 2) {
                const double lo = ff_to(s_lo[j]), hi = ff_to(s_hi[j]), vmax = ff_to(s_vm[j]);
                double x, v;
                if (seeded) {
                    if (p == 0) {
                        double c = j < 7 ? c_pop_c[VILLAR][j] : c_rel_mean64[j % 7];
                        if (j == 3) c = t_peak - 5.0;
                        x = fmin(fmax(c, lo), hi);
                        v = __dmul_rn(__dmul_rn(vmax, 0.2), __dsub_rn(2.0 * dr[j], 1.0));
                    } else {
                        const int o = D + 2 * D * (p - 1);
                        x = __dadd_rn(lo, __dmul_rn(dr[o + j], __dsub_rn(hi, lo)));
                        v = __dmul_rn(__dmul_rn(vmax, 0.2), __dsub_rn(2.0 * dr[o + D + j], 1.0));
                    }
                } else {
                    const int o = 2 * D * p;
                    x = __dadd_rn(lo, __dmul_rn(dr[o + 2 * j], __dsub_rn(hi, lo)));
                    v = __dmul_rn(__dmul_rn(vmax, 0.2), __dsub_rn(2.0 * dr[o + 2 * j + 1], 1.0));
                }
                const ff xf = ff_from(x), vf = ff_from(v);
                const size_t k = (size_t)j * JP + p;
                xh[k] = xf.hi;
                xl[k] = xf.lo;
                vh[k] = vf.hi;
                vl[k] = vf.lo;
                pbh[k] = xf.hi;
                pl[k] = xf.lo;
                xt[k] = xf.hi;
            }
        }
        __syncthreads();
        double c = live ? joint_cost(jb, obs, xt, p, h, pm) : INFINITY;
        double pbc = c;
        int evals = live && h == 0 ? 1 : 0;
        // global best after the sequential initial loop: the first strict
        // minimum, in particle order
        {
            __shared__ double s_min[J_THREADS / 32];
            double mn = c;
            for (int k = 16; k; k >>= 1) mn = fmin(mn, __shfl_xor_sync(FULL, mn, k));
            if ((tid & 31) == 0) s_min[tid >> 5] = mn;
            __syncthreads();
            double g = INFINITY;
            for (int w = 0; w < J_THREADS / 32; w++) g = fmin(g, s_min[w]);
            const int qt = block_first(live && h == 0 && c == g && g < INFINITY, s_warp);
            const int q = qt >= 0 ? qt >> 1 : -1;
            if (tid == 0) s_gc = q >= 0 ? g : INFINITY;
            if (tid < D) s_g[tid] = q >= 0 ? ffm(xh[(size_t)tid * JP + q], xl[(size_t)tid * JP + q]) : ffm(0.0f, 0.0f);
        }
        __syncthreads();
        const int base = seeded ? 2 * D * JP - D : 2 * D * JP;
        const double inv_iters = 1.0 / (double)J_MAXIT;
        int stall = 0, it = 0;
        double prev = s_gc;
        for (; it < J_MAXIT; it++) {
            const double wd = __dsub_rn(0.9, __dmul_rn(__dmul_rn(__dsub_rn(0.9, 0.4), (double)it), inv_iters));
            const ff w = ff_from(wd);
            const float2* r = d15 + base + (size_t)it * 2 * D * JP + (size_t)2 * D * p;
            // the move of this particle from its iteration-start state, the
            // pair's two threads taking alternate dimensions: trial (leading
            // floats to xt) or commit (the full state, and the personal best
            // when `to_pb`).  A plain loop: unrolling it by band needed ~128
            // registers a thread and measured 20 % slower.
            auto move = [&](bool commit, bool to_pb) {
                for (int j = h; j < D; j += 2) {
                    const size_t k = (size_t)j * JP + p;
                    ff xn, vn;
                    ff_move(ffm(xh[k], xl[k]), ffm(vh[k], vl[k]), ffm(pbh[k], pl[k]), s_g[j], w, r[2 * j],
                            r[2 * j + 1], s_vm[j], s_lo[j], s_hi[j], xn, vn);
                    if (commit) {
                        xh[k] = xn.hi;
                        xl[k] = xn.lo;
                        vh[k] = vn.hi;
                        vl[k] = vn.lo;
                        if (to_pb) {
                            pbh[k] = xn.hi;
                            pl[k] = xn.lo;
                        }
                    } else {
                        xt[k] = xn.hi;
                    }
                }
            };
            int start = 0;
            while (start < JP) {
                const bool active = live && p >= start;
                if (active) {
                    move(false, false);
                    __syncwarp(pm);  // the pair's trial dimensions, before its cost
                    c = joint_cost(jb, obs, xt, p, h, pm);
                    evals += h == 0;
                }
                const double gc = s_gc;
                const int qt = block_first(active && h == 0 && c < gc, s_warp);
                const int q = qt >= 0 ? qt >> 1 : -1;
                const int qe = q < 0 ? JP - 1 : q;
                if (active && p <= qe) {
                    const bool to_pb = c < pbc;
                    move(true, to_pb);
                    if (to_pb) pbc = c;
                }
                __syncthreads();
                if (q >= 0) {
                    if (tid < D) s_g[tid] = ffm(xh[(size_t)tid * JP + q], xl[(size_t)tid * JP + q]);
                    if (tid == 2 * q) s_gc = c;
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
        __syncthreads();
        if ((tid & 31) == 0) s_warp[tid >> 5] = tot;
        __syncthreads();
        JointResult& R = d.joint_res[(size_t)js * 3 + restart];
        if (tid == 0) {
            int all = 0;
            for (int w = 0; w < J_THREADS / 32; w++) all += s_warp[w];
            R.cost = s_gc;
            R.iters = it;
            R.evals = all;
            atomicAdd(&d.ctr->particle_obs_evals, (unsigned long long)all * (unsigned long long)jb.n_total);
        }
        if (tid < J_MAX_D) {
            R.params[tid] = tid < D ? s_g[tid].hi : 0.0f;
            R.params_lo[tid] = tid < D ? s_g[tid].lo : 0.0f;
        }
    }
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
            if (j >= 7) { o.pso_params[j] = NAN; continue; }
            const double ref = (double)R[br].params[j] + (double)R[br].params_lo[j];
            const double off = (double)R[br].params[7 * k + j] + (double)R[br].params_lo[7 * k + j];
            o.pso_params[j] = k == 0 ? ref : ref + off;
        }
    }
}

size_t joint_smem_bytes(int max_obs, int max_d) {
    (void)max_d;
    return (size_t)max_obs * sizeof(float4);
}

// Blocks of the persistent joint swarm: as many as are resident at once.
int joint_grid(int max_obs, int max_d, int num_sms) {
    const size_t smem = joint_smem_bytes(max_obs, max_d);
    int per_sm = 0;
    if (cudaFuncSetAttribute(joint_pso_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, joint_pso_kernel, J_THREADS, smem) != cudaSuccess)
        per_sm = 1;
    return std::max(1, per_sm) * num_sms;
}

int launch_joint(const DeviceBatch& d, cudaStream_t s) {
    if (d.n_joint == 0) return 0;
    size_t smem = joint_smem_bytes(d.joint_max_obs, d.joint_max_d);
    if (cudaFuncSetAttribute(joint_pso_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return -1;
    const int grid = std::min(d.joint_grid, 3 * d.n_joint);
    joint_pso_kernel<<<grid, J_THREADS, smem, s>>>(d);
    joint_pick_kernel<<<(d.n_joint + 127) / 128, 128, 0, s>>>(d);
    return 0;
}

}  // namespace lcf
