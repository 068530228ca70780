// pso.cu — band preparation and the persistent particle-swarm kernel.
//
// One warp runs one swarm (a PSO task: band x model x restart, a profile-t0
// run, or a MultiBazin run); lane p holds particle p (30 of 32 lanes).  The
// band's observations are staged once per task into the warp's slice of
// shared memory with a TMA bulk copy and read by all lanes at the same index
// (broadcast), so the inner loop touches no HBM.
//
// The reference updates the global best *inside* its particle loop
// (pso_minimize, src/parametric.rs:1698-1741): particle p moves towards the
// global best as left by particles 0..p-1 of the same iteration.  The warp
// reproduces that order exactly with speculative rounds: all particles move
// and are evaluated in parallel against the current best; the first lane q
// whose cost beats the best is accepted together with lanes < q, the best is
// updated, and lanes > q are moved again from their pre-iteration state.
// Every iteration therefore costs 1 + (number of global-best improvements)
// rounds.  The random draws are the reference's own: rand's SmallRng
// (xoshiro256++) seeded with 42/137/271 produces a stream that does not
// depend on the data, so the host generates each seed's stream once and the
// kernel indexes it by (iteration, particle, dimension) — a counter-based
// view of the reference's sequence.
#include <cuda_runtime.h>

#include <algorithm>

#include "lane_cost.cuh"
#include "lcf_internal.cuh"
#include "models_f32.cuh"
#include "swarm_cost.cuh"

namespace lcf {

#ifndef FULL
#define FULL 0xffffffffu
#endif

// ---------------------------------------------------------------------------
// Band preparation (src/parametric.rs:3581-3630): warp per band.
// ---------------------------------------------------------------------------
__global__ void prep_kernel(DeviceBatch d) {
    int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    if (warp >= d.n_bands) return;
    int b = warp;
    int64_t o0 = d.band_off[b], o1 = d.band_off[b + 1];
    int n = (int)(o1 - o0);
    BandStats st;
    st.off = o0;
    st.n = n;
    // source of this band and rank by count inside the source (stable)
    int lo = 0, hi = d.n_sources;
    while (hi - lo > 1) {
        int mid = (lo + hi) >> 1;
        if (d.src_off[mid] <= b) lo = mid; else hi = mid;
    }
    int s = lo;
    st.source = s;
    // peak flux: fold(f64::MIN, f64::max) (NaN ignored)
    double peak = -1.7976931348623157e308;
    double tmin = INFINITY, tmax = -INFINITY;
    for (int i = lane; i < n; i += 32) {
        double f = d.flux[o0 + i];
        peak = fmax(peak, f);
        double t = d.times[o0 + i];
        tmin = fmin(tmin, t);
        tmax = fmax(tmax, t);
    }
    for (int k = 16; k; k >>= 1) {
        peak = fmax(peak, __shfl_xor_sync(FULL, peak, k));
        tmin = fmin(tmin, __shfl_xor_sync(FULL, tmin, k));
        tmax = fmax(tmax, __shfl_xor_sync(FULL, tmax, k));
    }
    int valid = (n > 0 && peak > 0.0) ? 1 : 0;
    // rank: bands of the same source with more points, or equal points and a
    // lower index, come first; invalid bands are not ranked
    int rank = 0;
    if (valid) {
        for (int ob = d.src_off[s] + lane; ob < d.src_off[s + 1]; ob += 32) {
            if (ob == b) continue;
            int64_t q0 = d.band_off[ob], q1 = d.band_off[ob + 1];
            int nb = (int)(q1 - q0);
            bool v2 = false;
            if (nb > 0) {
                double pk = -1.7976931348623157e308;
                for (int64_t i = q0; i < q1; i++) pk = fmax(pk, d.flux[i]);
                v2 = pk > 0.0;
            }
            if (v2 && (nb > n || (nb == n && ob < b))) rank++;
        }
        for (int k = 16; k; k >>= 1) rank += __shfl_xor_sync(FULL, rank, k);
    }
    // first maximum of the normalised detections / of all fluxes (original order)
    double best_det = -INFINITY, best_all = -INFINITY;
    int idx_det = 0x7fffffff, idx_all = 0x7fffffff;
    for (int i = lane; i < n; i += 32) {
        double f = d.flux[o0 + i], e = d.err[o0 + i];
        double fn = f / peak;
        bool up = e > 0.0 && (f / e) < 3.0;
        if (!up && fn > best_det) { best_det = fn; idx_det = i; }
        if (fn > best_all) { best_all = fn; idx_all = i; }
    }
    for (int k = 16; k; k >>= 1) {
        double bd = __shfl_xor_sync(FULL, best_det, k);
        int id = __shfl_xor_sync(FULL, idx_det, k);
        if (bd > best_det || (bd == best_det && id < idx_det)) { best_det = bd; idx_det = id; }
        double ba = __shfl_xor_sync(FULL, best_all, k);
        int ia = __shfl_xor_sync(FULL, idx_all, k);
        if (ba > best_all || (ba == best_all && ia < idx_all)) { best_all = ba; idx_all = ia; }
    }
    st.valid = valid;
    st.rank = valid ? rank : -1;
    st.joint = d.joint_flag ? (int32_t)d.joint_flag[s] : 0;
    st.pad = 0;
    st.peak = peak;
    st.t_first = tmin;
    st.t_last = tmax;
    // peak_time starts at times[0] and is replaced by the first strict maximum
    st.t_peak = n > 0 ? d.times[o0 + (idx_det == 0x7fffffff ? 0 : idx_det)] : 0.0;
    st.t_peak_all = n > 0 ? d.times[o0 + (idx_all == 0x7fffffff ? 0 : idx_all)] : 0.0;
    // stable time order: position of observation i = #{j: t_j < t_i or (t_j == t_i and j < i)}
    bool sorted = true;
    for (int i = lane; i + 1 < n; i += 32)
        if (d.times[o0 + i + 1] < d.times[o0 + i]) sorted = false;
    sorted = __all_sync(FULL, sorted);
    // The double-float copy for the polish holds the band's detections first,
    // then its upper limits, each in time order: the lanes of one iteration of
    // its observation loop then take the same branch of the term.
    int n_det = 0;
    for (int i = lane; i < n; i += 32) {
        const double f = d.flux[o0 + i], e = d.err[o0 + i];
        n_det += (e > 0.0 && (f / e) < 3.0) ? 0 : 1;
    }
    for (int k = 16; k; k >>= 1) n_det += __shfl_xor_sync(FULL, n_det, k);
    int det_run = 0;
    for (int base = 0; base < n; base += 32) {
        const int i = base + lane;
        const bool in = i < n;
        double t = 0.0, f = 0.0, e = 0.0;
        bool up = false;
        if (in) {
            t = d.times[o0 + i];
            f = d.flux[o0 + i];
            e = d.err[o0 + i];
            up = e > 0.0 && (f / e) < 3.0;
        }
        const unsigned detm = __ballot_sync(FULL, in && !up);
        if (in) {
            int pos = i, pos_ff;
            if (!sorted) {
                pos = 0;
                int cls = 0;  // earlier observations of the same class
                for (int j = 0; j < n; j++) {
                    const double tj = d.times[o0 + j];
                    if (tj < t || (tj == t && j < i)) {
                        pos++;
                        const double fj = d.flux[o0 + j], ej = d.err[o0 + j];
                        cls += ((ej > 0.0 && (fj / ej) < 3.0) == up) ? 1 : 0;
                    }
                }
                pos_ff = up ? n_det + cls : cls;
            } else {
                const int det_before = det_run + __popc(detm & ((1u << lane) - 1u));
                pos_ff = up ? n_det + (i - det_before) : det_before;
            }
            const double fn = f / peak, fe = e / peak;
            const double uf = 3.0 * e / peak;
            const double var = fe * fe + 1e-10;
            const int64_t q = o0 + pos;
            const float th = (float)t;
            float4 rec;
            rec.x = th;
            rec.y = (float)(t - (double)th);
            rec.z = (float)(up ? uf : fn);
            rec.w = up ? -(float)var : (float)var;
            d.obs[q] = rec;
            d.t64[q] = t;
            d.f64[q] = fn;
            d.fe64[q] = fe;
            d.var64[q] = var;
            d.uf64[q] = uf;
            d.up[q] = up ? 1 : 0;
            {
                const double y = up ? uf : fn;
                const float yh = (float)y, vh = (float)var, vl = (float)(var - (double)vh);
                d.ffa[o0 + pos_ff] = make_float4(th, rec.y, yh, (float)(y - (double)yh));
                d.ffb[o0 + pos_ff] = up ? make_float2(-vh, -vl) : make_float2(vh, vl);
            }
            d.mag64[q] = -2.5 * log10(f) + 23.9;
        }
        det_run += __popc(detm);
    }
    if (lane == 0) d.stats[b] = st;
}

void launch_prep(const DeviceBatch& d, cudaStream_t s) {
    if (d.n_bands == 0) return;
    int block = 256;
    int grid = (int)(((int64_t)d.n_bands * 32 + block - 1) / block);
    prep_kernel<<<grid, block, 0, s>>>(d);
}

// ---------------------------------------------------------------------------
// TMA bulk copy of a band into shared memory (cp.async.bulk + mbarrier)
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// Issue the copy (one lane).  Sizes and addresses are multiples of 16 bytes.
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}
// Bounded wait on the barrier phase: at most `polls` polls; returns false if
// the bound expired (at once for polls = 0).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t phase, int polls) {
    uint32_t done = 0;
    for (int it = 0; it < polls; it++) {
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(smem_u32(bar)), "r"(phase)
            : "memory");
        if (done) return true;
    }
    return false;
}

// ---------------------------------------------------------------------------
// The PSO kernel
// ---------------------------------------------------------------------------
struct WarpSmem {
    uint64_t bar;
    uint64_t pad;
    // exact-trajectory swarms: box, velocity limit and global best of the
    // current run, double-float, one per swarm dimension
    ff lo[7], hi[7], vmax[7], g[7];
    // and the low halves of each lane's double-float state (the high halves
    // stay in registers): [state][dimension][lane], state = position,
    // velocity, personal best, position and velocity at the iteration start
    float lo_state[5][7][32];
    double s_pos[8];  // a position the warp evaluates in FP64 (MultiBazin K = 1 near ties)
};
// The MultiBazin instantiations (swarm dimensions 4K + 2 = 10, 14, 18): the
// same, with three state planes (position, velocity, personal best; the
// MultiBazin swarm recomputes a move instead of keeping its start state).
template <int MAXD>
struct WarpSmemMB {
    uint64_t bar;
    uint64_t pad;
    ff lo[MAXD], hi[MAXD], vmax[MAXD], g[MAXD];
    float lo_state[3][MAXD][32];
    double s_pos[MAXD];  // a position the warp evaluates in FP64 (near ties)
};
template <int MAXD>
struct WarpSmemOf {
    using type = WarpSmemMB<MAXD>;
};
template <>
struct WarpSmemOf<7> {
    using type = WarpSmem;
};

// One swarm run (pso_minimize / pso_minimize_seeded, src/parametric.rs:1646-1757,
// 1160-1266) of a task of kind KIND: warp = swarm, lane = particle.
template <int MAXD, int KIND>
__device__ __forceinline__ void run_swarm(const DeviceBatch& d, const PsoTask& task, const BandStats& bs, TaskCtx& t,
                                          int slot, int gwarp) {
    const int lane = threadIdx.x & 31;
    // dimensions and bounds
    float lo[MAXD], hi[MAXD], seedp[MAXD];
    bool seeded = (task.flags & TASK_SEEDED) != 0;
    if constexpr (KIND < KIND_MB1) {
        constexpr int m = KIND;
        t.model = m;
        t.np = n_params_of(m);
        t.t0i = t0_idx_of(m);
        double dlo[MAXP], dhi[MAXP];
        for (int j = 0; j < MAXP; j++) { dlo[j] = c_lo[m][j]; dhi[j] = c_hi[m][j]; }
        if (task.flags & TASK_T0_BOUNDS) {
            // data-informed t0 bounds, src/parametric.rs:1881-1909
            double t0_lo = fmax(bs.t_first - 30.0, dlo[t.t0i]);
            double t0_hi = fmin(bs.t_peak + 10.0, dhi[t.t0i]);
            if (t0_lo < t0_hi) { dlo[t.t0i] = t0_lo; dhi[t.t0i] = t0_hi; }
        }
        if (task.flags & TASK_T0_FIXED) {
            t.D = t.np - 1;
            int k = 0;
            for (int j = 0; j < t.np; j++) {
                if (j == t.t0i) continue;
                if (k < MAXD) { lo[k] = (float)dlo[j]; hi[k] = (float)dhi[j]; }
                k++;
            }
        } else {
            t.D = t.np;
            for (int j = 0; j < t.np && j < MAXD; j++) { lo[j] = (float)dlo[j]; hi[j] = (float)dhi[j]; }
        }
        if (seeded) {
            // seed particles of pso_fit_single_model, src/parametric.rs:1924-1964
            for (int j = 0; j < t.np && j < MAXD; j++) {
                double c = c_pop_c[m][j];
                double v = fmin(fmax(c, dlo[j]), dhi[j]);
                seedp[j] = (float)v;
            }
            double t0s = task.restart == 1 ? bs.t_peak - 5.0 : bs.t_first - 15.0;
            if (t.t0i < MAXD) seedp[t.t0i] = (float)fmin(fmax(t0s, dlo[t.t0i]), dhi[t.t0i]);
        }
    } else {
        constexpr int K = KIND - KIND_MB1 + 1;
        t.model = BAZIN;
        t.np = 4 * K + 2;
        t.D = t.np;
        t.t0i = -1;
        // multi_bazin_bounds, src/parametric.rs:958-970
        for (int c = 0; c < K && 4 * c + 3 < MAXD; c++) {
            lo[4 * c] = -3.0f; hi[4 * c] = 3.0f;
            lo[4 * c + 1] = (float)(bs.t_first - 30.0); hi[4 * c + 1] = (float)(bs.t_last + 30.0);
            lo[4 * c + 2] = -2.0f; hi[4 * c + 2] = 5.0f;
            lo[4 * c + 3] = -2.0f; hi[4 * c + 3] = 6.0f;
        }
        if (4 * K + 1 < MAXD) {
            lo[4 * K] = -0.3f; hi[4 * K] = 0.3f;
            lo[4 * K + 1] = -5.0f; hi[4 * K + 1] = 0.0f;
        }
        if (seeded && task.aux >= 0) {
            const double* sp = d.mb[task.aux].seed;
            for (int j = 0; j < t.np && j < MAXD; j++) seedp[j] = (float)sp[j];
        }
    }
    const int D = t.D;
    float vmax[MAXD];
#pragma unroll
    for (int j = 0; j < MAXD; j++) vmax[j] = j < D ? 0.5f * (hi[j] - lo[j]) : 0.0f;
    t.mscratch = d.scratch + (size_t)gwarp * (size_t)d.scratch_per_warp;
    const float* dr = d.draws + (size_t)task.restart * DRAWS_PER_SEED;
    const int p = lane;
    const bool live = p < NP;
    // ---- initialisation (src/parametric.rs:1677-1692, seeded :1189-1210)
    float x[MAXD], v[MAXD], pb[MAXD], g[MAXD];
    int base;
    if (seeded) {
        if (p == 0) {
#pragma unroll
            for (int j = 0; j < MAXD; j++) {
                if (j < D) { x[j] = seedp[j]; v[j] = vmax[j] * 0.2f * (2.0f * dr[j] - 1.0f); }
            }
        } else if (live) {
            int o = D + 2 * D * (p - 1);
#pragma unroll
            for (int j = 0; j < MAXD; j++) {
                if (j < D) {
                    x[j] = lo[j] + dr[o + j] * (hi[j] - lo[j]);
                    v[j] = vmax[j] * 0.2f * (2.0f * dr[o + D + j] - 1.0f);
                }
            }
        }
        base = 2 * D * NP - D;
    } else {
        if (live) {
            int o = 2 * D * p;
#pragma unroll
            for (int j = 0; j < MAXD; j++) {
                if (j < D) {
                    x[j] = lo[j] + dr[o + 2 * j] * (hi[j] - lo[j]);
                    v[j] = vmax[j] * 0.2f * (2.0f * dr[o + 2 * j + 1] - 1.0f);
                }
            }
        }
        base = 2 * D * NP;
    }
#pragma unroll
    for (int j = 0; j < MAXD; j++) {
        if (!live || j >= D) { x[j] = 0.0f; v[j] = 0.0f; }
        pb[j] = x[j];
        g[j] = 0.0f;
    }
    // one evaluation round over the particles of lanes start .. NP - 1
    // (lane-split, except MetzgerKN); lane p >= start receives its own cost
    auto eval_round = [&](int start) -> double {
        if constexpr (KIND == METZGER) {
            return (live && p >= start) ? particle_cost_k<KIND>(t, x) : INFINITY;
        } else {
            const int k = NP - start;
            const double cs = particle_cost_split<KIND>(t, x, start, k);
            const double co = __shfl_sync(FULL, cs, ((p - start) * split_lanes(k)) & 31);
            return (live && p >= start) ? co : INFINITY;
        }
    };
    double c = eval_round(0);
    int evals = 1;
    double pbc = c;
    double gc = INFINITY;
    {
        // global best after the sequential initial loop: first strict minimum
        double mn = c;
        for (int k = 16; k; k >>= 1) mn = fmin(mn, __shfl_xor_sync(FULL, mn, k));
        unsigned m = __ballot_sync(FULL, live && c == mn && mn < INFINITY);
        if (m) {
            int q = __ffs(m) - 1;
            gc = mn;
#pragma unroll
            for (int j = 0; j < MAXD; j++) g[j] = __shfl_sync(FULL, x[j], q);
        }
    }
    // ---- iterations
    int stall = 0;
    double prev = gc;
    const double inv_iters = 1.0 / (double)MAX_ITERS;
    int it = 0;
    for (; it < MAX_ITERS; it++) {
        const float w = (float)(0.9 - (0.9 - 0.4) * (double)it * inv_iters);
        float x0[MAXD], v0[MAXD];
#pragma unroll
        for (int j = 0; j < MAXD; j++) { x0[j] = x[j]; v0[j] = v[j]; }
        const float* r = dr + base + it * 2 * D * NP + 2 * D * p;
        int start = 0;
        while (start < NP) {
            bool active = live && p >= start;
            if (active) {
#pragma unroll
                for (int j = 0; j < MAXD; j++) {
                    if (j < D) {
                        float r1 = r[2 * j], r2 = r[2 * j + 1];
                        float vv = w * v0[j] + 1.5f * r1 * (pb[j] - x0[j]) + 1.5f * r2 * (g[j] - x0[j]);
                        vv = fminf(fmaxf(vv, -vmax[j]), vmax[j]);
                        float nx = x0[j] + vv;
                        if (nx <= lo[j]) { x[j] = lo[j]; v[j] = 0.0f; }
                        else if (nx >= hi[j]) { x[j] = hi[j]; v[j] = 0.0f; }
                        else { x[j] = nx; v[j] = vv; }
                    }
                }
            }
            {
                const double cr = eval_round(start);
                if (active) {
                    c = cr;
                    evals++;
                }
            }
            unsigned m = __ballot_sync(FULL, active && c < gc);
            int q = m ? __ffs(m) - 1 : NP - 1;
            bool acc = live && p >= start && p <= q;
            if (acc && c < pbc) {
                pbc = c;
#pragma unroll
                for (int j = 0; j < MAXD; j++) pb[j] = x[j];
            }
            if (m) {
                gc = __shfl_sync(FULL, c, q);
#pragma unroll
                for (int j = 0; j < MAXD; j++) g[j] = __shfl_sync(FULL, x[j], q);
            }
            start = q + 1;
        }
        bool improved = prev - gc > 0.01 * fmax(fabs(prev), 1e-10);
        if (improved) {
            stall = 0;
            prev = gc;
        } else if (++stall >= STALL_ITERS) {
            it++;
            break;
        }
    }
    // ---- result
    int tot_evals = live ? evals : 0;
    for (int k = 16; k; k >>= 1) tot_evals += __shfl_xor_sync(FULL, tot_evals, k);
    if (lane == 0) {
        PsoResult& R = d.pso_res[task.out];
        R.cost = gc;
        R.iters = it;
        R.evals = tot_evals;
        for (int j = 0; j < MB_MAXP; j++) R.params[j] = 0.0f;
#pragma unroll
        for (int j = 0; j < MAXD; j++)
            if (j < D) R.params[j] = g[j];
        atomicAdd(&d.ctr->particle_obs_evals, (unsigned long long)tot_evals * (unsigned long long)bs.n);
        if (KIND == METZGER) atomicAdd(&d.ctr->ode_steps, (unsigned long long)tot_evals * MetzgerF::NG);
        if (slot == 0) {
            atomicAdd(&d.ctr->slot0_evals[KIND], (unsigned long long)tot_evals * (unsigned long long)bs.n);
            atomicAdd(&d.ctr->slot0_particles[KIND], (unsigned long long)tot_evals);
        }
    }
}

// ---------------------------------------------------------------------------
// Exact-trajectory swarms: the models other than MetzgerKN, in model
// selection and the profile t0 search.  The reference's choice of model is
// chaotic at the 1e-7 level: with its own FP64 costs, rounding only the
// particle positions to FP32 changes the selected model for ~1.2 % of bands
// (measured with the FP64 restatement on 600 bands).  These swarms therefore
// follow the reference's trajectory at double-float precision:
//   * positions, velocities and bests are double-float pairs (high halves in
//     registers, low halves in shared memory), initialised with the
//     reference's FP64 draws and moved with its FP64 products 1.5 r
//     (c1 = c2 = 1.5), ~1e-14 from the reference's FP64 arithmetic;
//   * each particle's cost is evaluated in FP32 at the position's leading
//     float, lane-split as in the other swarms (deciding near-tied FP32
//     comparisons on accurate costs was measured and changed no result);
//   * the best position is stored as double-float pairs (pso_param); the
//     t0 search's runs report the accurate cost of their best position (the
//     polish's double-float cost, LaneLb) for the picks, and the polish
//     settles the model-selection restarts on accurate costs.
// ---------------------------------------------------------------------------

// Accurate cost of the double-float position pos[0..6] (every lane passes
// the same position): component j of the full parameter vector in lane j,
// t0 inserted for t0-fixed tasks.
template <int KIND>
__device__ __noinline__ double swarm_exact_cost(LaneLb<KIND>& lc, bool fixed, double t0_fixed, const ff* pos) {
    constexpr int t0i = t0_idx_of(KIND);
    const int j = threadIdx.x & 7;
    double v = (fixed && j == t0i) ? t0_fixed : 0.0;
#pragma unroll
    for (int m = 0; m < 7; m++) {
        const int k = (fixed && m >= t0i) ? m + 1 : m;
        if (k == j && !(fixed && j == t0i)) v = (double)pos[m].hi + (double)pos[m].lo;
    }
    double f, g_unused;
    lc.cost_grad(v, f, g_unused, false);
    return f;
}

// The band and cost options of a swarm task for swarm_exact_cost.
template <int KIND>
__device__ __forceinline__ void exact_cost_setup(LaneLb<KIND>& lc, const DeviceBatch& d, const BandStats& bs,
                                                 int flags) {
    lc.t = d.t64 + bs.off;
    lc.flux = d.f64 + bs.off;
    lc.var = d.var64 + bs.off;
    lc.uf = d.uf64 + bs.off;
    lc.up = d.up + bs.off;
    lc.fa = d.ffa + bs.off;
    lc.fb = d.ffb + bs.off;
    lc.t_first = bs.t_first;
    lc.t_last = bs.t_last;
    lc.n = bs.n;
    lc.nd = (double)max(bs.n, 1);
    lc.inv_nd = 1.0 / lc.nd;
    lc.lo_j = -INFINITY;
    lc.hi_j = INFINITY;
    lc.evals = 0;
    lc.iters = 0;
    lc.fp64_evals = 0;
    lc.with_prior = (flags & TASK_PRIOR) != 0;
}

template <int KIND>
__device__ __forceinline__ void run_swarm_exact(const DeviceBatch& d, const PsoTask& task, const BandStats& bs,
                                                TaskCtx& t, WarpSmem* ws, int slot) {
    constexpr int m = KIND, np = n_params_of(m), t0i = t0_idx_of(m), MAXD = 7;
    const int lane = threadIdx.x & 31;
    const int p = lane;
    const bool live = p < NP;
    const bool seeded = (task.flags & TASK_SEEDED) != 0;
    const bool fixed = (task.flags & TASK_T0_FIXED) != 0;
    t.model = m;
    t.np = np;
    t.t0i = t0i;
    t.D = fixed ? np - 1 : np;
    const int D = t.D;
    // low halves of this lane's state
    float* XL = &ws->lo_state[0][0][lane];
    float* VL = &ws->lo_state[1][0][lane];
    float* PL = &ws->lo_state[2][0][lane];
    float* X0L = &ws->lo_state[3][0][lane];
    float* V0L = &ws->lo_state[4][0][lane];
    // the box in FP64 (data-informed t0 bounds, src/parametric.rs:1881-1909);
    // swarm dimension k is parameter k, or k + 1 past t0 when t0 is fixed
    double blo[MAXD], bhi[MAXD], seed[MAXD];
    {
        double dlo[MAXP], dhi[MAXP];
#pragma unroll
        for (int j = 0; j < MAXP; j++) { dlo[j] = c_lo[m][j]; dhi[j] = c_hi[m][j]; }
        if (task.flags & TASK_T0_BOUNDS) {
            const double t0_lo = fmax(bs.t_first - 30.0, dlo[t0i]);
            const double t0_hi = fmin(bs.t_peak + 10.0, dhi[t0i]);
            if (t0_lo < t0_hi) { dlo[t0i] = t0_lo; dhi[t0i] = t0_hi; }
        }
#pragma unroll
        for (int k = 0; k < MAXD; k++) {
            const int jk = (fixed && k >= t0i) ? k + 1 : k;
            blo[k] = k < D ? dlo[jk] : 0.0;
            bhi[k] = k < D ? dhi[jk] : 0.0;
            seed[k] = 0.0;
        }
        if (seeded) {
            // seed particles of pso_fit_single_model, src/parametric.rs:1924-1964
#pragma unroll
            for (int j = 0; j < np; j++) seed[j] = fmin(fmax(c_pop_c[m][j], dlo[j]), dhi[j]);
            const double t0s = task.restart == 1 ? bs.t_peak - 5.0 : bs.t_first - 15.0;
            seed[t0i] = fmin(fmax(t0s, dlo[t0i]), dhi[t0i]);
        }
    }
    double vmaxd[MAXD];
#pragma unroll
    for (int k = 0; k < MAXD; k++) vmaxd[k] = __dmul_rn(0.5, __dsub_rn(bhi[k], blo[k]));
    __syncwarp();
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < MAXD; k++) {
            ws->lo[k] = ff_from(blo[k]);
            ws->hi[k] = ff_from(bhi[k]);
            ws->vmax[k] = ff_from(vmaxd[k]);
            ws->g[k] = ffm(0.0f, 0.0f);
        }
    }
    // ---- initialisation (src/parametric.rs:1677-1692, seeded :1189-1210) in
    // FP64 as the reference, without contractions
    const double* dr = d.draws64 + (size_t)task.restart * DRAWS_PER_SEED;
    const float2* d15 = d.draws15 + (size_t)task.restart * DRAWS_PER_SEED;
    float xh[MAXD], vh[MAXD], pbh[MAXD];
    int base;
    {
        double xi[MAXD], vi[MAXD];
#pragma unroll
        for (int k = 0; k < MAXD; k++) { xi[k] = 0.0; vi[k] = 0.0; }
        if (seeded) {
            if (p == 0) {
#pragma unroll
                for (int k = 0; k < MAXD; k++)
                    if (k < D) {
                        xi[k] = seed[k];
                        vi[k] = __dmul_rn(__dmul_rn(vmaxd[k], 0.2), __dsub_rn(2.0 * dr[k], 1.0));
                    }
            } else if (live) {
                const int o = D + 2 * D * (p - 1);
#pragma unroll
                for (int k = 0; k < MAXD; k++)
                    if (k < D) {
                        xi[k] = __dadd_rn(blo[k], __dmul_rn(dr[o + k], __dsub_rn(bhi[k], blo[k])));
                        vi[k] = __dmul_rn(__dmul_rn(vmaxd[k], 0.2), __dsub_rn(2.0 * dr[o + D + k], 1.0));
                    }
            }
            base = 2 * D * NP - D;
        } else {
            if (live) {
                const int o = 2 * D * p;
#pragma unroll
                for (int k = 0; k < MAXD; k++)
                    if (k < D) {
                        xi[k] = __dadd_rn(blo[k], __dmul_rn(dr[o + 2 * k], __dsub_rn(bhi[k], blo[k])));
                        vi[k] = __dmul_rn(__dmul_rn(vmaxd[k], 0.2), __dsub_rn(2.0 * dr[o + 2 * k + 1], 1.0));
                    }
            }
            base = 2 * D * NP;
        }
#pragma unroll
        for (int k = 0; k < MAXD; k++) {
            const ff xf = ff_from(xi[k]), vf = ff_from(vi[k]);
            xh[k] = xf.hi;
            XL[32 * k] = xf.lo;
            vh[k] = vf.hi;
            VL[32 * k] = vf.lo;
            pbh[k] = xf.hi;
            PL[32 * k] = xf.lo;
        }
    }
    __syncwarp();
    // one evaluation round over lanes start .. NP - 1 (lane-split FP32)
    auto eval_round = [&](int start) -> double {
        const int kk = NP - start;
        const double cs = particle_cost_split<KIND>(t, xh, start, kk);
        const double co = __shfl_sync(FULL, cs, ((p - start) * split_lanes(kk)) & 31);
        return (live && p >= start) ? co : INFINITY;
    };
    // the global best <- the position of lane q
    auto set_gbest = [&](int q) {
        ff gq[MAXD];
#pragma unroll
        for (int k = 0; k < MAXD; k++) gq[k] = ffm(__shfl_sync(FULL, xh[k], q), __shfl_sync(FULL, XL[32 * k], q));
        __syncwarp();
        if (lane == 0) {
#pragma unroll
            for (int k = 0; k < MAXD; k++) ws->g[k] = gq[k];
        }
        __syncwarp();
    };
    double c = eval_round(0);
    int evals = 1;
    double pbc = c;
    double gc = INFINITY;
    {
        // global best after the sequential initial loop: first strict minimum
        double mn = c;
        for (int k = 16; k; k >>= 1) mn = fmin(mn, __shfl_xor_sync(FULL, mn, k));
        const unsigned mm = __ballot_sync(FULL, live && c == mn && mn < INFINITY);
        if (mm) {
            const int q = __ffs(mm) - 1;
            gc = mn;
            set_gbest(q);
        }
    }
    // ---- iterations (src/parametric.rs:1694-1755)
    int stall = 0;
    double prev = gc;
    const double inv_iters = 1.0 / (double)MAX_ITERS;
    int it = 0;
    for (; it < MAX_ITERS; it++) {
        const double wd = __dsub_rn(0.9, __dmul_rn(__dmul_rn(__dsub_rn(0.9, 0.4), (double)it), inv_iters));
        const ff w = ff_from(wd);
        float x0h[MAXD], v0h[MAXD];
#pragma unroll
        for (int k = 0; k < MAXD; k++) {
            x0h[k] = xh[k];
            v0h[k] = vh[k];
            X0L[32 * k] = XL[32 * k];
            V0L[32 * k] = VL[32 * k];
        }
        const float2* r15 = d15 + base + it * 2 * D * NP + 2 * D * p;
        int start = 0;
        while (start < NP) {
            const bool active = live && p >= start;
            if (active) {
#pragma unroll
                for (int k = 0; k < MAXD; k++) {
                    if (k < D) {
                        const ff x0 = ffm(x0h[k], X0L[32 * k]), v0 = ffm(v0h[k], V0L[32 * k]);
                        const ff pbk = ffm(pbh[k], PL[32 * k]);
                        ff xn, vn;
                        ff_move(x0, v0, pbk, ws->g[k], w, r15[2 * k], r15[2 * k + 1], ws->vmax[k], ws->lo[k],
                                ws->hi[k], xn, vn);
                        xh[k] = xn.hi;
                        XL[32 * k] = xn.lo;
                        vh[k] = vn.hi;
                        VL[32 * k] = vn.lo;
                    }
                }
            }
            {
                const double cr = eval_round(start);
                if (active) {
                    c = cr;
                    evals++;
                }
            }
            const unsigned mq = __ballot_sync(FULL, active && c < gc);
            const int q = mq ? __ffs(mq) - 1 : NP - 1;
            const bool acc = live && p >= start && p <= q;
            if (acc && c < pbc) {
                pbc = c;
#pragma unroll
                for (int k = 0; k < MAXD; k++) {
                    pbh[k] = xh[k];
                    PL[32 * k] = XL[32 * k];
                }
            }
            if (mq) {
                gc = __shfl_sync(FULL, c, q);
                set_gbest(q);
            }
            start = q + 1;
        }
        bool improved = prev - gc > 0.01 * fmax(fabs(prev), 1e-10);
        if (improved) {
            stall = 0;
            prev = gc;
        } else if (++stall >= STALL_ITERS) {
            it++;
            break;
        }
    }
    // ---- result: for the t0 search, the accurate cost of the best position
    // (its picks compare it with the polished cost); model-selection runs
    // report the FP32 estimate, which the polish settles
    double rc = gc;
    if (fixed && gc < INFINITY) {
        LaneLb<KIND> lc;
        exact_cost_setup(lc, d, bs, task.flags);
        ff gp[MAXD];
#pragma unroll
        for (int k = 0; k < MAXD; k++) gp[k] = ws->g[k];
        rc = swarm_exact_cost<KIND>(lc, fixed, task.t0_fixed, gp);
    }
    int tot_evals = live ? evals : 0;
    for (int k = 16; k; k >>= 1) tot_evals += __shfl_xor_sync(FULL, tot_evals, k);
    if (lane == 0) {
        PsoResult& R = d.pso_res[task.out];
        R.cost = rc;
        R.iters = it;
        R.evals = tot_evals;
        for (int j = 0; j < MB_MAXP; j++) R.params[j] = R.params_lo[j] = 0.0f;
#pragma unroll
        for (int k = 0; k < MAXD; k++)
            if (k < D) {
                R.params[k] = ws->g[k].hi;
                R.params_lo[k] = ws->g[k].lo;
            }
        R.pad[0] = 1.0f;
        atomicAdd(&d.ctr->particle_obs_evals, (unsigned long long)tot_evals * (unsigned long long)bs.n);
        if (slot == 0) {
            atomicAdd(&d.ctr->slot0_evals[KIND], (unsigned long long)tot_evals * (unsigned long long)bs.n);
            atomicAdd(&d.ctr->slot0_particles[KIND], (unsigned long long)tot_evals);
        }
    }
    __syncwarp();
}

// ---------------------------------------------------------------------------
// FP64 MultiBazin cost (multi_bazin_cost, src/parametric.rs:973-1004, in the
// oracle's FP64 form) of the position pos[0 .. 4K + 1], read by every lane:
// the warp splits the band's observations, then sums its partial sums.  A
// non-finite prediction makes the cost 1e99, as in the reference.  Every lane
// of the warp must call it.  It gives each run's reported cost: the swarm
// compares FP32 costs, the reference reports (and fit_multi_bazin compares
// across restarts and K) the FP64 cost of the best position.
// ---------------------------------------------------------------------------
template <int K>
__device__ __noinline__ double mb_cost_fp64(const DeviceBatch& d, const BandStats& bs, const double* pos) {
    const int lane = threadIdx.x & 31;
    double a[K], t0[K], tr[K], tf[K];
#pragma unroll
    for (int c = 0; c < K; c++) {
        a[c] = exp(pos[4 * c]);
        t0[c] = pos[4 * c + 1];
        tr[c] = exp(pos[4 * c + 2]);
        tf[c] = exp(pos[4 * c + 3]);
    }
    const double B = pos[4 * K];
    const double se = exp(pos[4 * K + 1]);
    const double se2 = se * se;
    const double* t = d.t64 + bs.off;
    const double* f = d.f64 + bs.off;
    const double* var = d.var64 + bs.off;
    const double* uf = d.uf64 + bs.off;
    const uint8_t* up = d.up + bs.off;
    double nll = 0.0;
    int bad = 0;
    for (int i = lane; i < bs.n; i += 32) {
        double sum = 0.0;
#pragma unroll
        for (int c = 0; c < K; c++) {
            const double dt = t[i] - t0[c];
            sum += a[c] * exp(-dt / tf[c]) * (1.0 / (1.0 + exp(-dt / tr[c])));
        }
        const double pr = sum + B;
        if (!isfinite(pr)) {
            bad = 1;
            continue;
        }
        const double tv = var[i] + se2;
        if (up[i]) {
            nll -= log_normal_cdf_f64((uf[i] - pr) / sqrt(tv));
        } else {
            const double dd = pr - f[i];
            nll += dd * dd / tv + log(tv);
        }
    }
    for (int o = 16; o; o >>= 1) nll += __shfl_xor_sync(FULL, nll, o);
    if (__any_sync(FULL, bad)) return 1e99;
    return nll / (double)max(bs.n, 1);
}


// ---------------------------------------------------------------------------
// Exact-trajectory MultiBazin swarms (fit_multi_bazin's pso_minimize runs,
// src/parametric.rs:1008-1157).  With a 30-particle, 60-iteration swarm and
// no polish after it, the reference's K and costs are its swarm's end points:
// rounding only the swarm positions to FP32 in the FP64 restatement changes
// K for 3 of the 30 real ZTF sources and 4 of 200 uneven synthetic ones.  So
// these swarms follow the reference's trajectory in double-float as the
// model-selection swarms do, with one difference in the state kept: a lane's
// position, velocity and personal best are double-float (high halves in
// registers, low halves in shared memory, st[plane][dimension][lane]), and
// the iteration-start state is not copied.  A trial move is evaluated at its
// leading float and dropped; the lanes accepted in a round recompute the
// same move (same inputs, the global best not yet updated, so the same bits)
// and commit it, and lanes not yet accepted still hold the iteration start.
// One extra move per particle and iteration; 18 dimensions need 7.5 KB of
// shared memory a warp instead of 12.1 KB.
// ---------------------------------------------------------------------------
template <int MAXD, int KIND>
__device__ __forceinline__ void run_swarm_exact_mb(const DeviceBatch& d, const PsoTask& task, const BandStats& bs,
                                                   TaskCtx& t, ff* s_lo, ff* s_hi, ff* s_vm, ff* s_g, float* st,
                                                   double* s_pos, int slot) {
    constexpr int K = KIND - KIND_MB1 + 1, D = 4 * K + 2;
    static_assert(D <= MAXD, "MultiBazin swarm wider than the instantiation");
    const int lane = threadIdx.x & 31;
    const int p = lane;
    const bool live = p < NP;
    const bool seeded = (task.flags & TASK_SEEDED) != 0;
    t.model = BAZIN;
    t.np = D;
    t.D = D;
    t.t0i = -1;
    float* XL = st + lane;
    float* VL = st + 32 * MAXD + lane;
    float* PL = st + 64 * MAXD + lane;
    // the box in FP64 (multi_bazin_bounds, src/parametric.rs:958-970)
    double blo[D], bhi[D], vmaxd[D];
#pragma unroll
    for (int c = 0; c < K; c++) {
        blo[4 * c] = -3.0; bhi[4 * c] = 3.0;
        blo[4 * c + 1] = bs.t_first - 30.0; bhi[4 * c + 1] = bs.t_last + 30.0;
        blo[4 * c + 2] = -2.0; bhi[4 * c + 2] = 5.0;
        blo[4 * c + 3] = -2.0; bhi[4 * c + 3] = 6.0;
    }
    blo[4 * K] = -0.3; bhi[4 * K] = 0.3;
    blo[4 * K + 1] = -5.0; bhi[4 * K + 1] = 0.0;
#pragma unroll
    for (int k = 0; k < D; k++) vmaxd[k] = __dmul_rn(0.5, __dsub_rn(bhi[k], blo[k]));
    __syncwarp();
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < D; k++) {
            s_lo[k] = ff_from(blo[k]);
            s_hi[k] = ff_from(bhi[k]);
            s_vm[k] = ff_from(vmaxd[k]);
            s_g[k] = ffm(0.0f, 0.0f);
        }
    }
    // ---- initialisation (src/parametric.rs:1677-1692, seeded :1189-1210) in
    // FP64 as the reference, without contractions; the seed particle is the
    // K - 1 fit extended at the largest residual (mb_build_kernel)
    const double* dr = d.draws64 + (size_t)task.restart * DRAWS_PER_SEED;
    const float2* d15 = d.draws15 + (size_t)task.restart * DRAWS_PER_SEED;
    const double* seed = (seeded && task.aux >= 0) ? d.mb[task.aux].seed : nullptr;
    float xh[D], vh[D], pbh[D], xt[D];
#pragma unroll
    for (int k = 0; k < D; k++) {
        double xi = 0.0, vi = 0.0;
        if (seeded) {
            if (p == 0) {
                xi = seed ? seed[k] : 0.0;
                vi = __dmul_rn(__dmul_rn(vmaxd[k], 0.2), __dsub_rn(2.0 * dr[k], 1.0));
            } else if (live) {
                const int o = D + 2 * D * (p - 1);
                xi = __dadd_rn(blo[k], __dmul_rn(dr[o + k], __dsub_rn(bhi[k], blo[k])));
                vi = __dmul_rn(__dmul_rn(vmaxd[k], 0.2), __dsub_rn(2.0 * dr[o + D + k], 1.0));
            }
        } else if (live) {
            const int o = 2 * D * p;
            xi = __dadd_rn(blo[k], __dmul_rn(dr[o + 2 * k], __dsub_rn(bhi[k], blo[k])));
            vi = __dmul_rn(__dmul_rn(vmaxd[k], 0.2), __dsub_rn(2.0 * dr[o + 2 * k + 1], 1.0));
        }
        const ff xf = ff_from(xi), vf = ff_from(vi);
        xh[k] = xf.hi;
        XL[32 * k] = xf.lo;
        vh[k] = vf.hi;
        VL[32 * k] = vf.lo;
        pbh[k] = xf.hi;
        PL[32 * k] = xf.lo;
        xt[k] = xf.hi;
    }
    const int base = seeded ? 2 * D * NP - D : 2 * D * NP;
    __syncwarp();
    // one evaluation round over lanes start .. NP - 1 at the trial positions
    auto eval_round = [&](int start) -> double {
        const int kk = NP - start;
        const double cs = particle_cost_split<KIND>(t, xt, start, kk);
        const double co = __shfl_sync(FULL, cs, ((p - start) * split_lanes(kk)) & 31);
        return (live && p >= start) ? co : INFINITY;
    };
    auto set_gbest = [&](int q) {
        ff gq[D];
#pragma unroll
        for (int k = 0; k < D; k++) gq[k] = ffm(__shfl_sync(FULL, xh[k], q), __shfl_sync(FULL, XL[32 * k], q));
        __syncwarp();
        if (lane == 0) {
#pragma unroll
            for (int k = 0; k < D; k++) s_g[k] = gq[k];
        }
        __syncwarp();
    };
    double c = eval_round(0);
    int evals = 1;
    double pbc = c;
    double gc = INFINITY;
    {
        double mn = c;
        for (int k = 16; k; k >>= 1) mn = fmin(mn, __shfl_xor_sync(FULL, mn, k));
        const unsigned mm = __ballot_sync(FULL, live && c == mn && mn < INFINITY);
        if (mm) {
            gc = mn;
            set_gbest(__ffs(mm) - 1);
        }
    }
    // FP64 cost of the position lane `src` writes into s_pos (warp-uniform)
    auto fp64_of = [&](int src, auto&& write) -> double {
        if (lane == src) write();
        __syncwarp();
        const double v = mb_cost_fp64<K>(d, bs, s_pos);
        __syncwarp();
        return v;
    };
    auto fp64_g = [&]() -> double {
        return fp64_of(0, [&]() {
#pragma unroll
            for (int k = 0; k < D; k++) s_pos[k] = ff_to(s_g[k]);
        });
    };
    // ---- iterations (src/parametric.rs:1694-1755)
    int stall = 0;
    double prev = gc;
    const double inv_iters = 1.0 / (double)MAX_ITERS;
    int it = 0;
    for (; it < MAX_ITERS; it++) {
        const double wd = __dsub_rn(0.9, __dmul_rn(__dmul_rn(__dsub_rn(0.9, 0.4), (double)it), inv_iters));
        const ff w = ff_from(wd);
        const float2* r15 = d15 + base + it * 2 * D * NP + 2 * D * p;
        // the move from the iteration-start state against the current global
        // best: trial (leading floats to xt) or commit (the full state)
        auto move = [&](bool commit) {
#pragma unroll
            for (int k = 0; k < D; k++) {
                ff xn, vn;
                ff_move(ffm(xh[k], XL[32 * k]), ffm(vh[k], VL[32 * k]), ffm(pbh[k], PL[32 * k]), s_g[k], w,
                        r15[2 * k], r15[2 * k + 1], s_vm[k], s_lo[k], s_hi[k], xn, vn);
                if (commit) {
                    xh[k] = xn.hi;
                    XL[32 * k] = xn.lo;
                    vh[k] = vn.hi;
                    VL[32 * k] = vn.lo;
                } else {
                    xt[k] = xn.hi;
                }
            }
        };
        int start = 0;
        while (start < NP) {
            const bool active = live && p >= start;
            if (active) move(false);
            {
                const double cr = eval_round(start);
                if (active) {
                    c = cr;
                    evals++;
                }
            }
            const unsigned mq = __ballot_sync(FULL, active && c < gc);
            const int q = mq ? __ffs(mq) - 1 : NP - 1;
            if (active && p <= q) {
                move(true);
                if (c < pbc) {
                    pbc = c;
#pragma unroll
                    for (int k = 0; k < D; k++) {
                        pbh[k] = xh[k];
                        PL[32 * k] = XL[32 * k];
                    }
                }
            }
            __syncwarp();
            if (mq) {
                gc = __shfl_sync(FULL, c, q);
                set_gbest(q);
            }
            start = q + 1;
        }
        bool improved = prev - gc > 0.01 * fmax(fabs(prev), 1e-10);
        if (improved) {
            stall = 0;
            prev = gc;
        } else if (++stall >= STALL_ITERS) {
            it++;
            break;
        }
    }
    // ---- result: the FP64 cost of the best position, as the reference
    // reports it (fit_multi_bazin compares the restarts' costs and the BICs)
    const double rc = gc < INFINITY ? fp64_g() : gc;
    int tot_evals = live ? evals : 0;
    for (int k = 16; k; k >>= 1) tot_evals += __shfl_xor_sync(FULL, tot_evals, k);
    if (lane == 0) {
        PsoResult& R = d.pso_res[task.out];
        R.cost = rc;
        R.iters = it;
        R.evals = tot_evals;
        for (int j = 0; j < MB_MAXP; j++) R.params[j] = R.params_lo[j] = 0.0f;
#pragma unroll
        for (int k = 0; k < D; k++) {
            R.params[k] = s_g[k].hi;
            R.params_lo[k] = s_g[k].lo;
        }
        R.pad[0] = 1.0f;
        atomicAdd(&d.ctr->particle_obs_evals, (unsigned long long)tot_evals * (unsigned long long)bs.n);
        if (slot == 0) {
            atomicAdd(&d.ctr->slot0_evals[KIND], (unsigned long long)tot_evals * (unsigned long long)bs.n);
            atomicAdd(&d.ctr->slot0_particles[KIND], (unsigned long long)tot_evals);
        }
    }
    __syncwarp();
}

// MINB: blocks of 256 threads per SM the register budget is sized for.  Two
// (128 registers a thread, 16 warps) is the default: measured on GB300 it runs
// the swarms ~1.7x faster than one block without spills.  The 7-dimension
// swarm also has a three-block build (80 registers, 24 warps, more spills):
// on the 10k uneven workload it runs the model-selection launch 14 % faster
// (495 -> 426 ms) but the t0-search launches, fewer and longer tasks, 30 %
// slower, so the launch autotuner offers it for model selection only.
template <int MAXD, int MINB>
__global__ void __launch_bounds__(256, MINB)
    pso_kernel(DeviceBatch d, int slot, const PsoTask* tasks, int n_host, int smem_obs) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int nwarps = blockDim.x >> 5;
    float4* sobs = reinterpret_cast<float4*>(smem_raw) + (size_t)warp * smem_obs;
    using WS = typename WarpSmemOf<MAXD>::type;
    WS* ws = reinterpret_cast<WS*>(reinterpret_cast<float4*>(smem_raw) + (size_t)nwarps * smem_obs) + warp;
    if (lane == 0) mbar_init(&ws->bar);
    __syncwarp();
    uint32_t phase = 0;
    const int n_tasks = n_host >= 0 ? n_host : d.ctr->task_count[slot];
    const int gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;

    while (true) {
        int ti = 0;
        if (lane == 0) ti = atomicAdd(&d.ctr->task_head[slot], 1);
        ti = __shfl_sync(FULL, ti, 0);
        if (ti >= n_tasks) break;
        const PsoTask task = tasks[ti];
        const BandStats bs = d.stats[task.band];
        // tasks of bands the reference does not fit (or MultiBazin tasks of
        // bands that are not their source's rank-0 band with n >= 5) are no-ops
        if (!bs.valid || ((task.flags & TASK_RANK0) && (bs.rank != 0 || bs.n < 5))) continue;
        TaskCtx t;
        t.kind = task.kind;
        t.flags = task.flags;
        t.n = bs.n;
        t.inv_n = 1.0 / (double)max(bs.n, 1);
        t.t_last = (float)bs.t_last;
        t.t0_fixed = (float)task.t0_fixed;
        // stage the band
        const float4* gobs = d.obs + bs.off;
        if (bs.n <= smem_obs && bs.n > 0) {
            __syncwarp();
            if (lane == 0) bulk_copy_g2s(sobs, gobs, (uint32_t)bs.n * 16u, &ws->bar);
            // the lanes agree on the outcome, so the warp stays converged
            const bool ok = __all_sync(FULL, mbar_wait(&ws->bar, phase, d.wait_polls));
            if (!ok) {
                // the bound expired: record it, let the copy already issued
                // into this warp's stage land (a second bounded wait), and
                // stop taking tasks; the barrier is not re-armed and the
                // stage is not reused.  The tasks left behind keep their
                // "not run" results, and the host reports LCF_E_TIMEOUT.
                if (lane == 0) atomicCAS(&d.ctr->error, 0, LCF_E_TIMEOUT);
                mbar_wait(&ws->bar, phase, 1 << 24);
                __syncwarp();
                break;
            }
            phase ^= 1u;
            t.obs = sobs;
        } else {
            t.obs = gobs;
        }
        // one specialised swarm loop per task kind: the warps resident on an SM
        // (the queue is grouped by kind) run one kind's code
        if constexpr (MAXD != 7) {
            constexpr int KMB = KIND_MB1 + (MAXD - 2) / 4 - 1;  // D = 4K + 2
            if (task.kind == KMB)
                run_swarm_exact_mb<MAXD, KMB>(d, task, bs, t, ws->lo, ws->hi, ws->vmax, ws->g, &ws->lo_state[0][0][0],
                                              ws->s_pos, slot);
        } else switch (task.kind) {
            case BAZIN: run_swarm_exact<BAZIN>(d, task, bs, t, ws, slot); break;
            case VILLAR: run_swarm_exact<VILLAR>(d, task, bs, t, ws, slot); break;
            case TDE: run_swarm_exact<TDE>(d, task, bs, t, ws, slot); break;
            case ARNETT: run_swarm_exact<ARNETT>(d, task, bs, t, ws, slot); break;
            case MAGNETAR: run_swarm_exact<MAGNETAR>(d, task, bs, t, ws, slot); break;
            case SHOCK: run_swarm_exact<SHOCK>(d, task, bs, t, ws, slot); break;
            case AFTERGLOW: run_swarm_exact<AFTERGLOW>(d, task, bs, t, ws, slot); break;
            case METZGER: run_swarm<MAXD, METZGER>(d, task, bs, t, slot, gwarp); break;
            case KIND_MB1:
                run_swarm_exact_mb<MAXD, KIND_MB1>(d, task, bs, t, ws->lo, ws->hi, ws->vmax, ws->g,
                                                   &ws->lo_state[0][0][0], ws->s_pos, slot);
                break;
            default: break;
        }
        __syncwarp();
    }
}
// ---------------------------------------------------------------------------
// Peak probes: dependent FMA chains (FP32 pipe) and ex2.approx chains (SFU
// pipe), eight independent chains per thread, a full persistent grid.
// ---------------------------------------------------------------------------
__global__ void probe_fma_kernel(float* out, int iters) {
    float a[8];
    for (int k = 0; k < 8; k++) a[k] = threadIdx.x * 1e-7f + k;
    const float m = 0.999999f, c = 1e-7f;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int k = 0; k < 8; k++) a[k] = fmaf(a[k], m, c);
    }
    float s = 0.0f;
    for (int k = 0; k < 8; k++) s += a[k];
    if (s == 12345.0f) out[threadIdx.x] = s;
}
__global__ void probe_ex2_kernel(float* out, int iters) {
    float a[8];
    for (int k = 0; k < 8; k++) a[k] = -1e-3f * (threadIdx.x & 7) - 0.01f * k;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int k = 0; k < 8; k++) {
            float y;
            asm volatile("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(a[k]));
            a[k] = -y;
        }
    }
    float s = 0.0f;
    for (int k = 0; k < 8; k++) s += a[k];
    if (s == 12345.0f) out[threadIdx.x] = s;
}
static double time_probe(void (*k)(float*, int), int num_sms, int iters) {
    float* out = nullptr;
    cudaMalloc(&out, 1024 * sizeof(float));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    int grid = num_sms * 8, block = 256;
    k<<<grid, block>>>(out, iters / 10);
    cudaEventRecord(e0);
    k<<<grid, block>>>(out, iters);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    double ops = (double)grid * block * 8.0 * iters;
    return ms > 0.0f ? ops / (ms * 1e-3) : 0.0;
}
double probe_fp32_tflops(int num_sms) { return 2.0 * time_probe(probe_fma_kernel, num_sms, 1 << 16) * 1e-12; }
double probe_mufu_gops(int num_sms) { return time_probe(probe_ex2_kernel, num_sms, 1 << 14) * 1e-9; }

static size_t warp_smem_bytes(int max_dim) {
    return max_dim <= 7 ? sizeof(WarpSmem) : max_dim <= 10 ? sizeof(WarpSmemMB<10>)
         : max_dim <= 14 ? sizeof(WarpSmemMB<14>) : sizeof(WarpSmemMB<18>);
}

// Observations a warp stages in shared memory: smem_obs, except in the
// MultiBazin instantiations, whose larger swarm state would otherwise leave
// room for one block per SM; there as many (a multiple of 32) as keep two
// blocks of `block` threads within 220 KB.  Longer bands are read from
// global memory, with the same values.
int pso_stage_obs(int block, int smem_obs, int max_dim) {
    if (max_dim <= 7) return smem_obs;
    const size_t per_warp = (size_t)110 * 1024 / (size_t)(block / 32);
    const size_t ws = warp_smem_bytes(max_dim);
    int n = per_warp > ws ? (int)((per_warp - ws) / sizeof(float4)) : 0;
    n &= ~31;
    return std::max(32, std::min(smem_obs, n));
}

size_t pso_smem_bytes(int block, int smem_obs, int max_dim) {
    const int so = pso_stage_obs(block, smem_obs, max_dim);
    return (size_t)(block / 32) * ((size_t)so * sizeof(float4) + warp_smem_bytes(max_dim));
}

int pso_init_attributes(const int* blocks, const int* smem_obs, int n) {
    size_t m7 = 0, m10 = 0, m14 = 0, m18 = 0;
    for (int c = 0; c < n; c++) {
        m7 = std::max(m7, pso_smem_bytes(blocks[c], smem_obs[c], 7));
        m10 = std::max(m10, pso_smem_bytes(blocks[c], smem_obs[c], 10));
        m14 = std::max(m14, pso_smem_bytes(blocks[c], smem_obs[c], 14));
        m18 = std::max(m18, pso_smem_bytes(blocks[c], smem_obs[c], 18));
    }
    const cudaFuncAttribute a = cudaFuncAttributeMaxDynamicSharedMemorySize;
    cudaError_t e = cudaFuncSetAttribute(pso_kernel<7, 2>, a, (int)m7);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(pso_kernel<7, 3>, a, (int)m7);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(pso_kernel<10, 2>, a, (int)m10);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(pso_kernel<14, 2>, a, (int)m14);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(pso_kernel<18, 2>, a, (int)m18);
    return (int)e;
}

int pso_blocks_per_sm(int block, size_t smem, int minb) {
    int n = 0;
    cudaError_t e = minb == 3 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, pso_kernel<7, 3>, block, smem)
                              : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, pso_kernel<7, 2>, block, smem);
    return e == cudaSuccess ? n : 1;
}

void launch_pso(const DeviceBatch& d, int slot, const PsoTask* tasks, int n_host, int max_dim, int grid, int block,
                cudaStream_t s, int minb) {
    if (n_host == 0) return;
    const int smem_obs = pso_stage_obs(block, d.smem_obs, max_dim);
    const size_t smem = pso_smem_bytes(block, d.smem_obs, max_dim);
    if (max_dim <= 7 && minb == 3) pso_kernel<7, 3><<<grid, block, smem, s>>>(d, slot, tasks, n_host, smem_obs);
    else if (max_dim <= 7) pso_kernel<7, 2><<<grid, block, smem, s>>>(d, slot, tasks, n_host, smem_obs);
    else if (max_dim <= 10) pso_kernel<10, 2><<<grid, block, smem, s>>>(d, slot, tasks, n_host, smem_obs);
    else if (max_dim <= 14) pso_kernel<14, 2><<<grid, block, smem, s>>>(d, slot, tasks, n_host, smem_obs);
    else pso_kernel<18, 2><<<grid, block, smem, s>>>(d, slot, tasks, n_host, smem_obs);
}

// ---------------------------------------------------------------------------
// Device task sort (counting sort on 256 keys) for the task lists built on
// the device (t0 search, Bazin gate, MultiBazin K = 2..4): the same order as
// the host-built model-selection queue, so that the warps resident on an SM
// run one kind's code and the longest swarms start first.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int task_sort_key(const PsoTask& t, int n) {
    int grp = t.kind == METZGER ? 0 : 1 + t.kind;                      // 0..12
    int lb = (int)(2.0f * log2f((float)max(n, 1))) - 3;                // 16 length buckets
    lb = min(15, max(0, lb));
    return grp * 16 + (15 - lb);                                       // < 208
}

__global__ void task_hist_kernel(DeviceBatch d, int slot) {
    const int n_tasks = d.ctr->task_count[slot];
    int* hist = d.ctr->sort_hist[slot];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_tasks; i += gridDim.x * blockDim.x) {
        const PsoTask t = d.tasks[slot][i];
        atomicAdd(&hist[task_sort_key(t, d.stats[t.band].n)], 1);
    }
}

__global__ void task_scan_kernel(DeviceBatch d, int slot) {  // one block of 256 threads
    __shared__ int sh[256];
    const int i = threadIdx.x;
    const int v = d.ctr->sort_hist[slot][i];
    sh[i] = v;
    __syncthreads();
    for (int off = 1; off < 256; off <<= 1) {
        int a = i >= off ? sh[i - off] : 0;
        __syncthreads();
        sh[i] += a;
        __syncthreads();
    }
    d.ctr->sort_hist[slot][i] = sh[i] - v;  // exclusive prefix: first position of key i
}

__global__ void task_scatter_kernel(DeviceBatch d, int slot, PsoTask* out) {
    const int n_tasks = d.ctr->task_count[slot];
    int* pos = d.ctr->sort_hist[slot];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_tasks; i += gridDim.x * blockDim.x) {
        const PsoTask t = d.tasks[slot][i];
        int p = atomicAdd(&pos[task_sort_key(t, d.stats[t.band].n)], 1);
        out[p] = t;
    }
}

void launch_task_sort(const DeviceBatch& d, int slot, PsoTask* out, cudaStream_t s) {
    if (d.n_bands == 0 || d.task_cap[slot] == 0) return;
    int grid = (d.task_cap[slot] + 255) / 256;
    grid = grid < 1024 ? grid : 1024;
    task_hist_kernel<<<grid, 256, 0, s>>>(d, slot);
    task_scan_kernel<<<1, 256, 0, s>>>(d, slot);
    task_scatter_kernel<<<grid, 256, 0, s>>>(d, slot, out);
}

}  // namespace lcf
