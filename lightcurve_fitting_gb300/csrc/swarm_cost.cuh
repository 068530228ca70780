// swarm_cost.cuh — the FP32 particle cost shared by the swarm kernels and
// the likelihood API (PsoCost::cost_from_slice, src/parametric.rs:1303-1370,
// and multi_bazin_cost, :973-1004).  Its exp / log / division are those of
// the translation unit that includes it: the swarm units are compiled with
// nvcc's fast single-precision forms, the likelihood API's with the
// accurate library forms.
#pragma once

#include "lcf_internal.cuh"
#include "models_f32.cuh"

namespace lcf {

constexpr unsigned FULL_MASK = 0xffffffffu;

// ---------------------------------------------------------------------------
// Particle cost (PsoCost::cost_from_slice, src/parametric.rs:1303-1370, and
// multi_bazin_cost, :973-1004) for the particle of this lane.
// ---------------------------------------------------------------------------
struct TaskCtx {
    int kind, model, np, D, t0i, flags, n;
    float t0_fixed;
    float t_last;
    const float4* obs;
    float* mscratch;     // MetzgerKN scratch of this warp ([n][32])
    double inv_n;        // 1 / max(n, 1)
};

// Negative log-likelihood terms of observations i0, i0 + stride, ... < n.
template <class M>
__device__ __forceinline__ Nll nll_loop(const M& m, const float4* obs, int n, float se2, int i0 = 0, int stride = 1) {
    Nll acc;
    acc.reset();
#pragma unroll 2
    for (int i = i0; i < n; i += stride) {
        float4 o = obs[i];
        int st = ST_OK;
        float pr = m.eval(o.x, o.y, st);
        acc.obs(o, pr, st, se2);
    }
    return acc;
}

// MultiBazin prediction: sum of K Bazin components + B (src/parametric.rs:932-940)
template <int K>
__device__ __forceinline__ Nll nll_multibazin(const float* p, const float4* obs, int n, float se2, int i0 = 0,
                                              int stride = 1) {
    float la[K], t0[K], itr[K], itf[K], dif[K];
#pragma unroll
    for (int c = 0; c < K; c++) {
        la[c] = p[4 * c];
        t0[c] = p[4 * c + 1];
        itr[c] = expf(-p[4 * c + 2]);
        itf[c] = expf(-p[4 * c + 3]);
        dif[c] = itr[c] * expm1f(p[4 * c + 2] - p[4 * c + 3]);
    }
    float B = p[4 * K];
    Nll acc;
    acc.reset();
    for (int i = i0; i < n; i += stride) {
        float4 o = obs[i];
        float sum = 0.0f, bigL = -INFINITY;
        int st = ST_OK;
#pragma unroll
        for (int c = 0; c < K; c++) {
            // one Bazin component in log space (as BazinF::eval)
            float dt = (o.x - t0[c]) + o.y;
            float xf = -dt * itf[c], xr = -dt * itr[c];
            if (xf > 80.0f) {
                if (xf > LN_DBL_MAX || la[c] + xf > LN_DBL_MAX) { st = ST_NONFINITE; continue; }
                if (xr > LN_DBL_MAX) continue;  // exact zero in FP64
            }
            float L = la[c] + (xr > 0.0f ? -dt * dif[c] : xf) - log1pf(expf(-fabsf(xr)));
            if (L > BIG_L) bigL = fmaxf(bigL, L) + log1pf(expf(-fabsf(bigL - L)));
            else sum += expf(L);
        }
        float pr = 0.0f;
        if (st == ST_OK && bigL > -INFINITY) {
            // FP64 sum overflows to +inf past ln DBL_MAX: non-finite prediction
            if (bigL > LN_DBL_MAX) st = ST_NONFINITE;
            else { st = ST_BIG; pr = bigL; }
        } else {
            pr = sum + B;
        }
        acc.obs(o, pr, st, se2);
    }
    return acc;
}

template <class M>
__device__ __forceinline__ void model_init(M& e, const float* p, const double* pd) {
    if (pd) e.init64(pd);
    else e.init(p);
}

// Cost of one particle of a task of kind KIND (PsoCost::cost_from_slice,
// src/parametric.rs:1303-1370, or the MultiBazin cost :985-1006).
// pd: optional FP64 parameter vector (same values as p) for callers whose
// parameters are FP64; the per-particle constants are then formed in FP64.
template <int KIND>
__device__ __forceinline__ double particle_cost_k(const TaskCtx& t, const float* x, const double* pd = nullptr) {
    if constexpr (KIND >= KIND_MB1) {
        constexpr int K = KIND - KIND_MB1 + 1;
        float p[4 * K + 2];
#pragma unroll
        for (int i = 0; i < 4 * K + 2; i++) p[i] = x[i];
        float se = expf(p[4 * K + 1]);
        Nll acc = nll_multibazin<K>(p, t.obs, t.n, se * se);
        return acc.finish(0.0, t.inv_n);
    } else {
        constexpr int m = KIND;
        constexpr int np = n_params_of(m);
        // rebuild the full parameter vector (profile t0 search: t0 held fixed)
        float p[MAXP];
        if (t.flags & TASK_T0_FIXED) {
            constexpr int t0i = t0_idx_of(m);
#pragma unroll
            for (int i = 0; i < np; i++) p[i] = i < t0i ? x[i] : (i == t0i ? t.t0_fixed : x[i - 1]);
        } else {
#pragma unroll
            for (int i = 0; i < np; i++) p[i] = x[i];
        }
        if constexpr (m == VILLAR) {
            float c = VillarF::constraint(p);
            if (c > 0.0f) return 1e12 + 10000.0 * (double)c;
        }
        double prior = 0.0;
        if (t.flags & TASK_PRIOR) {
            float s = 0.0f;
#pragma unroll
            for (int j = 0; j < np; j++) {
                float w = (float)c_pop_w[m][j];
                if (w > 0.0f) {
                    float z = (p[j] - (float)c_pop_c[m][j]) / w;
                    s += 0.5f * z * z;
                }
            }
            prior = (double)s;
        }
        float se = pd ? (float)exp(pd[se_idx_of(m)]) : expf(p[se_idx_of(m)]);
        float se2 = se * se;
        Nll acc;
        if constexpr (m == BAZIN) { BazinF e; model_init(e, p, pd); acc = nll_loop(e, t.obs, t.n, se2); }
        else if constexpr (m == VILLAR) { VillarF e; model_init(e, p, pd); acc = nll_loop(e, t.obs, t.n, se2); }
        else if constexpr (m == TDE) { TdeF e; model_init(e, p, pd); acc = nll_loop(e, t.obs, t.n, se2); }
        else if constexpr (m == ARNETT) { ArnettF e; model_init(e, p, pd); acc = nll_loop(e, t.obs, t.n, se2); }
        else if constexpr (m == MAGNETAR) { MagnetarF e; model_init(e, p, pd); acc = nll_loop(e, t.obs, t.n, se2); }
        else if constexpr (m == SHOCK) { ShockF e; model_init(e, p, pd); acc = nll_loop(e, t.obs, t.n, se2); }
        else if constexpr (m == AFTERGLOW) { AfterglowF e; model_init(e, p, pd); acc = nll_loop(e, t.obs, t.n, se2); }
        else {
            // MetzgerKN: ODE sweep -> unnormalised interpolants in scratch
            struct ObsT {
                const float4* o;
                __device__ float t(int j) const { return o[j].x + o[j].y; }
            } ot{t.obs};
            int lane = threadIdx.x & 31;
            float* lv = t.mscratch + lane;
            float l_peak = 0.0f;
            bool ok = MetzgerF::sweep(p, t.t_last, ot, t.n, lv, 32, l_peak);
            acc.reset();
            float scale = 1.0f;
            if (ok) {
                float inv = 1.0f / l_peak;
                float mx = -INFINITY;
                for (int j = 0; j < t.n; j++)
                    if (t.obs[j].w >= 0.0f) mx = fmaxf(mx, lv[j * 32] * inv);
                scale = inv;
                if (mx > 1e-10f && isfinite(mx)) scale = inv * fminf(fmaxf(1.0f / mx, 0.1f), 10.0f);
            }
            for (int j = 0; j < t.n; j++) {
                float4 o = t.obs[j];
                float pr = ok ? lv[j * 32] * scale : 0.0f;
                acc.obs(o, pr, ST_OK, se2);
            }
        }
        return acc.finish(prior, t.inv_n);
    }
}

// ---------------------------------------------------------------------------
// Lane-split particle cost for the swarm's evaluation rounds.  A round
// evaluates the k particles held by lanes base .. base + k - 1 (the
// speculative rounds that reproduce the reference's in-loop global best
// re-evaluate only the particles after the first improver, so k shrinks
// within an iteration).  Each particle is evaluated by s = split_lanes(k)
// consecutive lanes, lane u of the group taking observations u, u + s, ...;
// the groups' compensated partial sums are combined in FP64 in lane order.
// Every lane of group g returns particle base + g's cost.  MetzgerKN (whose
// cost is dominated by the per-particle ODE sweep) does not use it.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int split_lanes(int k) {
    const int s = 32 / k;
    return s > 8 ? 8 : s;
}

template <int KIND>
__device__ __forceinline__ double particle_cost_split(const TaskCtx& t, const float* x, int base, int k) {
    const int lane = threadIdx.x & 31;
    const int s = split_lanes(k);
    const int g = lane / s, u = lane - g * s;
    const bool on = g < k;
    const int src = on ? base + g : lane;
    constexpr bool MB = KIND >= KIND_MB1;
    constexpr int NX = MB ? 4 * (KIND - KIND_MB1 + 1) + 2 : n_params_of(KIND);
    float xs[NX];
#pragma unroll
    for (int j = 0; j < NX; j++) xs[j] = __shfl_sync(FULL_MASK, x[j], src);
    Nll acc;
    acc.reset();
    double prior = 0.0;
    float villar_c = 0.0f;
    if constexpr (MB) {
        constexpr int K = KIND - KIND_MB1 + 1;
        float se = expf(xs[4 * K + 1]);
        if (on) acc = nll_multibazin<K>(xs, t.obs, t.n, se * se, u, s);
    } else {
        constexpr int m = KIND;
        constexpr int np = n_params_of(m);
        float p[MAXP];
        if (t.flags & TASK_T0_FIXED) {
            constexpr int t0i = t0_idx_of(m);
#pragma unroll
            for (int i = 0; i < np; i++) p[i] = i < t0i ? xs[i] : (i == t0i ? t.t0_fixed : xs[i - 1]);
        } else {
#pragma unroll
            for (int i = 0; i < np; i++) p[i] = xs[i];
        }
        if constexpr (m == VILLAR) villar_c = VillarF::constraint(p);
        if (t.flags & TASK_PRIOR) {
            float sp = 0.0f;
#pragma unroll
            for (int j = 0; j < np; j++) {
                float w = (float)c_pop_w[m][j];
                if (w > 0.0f) {
                    float z = (p[j] - (float)c_pop_c[m][j]) / w;
                    sp += 0.5f * z * z;
                }
            }
            prior = (double)sp;
        }
        float se = expf(p[se_idx_of(m)]);
        float se2 = se * se;
        if (on && !(villar_c > 0.0f)) {
            if constexpr (m == BAZIN) { BazinF e; e.init(p); acc = nll_loop(e, t.obs, t.n, se2, u, s); }
            else if constexpr (m == VILLAR) { VillarF e; e.init(p); acc = nll_loop(e, t.obs, t.n, se2, u, s); }
            else if constexpr (m == TDE) { TdeF e; e.init(p); acc = nll_loop(e, t.obs, t.n, se2, u, s); }
            else if constexpr (m == ARNETT) { ArnettF e; e.init(p); acc = nll_loop(e, t.obs, t.n, se2, u, s); }
            else if constexpr (m == MAGNETAR) { MagnetarF e; e.init(p); acc = nll_loop(e, t.obs, t.n, se2, u, s); }
            else if constexpr (m == SHOCK) { ShockF e; e.init(p); acc = nll_loop(e, t.obs, t.n, se2, u, s); }
            else if constexpr (m == AFTERGLOW) { AfterglowF e; e.init(p); acc = nll_loop(e, t.obs, t.n, se2, u, s); }
        }
    }
    double tot;
    float big;
    int nonfinite, inf;
    if (s == 1) {
        tot = (double)acc.s - (double)acc.c;
        big = acc.big;
        nonfinite = acc.nonfinite;
        inf = acc.inf;
    } else {
        tot = 0.0;
        big = -INFINITY;
        nonfinite = 0;
        inf = 0;
        const int flags = acc.nonfinite | (acc.inf << 1);
        for (int v = 0; v < s; v++) {
            const int sl = (g * s + v) & 31;
            const float ps = __shfl_sync(FULL_MASK, acc.s, sl), pc = __shfl_sync(FULL_MASK, acc.c, sl);
            const float pb = __shfl_sync(FULL_MASK, acc.big, sl);
            const int pf = __shfl_sync(FULL_MASK, flags, sl);
            tot += (double)ps - (double)pc;
            if (pb > -INFINITY) big = big > -INFINITY ? fmaxf(big, pb) + log1pf(expf(-fabsf(big - pb))) : pb;
            nonfinite |= pf & 1;
            inf |= pf >> 1;
        }
    }
    if constexpr (!MB && KIND == VILLAR) {
        if (villar_c > 0.0f) return 1e12 + 10000.0 * (double)villar_c;
    }
    return Nll::finish_sum(tot, big, nonfinite, inf, prior, t.inv_n);
}

// Runtime dispatch on the task kind (the likelihood API).
__device__ inline double particle_cost(const TaskCtx& t, const float* x, const double* pd = nullptr) {
    switch (t.kind) {
        case BAZIN: return particle_cost_k<BAZIN>(t, x, pd);
        case VILLAR: return particle_cost_k<VILLAR>(t, x, pd);
        case TDE: return particle_cost_k<TDE>(t, x, pd);
        case ARNETT: return particle_cost_k<ARNETT>(t, x, pd);
        case MAGNETAR: return particle_cost_k<MAGNETAR>(t, x, pd);
        case SHOCK: return particle_cost_k<SHOCK>(t, x, pd);
        case AFTERGLOW: return particle_cost_k<AFTERGLOW>(t, x, pd);
        default: return particle_cost_k<METZGER>(t, x, pd);
    }
}


}  // namespace lcf
