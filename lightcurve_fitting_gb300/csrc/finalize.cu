// finalize.cu — the FP64 stages after model selection and the dependent
// PSO stages' task builders:
//   * Laplace (laplace_fit, src/parametric.rs:2623-2693): central finite
//     difference Hessian of the unnormalised negative log-posterior over the
//     shape parameters, Jacobi eigen-decomposition, eigenvalue clamp 1e-6;
//   * profile_t0_refine (:2788-3008), profile_refine_all (:2705-2786) and the
//     magnitude-space chi2 (:3680-3711);
//   * the profile t0 search (:1767-1849) and the greedy MultiBazin K = 1..4
//     fit (:1008-1157), whose PSO runs execute in pso.cu and whose task lists
//     are appended here on the device, so the whole sequence needs no host
//     round trip.
// One warp per band; the lanes split the observations, the FP64 sums are
// reduced across the warp.
#include <cuda_runtime.h>

#include "lcf_internal.cuh"
#include "models_f32.cuh"
#include "models_f64.cuh"

namespace lcf {

#define FULL 0xffffffffu

__device__ __forceinline__ double wsum(double v) {
    for (int k = 16; k; k >>= 1) v += __shfl_xor_sync(FULL, v, k);
    return v;
}
__device__ __forceinline__ double wmax(double v) {
    for (int k = 16; k; k >>= 1) v = fmax(v, __shfl_xor_sync(FULL, v, k));
    return v;
}

struct BandView {
    const double *t, *f, *fe, *var, *uf, *mag;
    const uint8_t* up;
    int n;
    double peak;
};
__device__ __forceinline__ BandView band_view(const DeviceBatch& d, const BandStats& bs) {
    BandView v;
    v.t = d.t64 + bs.off; v.f = d.f64 + bs.off; v.fe = d.fe64 + bs.off; v.var = d.var64 + bs.off;
    v.uf = d.uf64 + bs.off; v.mag = d.mag64 + bs.off; v.up = d.up + bs.off;
    v.n = bs.n; v.peak = bs.peak;
    return v;
}

// Prediction of observation i (lanes call with their own i).  For MetzgerKN
// the whole band is first evaluated by lane 0 into `scr` (the sweep is
// sequential over the grid).
struct Predictor {
    int m;
    const double* p;
    const double* scr;
    Model64 mod;
    __device__ Predictor(int m_, const double* p_, const double* s_) : m(m_), p(p_), scr(s_) {
        if (m != 7) mod.init(m, p);
    }
    __device__ double operator()(const BandView& b, int i) const {
        return m == 7 ? scr[i] : mod.eval(b.t[i], nullptr);
    }
};
__device__ void metzger_prepare(int m, const double* p, const BandView& b, double* scr) {
    if (m != 7) return;
    if ((threadIdx.x & 31) == 0) metzger_f64(p, b.t, b.n, scr);
    __syncwarp();
}

// MetzgerKN rescale of the non-upper peak to 1 (src/parametric.rs:1325-1337)
__device__ double metzger_scale(const Predictor& P, const BandView& b) {
    int lane = threadIdx.x & 31;
    double mx = -INFINITY;
    for (int i = lane; i < b.n; i += 32)
        if (!b.up[i]) mx = fmax(mx, P(b, i));
    mx = wmax(mx);
    if (mx > 1e-10 && isfinite(mx)) return fmin(fmax(1.0 / mx, 0.1), 10.0);
    return 1.0;
}

// neg_log_posterior, src/parametric.rs:2464-2511
__device__ double neg_log_posterior_w(int m, const BandView& b, const double* p, double* scr) {
    int lane = threadIdx.x & 31;
    metzger_prepare(m, p, b, scr);
    Predictor P(m, p, scr);
    double scale = m == 7 ? metzger_scale(P, b) : 1.0;
    double se2 = exp(2.0 * p[se_idx_of(m)]);
    double nll = 0.0;
    int nonfinite = 0;
    for (int i = lane; i < b.n; i += 32) {
        double pr = P(b, i) * scale;
        if (!isfinite(pr)) { nonfinite = 1; continue; }
        double tv = b.var[i] + se2;
        if (b.up[i]) nll -= log_normal_cdf_f64((b.uf[i] - pr) / sqrt(tv));
        else {
            double dd = pr - b.f[i];
            nll += 0.5 * (dd * dd / tv + log(2.0 * 3.14159265358979323846 * tv));
        }
    }
    if (__any_sync(FULL, nonfinite)) return 1e99;
    nll = wsum(nll);
    double nlp = 0.0;
    for (int j = 0; j < n_params_of(m); j++) {
        double w = c_pri_w[m][j], dd = p[j] - c_pri_c[m][j];
        nlp += 0.5 * dd * dd / (w * w);
    }
    __syncwarp();
    return nll + nlp;
}

// Band log-likelihood skipping non-finite predictions (the profile scans,
// src/parametric.rs:2716-2726, :2916-2932)
__device__ double band_ll_w(int m, const BandView& b, const double* p, double* scr, bool metzger_rescale) {
    int lane = threadIdx.x & 31;
    metzger_prepare(m, p, b, scr);
    Predictor P(m, p, scr);
    double scale = (m == 7 && metzger_rescale) ? metzger_scale(P, b) : 1.0;
    double se2 = exp(2.0 * p[se_idx_of(m)]);
    double ll = 0.0;
    for (int i = lane; i < b.n; i += 32) {
        double pr = P(b, i) * scale;
        if (!isfinite(pr)) continue;
        double tv = b.var[i] + se2;
        if (b.up[i]) ll += log_normal_cdf_f64((b.uf[i] - pr) / sqrt(tv));
        else {
            double r = b.f[i] - pr;
            ll += -0.5 * (r * r / tv + log(2.0 * 3.14159265358979323846 * tv));
        }
    }
    ll = wsum(ll);
    __syncwarp();
    return ll;
}

// ---------------------------------------------------------------------------
// The refinement scans of models other than MetzgerKN evaluate the model in
// FP32 (the evaluators of models_f32.cuh, on the band's FP32 time records)
// and form each observation's term in FP64 from per-band constants that do
// not change across the scans (sigma_extra is fixed there): 1/tv, 1/sqrt(tv)
// and ln(2 pi tv).  The scans compare log-likelihoods against thresholds
// 0.5 apart and pick grid points, so FP32 prediction rounding (1e-7
// relative) moves no decision except a value within ~1e-5 of a threshold.
// ---------------------------------------------------------------------------
__device__ void scan_constants(const BandView& b, double se2, double* cst) {
    for (int i = threadIdx.x & 31; i < b.n; i += 32) {
        double tv = b.var[i] + se2;
        cst[3 * i] = 1.0 / tv;
        cst[3 * i + 1] = 1.0 / sqrt(tv);
        cst[3 * i + 2] = log(2.0 * 3.14159265358979323846 * tv);
    }
    __syncwarp();
}

// FP32 prediction -> FP64 value; false for a prediction the reference finds
// non-finite (skipped by the scans).  Huge predictions come back through
// their logarithm (ST_BIG) and are finite in FP64.
__device__ __forceinline__ bool pred_f64(float pf, int st, double& pr) {
    if (st == ST_NONFINITE) return false;
    pr = st == ST_BIG ? exp((double)pf) : (double)pf;
    return true;
}

__device__ __forceinline__ double ll_term(const BandView& b, int i, double pr, const double* cst) {
    const double* c = cst + 3 * i;
    if (b.up[i]) {
        double z = (b.uf[i] - pr) * c[1];
        if (z > -1e15) return (double)log_normal_cdf_f((float)z);
        return -0.5 * z * z - 0.9189385332046727 - log(-z);
    }
    double r = b.f[i] - pr;
    return -0.5 * (r * r * c[0] + c[2]);
}

template <class F>
__device__ double ll_scan_t(const double* p, const float4* obs, const BandView& b, const double* cst) {
    F e;
    e.init64(p);
    double ll = 0.0;
    for (int i = threadIdx.x & 31; i < b.n; i += 32) {
        float4 o = obs[i];
        int st = ST_OK;
        float pf = e.eval(o.x, o.y, st);
        double pr;
        if (!pred_f64(pf, st, pr)) continue;
        ll += ll_term(b, i, pr, cst);
    }
    return wsum(ll);
}

// band_ll_w for the models other than MetzgerKN, FP32 evaluation
__device__ double band_ll_fast(int m, const double* p, const float4* obs, const BandView& b, const double* cst) {
    switch (m) {
        case BAZIN: return ll_scan_t<BazinF>(p, obs, b, cst);
        case VILLAR: return ll_scan_t<VillarF>(p, obs, b, cst);
        case TDE: return ll_scan_t<TdeF>(p, obs, b, cst);
        case ARNETT: return ll_scan_t<ArnettF>(p, obs, b, cst);
        case MAGNETAR: return ll_scan_t<MagnetarF>(p, obs, b, cst);
        case SHOCK: return ll_scan_t<ShockF>(p, obs, b, cst);
        default: return ll_scan_t<AfterglowF>(p, obs, b, cst);
    }
}

// Weighted sums of the unit-amplitude shape for the amplitude (and baseline)
// solve of profile_t0_refine: sw, sy, sf, syf, sff over detections.
template <class F>
__device__ void shape_sums_t(const double* p, const float4* obs, const BandView& b, const double* cst, double* s5) {
    F e;
    e.init64(p);
    double sw = 0, sy = 0, sf = 0, syf = 0, sff = 0;
    for (int i = threadIdx.x & 31; i < b.n; i += 32) {
        if (b.up[i]) continue;
        float4 o = obs[i];
        int st = ST_OK;
        float pf = e.eval(o.x, o.y, st);
        double sh;
        if (!pred_f64(pf, st, sh) || !isfinite(sh)) continue;
        double w = cst[3 * i];
        sw += w; sy += w * b.f[i]; sf += w * sh; syf += w * b.f[i] * sh; sff += w * sh * sh;
    }
    s5[0] = wsum(sw); s5[1] = wsum(sy); s5[2] = wsum(sf); s5[3] = wsum(syf); s5[4] = wsum(sff);
}

__device__ void shape_sums_fast(int m, const double* p, const float4* obs, const BandView& b, const double* cst,
                                double* s5) {
    switch (m) {
        case BAZIN: shape_sums_t<BazinF>(p, obs, b, cst, s5); break;
        case VILLAR: shape_sums_t<VillarF>(p, obs, b, cst, s5); break;
        case TDE: shape_sums_t<TdeF>(p, obs, b, cst, s5); break;
        case ARNETT: shape_sums_t<ArnettF>(p, obs, b, cst, s5); break;
        case MAGNETAR: shape_sums_t<MagnetarF>(p, obs, b, cst, s5); break;
        case SHOCK: shape_sums_t<ShockF>(p, obs, b, cst, s5); break;
        default: shape_sums_t<AfterglowF>(p, obs, b, cst, s5); break;
    }
}

// ---------------------------------------------------------------------------
// MetzgerKN refinement scans, one scan point per lane.  The scans evaluate
// up to ~140 independent parameter vectors per band; each lane integrates
// its own vector's ODE (FP64, metzger_sweep64 — the arithmetic of
// metzger_f64) twice: the first sweep finds the peak the predictions are
// normalised by (and the largest detection prediction for the rescale), the
// second forms the band's terms in observation order.
// ---------------------------------------------------------------------------
struct MzPeak {
    const uint8_t* up;
    double mx;  // largest unnormalised detection interpolant
    __device__ void operator()(int j, double l) {
        if (!up[j]) mx = fmax(mx, l);
    }
};

struct MzLl {
    const BandView* b;
    const double* cst;
    double inv_peak, scale, ll;
    __device__ void term(int j, double pr) {
        if (!isfinite(pr)) return;
        const double* c = cst + 3 * j;
        if (b->up[j]) {
            ll += log_normal_cdf_f64((b->uf[j] - pr) * c[1]);
        } else {
            double r = b->f[j] - pr;
            ll += -0.5 * (r * r * c[0] + c[2]);
        }
    }
    __device__ void operator()(int j, double l) { term(j, l * inv_peak * scale); }
};

// Bands of at most MZ_KEEP observations keep the first sweep's interpolants
// in shared memory (lane-interleaved: entry j of a lane at keep[32 j]) and
// form the terms from them, in the second sweep's order, instead of
// integrating the ODE again; longer bands sweep twice.
constexpr int MZ_KEEP = 32;
struct MzKeep {
    const uint8_t* up;
    double* keep;
    double mx;
    __device__ void operator()(int j, double l) {
        if (!up[j]) mx = fmax(mx, l);
        keep[32 * j] = l;
    }
};
__device__ __forceinline__ bool metzger_first_sweep(const double* p, const BandView& b, double* keep, double& mx,
                                                    int& j_start, double& l_peak) {
    if (keep) {
        MzKeep kp{b.up, keep, -INFINITY};
        bool ok = metzger_sweep64(p, b.t, b.n, kp, j_start, l_peak);
        mx = kp.mx;
        return ok;
    }
    MzPeak pk{b.up, -INFINITY};
    bool ok = metzger_sweep64(p, b.t, b.n, pk, j_start, l_peak);
    mx = pk.mx;
    return ok;
}

// band_ll_w for MetzgerKN by one lane (rescale: the PSO cost's peak rescale);
// keep: this lane's interpolant slots (nullptr: sweep twice)
__device__ double metzger_ll_lane(const double* p, const BandView& b, const double* cst, bool rescale,
                                  double* keep) {
    if (b.n > MZ_KEEP) keep = nullptr;
    MzPeak pk{b.up, -INFINITY};
    int j_start;
    double l_peak;
    bool ok = metzger_first_sweep(p, b, keep, pk.mx, j_start, l_peak);
    bool valid = ok && l_peak > 0.0 && isfinite(l_peak);
    double scale = 1.0;
    if (rescale) {
        // largest normalised detection prediction; invalid sweeps and the
        // observations before t0 predict 0
        double mx = -INFINITY;
        int z_end = valid ? j_start : b.n;
        for (int j = 0; j < z_end; j++)
            if (!b.up[j]) mx = fmax(mx, 0.0);
        if (valid) mx = fmax(mx, pk.mx / l_peak);
        if (mx > 1e-10 && isfinite(mx)) scale = fmin(fmax(1.0 / mx, 0.1), 10.0);
    }
    MzLl acc{&b, cst, valid ? 1.0 / l_peak : 0.0, scale, 0.0};
    int z_end = valid ? j_start : b.n;
    for (int j = 0; j < z_end; j++) acc.term(j, 0.0 * scale);
    if (valid) {
        // the same interpolants, normalised
        struct Norm {
            MzLl* a;
            double lpk;
            __device__ void operator()(int j, double l) { a->term(j, l / lpk * a->scale); }
        } nv{&acc, l_peak};
        if (keep) {
            for (int j = j_start; j < b.n; j++) nv(j, keep[32 * j]);
        } else {
            int js;
            double lp;
            metzger_sweep64(p, b.t, b.n, nv, js, lp);
        }
    }
    return acc.ll;
}

// shape sums of profile_t0_refine for MetzgerKN by one lane: sw, sy, sf,
// syf, sff over detections of the normalised prediction
__device__ void metzger_shape_lane(const double* p, const BandView& b, const double* cst, double* s5, double* keep) {
    if (b.n > MZ_KEEP) keep = nullptr;
    double mx_unused;
    int j_start;
    double l_peak;
    bool ok = metzger_first_sweep(p, b, keep, mx_unused, j_start, l_peak);
    bool valid = ok && l_peak > 0.0 && isfinite(l_peak);
    double sw = 0, sy = 0, sf = 0, syf = 0, sff = 0;
    int z_end = valid ? j_start : b.n;
    for (int j = 0; j < z_end; j++) {
        if (b.up[j]) continue;
        double w = cst[3 * j];
        sw += w; sy += w * b.f[j];
    }
    if (valid) {
        struct Sums {
            const BandView* b;
            const double* cst;
            double lpk, sw, sy, sf, syf, sff;
            __device__ void operator()(int j, double l) {
                if (b->up[j]) return;
                double sh = l / lpk;
                if (!isfinite(sh)) return;
                double w = cst[3 * j], fj = b->f[j];
                sw += w; sy += w * fj; sf += w * sh; syf += w * fj * sh; sff += w * sh * sh;
            }
        } su{&b, cst, l_peak, sw, sy, sf, syf, sff};
        if (keep) {
            for (int j = j_start; j < b.n; j++) su(j, keep[32 * j]);
        } else {
            int js;
            double lp;
            metzger_sweep64(p, b.t, b.n, su, js, lp);
        }
        sw = su.sw; sy = su.sy; sf = su.sf; syf = su.syf; sff = su.sff;
    }
    s5[0] = sw; s5[1] = sy; s5[2] = sf; s5[3] = syf; s5[4] = sff;
}

// profile_t0_refine + profile_refine_all for a MetzgerKN band (np = 5,
// t0 = p[3], sigma_extra = p[4]; no baseline parameter), lanes over scan
// points; the sequential decisions run uniformly on the gathered values.
__device__ void refine_metzger(const BandStats& bs, const BandView& b, const double* cst, double* mu, double* ls,
                               double* keep) {
    const int lane = threadIdx.x & 31;
    constexpr int m = METZGER, np = 5, se = 4, t0i = 3, NG = 25;
    double t0_lo = bs.t_first - 30.0, t0_hi = bs.t_peak_all + 5.0;
    if (t0_lo < t0_hi) {
        auto grid = [&](int gi) { return t0_lo + (t0_hi - t0_lo) * (double)gi / (double)(NG - 1); };
        // profiled amplitude at each grid t0, then its log-likelihood (rescaled)
        double my_ll = -INFINITY;
        if (lane < NG) {
            double p[MAXP];
            for (int j = 0; j < np; j++) p[j] = mu[j];
            p[t0i] = grid(lane);
            double saved_la = p[0];
            p[0] = 0.0;
            double s5[5];
            metzger_shape_lane(p, b, cst, s5, keep);
            double syf = s5[3], sff = s5[4];
            if (sff > 1e-20 && syf / sff > 1e-10) p[0] = log(syf / sff);
            else p[0] = saved_la;
            my_ll = metzger_ll_lane(p, b, cst, true, keep);
        }
        double best_t0 = mu[t0i], best_ll = -INFINITY;
        for (int gi = 0; gi < NG; gi++) {
            double l = __shfl_sync(FULL, my_ll, gi);
            if (l > best_ll) { best_ll = l; best_t0 = grid(gi); }
        }
        // log-likelihood at mu with t0 on each grid point (no rescale)
        double e_ll = -INFINITY;
        if (lane < NG) {
            double p[MAXP];
            for (int j = 0; j < np; j++) p[j] = mu[j];
            p[t0i] = grid(lane);
            e_ll = metzger_ll_lane(p, b, cst, false, keep);
        }
        double lo1 = best_t0, hi1 = best_t0, thr = best_ll - 0.5;
        for (int gi = NG - 1; gi >= 0; gi--) {
            double t0 = grid(gi);
            double l = __shfl_sync(FULL, e_ll, gi);
            if (t0 >= best_t0) continue;
            if (l >= thr) lo1 = t0;
            else break;
        }
        for (int gi = 0; gi < NG; gi++) {
            double t0 = grid(gi);
            double l = __shfl_sync(FULL, e_ll, gi);
            if (t0 <= best_t0) continue;
            if (l >= thr) hi1 = t0;
            else break;
        }
        mu[t0i] = best_t0;
        ls[t0i] = log(fmax((hi1 - lo1) / 2.0, 0.1));
    }
    // profile_refine_all: evaluation 0 = mu, 1 + 15 j + gi = parameter j on
    // grid point gi; two rounds of 32 lanes
    constexpr int NE = 1 + 4 * 15;
    double r_ll[2];
    for (int round = 0; round < 2; round++) {
        int e = round * 32 + lane;
        r_ll[round] = -INFINITY;
        if (e < NE) {
            double p[MAXP];
            for (int k = 0; k < np; k++) p[k] = mu[k];
            if (e > 0) {
                int j = (e - 1) / 15, gi = (e - 1) % 15;
                double slo = c_lo[m][j], shi = c_hi[m][j];
                p[j] = slo + (shi - slo) * (double)gi / 14.0;
            }
            r_ll[round] = metzger_ll_lane(p, b, cst, false, keep);
        }
    }
    auto get = [&](int e) {
        double a = __shfl_sync(FULL, r_ll[0], e & 31), c = __shfl_sync(FULL, r_ll[1], e & 31);
        return e < 32 ? a : c;
    };
    double thr = get(0) - 0.5;
    for (int j = 0; j < np; j++) {
        if (j == se) continue;
        double mu_j = mu[j], svi_sigma = exp(ls[j]);
        double slo = c_lo[m][j], shi = c_hi[m][j];
        if (shi - slo < 1e-10) continue;
        double l1 = mu_j, h1 = mu_j;
        for (int gi = 0; gi < 15; gi++) {
            double val = slo + (shi - slo) * (double)gi / 14.0;
            if (get(1 + j * 15 + gi) >= thr) { l1 = fmin(l1, val); h1 = fmax(h1, val); }
        }
        double prof = fmax((h1 - l1) / 2.0, 1e-6);
        ls[j] = log(fmax(fmax(svi_sigma, prof), c_pop_w[m][j]));
    }
}

// symmetric_eigen (Jacobi), src/parametric.rs:2517-2587
__device__ void jacobi_eigen(double* a, int n, double* ev, double* V) {
    for (int i = 0; i < n * n; i++) V[i] = 0.0;
    for (int i = 0; i < n; i++) V[i * n + i] = 1.0;
    int max_iter = 100 * n * n;
    for (int itr = 0; itr < max_iter; itr++) {
        double mv = 0.0;
        int p = 0, q = 1;
        for (int i = 0; i < n; i++)
            for (int j = i + 1; j < n; j++) {
                double v = fabs(a[i * n + j]);
                if (v > mv) { mv = v; p = i; q = j; }
            }
        double app = a[p * n + p], aqq = a[q * n + q], apq = a[p * n + q];
        // the reference stops below 1e-15 absolute, which a Hessian with
        // entries ~1e6 never reaches (its rotations leave ~1e-10): it then
        // runs all 100 n^2 rotations, each of them below rounding level once
        // the largest off-diagonal element is below 1e-15 of its diagonal
        // pair.  Stopping there too changes the eigenvalues at rounding level
        // and spares the FP64 trigonometry of those rotations.
        if (mv < 1e-15 || mv <= 1e-15 * sqrt(fabs(app * aqq))) break;
        double th = fabs(app - aqq) < 1e-30 ? 0.78539816339744830962 : 0.5 * atan(2.0 * apq / (app - aqq));
        double c = cos(th), s = sin(th);
        for (int i = 0; i < n; i++) {
            double aip = a[i * n + p], aiq = a[i * n + q];
            a[i * n + p] = c * aip + s * aiq;
            a[i * n + q] = -s * aip + c * aiq;
        }
        for (int j = 0; j < n; j++) {
            double apj = a[p * n + j], aqj = a[q * n + j];
            a[p * n + j] = c * apj + s * aqj;
            a[q * n + j] = -s * apj + c * aqj;
        }
        a[p * n + p] = c * c * app + 2.0 * c * s * apq + s * s * aqq;
        a[q * n + q] = s * s * app - 2.0 * c * s * apq + c * c * aqq;
        a[p * n + q] = 0.0;
        a[q * n + p] = 0.0;
        for (int i = 0; i < n; i++) {
            double vip = V[i * n + p], viq = V[i * n + q];
            V[i * n + p] = c * vip + s * viq;
            V[i * n + q] = -s * vip + c * viq;
        }
    }
    for (int i = 0; i < n; i++) ev[i] = a[i * n + i];
}

// ---------------------------------------------------------------------------
// Bands grouped by their selected model (counting sort on 9 keys: MetzgerKN,
// whose uncertainty and refinements cost the most, first, then models 0..6,
// then the unfitted bands).  The per-band kernels take band_order[warp], so
// the warps resident on an SM run one model's code and no warp slot is spent
// on a band that selected another model.  The order inside a key is not
// fixed; each band's computation does not depend on it.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int band_order_key(const DeviceBatch& d, int b) {
    const int m = d.out[b].model;
    if (!d.stats[b].valid || m < 0) return 8;
    return m == METZGER ? 0 : 1 + m;
}
__global__ void band_hist_kernel(DeviceBatch d) {
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < d.n_bands; b += gridDim.x * blockDim.x)
        atomicAdd(&d.ctr->band_hist[band_order_key(d, b)], 1);
}
__global__ void band_scan_kernel(DeviceBatch d) {  // one thread
    int run = 0;
    for (int k = 0; k < 9; k++) {
        const int v = d.ctr->band_hist[k];
        d.ctr->band_hist[k] = run;
        run += v;
    }
}
__global__ void band_scatter_kernel(DeviceBatch d) {
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < d.n_bands; b += gridDim.x * blockDim.x)
        d.band_order[atomicAdd(&d.ctr->band_hist[band_order_key(d, b)], 1)] = b;
}
void launch_band_order(const DeviceBatch& d, cudaStream_t s) {
    if (d.n_bands == 0) return;
    int grid = (d.n_bands + 255) / 256;
    grid = grid < 1024 ? grid : 1024;
    band_hist_kernel<<<grid, 256, 0, s>>>(d);
    band_scan_kernel<<<1, 1, 0, s>>>(d);
    band_scatter_kernel<<<grid, 256, 0, s>>>(d);
}

// neg_log_posterior (src/parametric.rs:2464-2511) of MetzgerKN at one
// parameter vector, by one lane: a first FP64 sweep for the rescale's peak
// (the largest non-upper prediction), a second for the terms in observation
// order, as the reference sums them.
__device__ double metzger_nlp_lane(const BandView& b, const double* p) {
    struct Peak {
        const uint8_t* up;
        double mx;
        __device__ void operator()(int j, double l) {
            if (!up[j]) mx = fmax(mx, l);
        }
    } pk{b.up, -INFINITY};
    int j_start;
    double l_peak;
    bool ok = metzger_sweep64(p, b.t, b.n, pk, j_start, l_peak) && l_peak > 0.0 && isfinite(l_peak);
    // the predictions before the first visited observation are 0
    double mx = pk.mx / l_peak;
    for (int j = 0; j < (ok ? j_start : b.n); j++)
        if (!b.up[j]) mx = ok ? fmax(mx, 0.0) : 0.0;
    if (!ok) mx = b.n > 0 ? 0.0 : -INFINITY;
    const double scale = (mx > 1e-10 && isfinite(mx)) ? fmin(fmax(1.0 / mx, 0.1), 10.0) : 1.0;
    const double se2 = exp(2.0 * p[se_idx_of(METZGER)]);
    struct Terms {
        const BandView* b;
        double peak, scale, se2, nll;
        int nonfinite;
        __device__ void term(int i, double pr) {
            if (!isfinite(pr)) { nonfinite = 1; return; }
            const double tv = b->var[i] + se2;
            if (b->up[i]) nll -= log_normal_cdf_f64((b->uf[i] - pr) / sqrt(tv));
            else {
                const double dd = pr - b->f[i];
                nll += 0.5 * (dd * dd / tv + log(2.0 * 3.14159265358979323846 * tv));
            }
        }
        __device__ void operator()(int j, double l) { term(j, (l / peak) * scale); }
    } tm{&b, l_peak, scale, se2, 0.0, 0};
    if (ok) {
        for (int j = 0; j < j_start; j++) tm.term(j, 0.0 * scale);
        metzger_sweep64(p, b.t, b.n, tm, j_start, l_peak);
    } else {
        for (int j = 0; j < b.n; j++) tm.term(j, 0.0 * scale);
    }
    if (tm.nonfinite) return 1e99;
    double nlp = 0.0;
    for (int j = 0; j < n_params_of(METZGER); j++) {
        const double w = c_pri_w[METZGER][j], dd = p[j] - c_pri_c[METZGER][j];
        nlp += 0.5 * dd * dd / (w * w);
    }
    return tm.nll + nlp;
}

// MetzgerKN's Laplace Hessian as the reference takes it (central differences
// of the cost, :2623-2693), with the stencil's points spread over the lanes:
// point 0 is the MAP (its cost f0), points 1 + 4k .. 4 + 4k the four
// evaluations of the k-th pair (si <= sj).  Warp-collective.
__device__ void laplace_fd_metzger(const BandView& b, const double* mp, const int* idx, int ns, double* H,
                                   double& f0) {
    const int lane = threadIdx.x & 31;
    const int npts = 1 + 2 * ns * (ns + 1);
    double c[2] = {0.0, 0.0};
    for (int r = 0; r < 2; r++) {
        const int pt = lane + 32 * r;
        if (pt >= npts) continue;
        double q[MAXP];
        for (int t = 0; t < n_params_of(METZGER); t++) q[t] = mp[t];
        if (pt > 0) {
            int k = (pt - 1) >> 2, si = 0;
            while (k >= ns - si) { k -= ns - si; si++; }
            const int sj = si + k, s4 = (pt - 1) & 3;
            const int i = idx[si], j = idx[sj];
            const double hi = 1e-4 * fmax(fabs(mp[i]), 1.0), hj = 1e-4 * fmax(fabs(mp[j]), 1.0);
            q[i] += (s4 < 2 ? 1.0 : -1.0) * hi;
            q[j] += ((s4 & 1) == 0 ? 1.0 : -1.0) * hj;
        }
        c[r] = metzger_nlp_lane(b, q);
    }
    auto cost = [&](int pt) {
        const double v = pt < 32 ? c[0] : c[1];
        return __shfl_sync(FULL, v, pt & 31);
    };
    f0 = cost(0);
    int k = 0;
    for (int si = 0; si < ns; si++) {
        const double hi = 1e-4 * fmax(fabs(mp[idx[si]]), 1.0);
        for (int sj = si; sj < ns; sj++, k++) {
            const double hj = 1e-4 * fmax(fabs(mp[idx[sj]]), 1.0);
            const double h = (cost(1 + 4 * k) - cost(2 + 4 * k) - cost(3 + 4 * k) + cost(4 + 4 * k)) / (4.0 * hi * hj);
            H[si * ns + sj] = h;
            H[sj * ns + si] = h;
        }
    }
}

// Analytic Hessian of neg_log_posterior (src/parametric.rs:2464-2507) over the
// shape parameters idx[0..ns), sigma_extra held fixed as laplace_fit holds
// it (:2623-2693).  Forward mode over the analytic gradient: column k is the
// derivative along parameter idx[k] of
//   sum_i dl_i/dpred * grad pred_i + the prior's gradient,
// i.e. sum_i (d2l_i/dpred2 g_j g_k + dl_i/dpred h_jk) + the prior's 1 / w^2
// on the diagonal, with g = grad pred and its column h from the model
// gradient evaluated on Dual numbers, and the upper-limit term's log-CDF
// derivatives from a second-order Taylor number.  The reference takes the
// same matrix by central differences of its cost (4 evaluations per pair,
// step 1e-4 max(|theta|, 1)).  Models 0..6; warp-collective, lanes over
// observations.  Returns false when a prediction or an entry is not finite
// (the caller then takes the reference's finite differences).
__device__ bool laplace_hessian_analytic(int m, const BandView& b, const double* mp, const int* idx, int ns,
                                         double* H) {
    const int lane = threadIdx.x & 31;
    const int nf = n_params_of(m), se = se_idx_of(m);
    const double se2 = exp(2.0 * mp[se]);
    int bad = 0;
    for (int sk = 0; sk < ns; sk++) {
        Dual q[MAXP];
        for (int j = 0; j < nf; j++) q[j] = Dual(mp[j], j == idx[sk] ? 1.0 : 0.0);
        double col[MAXP];
        for (int sj = 0; sj < ns; sj++) col[sj] = 0.0;
        for (int i = lane; i < b.n; i += 32) {
            Dual g[MAXP];
            model_grad_t<Dual>(m, q, Dual(b.t[i]), g);
            const double pr = eval_model_f64(m, mp, b.t[i]);
            if (!isfinite(pr)) {
                bad = 1;
                continue;
            }
            const double tv = b.var[i] + se2;
            double a1, a2;  // dl / dpred and d2l / dpred2
            if (b.up[i]) {
                // l = -log Phi(z), z = (u - pred) / s
                const double s = sqrt(tv);
                const Jet2 L = log_normal_cdf_jet(Jet2((b.uf[i] - pr) / s, 1.0, 0.0));
                a1 = L.c1 / s;
                a2 = -2.0 * L.c2 / tv;
            } else {
                // l = ((pred - y)^2 / tv + ln(2 pi tv)) / 2
                a1 = (pr - b.f[i]) / tv;
                a2 = 1.0 / tv;
            }
            const double gk = g[idx[sk]].v;
            for (int sj = 0; sj < ns; sj++) col[sj] += a2 * g[idx[sj]].v * gk + a1 * g[idx[sj]].d;
        }
        for (int sj = 0; sj < ns; sj++) {
            double v = wsum(col[sj]);
            if (sj == sk) {
                const double w = c_pri_w[m][idx[sj]];
                v += 1.0 / (w * w);
            }
            H[sj * ns + sk] = v;
        }
    }
    for (int a = 0; a < ns; a++)
        for (int c = a; c < ns; c++) {
            const double v = 0.5 * (H[a * ns + c] + H[c * ns + a]);
            H[a * ns + c] = v;
            H[c * ns + a] = v;
            if (!isfinite(v)) bad = 1;
        }
    return !__any_sync(FULL, bad);
}

__global__ void laplace_kernel(DeviceBatch d) {
    int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (warp >= d.n_bands) return;
    warp = d.band_order[warp];
    BandStats bs = d.stats[warp];
    BandOut& o = d.out[warp];
    if (!bs.valid || o.model < 0) return;
    BandView b = band_view(d, bs);
    int m = o.model, nf = n_params_of(m), se = se_idx_of(m);
    double* scr = d.scratch64 + 5 * bs.off;
    double mp[MAXP];
    for (int j = 0; j < nf; j++) mp[j] = o.pso_params[j];
    int idx[MAXP], ns = 0;
    for (int i = 0; i < nf; i++)
        if (i != se) idx[ns++] = i;
    double H[36];
    // the analytic Hessian (forward over the adjoint); MetzgerKN, whose
    // gradient is itself a finite difference in the reference, and points
    // with non-finite predictions keep the reference's central differences
    // (MetzgerKN's with one stencil point per lane)
    double f0;
    if (m == METZGER) laplace_fd_metzger(b, mp, idx, ns, H, f0);
    else f0 = neg_log_posterior_w(m, b, mp, scr);
    const bool analytic = m == METZGER || (f0 < 1e99 && laplace_hessian_analytic(m, b, mp, idx, ns, H));
    for (int si = 0; si < ns && !analytic; si++) {
        int i = idx[si];
        double hi = 1e-4 * fmax(fabs(mp[i]), 1.0);
        for (int sj = si; sj < ns; sj++) {
            int j = idx[sj];
            double hj = 1e-4 * fmax(fabs(mp[j]), 1.0);
            double q[MAXP];
            double fv[4];
            const double si_[4] = {1, 1, -1, -1}, sj_[4] = {1, -1, 1, -1};
            for (int k = 0; k < 4; k++) {
                for (int t = 0; t < nf; t++) q[t] = mp[t];
                q[i] += si_[k] * hi;
                q[j] += sj_[k] * hj;
                fv[k] = neg_log_posterior_w(m, b, q, scr);
            }
            double h = (fv[0] - fv[1] - fv[2] + fv[3]) / (4.0 * hi * hj);
            H[si * ns + sj] = h;
            H[sj * ns + si] = h;
        }
    }
    if ((threadIdx.x & 31) == 0) {
        double ev[MAXP], V[36];
        jacobi_eigen(H, ns, ev, V);
        double sls[MAXP];
        for (int i = 0; i < ns; i++) {
            double sum = 0.0;
            for (int k = 0; k < ns; k++) sum += V[i * ns + k] * V[i * ns + k] * (1.0 / fmax(ev[k], 1e-6));
            sls[i] = 0.5 * log(fmax(sum, 1e-30));
        }
        int s2 = 0;
        for (int i = 0; i < MAXP; i++) {
            o.mu[i] = i < nf ? mp[i] : NAN;
            if (i >= nf) o.log_sigma[i] = NAN;
            else if (i == se) o.log_sigma[i] = log(c_pri_w[m][i]);
            else o.log_sigma[i] = sls[s2++];
        }
        o.elbo = -f0;
        o.svi_steps = 0;
    }
}

void launch_laplace(const DeviceBatch& d, cudaStream_t s) {
    if (d.n_bands == 0) return;
    int64_t threads = (int64_t)d.n_bands * 32;
    laplace_kernel<<<(int)((threads + 127) / 128), 128, 0, s>>>(d);
}

// profile_t0_refine + profile_refine_all + mag chi2
#ifndef LCF_REFINE_BLOCK
#define LCF_REFINE_BLOCK 128
#endif
__global__ void refine_kernel(DeviceBatch d) {
    int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    if (warp >= d.n_bands) return;
    warp = d.band_order[warp];
    BandStats bs = d.stats[warp];
    BandOut& o = d.out[warp];
    if (!bs.valid || o.model < 0) return;
    BandView b = band_view(d, bs);
    int m = o.model, np = n_params_of(m), se = se_idx_of(m), t0i = t0_idx_of(m);
    double* scr = d.scratch64 + 5 * bs.off;
    double mu[MAXP], ls[MAXP];
    for (int j = 0; j < np; j++) { mu[j] = o.mu[j]; ls[j] = o.log_sigma[j]; }
    // scans of the models other than MetzgerKN: FP32 evaluation, FP64 terms;
    // MetzgerKN: FP64 sweeps, one scan point per lane
    const bool fast = m != METZGER;
    const float4* obs = d.obs + bs.off;
    scan_constants(b, exp(2.0 * mu[se]), scr);
    if (!fast) {
        extern __shared__ double rf_keep[];
        refine_metzger(bs, b, scr, mu, ls, rf_keep + (size_t)(threadIdx.x >> 5) * 32 * MZ_KEEP + lane);
    }
    auto scan_ll = [&](const double* p, bool rescale) {
        return fast ? band_ll_fast(m, p, obs, b, scr) : band_ll_w(m, b, p, scr, rescale);
    };
    // ---- profile_t0_refine
    if (fast) {
        double t0_lo = bs.t_first - 30.0, t0_hi = bs.t_peak_all + 5.0;
        if (t0_lo < t0_hi) {
            const int NG = 25;
            double sx2 = exp(2.0 * mu[se]);
            bool has_b = (m == BAZIN || m == TDE);
            double best_t0 = mu[t0i], best_ll = -INFINITY;
            for (int gi = 0; gi < NG; gi++) {
                double t0 = t0_lo + (t0_hi - t0_lo) * (double)gi / (double)(NG - 1);
                double p[MAXP];
                for (int j = 0; j < np; j++) p[j] = mu[j];
                p[t0i] = t0;
                double saved_la = p[0];
                p[0] = 0.0;
                double saved_b = 0.0;
                if (has_b) { saved_b = p[1]; p[1] = 0.0; }
                double sw = 0, sy = 0, sf = 0, syf = 0, sff = 0;
                if (fast) {
                    double s5[5];
                    shape_sums_fast(m, p, obs, b, scr, s5);
                    sw = s5[0]; sy = s5[1]; sf = s5[2]; syf = s5[3]; sff = s5[4];
                } else {
                    metzger_prepare(m, p, b, scr);
                    Predictor P(m, p, scr);
                    for (int i = lane; i < b.n; i += 32) {
                        double sh = P(b, i);
                        if (b.up[i] || !isfinite(sh)) continue;
                        double w = 1.0 / (b.var[i] + sx2);
                        sw += w; sy += w * b.f[i]; sf += w * sh; syf += w * b.f[i] * sh; sff += w * sh * sh;
                    }
                    sw = wsum(sw); sy = wsum(sy); sf = wsum(sf); syf = wsum(syf); sff = wsum(sff);
                    __syncwarp();
                }
                if (has_b) {
                    double det = sw * sff - sf * sf;
                    if (fabs(det) > 1e-20) {
                        double a_opt = (sw * syf - sf * sy) / det, b_opt = (sff * sy - sf * syf) / det;
                        if (a_opt > 1e-10) { p[0] = log(a_opt); p[1] = b_opt; }
                        else { p[0] = saved_la; p[1] = saved_b; }
                    } else { p[0] = saved_la; p[1] = saved_b; }
                } else {
                    if (sff > 1e-20 && syf / sff > 1e-10) p[0] = log(syf / sff);
                    else p[0] = saved_la;
                }
                double ll = scan_ll(p, true);
                if (ll > best_ll) { best_ll = ll; best_t0 = t0; }
            }
            double lo1 = best_t0, hi1 = best_t0, thr = best_ll - 0.5;
            for (int gi = NG - 1; gi >= 0; gi--) {
                double t0 = t0_lo + (t0_hi - t0_lo) * (double)gi / (double)(NG - 1);
                if (t0 >= best_t0) continue;
                double p[MAXP];
                for (int j = 0; j < np; j++) p[j] = mu[j];
                p[t0i] = t0;
                if (scan_ll(p, false) >= thr) lo1 = t0;
                else break;
            }
            for (int gi = 0; gi < NG; gi++) {
                double t0 = t0_lo + (t0_hi - t0_lo) * (double)gi / (double)(NG - 1);
                if (t0 <= best_t0) continue;
                double p[MAXP];
                for (int j = 0; j < np; j++) p[j] = mu[j];
                p[t0i] = t0;
                if (scan_ll(p, false) >= thr) hi1 = t0;
                else break;
            }
            mu[t0i] = best_t0;
            ls[t0i] = log(fmax((hi1 - lo1) / 2.0, 0.1));
        }
    }
    // ---- profile_refine_all
    if (fast) {
        double map_ll = scan_ll(mu, false);
        double thr = map_ll - 0.5;
        for (int j = 0; j < np; j++) {
            if (j == se) continue;
            double mu_j = mu[j];
            double svi_sigma = exp(ls[j]);
            double slo = c_lo[m][j], shi = c_hi[m][j];
            if (shi - slo < 1e-10) continue;
            double l1 = mu_j, h1 = mu_j;
            for (int gi = 0; gi < 15; gi++) {
                double val = slo + (shi - slo) * (double)gi / 14.0;
                double p[MAXP];
                for (int k = 0; k < np; k++) p[k] = mu[k];
                p[j] = val;
                double ll = scan_ll(p, false);
                if (ll >= thr) { l1 = fmin(l1, val); h1 = fmax(h1, val); }
            }
            double prof = fmax((h1 - l1) / 2.0, 1e-6);
            double prior_sigma = c_pop_w[m][j];
            ls[j] = log(fmax(fmax(svi_sigma, prof), prior_sigma));
        }
    }
    // ---- magnitude-space chi2 with the refined mu (PSO params if fewer
    // than half of the predictions are positive)
    double msum = 0.0;
    int mcount = 0;
    {
        metzger_prepare(m, mu, b, scr);
        Predictor P(m, mu, scr);
        int npos = 0;
        for (int i = lane; i < b.n; i += 32) npos += (P(b, i) * b.peak > 0.0) ? 1 : 0;
        for (int k = 16; k; k >>= 1) npos += __shfl_xor_sync(FULL, npos, k);
        __syncwarp();
        const double* use = mu;
        double pso[MAXP];
        // the joint fit always takes mu (src/parametric.rs:4057-4073)
        if (npos < b.n / 2 && !bs.joint) {
            for (int j = 0; j < np; j++) pso[j] = o.pso_params[j];
            use = pso;
        }
        metzger_prepare(m, use, b, scr);
        Predictor Q(m, use, scr);
        for (int i = lane; i < b.n; i += 32) {
            double pf = Q(b, i) * b.peak;
            if (pf > 0.0 && b.f[i] > 0.0) {
                double mpred = -2.5 * log10(pf) + 23.9;
                double merr = 1.0857 * b.fe[i] / b.f[i];
                if (merr > 0.0) {
                    double r = b.mag[i] - mpred;
                    msum += r * r / (merr * merr);
                    mcount++;
                }
            }
        }
        msum = wsum(msum);
        for (int k = 16; k; k >>= 1) mcount += __shfl_xor_sync(FULL, mcount, k);
    }
    if (lane == 0) {
        for (int j = 0; j < np; j++) { o.mu[j] = mu[j]; o.log_sigma[j] = ls[j]; }
        o.mag_chi2 = mcount > 0 ? msum / (double)mcount : NAN;
    }
}

void launch_refine(const DeviceBatch& d, cudaStream_t s) {
    if (d.n_bands == 0) return;
    int64_t threads = (int64_t)d.n_bands * 32;
    const size_t smem = (size_t)(LCF_REFINE_BLOCK / 32) * 32 * MZ_KEEP * sizeof(double);
    refine_kernel<<<(int)((threads + LCF_REFINE_BLOCK - 1) / LCF_REFINE_BLOCK), LCF_REFINE_BLOCK, smem, s>>>(d);
}

// ---------------------------------------------------------------------------
// Profile t0 search (SVI mode, rank-0 band): task builders and pickers.
// Coarse: 5 runs on linspace(t0_min, t0_max, 5); fine: 3 runs on
// linspace(best_t0 -/+ 0.5 clipped); results in t0 slots (band * 8 + k).
// ---------------------------------------------------------------------------
__device__ __forceinline__ double lin_at(double a, double b, int n, int i) {
    return n <= 1 ? a : a + (double)i * ((b - a) / (double)(n - 1));
}

__global__ void t0_build_kernel(DeviceBatch d, int slot, int fine, int64_t t0_base) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= d.n_bands) return;
    BandStats bs = d.stats[b];
    BandOut& o = d.out[b];
    if (!bs.valid || bs.rank != 0 || o.model < 0 || bs.joint) return;  // no t0 search in the joint fit
    int m = o.model, t0i = t0_idx_of(m);
    double* ts = d.t0_state + 3 * (int64_t)b;
    if (!fine) {
        double pilot = o.pso_params[t0i];
        ts[0] = fmax(pilot - 5.0, bs.t_first - 10.0);
        ts[1] = pilot + 5.0;
        ts[2] = pilot;
    }
    double t0_min = ts[0], t0_max = ts[1];
    int cnt = fine ? 3 : 5;
    double a = t0_min, z = t0_max;
    if (fine) {
        a = fmax(ts[2] - 0.5, t0_min);
        z = fmin(ts[2] + 0.5, t0_max);
    }
    int base = atomicAdd(&d.ctr->task_count[slot], cnt);
    for (int k = 0; k < cnt; k++) {
        PsoTask t;
        t.band = b;
        t.kind = (int16_t)m;
        t.restart = 0;
        t.flags = TASK_T0_FIXED;
        t.out = (int)(t0_base + (int64_t)b * 8 + (fine ? 5 : 0) + k);
        t.aux = -1;
        t.t0_fixed = lin_at(a, z, cnt, k);
        d.tasks[slot][base + k] = t;
    }
}

__global__ void t0_pick_kernel(DeviceBatch d, int fine, int64_t t0_base) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= d.n_bands) return;
    BandStats bs = d.stats[b];
    BandOut& o = d.out[b];
    if (!bs.valid || bs.rank != 0 || o.model < 0 || bs.joint) return;
    int m = o.model, np = n_params_of(m), t0i = t0_idx_of(m);
    double* ts = d.t0_state + 3 * (int64_t)b;
    double t0_min = ts[0], t0_max = ts[1];
    double best_c = o.pso_cost;
    double best_t0 = ts[2];
    double a = t0_min, z = t0_max;
    int cnt = fine ? 3 : 5;
    if (fine) { a = fmax(best_t0 - 0.5, t0_min); z = fmin(best_t0 + 0.5, t0_max); }
    int best_k = -1;
    for (int k = 0; k < cnt; k++) {
        const PsoResult& R = d.pso_res[t0_base + (int64_t)b * 8 + (fine ? 5 : 0) + k];
        if (R.cost < best_c) { best_c = R.cost; best_k = k; if (!fine) best_t0 = lin_at(a, z, cnt, k); }
    }
    if (!fine) ts[2] = best_t0;
    if (best_k >= 0) {
        const PsoResult& R = d.pso_res[t0_base + (int64_t)b * 8 + (fine ? 5 : 0) + best_k];
        double t0v = lin_at(a, z, cnt, best_k);
        int fi = 0;
        for (int i = 0; i < np - 1; i++) {
            if (i == t0i) o.pso_params[fi++] = t0v;
            o.pso_params[fi++] = pso_param(R, i);
        }
        if (t0i >= np - 1) o.pso_params[fi] = t0v;
        o.pso_cost = best_c;
    }
}

void launch_t0_build(const DeviceBatch& d, int slot, int fine, cudaStream_t s) {
    if (d.n_bands == 0) return;
    t0_build_kernel<<<(d.n_bands + 127) / 128, 128, 0, s>>>(d, slot, fine, d.t0_slot_base);
}
void launch_t0_pick(const DeviceBatch& d, int slot, int fine, cudaStream_t s) {
    (void)slot;
    if (d.n_bands == 0) return;
    t0_pick_kernel<<<(d.n_bands + 127) / 128, 128, 0, s>>>(d, fine, d.t0_slot_base);
}

// Bazin gate of fit_all_models == false (src/parametric.rs:2037): the bands
// whose polished Bazin cost is >= 2 get the remaining seven models.
__global__ void gate_build_kernel(DeviceBatch d, int slot) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= d.n_bands) return;
    BandStats bs = d.stats[b];
    if (!bs.valid) return;
    if (!(d.fits[b * 8 + BAZIN].cost >= 2.0)) return;
    int base = atomicAdd(&d.ctr->task_count[slot], 21);
    int k = 0;
    for (int mi = 1; mi < 8; mi++) {
        int m = c_select_order[mi];
        for (int r = 0; r < 3; r++) {
            PsoTask t;
            t.band = b;
            t.kind = (int16_t)m;
            t.restart = (int8_t)r;
            t.flags = TASK_PRIOR | TASK_T0_BOUNDS | (r > 0 ? TASK_SEEDED : 0);
            t.out = (b * 8 + m) * 3 + r;
            t.aux = -1;
            t.t0_fixed = 0.0;
            d.tasks[slot][base + k++] = t;
        }
    }
}
void launch_gate_build(const DeviceBatch& d, int slot, cudaStream_t s) {
    if (d.n_bands == 0) return;
    gate_build_kernel<<<(d.n_bands + 127) / 128, 128, 0, s>>>(d, slot);
}

// ---------------------------------------------------------------------------
// MultiBazin (fit_multi_bazin, src/parametric.rs:1008-1157) on rank-0 bands
// with n >= 5.  Results of K live in slots mb_base + (band * 4 + K - 1) * 3 + r.
// ---------------------------------------------------------------------------
__device__ double mb_eval(const double* p, int k, double t) {
    double sum = 0.0;
    for (int c = 0; c < k; c++) {
        const double* q = p + 4 * c;
        double dt = t - q[1];
        sum += exp(q[0]) * exp(-dt / exp(q[3])) * (1.0 / (1.0 + exp(-dt / exp(q[2]))));
    }
    return sum + p[4 * k];
}

__global__ void mb_pick_kernel(DeviceBatch d, int k, int64_t mb_base) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= d.n_bands) return;
    BandStats bs = d.stats[b];
    if (!bs.valid || bs.rank != 0 || bs.n < 5) return;
    MbState& S = d.mb[b];
    if (k == 1) {
        S.best_k = 1; S.done = 0; S.k_done = 0;
        S.best_cost = INFINITY; S.best_bic = INFINITY;
        for (int i = 0; i < LCF_MB_MAX_K; i++) { S.per_k_cost[i] = NAN; S.per_k_bic[i] = NAN; }
    }
    if (S.done) return;
    const PsoResult* R = d.pso_res + mb_base + ((int64_t)b * 4 + (k - 1)) * 3;
    int np = 4 * k + 2;
    int best = 0;
    double c1 = R[0].cost;
    if (k > 1 && R[1].cost < c1) { c1 = R[1].cost; best = 1; }
    if (R[2].cost < c1) { c1 = R[2].cost; best = 2; }
    double nf = (double)bs.n;
    double kb = 2.0 * c1 * nf + (double)np * log(nf);
    S.per_k_cost[k - 1] = c1;
    S.per_k_bic[k - 1] = kb;
    if (kb < S.best_bic) {
        S.best_bic = kb;
        S.best_cost = c1;
        S.best_k = k;
        for (int j = 0; j < MB_MAXP; j++) S.best_params[j] = j < np ? pso_param(R[best], j) : NAN;
    }
    for (int j = 0; j < MB_MAXP; j++) S.prev_params[j] = j < np ? pso_param(R[best], j) : NAN;
    S.k_done = k;
    if (k > 1 && kb > S.per_k_bic[k - 2] + 2.0) S.done = 1;
}

// Builds the K tasks (K >= 2): the seed particle extends the K-1 fit with a
// component at the largest positive residual of a detection.
__global__ void mb_build_kernel(DeviceBatch d, int slot, int k, int64_t mb_base) {
    int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    if (warp >= d.n_bands) return;
    int b = warp;
    BandStats bs = d.stats[b];
    if (!bs.valid || bs.rank != 0 || bs.n < 5) return;
    MbState& S = d.mb[b];
    if (S.done || S.k_done != k - 1) return;
    BandView v = band_view(d, bs);
    const double* prev = S.prev_params;
    double best = -INFINITY;
    int bi = 0x7fffffff;
    for (int i = lane; i < v.n; i += 32) {
        if (v.up[i]) continue;
        double res = v.f[i] - mb_eval(prev, k - 1, v.t[i]);
        if (res > best) { best = res; bi = i; }
    }
    for (int s = 16; s; s >>= 1) {
        double ob = __shfl_xor_sync(FULL, best, s);
        int oi = __shfl_xor_sync(FULL, bi, s);
        if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
    }
    if (lane != 0) return;
    if (bi == 0x7fffffff) bi = 0;
    int np = 4 * k + 2, pn = 4 * (k - 1);
    double init[MB_MAXP];
    for (int j = 0; j < pn; j++) init[j] = prev[j];
    init[pn] = log(fmax(best, 1e-10));
    init[pn + 1] = v.t[bi];
    init[pn + 2] = 1.0;
    init[pn + 3] = 1.0;
    init[pn + 4] = prev[pn];
    init[pn + 5] = prev[pn + 1];
    for (int c = 0; c < k; c++) {
        const double lo[4] = {-3.0, bs.t_first - 30.0, -2.0, -2.0}, hi[4] = {3.0, bs.t_last + 30.0, 5.0, 6.0};
        for (int q = 0; q < 4; q++) init[4 * c + q] = fmin(fmax(init[4 * c + q], lo[q]), hi[q]);
    }
    init[4 * k] = fmin(fmax(init[4 * k], -0.3), 0.3);
    init[4 * k + 1] = fmin(fmax(init[4 * k + 1], -5.0), 0.0);
    for (int j = 0; j < MB_MAXP; j++) S.seed[j] = j < np ? init[j] : 0.0;
    int base = atomicAdd(&d.ctr->task_count[slot], 3);
    for (int r = 0; r < 3; r++) {
        PsoTask t;
        t.band = b;
        t.kind = (int16_t)(KIND_MB1 + k - 1);
        t.restart = (int8_t)r;
        t.flags = r == 1 ? TASK_SEEDED : 0;
        t.out = (int)(mb_base + ((int64_t)b * 4 + (k - 1)) * 3 + r);
        t.aux = r == 1 ? b : -1;
        t.t0_fixed = 0.0;
        d.tasks[slot][base + r] = t;
    }
}

void launch_mb_pick(const DeviceBatch& d, int k, cudaStream_t s) {
    if (d.n_bands == 0) return;
    mb_pick_kernel<<<(d.n_bands + 127) / 128, 128, 0, s>>>(d, k, d.mb_slot_base);
}
void launch_mb_build(const DeviceBatch& d, int slot, int k, cudaStream_t s) {
    if (d.n_bands == 0) return;
    int64_t threads = (int64_t)d.n_bands * 32;
    mb_build_kernel<<<(int)((threads + 127) / 128), 128, 0, s>>>(d, slot, k, d.mb_slot_base);
}

}  // namespace lcf
