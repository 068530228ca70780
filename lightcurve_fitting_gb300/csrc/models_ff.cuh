// models_ff.cuh — the L-BFGS polish's observation term in double-float (ff)
// arithmetic: the prediction and its analytic gradient (src/parametric.rs:
// 199-509) and one observation's share of PsoCost::cost_from_slice and
// PsoCost::gradient (:1303-1446), to ~1e-14 of the FP64 values.
//
// The formulas are the reference's, rearranged where a factor would leave
// FP32's exponent range before the product does:
//   * logistic functions are formed from e^-|x| (both sigma and 1 - sigma);
//   * softplus ln(1 + e^ph) as ph + ln(1 + e^-ph) for ph > 0;
//   * Bazin's e^(-dt/tau_f) sigma(dt/tau_r) as one exponential for dt < 0;
//   * Villar's w e^(u/tau_f) as e^(u (1/tau_f - 10)) / (1 + e^(-10 u)) for
//     u > 0 (its exponent is negative: 1/tau_f < e^-1 inside the bounds);
//   * Afterglow's (u1 + u2)^(-1/2) and u_k / (u1 + u2) by log-sum-exp;
//   * the upper-limit cost ln(0.5 poly e^(-a^2)) as ln(0.5 poly) - a^2.
// ff_range_ok() bounds, once per evaluation, every exponent and the
// prediction over the band's time span; an evaluation outside them runs the
// FP64 term (models_f64.cuh) instead, so results there are the FP64 ones.
#pragma once

#include "ff.cuh"
#include "lcf_internal.cuh"

#ifndef LCF_FF_MID
#define LCF_FF_MID __device__ __forceinline__
#endif
// the upper-limit term runs for ~1/4 of the observations: out of line it keeps
// the observation loop's hot code smaller (measured 1.5 % faster polish)
#ifndef LCF_FF_UPPER
#define LCF_FF_UPPER static __device__ __noinline__
#endif

namespace lcf {

// logistic sigma(x) = 1 / (1 + e^-x) and 1 - sigma(x)
LCF_FF_MID void ff_sigmoid(ff x, ff& sig, ff& oms) {
    const bool pos = x.hi >= 0.0f;
    const ff s = ff_exp(pos ? ff_neg(x) : x);  // e^-|x| <= 1
    const ff r = ff_rcp(ff_add(s, 1.0f));
    const ff sr = ff_mul(s, r);
    sig = pos ? r : sr;
    oms = pos ? sr : r;
}

// phase_soft (src/parametric.rs:306): ps = ln(1 + e^ph) + 1e-6, and
// sp = d ps / d ph = e^ph / (1 + e^ph)
LCF_FF_MID void ff_softplus(ff ph, ff& ps, ff& sp) {
    const bool pos = ph.hi > 0.0f;
    const ff s = ff_exp(pos ? ff_neg(ph) : ph);  // e^-|ph|
    const ff q = ff_add(s, 1.0f);
    const ff l = ff_log(q);
    const ff r = ff_rcp(q);
    ps = ff_add(pos ? ff_add(ph, l) : l, ffm(9.999999974752427e-07f, 2.5247572468697606e-15f));
    sp = pos ? r : ff_mul(s, r);
}

__device__ __forceinline__ ff shfl_ff(ff v, int src) {
    return ffm(__shfl_sync(0xffffffffu, v.hi, src), __shfl_sync(0xffffffffu, v.lo, src));
}
__device__ __forceinline__ ff shfl_xor_ff(ff v, int m) {
    return ffm(__shfl_xor_sync(0xffffffffu, v.hi, m), __shfl_xor_sync(0xffffffffu, v.lo, m));
}
__device__ __forceinline__ ff warp_sum_ff(ff v) {
    for (int k = 16; k; k >>= 1) v = ff_add(v, shfl_xor_ff(v, k));
    return v;
}
// Sums 8 per-lane ff values over the warp by recursive halving (4 + 2 + 1
// exchanges, then two more); lane l returns the total of v[(l >> 2) & 7].
__device__ __forceinline__ ff reduce_scatter8_ff(const ff* v) {
    const int lane = threadIdx.x & 31;
    const bool b4 = lane & 16, b3 = lane & 8, b2 = lane & 4;
    ff a[4], b[2];
#pragma unroll
    for (int i = 0; i < 4; i++) a[i] = ff_add(b4 ? v[4 + i] : v[i], shfl_xor_ff(b4 ? v[i] : v[4 + i], 16));
#pragma unroll
    for (int i = 0; i < 2; i++) b[i] = ff_add(b3 ? a[2 + i] : a[i], shfl_xor_ff(b3 ? a[i] : a[2 + i], 8));
    ff c = ff_add(b2 ? b[1] : b[0], shfl_xor_ff(b2 ? b[0] : b[1], 4));
    c = ff_add(c, shfl_xor_ff(c, 2));
    return ff_add(c, shfl_xor_ff(c, 1));
}

template <int MODEL>
struct FfModel;

// Bazin (:200-228)
template <>
struct FfModel<BAZIN> {
    ff a, b, t0, itr, itf, dif;
    __device__ void init(const double* q, const ff* ef, const ff* rf) {
        a = ef[0]; b = ff_from(q[1]); t0 = ff_from(q[2]); itr = rf[3]; itf = rf[4];
        dif = ff_sub(rf[3], rf[4]);
    }
    __device__ __forceinline__ ff eval(ff t, ff* g) const {
        const ff dt = ff_sub(t, t0);
        const bool pos = dt.hi >= 0.0f;
        // dt >= 0: e^(-dt itf) / (1 + e^(-dt itr)); dt < 0: e^(dt (itr - itf)) / (1 + e^(dt itr))
        const ff dtr = ff_mul(dt, itr);
        const ff s = ff_exp(pos ? ff_neg(dtr) : dtr);
        const ff rd = ff_rcp(ff_add(s, 1.0f));
        const ff e1 = ff_exp(pos ? ff_neg(ff_mul(dt, itf)) : ff_mul(dt, dif));
        const ff base = ff_mul(ff_mul(a, e1), rd);
        if (g) {
            const ff oms = pos ? ff_mul(s, rd) : rd;  // 1 - sigma
            g[0] = base;
            g[1] = ffm(1.0f, 0.0f);
            g[2] = ff_mul(base, ff_sub(itf, ff_mul(oms, itr)));
            g[3] = ff_neg(ff_mul(ff_mul(base, oms), dtr));
            g[4] = ff_mul(base, ff_mul(dt, itf));
        }
        return ff_add(base, b);
    }
};

// Villar (:231-294)
template <>
struct FfModel<VILLAR> {
    ff a, beta, gam, t0, itr, itf, omb, itfm10;
    __device__ void init(const double* q, const ff* ef, const ff* rf) {
        a = ef[0]; beta = ff_from(q[1]); gam = ef[2]; t0 = ff_from(q[3]); itr = rf[4]; itf = rf[5];
        omb = ff_sub(ffm(1.0f, 0.0f), ff_mul(beta, gam)); itfm10 = ff_add(itf, -10.0f);
    }
    __device__ __forceinline__ ff eval(ff t, ff* g) const {
        const ff ph = ff_sub(t, t0);
        ff sig, oms;
        ff_sigmoid(ff_mul(ph, itr), sig, oms);
        // w = sigma(10 (ph - gamma)) = 1 / (1 + e^(10 u)), u = gamma - ph
        const ff u = ff_sub(gam, ph);
        const bool upos = u.hi > 0.0f;
        const ff sw = ff_exp(ff_mul(upos ? ff_neg(u) : u, 10.0f));  // e^(-10 |u|)
        const ff rw = ff_rcp(ff_add(sw, 1.0f));
        const ff sww = ff_mul(sw, rw);
        const ff w = upos ? sww : rw, omw = upos ? rw : sww;
        // wed = w e^(u itf)
        const ff wed = ff_mul(ff_exp(ff_mul(u, upos ? itfm10 : itf)), rw);
        const ff pl = ff_sub(ffm(1.0f, 0.0f), ff_mul(beta, ph));
        const ff bw = ff_mul(omb, wed);  // w pr
        const ff piece = ff_add(ff_mul(omw, pl), bw);
        const ff as = ff_mul(a, sig);
        if (g) {
            g[0] = ff_mul(as, piece);
            g[1] = ff_neg(ff_mul(as, ff_add(ff_mul(omw, ph), ff_mul(gam, wed))));
            // -k w (1 - w) (pr - pl), k = 10
            const ff kk = ff_mul(ff_mul(omw, ff_sub(bw, ff_mul(w, pl))), -10.0f);
            g[2] = ff_mul(ff_mul(as, gam), ff_add(kk, ff_mul(wed, ff_sub(ff_mul(omb, itf), beta))));
            const ff dpdt0 = ff_add(ff_add(kk, ff_mul(omw, beta)), ff_mul(bw, itf));
            const ff sos = ff_mul(sig, oms);
            g[3] = ff_mul(a, ff_sub(ff_mul(sig, dpdt0), ff_mul(ff_mul(sos, itr), piece)));
            g[4] = ff_neg(ff_mul(ff_mul(ff_mul(a, piece), sos), ff_mul(ph, itr)));
            g[5] = ff_neg(ff_mul(ff_mul(as, bw), ff_mul(u, itf)));
        }
        return ff_mul(as, piece);
    }
};

// TDE (:297-336)
template <>
struct FfModel<TDE> {
    ff a, b, t0, itr, itf, al;
    __device__ void init(const double* q, const ff* ef, const ff* rf) {
        a = ef[0]; b = ff_from(q[1]); t0 = ff_from(q[2]); itr = rf[3]; itf = rf[4]; al = ff_from(q[5]);
    }
    __device__ __forceinline__ ff eval(ff t, ff* g) const {
        const ff ph = ff_sub(t, t0);
        ff sig, oms, ps, sp;
        ff_sigmoid(ff_mul(ph, itr), sig, oms);
        ff_softplus(ph, ps, sp);
        const ff w = ff_add(ff_mul(ps, itf), 1.0f);
        const ff lw = ff_log(w);
        const ff decay = ff_exp(ff_neg(ff_mul(al, lw)));
        const ff as = ff_mul(a, sig);
        if (g) {
            const ff wm1 = ff_mul(decay, ff_rcp(w));
            const ff sos = ff_mul(sig, oms);
            g[0] = ff_mul(as, decay);
            g[1] = ffm(1.0f, 0.0f);
            // a (sig al wm1 sp itf - sig (1 - sig) itr decay)
            g[2] = ff_sub(ff_mul(ff_mul(as, al), ff_mul(wm1, ff_mul(sp, itf))),
                          ff_mul(ff_mul(a, decay), ff_mul(sos, itr)));
            g[3] = ff_neg(ff_mul(ff_mul(a, decay), ff_mul(sos, ff_mul(ph, itr))));
            g[4] = ff_mul(ff_mul(as, al), ff_mul(wm1, ff_mul(ps, itf)));
            g[5] = ff_neg(ff_mul(ff_mul(as, lw), decay));
        }
        return ff_add(ff_mul(as, decay), b);
    }
};

// Arnett (:339-384)
template <>
struct FfModel<ARNETT> {
    ff a, t0, itm, f, omf;
    __device__ void init(const double* q, const ff* ef, const ff* rf) {
        a = ef[0]; t0 = ff_from(q[1]); itm = rf[2];
        f = ff_rcp(ff_add(rf[3], 1.0f));  // 1 / (1 + e^-p3)
        omf = ff_mul(rf[3], f);
    }
    __device__ __forceinline__ ff eval(ff t, ff* g) const {
        const ff I88 = ffm(0.11363636702299118f, -3.3866276449856514e-09f);    // 1 / 8.8
        const ff I1113 = ffm(0.008984725922346115f, 4.351192670060122e-11f);  // 1 / 111.3
        const ff ph = ff_sub(t, t0);
        ff ps, sp;
        ff_softplus(ph, ps, sp);
        const ff eni = ff_exp(ff_neg(ff_mul(ps, I88))), eco = ff_exp(ff_neg(ff_mul(ps, I1113)));
        const ff heat = ff_add(ff_mul(f, eni), ff_mul(omf, eco));
        const ff x = ff_mul(ps, itm);
        const ff x2 = ff_sqr(x);
        const ff ex2 = ff_exp(ff_neg(x2));
        const ff trap = ff_sub(ffm(1.0f, 0.0f), ex2);
        const ff ah = ff_mul(a, heat);
        if (g) {
            const ff dheat = ff_neg(ff_add(ff_mul(ff_mul(f, eni), I88), ff_mul(ff_mul(omf, eco), I1113)));
            const ff dtrap = ff_scale(ff_mul(ff_mul(ps, ex2), ff_sqr(itm)), 2.0f);
            g[0] = ff_mul(ah, trap);
            g[1] = ff_neg(ff_mul(ff_mul(a, sp), ff_add(ff_mul(dheat, trap), ff_mul(heat, dtrap))));
            g[2] = ff_scale(ff_neg(ff_mul(ff_mul(ah, ex2), x2)), 2.0f);
            g[3] = ff_mul(ff_mul(a, trap), ff_mul(ff_sub(eni, eco), ff_mul(f, omf)));
        }
        return ff_mul(ah, trap);
    }
};

// Magnetar (:387-424)
template <>
struct FfModel<MAGNETAR> {
    ff a, t0, itsd, itd;
    __device__ void init(const double* q, const ff* ef, const ff* rf) {
        a = ef[0]; t0 = ff_from(q[1]); itsd = rf[2]; itd = rf[3];
    }
    __device__ __forceinline__ ff eval(ff t, ff* g) const {
        const ff ph = ff_sub(t, t0);
        ff ps, sp;
        ff_softplus(ph, ps, sp);
        const ff w = ff_add(ff_mul(ps, itsd), 1.0f);
        const ff rw = ff_rcp(w);
        const ff sd = ff_sqr(rw);
        const ff x = ff_mul(ps, itd);
        const ff x2 = ff_sqr(x);
        const ff ex2 = ff_exp(ff_neg(x2));
        const ff trap = ff_sub(ffm(1.0f, 0.0f), ex2);
        const ff asd = ff_mul(a, sd);
        if (g) {
            const ff w3 = ff_mul(sd, rw);
            g[0] = ff_mul(asd, trap);
            const ff t1 = ff_scale(ff_mul(ff_neg(ff_mul(w3, itsd)), trap), 2.0f);
            const ff t2 = ff_scale(ff_mul(sd, ff_mul(ff_mul(ps, ex2), ff_sqr(itd))), 2.0f);
            g[1] = ff_neg(ff_mul(ff_mul(a, sp), ff_add(t1, t2)));
            g[2] = ff_scale(ff_mul(ff_mul(a, trap), ff_mul(ps, ff_mul(w3, itsd))), 2.0f);
            g[3] = ff_scale(ff_neg(ff_mul(ff_mul(asd, ex2), x2)), 2.0f);
        }
        return ff_mul(asd, trap);
    }
};

// ShockCooling (:427-465)
template <>
struct FfModel<SHOCK> {
    ff a, t0, n, ittr;
    __device__ void init(const double* q, const ff* ef, const ff* rf) {
        a = ef[0]; t0 = ff_from(q[1]); n = ff_from(q[2]); ittr = rf[3];
    }
    __device__ __forceinline__ ff eval(ff t, ff* g) const {
        const ff ph = ff_sub(t, t0);
        ff sig5, oms5, ps, sp;
        ff_sigmoid(ff_mul(ph, 5.0f), sig5, oms5);
        ff_softplus(ph, ps, sp);
        const ff lps = ff_log(ps);
        const ff r = ff_mul(ps, ittr);
        const ff r2 = ff_sqr(r);
        // ps^-n e^(-r^2) as one exponential
        const ff base = ff_exp(ff_neg(ff_add(ff_mul(n, lps), r2)));
        const ff flux = ff_mul(ff_mul(a, sig5), base);
        if (g) {
            g[0] = flux;
            const ff inner = ff_add(ff_mul(n, ff_rcp(ps)), ff_scale(ff_mul(ps, ff_sqr(ittr)), 2.0f));
            const ff br = ff_sub(ff_mul(ff_mul(sig5, sp), inner), ff_mul(ff_mul(sig5, oms5), 5.0f));
            g[1] = ff_mul(ff_mul(a, base), br);
            g[2] = ff_neg(ff_mul(flux, lps));
            g[3] = ff_scale(ff_mul(flux, r2), 2.0f);
        }
        return flux;
    }
};

// Afterglow (:468-510): u = u1 + u2, u_k = e^(s_k), s_k = 2 a_k lr,
// lr = ln ps - ln t_b; flux = A u^(-1/2), with ln u by log-sum-exp
template <>
struct FfModel<AFTERGLOW> {
    ff a, t0, ltb, a1x2, a2x2;
    __device__ void init(const double* q, const ff* ef, const ff* rf) {
        a = ef[0]; t0 = ff_from(q[1]); ltb = ff_from(q[2]); a1x2 = ff_from(2.0 * q[3]); a2x2 = ff_from(2.0 * q[4]);
    }
    __device__ __forceinline__ ff eval(ff t, ff* g) const {
        const ff ph = ff_sub(t, t0);
        ff ps, sp;
        ff_softplus(ph, ps, sp);
        const ff lr = ff_sub(ff_log(ps), ltb);
        const ff s1 = ff_mul(a1x2, lr), s2 = ff_mul(a2x2, lr);
        const ff ds = ff_sub(s1, s2);
        const bool first = ds.hi >= 0.0f;
        const ff m = first ? s1 : s2;
        const ff lu = ff_add(m, ff_log(ff_add(ff_exp(first ? ff_neg(ds) : ds), 1.0f)));
        const ff iu = ff_exp(ff_scale(ff_neg(lu), 0.5f));
        const ff aiu = ff_mul(a, iu);
        if (g) {
            const ff f1 = ff_exp(ff_sub(s1, lu)), f2 = ff_exp(ff_sub(s2, lu));  // u_k / u
            const ff S = ff_add(ff_mul(a1x2, f1), ff_mul(a2x2, f2));
            const ff hs = ff_scale(ff_mul(aiu, S), 0.5f);
            g[0] = aiu;
            g[1] = ff_mul(hs, ff_mul(sp, ff_rcp(ps)));
            g[2] = hs;
            const ff al = ff_mul(aiu, lr);
            g[3] = ff_neg(ff_mul(al, f1));
            g[4] = ff_neg(ff_mul(al, f2));
        }
        return aiu;
    }
};

// MetzgerKN is not polished (src/parametric.rs:1992-1996); this stands in
// for the template instantiation only, and ff_range_ok sends it to FP64.
template <>
struct FfModel<METZGER> {
    __device__ void init(const double*, const ff*, const ff*) {}
    __device__ __forceinline__ ff eval(ff, ff*) const { return ffm(0.0f, 0.0f); }
};

// Exponent and prediction bounds of one evaluation over the band's phase
// span [ph_lo, ph_hi] (phase = t - t0): true when every exponential of the
// ff forms above stays below 80 and every prediction below e^20 (so a
// band's summed chi^2 terms stay below 1e30), so that no ff quantity leaves
// FP32's range; false sends the evaluation to FP64.
// The phase itself stays below 700 (the reference's e^phase overflows at
// 709.78, which the ff softplus does not).
template <int MODEL>
__device__ __forceinline__ bool ff_range_ok(const double* q, const ff* rf, double ph_lo, double ph_hi) {
    if (MODEL == METZGER || ph_hi > 700.0 || ph_lo < -700.0) return false;
    if (MODEL == BAZIN) {
        // dt < 0: exponent |dt| (itf - itr)
        const float e = ph_lo < 0.0 ? -(float)ph_lo * fmaxf(rf[4].hi - rf[3].hi, 0.0f) * 1.0001f : 0.0f;
        return e < 80.0f && (float)q[0] + e < 20.0f;
    }
    if (MODEL == AFTERGLOW) {
        // -ln(u) / 2 <= -max(a1, a2 lines) over ln ps - ln t_b, ps increasing
        // in the phase (FP32 with a margin: the bound only picks the arithmetic)
        auto sp = [](float x) { return x > 30.0f ? x : log1pf(expf(x)); };
        const float ltb = (float)q[2], a1 = (float)q[3], a2 = (float)q[4];
        const float l0 = logf(sp((float)ph_lo) + 1e-6f) - ltb, l1 = logf(sp((float)ph_hi) + 1e-6f) - ltb;
        const float b = fmaxf(fmaxf(-fmaxf(a1 * l0, a2 * l0), -fmaxf(a1 * l1, a2 * l1)), 0.0f) + 1.0f;
        return b < 80.0f && (float)q[0] + b < 20.0f;
    }
    return true;
}

// 0.5 ln(2 pi), ln(1e-300), the A&S 7.1.26 constants, as ff
__device__ __forceinline__ ff ff_poly_as(ff t) {
    const ff c1 = ffm(0.2548295855522156f, 6.447784528518241e-09f), c2 = ffm(-0.2844967246055603f, -1.1394440058154487e-08f),
             c3 = ffm(1.421413779258728f, -3.8258729517792744e-08f), c4 = ffm(-1.453152060508728f, 3.350872646024072e-08f),
             c5 = ffm(1.0614054203033447f, 8.696654951734217e-09f);
    ff p = ff_add(ff_mul(t, c5), c4);
    p = ff_add(ff_mul(t, p), c3);
    p = ff_add(ff_mul(t, p), c2);
    p = ff_add(ff_mul(t, p), c1);
    return ff_mul(t, p);
}

// upper_cost_ratio (models_f64.cuh) in ff: returns log Phi(z) (the cost is
// its negative) and, with want_ratio, the Gaussian pdf / CDF ratio of the
// gradient.  For z <= 0 the cost is ln(0.5 poly) - a^2, the reference's
// ln(0.5 poly e^(-a^2)) without forming e^(-a^2).  The ratio keeps the
// reference's CDF 0.5 (1 + erf) for z < 0, whose FP64 form cancels
// (0.5 (1 - fl64(1 - poly e^(-a^2))): relative error 2^-53 / CDF, exactly 0
// below z ~ -8.3, where the 1e-300 floor makes the ratio up to ~1e285); it is
// therefore formed in FP64 from the ff pieces, and a ratio beyond FP32's
// range sets `redo` (the evaluation is then repeated in FP64).
LCF_FF_UPPER ff ff_upper(ff z, bool want_ratio, ff& ratio, int& redo) {
    const ff az = z.hi < 0.0f ? ff_neg(z) : z;
    const ff a = ff_mul(az, ffm(0.7071067690849304f, 1.2101617485882343e-08f));
    const ff t = ff_rcp(ff_add(ff_mul(a, ffm(0.32759109139442444f, 8.605575807507648e-09f)), 1.0f));
    const ff poly = ff_poly_as(t);
    const ff a2 = ff_sqr(a);
    if (z.hi > 0.0f) {
        const ff e = ff_exp(ff_neg(a2));
        const ff cdf = ff_sub(ffm(1.0f, 0.0f), ff_scale(ff_mul(poly, e), 0.5f));
        if (want_ratio) ratio = ff_mul(ff_mul(e, ffm(0.3989422917366028f, -1.1335170135851058e-08f)), ff_rcp(cdf));
        return z.hi > 8.0f ? ffm(0.0f, 0.0f) : ff_log(cdf);
    }
    const ff lphi = ff_sub(ff_log(ff_scale(poly, 0.5f)), a2);
    const ff LN_FLOOR = ffm(-690.7755126953125f, -1.5202901522570755e-05f);  // ln 1e-300
    if (want_ratio) {
        const double ed = exp(-ff_to(a2));
        const double v = 1.0 - ff_to(poly) * ed;
        const double r = ed * 0.39894228040143267794 / fmax(0.5 * (1.0 + (-v)), 1e-300);
        if (r < 1e30) ratio = ff_from(r);
        else { ratio = ffm(0.0f, 0.0f); redo = 1; }
    }
    if (z.hi < -30.0f)  // -z^2/2 - ln(2 pi)/2 - ln(-z)
        return ff_neg(ff_add(ff_add(ff_scale(ff_sqr(z), 0.5f), ffm(0.9189385175704956f, 1.563417661998301e-08f)), ff_log(az)));
    return lphi.hi >= LN_FLOOR.hi ? lphi : LN_FLOOR;
}

// One observation's term of PsoCost::cost_from_slice / PsoCost::gradient
// (as lb_obs_term): A = (t hi, t lo, y hi, y lo) with y the normalised flux
// or, for an upper limit, the upper flux; B = obs_var (hi, lo), negated for
// upper limits.
template <int MODEL>
__device__ __forceinline__ void ff_obs_term(const FfModel<MODEL>& mod, float4 A, float2 B, ff se2, bool want_grad,
                                            ff& nll, ff* gl, int& nonfinite, int& redo) {
    constexpr int np = n_params_of(MODEL), se = se_idx_of(MODEL);
    const bool up = B.x < 0.0f;
    const ff var = up ? ffm(-B.x, -B.y) : ffm(B.x, B.y);
    ff mg[MAXP];
    const ff pr = mod.eval(ffm(A.x, A.y), want_grad ? mg : nullptr);
    if (!isfinite(pr.hi)) { nonfinite = 1; return; }
    const ff y = ffm(A.z, A.w);
    const ff tv = ff_add(var, se2);
    if (up) {
        const ff isv = ff_rsqrt(tv);
        const ff z = ff_mul(ff_sub(y, pr), isv);
        ff ratio;
        nll = ff_sub(nll, ff_upper(z, want_grad, ratio, redo));
        if (want_grad) {
            const ff ri = ff_mul(ratio, isv);
#pragma unroll
            for (int k = 0; k < np; k++)
                if (k != se) gl[k] = ff_add(gl[k], ff_mul(ri, mg[k]));
            gl[se] = ff_add(gl[se], ff_mul(ff_mul(ratio, z), ff_mul(se2, ff_sqr(isv))));
        }
    } else {
        const ff dd = ff_sub(pr, y);
        const ff itv = ff_rcp(tv);
        const ff d2 = ff_mul(ff_sqr(dd), itv);
        nll = ff_add(nll, ff_add(d2, ff_log(tv)));
        if (want_grad) {
            const ff sc = ff_scale(ff_mul(dd, itv), 2.0f);
#pragma unroll
            for (int k = 0; k < np; k++)
                if (k != se) gl[k] = ff_add(gl[k], ff_mul(sc, mg[k]));
            gl[se] = ff_add(gl[se], ff_scale(ff_mul(ff_sub(itv, ff_mul(d2, itv)), se2), 2.0f));
        }
    }
}

}  // namespace lcf
