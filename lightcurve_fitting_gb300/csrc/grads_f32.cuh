// grads_f32.cuh — FP32 prediction + analytic parameter gradient of each
// model, restating the reference's *_flux_grad functions
// (src/parametric.rs:213-509) in numerically safe FP32 forms.  They feed the
// L-BFGS polish (PsoCost::gradient, src/parametric.rs:1387-1445) and the SVI
// adjoint (svi_fit, src/parametric.rs:2330-2393): the gradient of the
// negative log-likelihood is accumulated as adjoint(pred) * d pred / d theta.
//
// Where the FP64 reference produces NaN components — phase beyond 709.78
// days, where ln(1 + e^phase) overflows and its derivative e^p/(1+e^p)
// becomes inf/inf — the same components are returned as NaN, since the
// reference's consumers treat them differently (SVI skips them, the L-BFGS
// gradient propagates them).  `st` reports ST_NONFINITE when the prediction
// itself is non-finite in FP64.
#pragma once

#include "lcf_internal.cuh"

#include "models_f32.cuh"

namespace lcf {

__device__ __forceinline__ float sigmoidf_stable(float x) {
    // 1 / (1 + e^-x), correct at both ends
    return x >= 0.0f ? 1.0f / (1.0f + expf(-x)) : expf(x) / (1.0f + expf(x));
}

// Returns the prediction; g[0..np-1] gets d pred / d theta (sigma_extra slot 0).
__device__ __forceinline__ float model_grad_f32(int m, const float* p, float th, float tl, float* g, int& st) {
    const float qnan = __int_as_float(0x7fffffff);
    st = ST_OK;
    switch (m) {
        case BAZIN: {
            float la = p[0], a = expf(p[0]), t0 = p[2], itr = expf(-p[3]), itf = expf(-p[4]);
            float dt = (th - t0) + tl;
            float xf = -dt * itf, xr = -dt * itr;
            if (xf > LN_DBL_MAX || la + xf > LN_DBL_MAX) { st = ST_NONFINITE; return 0.0f; }
            float base;
            float sig = sigmoidf_stable(-xr);       // 1 / (1 + e^{xr})
            float oms = sigmoidf_stable(xr);        // 1 - sig
            if (xf < 80.0f && xr < 80.0f) base = a * expf(xf) * sig;
            else if (xr > LN_DBL_MAX) base = 0.0f;
            else base = expf(la + xf - softplus_f(xr));
            g[0] = base;
            g[1] = 1.0f;
            g[2] = base * (itf - oms * itr);
            g[3] = -base * oms * dt * itr;
            g[4] = base * dt * itf;
            g[5] = 0.0f;
            return base + p[1];
        }
        case VILLAR: {
            float a = expf(p[0]), beta = p[1], gamma = expf(p[2]), t0 = p[3];
            float itr = expf(-p[4]), itf = expf(-p[5]);
            float ph = (th - t0) + tl;
            const float k = 10.0f;
            float sig = sigmoidf_stable(ph * itr);
            float w = sigmoidf_stable(k * (ph - gamma));
            float pl = 1.0f - beta * ph;
            float ed = expf((gamma - ph) * itf);
            float omb = 1.0f - beta * gamma;
            float pr = omb * ed;
            float piece = (1.0f - w) * pl + w * pr;
            float flux = a * sig * piece;
            g[0] = flux;
            g[1] = a * sig * ((1.0f - w) * (-ph) + w * (-gamma * ed));
            float wwm = w * (1.0f - w);
            float dw_dlg = -k * wwm * gamma;
            float dpr_dlg = ed * (-beta + omb * itf) * gamma;
            g[2] = a * sig * (dw_dlg * (pr - pl) + w * dpr_dlg);
            float dsig_dt0 = -sig * (1.0f - sig) * itr;
            float dw_dt0 = -k * wwm;
            float d_piece_dt0 = dw_dt0 * (pr - pl) + (1.0f - w) * beta + w * (omb * ed * itf);
            g[3] = a * (dsig_dt0 * piece + sig * d_piece_dt0);
            g[4] = a * piece * sig * (1.0f - sig) * (-ph * itr);
            g[5] = a * sig * w * (pr * (ph - gamma) * itf);
            g[6] = 0.0f;
            return flux;
        }
        case TDE: {
            float a = expf(p[0]), t0 = p[2], itr = expf(-p[3]), itf = expf(-p[4]), alpha = p[5];
            float ph = (th - t0) + tl;
            float sig = sigmoidf_stable(ph * itr);
            float ps;
            g[1] = 1.0f;
            g[6] = 0.0f;
            if (!phase_soft_f(ph, ps)) {
                g[0] = 0.0f; g[2] = qnan; g[3] = 0.0f; g[4] = qnan; g[5] = qnan;
                return p[1];
            }
            float sp = sigmoidf_stable(ph);
            float lw = log1pf(ps * itf);
            float decay = expf(-alpha * lw);
            float wm1 = decay / (1.0f + ps * itf);   // w^(-alpha-1)
            float base = a * sig * decay;
            g[0] = base;
            g[2] = a * (-sig * (1.0f - sig) * itr * decay + sig * alpha * wm1 * sp * itf);
            g[3] = a * decay * (-sig * (1.0f - sig) * ph * itr);
            g[4] = a * sig * alpha * wm1 * ps * itf;
            g[5] = a * sig * (-lw) * decay;
            return base + p[1];
        }
        case ARNETT: {
            float a = expf(p[0]), t0 = p[1], itm = expf(-p[2]), lf = p[3];
            float ph = (th - t0) + tl;
            float f = sigmoidf_stable(lf);
            float ps;
            g[4] = 0.0f;
            if (!phase_soft_f(ph, ps)) {
                g[0] = 0.0f; g[1] = qnan; g[2] = qnan; g[3] = 0.0f;
                return 0.0f;
            }
            float sp = sigmoidf_stable(ph);
            float e_ni = expf(-ps * (1.0f / 8.8f)), e_co = expf(-ps * (1.0f / 111.3f));
            float heat = f * e_ni + (1.0f - f) * e_co;
            float x = ps * itm;
            float ex2 = expf(-x * x);
            float trap = -expm1f(-x * x);
            float flux = a * heat * trap;
            g[0] = flux;
            float dheat = -f * e_ni * (1.0f / 8.8f) - (1.0f - f) * e_co * (1.0f / 111.3f);
            float dtrap = 2.0f * ps * ex2 * itm * itm;
            g[1] = a * (-sp) * (dheat * trap + heat * dtrap);
            g[2] = -2.0f * a * heat * ex2 * x * x;
            g[3] = a * trap * (e_ni - e_co) * f * (1.0f - f);
            return flux;
        }
        case MAGNETAR: {
            float a = expf(p[0]), t0 = p[1], itsd = expf(-p[2]), itd = expf(-p[3]);
            float ph = (th - t0) + tl;
            float ps;
            g[4] = 0.0f;
            if (!phase_soft_f(ph, ps)) {
                g[0] = 0.0f; g[1] = qnan; g[2] = qnan; g[3] = qnan;
                return 0.0f;
            }
            float sp = sigmoidf_stable(ph);
            float w = 1.0f + ps * itsd;
            float iw = 1.0f / w;
            float sd = iw * iw;
            float x = ps * itd;
            float ex2 = expf(-x * x);
            float trap = -expm1f(-x * x);
            float flux = a * sd * trap;
            g[0] = flux;
            float w3 = sd * iw;
            float dsd = -2.0f * w3 * itsd;
            float dtrap = 2.0f * ps * ex2 * itd * itd;
            g[1] = a * (-sp) * (dsd * trap + sd * dtrap);
            g[2] = a * trap * 2.0f * ps * w3 * itsd;
            g[3] = -2.0f * a * sd * ex2 * x * x;
            return flux;
        }
        case SHOCK: {
            float a = expf(p[0]), t0 = p[1], n = p[2], ittr = expf(-p[3]);
            float ph = (th - t0) + tl;
            float ps;
            g[4] = 0.0f;
            if (!phase_soft_f(ph, ps)) {
                g[0] = 0.0f; g[1] = qnan; g[2] = qnan; g[3] = qnan;
                return 0.0f;
            }
            float sig5 = sigmoidf_stable(5.0f * ph);
            float sp = sigmoidf_stable(ph);
            float lps = logf(ps);
            float r = ps * ittr;
            float base = expf(-n * lps - r * r);   // cooling * cutoff
            float flux = a * sig5 * base;
            g[0] = flux;
            g[1] = a * base * (-5.0f * sig5 * (1.0f - sig5) + sig5 * sp * (n / ps + 2.0f * ps * ittr * ittr));
            g[2] = -flux * lps;
            g[3] = flux * 2.0f * r * r;
            return flux;
        }
        default: {  // AFTERGLOW
            float la = p[0], t0 = p[1], ltb = p[2], a1 = p[3], a2 = p[4];
            float ph = (th - t0) + tl;
            float ps;
            g[5] = 0.0f;
            if (!phase_soft_f(ph, ps)) {
                g[0] = 0.0f; g[1] = qnan; g[2] = qnan; g[3] = qnan; g[4] = qnan;
                return 0.0f;
            }
            float sp = sigmoidf_stable(ph);
            float lr = logf(ps) - ltb;
            float s1 = 2.0f * a1 * lr, s2 = 2.0f * a2 * lr;
            // work relative to the larger exponent: u = e^mx (e1 + e2)
            float mx = fmaxf(s1, s2);
            float e1 = expf(s1 - mx), e2 = expf(s2 - mx);
            float lu = mx + logf(e1 + e2);
            float flux = expf(la - 0.5f * lu);
            // u^-1.5 * (2 a1 u1 + 2 a2 u2) = flux / a * (2 a1 e1 + 2 a2 e2) / (e1 + e2)
            float wsum = (2.0f * a1 * e1 + 2.0f * a2 * e2) / (e1 + e2);
            g[0] = flux;
            g[1] = -0.5f * flux * wsum / ps * (-sp);
            g[2] = -0.5f * flux * (-wsum);
            g[3] = -0.5f * flux * 2.0f * lr * e1 / (e1 + e2);
            g[4] = -0.5f * flux * 2.0f * lr * e2 / (e1 + e2);
            return flux;
        }
    }
}

// Upper-limit adjoint factor phi(z) / max(cdf(z), 1e-300) of the reference
// (src/parametric.rs:1415-1417, :2349-2352), with cdf(z) =
// 0.5 * (1 + erf_approx(z / sqrt 2)).  For z < 0 the FP64 sum 1 + erf
// quantises P = poly * e^{-z^2/2} to multiples of 2^-53 (exact as
// 1 - fl(1 - P)); that quantisation is reproduced.  Where it leaves fewer
// than 64 units (P * 2^53 < 63.5) the step between neighbouring units is too
// coarse for an FP32 estimate of P to pick the reference's: at 0 units the
// CDF is the 1e-300 floor and the ratio phi / 1e-300 reaches ~1e285 (beyond
// FP32), at 1 unit it is ~10.  There `defer` is set, 0 is returned, and the
// caller forms that observation's gradient terms itself (svi_deferred_pass:
// at full magnitude, with the unit count decided in FP64 near the boundary).
__device__ __forceinline__ float upper_ratio_f32(float z, bool& defer) {
    defer = false;
    const float inv_sqrt_2pi = 0.3989422804014327f;
    float x = fabsf(z) * 0.70710678118654752f;
    float t = 1.0f / (1.0f + 0.3275911f * x);
    float poly = t * (0.254829592f + t * (-0.284496736f + t * (1.421413741f + t * (-1.453152027f + t * 1.061405429f))));
    float e = expf(-x * x);
    if (z >= 0.0f) {
        float cdf = 1.0f - 0.5f * poly * e;
        return inv_sqrt_2pi * e / cdf;
    }
    float P = poly * e;
    if (P < 2.0e-9f) {
        // FP64: 1 - fl(1 - P) = round_half_even(P * 2^53) * 2^-53
        const float kq = P * 9007199254740992.0f;
        if (kq < 63.5f) {
            // below z = -38.7 the reference's pdf e^(-z^2/2) / sqrt(2 pi) is
            // exactly 0 in FP64 (past -745.13 in the exponent), so are its
            // gradient terms for this limit: nothing to defer
            if (z < -38.7f) return 0.0f;
            defer = true;
            return 0.0f;
        }
        const float k = rintf(kq);
        return inv_sqrt_2pi * e / (0.5f * k * 1.1102230246251565e-16f);
    }
    return inv_sqrt_2pi * 2.0f / poly;
}

// P * 2^53 of upper_ratio_f32 for z < 0 (the unit count of the reference's
// quantised CDF before rounding).
__device__ __forceinline__ float upper_units_f32(float z) {
    float x = fabsf(z) * 0.70710678118654752f;
    float t = 1.0f / (1.0f + 0.3275911f * x);
    float poly = t * (0.254829592f + t * (-0.284496736f + t * (1.421413741f + t * (-1.453152027f + t * 1.061405429f))));
    return poly * expf(-x * x) * 9007199254740992.0f;
}

}  // namespace lcf
