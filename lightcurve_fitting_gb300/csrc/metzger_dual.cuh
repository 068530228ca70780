// metzger_dual.cuh — MetzgerKN prediction and its derivatives with respect to
// (log10 M_ej, log10 v_ej, log10 kappa, t0) by forward-mode differentiation in
// FP32 (dual numbers with four tangents).
//
// The reference differentiates MetzgerKN for SVI by forward differences of
// its FP64 model with step 1e-5 (metzger_kn_grad_batch_into,
// src/parametric.rs:843-860): five sequential ODE solves per sample.  In FP32
// a 1e-5 difference would lose the derivative to rounding, so the sweep of
// models_f32.cuh (MetzgerF::sweep) is carried out on dual numbers instead: the
// tangents give the derivative of the same piecewise formula (grid, Euler
// recurrence with its clamps, linear interpolation, peak normalisation) that
// the forward difference approximates to O(1e-5).
#pragma once

#include <math.h>

namespace lcf {

struct D4 {
    float v, d[4];
    __device__ D4() {}
    __device__ explicit D4(float x) : v(x) { d[0] = d[1] = d[2] = d[3] = 0.0f; }
};
__device__ __forceinline__ D4 mk(float v, float s, const D4& a) {  // v with tangent s * a.d
    D4 r;
    r.v = v;
    for (int k = 0; k < 4; k++) r.d[k] = s * a.d[k];
    return r;
}
__device__ __forceinline__ D4 operator+(const D4& a, const D4& b) {
    D4 r; r.v = a.v + b.v; for (int k = 0; k < 4; k++) r.d[k] = a.d[k] + b.d[k]; return r;
}
__device__ __forceinline__ D4 operator-(const D4& a, const D4& b) {
    D4 r; r.v = a.v - b.v; for (int k = 0; k < 4; k++) r.d[k] = a.d[k] - b.d[k]; return r;
}
__device__ __forceinline__ D4 operator*(const D4& a, const D4& b) {
    D4 r; r.v = a.v * b.v; for (int k = 0; k < 4; k++) r.d[k] = a.d[k] * b.v + a.v * b.d[k]; return r;
}
__device__ __forceinline__ D4 operator/(const D4& a, const D4& b) {
    D4 r; float ib = 1.0f / b.v; r.v = a.v * ib;
    for (int k = 0; k < 4; k++) r.d[k] = (a.d[k] - r.v * b.d[k]) * ib;
    return r;
}
__device__ __forceinline__ D4 operator+(const D4& a, float c) { D4 r = a; r.v += c; return r; }
__device__ __forceinline__ D4 operator-(const D4& a, float c) { D4 r = a; r.v -= c; return r; }
__device__ __forceinline__ D4 operator*(const D4& a, float c) { return mk(a.v * c, c, a); }
__device__ __forceinline__ D4 operator*(float c, const D4& a) { return mk(a.v * c, c, a); }
__device__ __forceinline__ D4 dexp(const D4& a) { float e = expf(a.v); return mk(e, e, a); }
__device__ __forceinline__ D4 dlog(const D4& a) { return mk(logf(a.v), 1.0f / a.v, a); }
__device__ __forceinline__ D4 dlog1p(const D4& a) { return mk(log1pf(a.v), 1.0f / (1.0f + a.v), a); }
__device__ __forceinline__ D4 dsqrt(const D4& a) { float s = sqrtf(a.v); return mk(s, 0.5f / s, a); }
__device__ __forceinline__ D4 dpowc(const D4& a, float c) {  // a^c, a > 0
    float p = exp2f(c * log2f(a.v));
    return mk(p, c * p / a.v, a);
}
__device__ __forceinline__ D4 datan(const D4& a) { return mk(atanf(a.v), 1.0f / (1.0f + a.v * a.v), a); }
__device__ __forceinline__ D4 dconst(float v) { return D4(v); }

// Writes, for the sorted observation times `t[j]` (stride 1), the normalised
// prediction and its four derivatives to out[j * 5 + {0..4}].  Returns false
// when the reference returns all zeros (phase_max <= 0.01, or a non-positive
// or non-finite peak); out is then zero.
template <class Times>
__device__ bool metzger_dual_sweep(const float* pv, float t_last, const Times& t, int n, float* out) {
    const float MSUN30 = 1.989e3f, C = 2.998e10f, SPD = 86400.0f, PI_F = 3.14159265358979f, LN10F = 2.302585093f;
    D4 p0(pv[0]), p1(pv[1]), p2(pv[2]), t0(pv[3]);
    p0.d[0] = 1.0f; p1.d[1] = 1.0f; p2.d[2] = 1.0f; t0.d[3] = 1.0f;
    D4 m30 = dexp(p0 * LN10F) * MSUN30;
    D4 v = dexp(p1 * LN10F) * C;
    D4 kappa_r = dexp(p2 * LN10F);
    float pm = t_last - t0.v;
    for (int j = 0; j < n * 5; j++) out[j] = 0.0f;
    if (!(pm > 0.01f)) return false;
    D4 phase_max = (t0 * -1.0f) + t_last;
    const float lmin = -4.605170185988091f;
    D4 lmax = dlog(phase_max * 1.05f);
    D4 dl = (lmax - lmin) * (1.0f / 199.0f);
    const float xn0 = 0.8f, xr = 0.2f;
    D4 vs = v * 1e-5f;
    D4 e_th = m30 * vs * vs * 0.5f;
    D4 e_kin = e_th;
    D4 t_day = dconst(0.01f);
    D4 r = t_day * v * SPD;
    D4 mos = m30 * 1e-10f;
    D4 diff_k = m30 * (3.0f / (4.0f * PI_F * C) * 1e30f);
    D4 l_peak = dconst(-INFINITY);
    D4 prev_t = t_day, prev_l = dconst(0.0f);
    int j = 0;
    while (j < n && t(j) - t0.v <= 0.0f) j++;  // zeros already written
    for (int i = 0; i < 200; i++) {
        D4 t_next = dexp(dl * (float)(i + 1) + lmin);
        D4 t_sec = t_day * SPD;
        D4 ef = dpowc(t_day, 0.74f) * 0.34f;
        D4 eth = (dexp(t_day * -0.56f) + (ef.v > 1e-10f ? dlog1p(ef) / ef : dconst(1.0f))) * 0.36f;
        D4 xn = dexp(t_sec * (-1.0f / 900.0f)) * xn0;
        D4 tt = datan(dconst(0.11f) / (t_sec - 1.3f)) * (1.0f / PI_F);
        if (tt.v < 1e-30f) tt = dconst(1e-30f);
        D4 eps_rp = eth * dpowc(tt, 1.3f) * 2e18f;
        D4 l_heat = mos * (xn * 3.2e14f + eps_rp);
        D4 kappa_eff = (dconst(xn0) - xn) * 0.4f + kappa_r * xr;
        D4 t_diff = kappa_eff * diff_k / (v * t_sec) + r * (1.0f / C);
        D4 l_rad = (e_th.v > 0.0f && t_diff.v > 0.0f) ? e_th / t_diff : dconst(0.0f);
        if (l_rad.v > l_peak.v) l_peak = l_rad;
        if (i == 0) {
            while (j < n && t(j) - t0.v <= t_day.v) {
                for (int k = 0; k < 5; k++) out[j * 5 + k] = k == 0 ? l_rad.v : l_rad.d[k - 1];
                j++;
            }
        } else {
            while (j < n) {
                float phv = t(j) - t0.v;
                if (phv > t_day.v) break;
                D4 ph = (t0 * -1.0f) + t(j);
                D4 lv = prev_l + (ph - prev_t) / (t_day - prev_t) * (l_rad - prev_l);
                out[j * 5] = lv.v;
                for (int k = 0; k < 4; k++) out[j * 5 + 1 + k] = lv.d[k];
                j++;
            }
        }
        prev_t = t_day;
        prev_l = l_rad;
        D4 l_pdv = r.v > 0.0f ? e_th * v / r : dconst(0.0f);
        if (i < 199) {
            D4 dts = (t_next - t_day) * SPD;
            e_th = e_th + (l_heat - l_pdv - l_rad) * dts;
            if (e_th.v < 0.0f) e_th = dconst(0.0f);
            e_kin = e_kin + l_pdv * dts;
            D4 vn = dsqrt(e_kin * 2.0f / mos);
            v = vn.v < C ? vn : dconst(C);
            r = r + v * dts;
        }
        t_day = t_next;
    }
    while (j < n) {
        out[j * 5] = prev_l.v;
        for (int k = 0; k < 4; k++) out[j * 5 + 1 + k] = prev_l.d[k];
        j++;
    }
    if (!(l_peak.v > 0.0f) || !isfinite(l_peak.v)) {
        for (int q = 0; q < n * 5; q++) out[q] = 0.0f;
        return false;
    }
    // normalise by the peak (its tangent included, as the difference quotient has it)
    float ip = 1.0f / l_peak.v;
    for (int q = 0; q < n; q++) {
        float y = out[q * 5] * ip;
        for (int k = 0; k < 4; k++) out[q * 5 + 1 + k] = (out[q * 5 + 1 + k] - y * l_peak.d[k]) * ip;
        out[q * 5] = y;
    }
    return true;
}

}  // namespace lcf
