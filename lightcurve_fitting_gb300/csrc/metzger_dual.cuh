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

// A value with K tangents (forward-mode dual number).
template <int K>
struct DN {
    float v, d[K];
    __device__ DN() {}
    __device__ explicit DN(float x) : v(x) {
#pragma unroll
        for (int k = 0; k < K; k++) d[k] = 0.0f;
    }
};
template <int K>
__device__ __forceinline__ DN<K> mk(float v, float s, const DN<K>& a) {  // v with tangent s * a.d
    DN<K> r;
    r.v = v;
#pragma unroll
    for (int k = 0; k < K; k++) r.d[k] = s * a.d[k];
    return r;
}
template <int K>
__device__ __forceinline__ DN<K> operator+(const DN<K>& a, const DN<K>& b) {
    DN<K> r; r.v = a.v + b.v;
#pragma unroll
    for (int k = 0; k < K; k++) r.d[k] = a.d[k] + b.d[k];
    return r;
}
template <int K>
__device__ __forceinline__ DN<K> operator-(const DN<K>& a, const DN<K>& b) {
    DN<K> r; r.v = a.v - b.v;
#pragma unroll
    for (int k = 0; k < K; k++) r.d[k] = a.d[k] - b.d[k];
    return r;
}
template <int K>
__device__ __forceinline__ DN<K> operator*(const DN<K>& a, const DN<K>& b) {
    DN<K> r; r.v = a.v * b.v;
#pragma unroll
    for (int k = 0; k < K; k++) r.d[k] = a.d[k] * b.v + a.v * b.d[k];
    return r;
}
template <int K>
__device__ __forceinline__ DN<K> operator/(const DN<K>& a, const DN<K>& b) {
    DN<K> r; float ib = 1.0f / b.v; r.v = a.v * ib;
#pragma unroll
    for (int k = 0; k < K; k++) r.d[k] = (a.d[k] - r.v * b.d[k]) * ib;
    return r;
}
template <int K>
__device__ __forceinline__ DN<K> operator+(const DN<K>& a, float c) { DN<K> r = a; r.v += c; return r; }
template <int K>
__device__ __forceinline__ DN<K> operator-(const DN<K>& a, float c) { DN<K> r = a; r.v -= c; return r; }
template <int K>
__device__ __forceinline__ DN<K> operator*(const DN<K>& a, float c) { return mk(a.v * c, c, a); }
template <int K>
__device__ __forceinline__ DN<K> operator*(float c, const DN<K>& a) { return mk(a.v * c, c, a); }
template <int K>
__device__ __forceinline__ DN<K> dexp(const DN<K>& a) { float e = expf(a.v); return mk(e, e, a); }
template <int K>
__device__ __forceinline__ DN<K> dlog(const DN<K>& a) { return mk(logf(a.v), 1.0f / a.v, a); }
template <int K>
__device__ __forceinline__ DN<K> dlog1p(const DN<K>& a) { return mk(log1pf(a.v), 1.0f / (1.0f + a.v), a); }
template <int K>
__device__ __forceinline__ DN<K> dsqrt(const DN<K>& a) { float s = sqrtf(a.v); return mk(s, 0.5f / s, a); }
template <int K>
__device__ __forceinline__ DN<K> dpowc(const DN<K>& a, float c) {  // a^c, a > 0
    float p = exp2f(c * log2f(a.v));
    return mk(p, c * p / a.v, a);
}
template <int K>
__device__ __forceinline__ DN<K> datan(const DN<K>& a) { return mk(atanf(a.v), 1.0f / (1.0f + a.v * a.v), a); }

// The sweep with the tangents of parameters tan0 .. tan0 + K - 1 (of
// log10 M_ej, log10 v_ej, log10 kappa, t0): writes, for the sorted
// observation times `t[j]`, the unnormalised interpolant to out[j * 5] and
// its tangents to out[j * 5 + 1 + tan0 + k]; lp_v / lp_d receive the peak
// and its tangents.  Returns false when the reference returns all zeros
// (phase_max <= 0.01, or a non-positive or non-finite peak).  The same
// arithmetic for every K: instances with fewer tangents (one parameter per
// lane) split the work of the four-tangent sweep across lanes.
template <int K, class Times>
__device__ bool metzger_dual_raw(const float* pv, int tan0, float t_last, const Times& t, int n, float* out,
                                 float& lp_v, float* lp_d) {
    using D = DN<K>;
    const float MSUN30 = 1.989e3f, C = 2.998e10f, SPD = 86400.0f, PI_F = 3.14159265358979f, LN10F = 2.302585093f;
    D p0(pv[0]), p1(pv[1]), p2(pv[2]), t0(pv[3]);
#pragma unroll
    for (int k = 0; k < K; k++) {
        const int q = tan0 + k;
        if (q == 0) p0.d[k] = 1.0f;
        if (q == 1) p1.d[k] = 1.0f;
        if (q == 2) p2.d[k] = 1.0f;
        if (q == 3) t0.d[k] = 1.0f;
    }
    D m30 = dexp(p0 * LN10F) * MSUN30;
    D v = dexp(p1 * LN10F) * C;
    D kappa_r = dexp(p2 * LN10F);
    float pm = t_last - t0.v;
    for (int j = 0; j < n; j++) {
        out[j * 5] = 0.0f;
#pragma unroll
        for (int k = 0; k < K; k++) out[j * 5 + 1 + tan0 + k] = 0.0f;
    }
    lp_v = 0.0f;
#pragma unroll
    for (int k = 0; k < K; k++) lp_d[k] = 0.0f;
    if (!(pm > 0.01f)) return false;
    D phase_max = (t0 * -1.0f) + t_last;
    const float lmin = -4.605170185988091f;
    D lmax = dlog(phase_max * 1.05f);
    D dl = (lmax - lmin) * (1.0f / 199.0f);
    const float xn0 = 0.8f, xr = 0.2f;
    D vs = v * 1e-5f;
    D e_th = m30 * vs * vs * 0.5f;
    D e_kin = e_th;
    D t_day = D(0.01f);
    D r = t_day * v * SPD;
    D mos = m30 * 1e-10f;
    D diff_k = m30 * (3.0f / (4.0f * PI_F * C) * 1e30f);
    D l_peak = D(-INFINITY);
    D prev_t = t_day, prev_l = D(0.0f);
    int j = 0;
    while (j < n && t(j) - t0.v <= 0.0f) j++;  // zeros already written
    for (int i = 0; i < 200; i++) {
        D t_next = dexp(dl * (float)(i + 1) + lmin);
        D t_sec = t_day * SPD;
        D ef = dpowc(t_day, 0.74f) * 0.34f;
        D eth = (dexp(t_day * -0.56f) + (ef.v > 1e-10f ? dlog1p(ef) / ef : D(1.0f))) * 0.36f;
        D xn = dexp(t_sec * (-1.0f / 900.0f)) * xn0;
        D tt = datan(D(0.11f) / (t_sec - 1.3f)) * (1.0f / PI_F);
        if (tt.v < 1e-30f) tt = D(1e-30f);
        D eps_rp = eth * dpowc(tt, 1.3f) * 2e18f;
        D l_heat = mos * (xn * 3.2e14f + eps_rp);
        D kappa_eff = (D(xn0) - xn) * 0.4f + kappa_r * xr;
        D t_diff = kappa_eff * diff_k / (v * t_sec) + r * (1.0f / C);
        D l_rad = (e_th.v > 0.0f && t_diff.v > 0.0f) ? e_th / t_diff : D(0.0f);
        if (l_rad.v > l_peak.v) l_peak = l_rad;
        if (i == 0) {
            while (j < n && t(j) - t0.v <= t_day.v) {
                out[j * 5] = l_rad.v;
#pragma unroll
                for (int k = 0; k < K; k++) out[j * 5 + 1 + tan0 + k] = l_rad.d[k];
                j++;
            }
        } else {
            while (j < n) {
                float phv = t(j) - t0.v;
                if (phv > t_day.v) break;
                D ph = (t0 * -1.0f) + t(j);
                D lv = prev_l + (ph - prev_t) / (t_day - prev_t) * (l_rad - prev_l);
                out[j * 5] = lv.v;
#pragma unroll
                for (int k = 0; k < K; k++) out[j * 5 + 1 + tan0 + k] = lv.d[k];
                j++;
            }
        }
        prev_t = t_day;
        prev_l = l_rad;
        D l_pdv = r.v > 0.0f ? e_th * v / r : D(0.0f);
        if (i < 199) {
            D dts = (t_next - t_day) * SPD;
            e_th = e_th + (l_heat - l_pdv - l_rad) * dts;
            if (e_th.v < 0.0f) e_th = D(0.0f);
            e_kin = e_kin + l_pdv * dts;
            D vn = dsqrt(e_kin * 2.0f / mos);
            v = vn.v < C ? vn : D(C);
            r = r + v * dts;
        }
        t_day = t_next;
    }
    while (j < n) {
        out[j * 5] = prev_l.v;
#pragma unroll
        for (int k = 0; k < K; k++) out[j * 5 + 1 + tan0 + k] = prev_l.d[k];
        j++;
    }
    lp_v = l_peak.v;
#pragma unroll
    for (int k = 0; k < K; k++) lp_d[k] = l_peak.d[k];
    return l_peak.v > 0.0f && isfinite(l_peak.v);
}

// Writes, for the sorted observation times `t[j]` (stride 1), the normalised
// prediction and its four derivatives to out[j * 5 + {0..4}].  Returns false
// when the reference returns all zeros (phase_max <= 0.01, or a non-positive
// or non-finite peak); out is then zero.
template <class Times>
__device__ bool metzger_dual_sweep(const float* pv, float t_last, const Times& t, int n, float* out) {
    float lp_v, lp_d[4];
    if (!metzger_dual_raw<4>(pv, 0, t_last, t, n, out, lp_v, lp_d)) {
        for (int q = 0; q < n * 5; q++) out[q] = 0.0f;
        return false;
    }
    // normalise by the peak (its tangent included, as the difference quotient has it)
    float ip = 1.0f / lp_v;
    for (int q = 0; q < n; q++) {
        float y = out[q * 5] * ip;
        for (int k = 0; k < 4; k++) out[q * 5 + 1 + k] = (out[q * 5 + 1 + k] - y * lp_d[k]) * ip;
        out[q * 5] = y;
    }
    return true;
}

}  // namespace lcf
