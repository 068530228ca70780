// models_f64.cuh — FP64 device evaluation of the reference's model formulas
// (src/parametric.rs:199-538, MetzgerKN :544-648, log-normal CDF :866-901).
// Used where the reference's arithmetic is kept in FP64 on the device: the
// Laplace finite-difference Hessian, the profile refinements, the
// magnitude-space chi2, the MetzgerKN SVI finite differences and the
// drop-in `launch_*` exports.
#pragma once

#include <math.h>

namespace lcf {

__device__ __forceinline__ double sp64(double x) { return log(1.0 + exp(x)) + 1e-6; }

__device__ inline double eval_model_f64(int m, const double* p, double t) {
    switch (m) {
        case 0: {
            double a = exp(p[0]), b = p[1], dt = t - p[2], tr = exp(p[3]), tf = exp(p[4]);
            return a * exp(-dt / tf) * (1.0 / (1.0 + exp(-dt / tr))) + b;
        }
        case 1: {
            double a = exp(p[0]), beta = p[1], gamma = exp(p[2]), ph = t - p[3], tr = exp(p[4]), tf = exp(p[5]);
            double sig = 1.0 / (1.0 + exp(-ph / tr));
            double w = 1.0 / (1.0 + exp(-10.0 * (ph - gamma)));
            double pl = 1.0 - beta * ph;
            double pr = (1.0 - beta * gamma) * exp((gamma - ph) / tf);
            return a * sig * ((1.0 - w) * pl + w * pr);
        }
        case 2: {
            double a = exp(p[0]), b = p[1], ph = t - p[2], tr = exp(p[3]), tf = exp(p[4]), al = p[5];
            double sig = 1.0 / (1.0 + exp(-ph / tr));
            double w = 1.0 + sp64(ph) / tf;
            return a * sig * pow(w, -al) + b;
        }
        case 3: {
            double a = exp(p[0]), ph = t - p[1], tm = exp(p[2]);
            double ps = sp64(ph);
            double f = 1.0 / (1.0 + exp(-p[3]));
            double heat = f * exp(-ps / 8.8) + (1.0 - f) * exp(-ps / 111.3);
            double x = ps / tm;
            return a * heat * (1.0 - exp(-x * x));
        }
        case 4: {
            double a = exp(p[0]), ph = t - p[1], tsd = exp(p[2]), td = exp(p[3]);
            double ps = sp64(ph);
            double w = 1.0 + ps / tsd;
            double x = ps / td;
            return a * (1.0 / (w * w)) * (1.0 - exp(-x * x));
        }
        case 5: {
            double a = exp(p[0]), ph = t - p[1], n = p[2], ttr = exp(p[3]);
            double sig5 = 1.0 / (1.0 + exp(-ph * 5.0));
            double ps = sp64(ph);
            double r = ps / ttr;
            return a * sig5 * pow(ps, -n) * exp(-r * r);
        }
        default: {
            double a = exp(p[0]), ph = t - p[1], tb = exp(p[2]), a1 = p[3], a2 = p[4];
            double ps = sp64(ph);
            double lr = log(ps / tb);
            double u = exp(2.0 * a1 * lr) + exp(2.0 * a2 * lr);
            return a * pow(u, -0.5);
        }
    }
}

__device__ __forceinline__ double erf_approx_f64(double x) {
    double a = fabs(x);
    double t = 1.0 / (1.0 + 0.3275911 * a);
    double poly = t * (0.254829592 + t * (-0.284496736 + t * (1.421413741 + t * (-1.453152027 + t * 1.061405429))));
    double v = 1.0 - poly * exp(-a * a);
    return x >= 0.0 ? v : -v;
}

__device__ __forceinline__ double log_normal_cdf_f64(double x) {
    if (x > 8.0) return 0.0;
    if (x < -30.0) return -0.5 * x * x - 0.5 * log(2.0 * 3.14159265358979323846) - log(-x);
    double z = -x * 0.70710678118654752440;
    double t = 1.0 / (1.0 + 0.3275911 * fabs(z));
    double poly = t * (0.254829592 + t * (-0.284496736 + t * (1.421413741 + t * (-1.453152027 + t * 1.061405429))));
    double e = poly * exp(-z * z);
    double phi = z >= 0.0 ? 0.5 * e : 1.0 - 0.5 * e;
    return log(fmax(phi, 1e-300));
}

// MetzgerKN over a band whose times are sorted ascending (phase_max over all
// of them), exactly as metzger_kn_eval_batch; writes n predictions.
__device__ inline void metzger_f64(const double* p, const double* times, int n, double* out) {
    const double MSUN = 1.989e33, C = 2.998e10, SPD = 86400.0, PI = 3.14159265358979323846;
    double m_ej = pow(10.0, p[0]) * MSUN, v_ej = pow(10.0, p[1]) * C, kappa_r = pow(10.0, p[2]), t0 = p[3];
    double phase_max = 0.01;
    for (int i = 0; i < n; i++) phase_max = fmax(phase_max, times[i] - t0);
    if (phase_max <= 0.01) {
        for (int i = 0; i < n; i++) out[i] = 0.0;
        return;
    }
    const int NG = 200;
    double lmin = log(0.01), lmax = log(phase_max * 1.05);
    double e0 = 0.5 * m_ej * v_ej * v_ej;
    double e_th = e0 / 1e40, e_kin = e0 / 1e40, v = v_ej;
    double gt0 = exp(lmin);
    double r = gt0 * SPD * v;
    double l_peak = -INFINITY;
    double prev_t = gt0, prev_l = 0.0;
    double t_day = gt0;
    int j = 0;
    while (j < n && times[j] - t0 <= 0.0) { out[j] = 0.0; j++; }
    int j_start = j;
    for (int i = 0; i < NG; i++) {
        double t_next = exp(lmin + (lmax - lmin) * (double)(i + 1) / (double)(NG - 1));
        double t_sec = t_day * SPD;
        double ef = 0.34 * pow(t_day, 0.74);
        double eth = 0.36 * (exp(-0.56 * t_day) + (ef > 1e-10 ? log(1.0 + ef) / ef : 1.0));
        double xn = 0.8 * exp(-t_sec / 900.0);
        double tt = fmax(0.5 - atan((t_sec - 1.3) / 0.11) / PI, 1e-30);
        double eps_rp = 2e18 * eth * pow(tt, 1.3);
        double l_heat = m_ej * (3.2e14 * xn + eps_rp) / 1e40;
        double kappa_eff = 0.4 * (0.8 - xn) + kappa_r * 0.2;
        double t_diff = 3.0 * kappa_eff * m_ej / (4.0 * PI * C * v * t_sec) + r / C;
        double l_rad = (e_th > 0.0 && t_diff > 0.0) ? e_th / t_diff : 0.0;
        l_peak = fmax(l_peak, l_rad);
        if (i == 0) {
            while (j < n && times[j] - t0 <= t_day) { out[j] = l_rad; j++; }
        } else {
            while (j < n) {
                double ph = times[j] - t0;
                if (ph > t_day) break;
                double frac = (ph - prev_t) / (t_day - prev_t);
                out[j] = prev_l + frac * (l_rad - prev_l);
                j++;
            }
        }
        prev_t = t_day;
        prev_l = l_rad;
        double l_pdv = r > 0.0 ? e_th * v / r : 0.0;
        if (i < NG - 1) {
            double dts = (t_next - t_day) * SPD;
            e_th += (l_heat - l_pdv - l_rad) * dts;
            if (e_th < 0.0) e_th = 0.0;
            e_kin += l_pdv * dts;
            v = fmin(sqrt(2.0 * e_kin * 1e40 / m_ej), C);
            r += v * dts;
        }
        t_day = t_next;
    }
    while (j < n) { out[j] = prev_l; j++; }
    if (l_peak <= 0.0 || !isfinite(l_peak)) {
        for (int i = 0; i < n; i++) out[i] = 0.0;
        return;
    }
    for (int i = j_start; i < n; i++) out[i] /= l_peak;
}

}  // namespace lcf
