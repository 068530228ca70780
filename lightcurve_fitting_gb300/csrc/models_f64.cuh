// models_f64.cuh — FP64 device evaluation of the reference's model formulas
// (src/parametric.rs:199-538, MetzgerKN :544-648, log-normal CDF :866-901).
// Used where the reference's arithmetic is kept in FP64 on the device: the
// Laplace finite-difference Hessian, the profile refinements, the
// magnitude-space chi2, the MetzgerKN SVI finite differences and the
// drop-in `launch_*` exports.
#pragma once

#include <math.h>

#include "dual64.cuh"

namespace lcf {

__device__ __forceinline__ double sp64(double x) { return log(1.0 + exp(x)) + 1e-6; }
template <class T>
__device__ __forceinline__ T sp64_t(T x) { return mlog(1.0 + mexp(x)) + 1e-6; }

// The model formulas on a scalar type T: double (eval_model_f64 and
// model_grad_f64 below) or the forward-mode Dual of dual64.cuh (the Laplace
// Hessian).
template <class T>
__device__ inline T eval_model_t(int m, const T* p, T t) {
    switch (m) {
        case 0: {
            T a = mexp(p[0]), b = p[1], dt = t - p[2], tr = mexp(p[3]), tf = mexp(p[4]);
            return a * mexp(-dt / tf) * (1.0 / (1.0 + mexp(-dt / tr))) + b;
        }
        case 1: {
            T a = mexp(p[0]), beta = p[1], gamma = mexp(p[2]), ph = t - p[3], tr = mexp(p[4]), tf = mexp(p[5]);
            T sig = 1.0 / (1.0 + mexp(-ph / tr));
            T w = 1.0 / (1.0 + mexp(-10.0 * (ph - gamma)));
            T pl = 1.0 - beta * ph;
            T pr = (1.0 - beta * gamma) * mexp((gamma - ph) / tf);
            return a * sig * ((1.0 - w) * pl + w * pr);
        }
        case 2: {
            T a = mexp(p[0]), b = p[1], ph = t - p[2], tr = mexp(p[3]), tf = mexp(p[4]), al = p[5];
            T sig = 1.0 / (1.0 + mexp(-ph / tr));
            T w = 1.0 + sp64_t(ph) / tf;
            return a * sig * mpow(w, -al) + b;
        }
        case 3: {
            T a = mexp(p[0]), ph = t - p[1], tm = mexp(p[2]);
            T ps = sp64_t(ph);
            T f = 1.0 / (1.0 + mexp(-p[3]));
            T heat = f * mexp(-ps / 8.8) + (1.0 - f) * mexp(-ps / 111.3);
            T x = ps / tm;
            return a * heat * (1.0 - mexp(-x * x));
        }
        case 4: {
            T a = mexp(p[0]), ph = t - p[1], tsd = mexp(p[2]), td = mexp(p[3]);
            T ps = sp64_t(ph);
            T w = 1.0 + ps / tsd;
            T x = ps / td;
            return a * (1.0 / (w * w)) * (1.0 - mexp(-x * x));
        }
        case 5: {
            T a = mexp(p[0]), ph = t - p[1], n = p[2], ttr = mexp(p[3]);
            T sig5 = 1.0 / (1.0 + mexp(-ph * 5.0));
            T ps = sp64_t(ph);
            T r = ps / ttr;
            return a * sig5 * mpow(ps, -n) * mexp(-r * r);
        }
        default: {
            T a = mexp(p[0]), ph = t - p[1], tb = mexp(p[2]), a1 = p[3], a2 = p[4];
            T ps = sp64_t(ph);
            T lr = mlog(ps / tb);
            T u = mexp(2.0 * a1 * lr) + mexp(2.0 * a2 * lr);
            return a * mpow(u, -0.5);
        }
    }
}
__device__ inline double eval_model_f64(int m, const double* p, double t) { return eval_model_t<double>(m, p, t); }

// Analytic d flux / d theta (src/parametric.rs:213-509); the sigma_extra
// slot is 0.
template <class T>
__device__ inline void model_grad_t(int m, const T* p, T t, T* o) {
    switch (m) {
        case 0: {
            T a = mexp(p[0]), dt = t - p[2], tr = mexp(p[3]), tf = mexp(p[4]);
            T sig = 1.0 / (1.0 + mexp(-dt / tr));
            T base = a * mexp(-dt / tf) * sig;
            o[0] = base; o[1] = T(1.0);
            o[2] = base * (1.0 / tf - (1.0 - sig) / tr);
            o[3] = -base * (1.0 - sig) * dt / tr;
            o[4] = base * dt / tf;
            o[5] = T(0.0);
            return;
        }
        case 1: {
            T a = mexp(p[0]), beta = p[1], gamma = mexp(p[2]), ph = t - p[3], tr = mexp(p[4]), tf = mexp(p[5]);
            const double k = 10.0;
            T sig = 1.0 / (1.0 + mexp(-ph / tr));
            T w = 1.0 / (1.0 + mexp(-k * (ph - gamma)));
            T pl = 1.0 - beta * ph;
            T ed = mexp((gamma - ph) / tf);
            T pr = (1.0 - beta * gamma) * ed;
            T piece = (1.0 - w) * pl + w * pr;
            o[0] = a * sig * piece;
            o[1] = a * sig * ((1.0 - w) * (-ph) + w * (-gamma * ed));
            T dwdlg = -k * w * (1.0 - w) * gamma;
            T dprdlg = ed * (-beta + (1.0 - beta * gamma) / tf) * gamma;
            o[2] = a * sig * (dwdlg * (pr - pl) + w * dprdlg);
            T dsig_dt0 = -(sig * (1.0 - sig) / tr);
            T dw_dt0 = -(k * w * (1.0 - w));
            T dpdt0 = dw_dt0 * (pr - pl) + (1.0 - w) * beta + w * ((1.0 - beta * gamma) * ed / tf);
            o[3] = a * (dsig_dt0 * piece + sig * dpdt0);
            o[4] = a * piece * sig * (1.0 - sig) * (-ph / tr);
            o[5] = a * sig * w * (pr * (ph - gamma) / tf);
            o[6] = T(0.0);
            return;
        }
        case 2: {
            T a = mexp(p[0]), ph = t - p[2], tr = mexp(p[3]), tf = mexp(p[4]), al = p[5];
            T sig = 1.0 / (1.0 + mexp(-ph / tr));
            T ps = sp64_t(ph);
            T sp = mexp(ph) / (1.0 + mexp(ph));
            T w = 1.0 + ps / tf;
            T decay = mpow(w, -al);
            o[0] = a * sig * decay; o[1] = T(1.0);
            T dsig_dt0 = -sig * (1.0 - sig) / tr;
            T dd_dt0 = al * mpow(w, -al - 1.0) * sp / tf;
            o[2] = a * (dsig_dt0 * decay + sig * dd_dt0);
            o[3] = a * decay * (-sig * (1.0 - sig) * ph / tr);
            o[4] = a * sig * al * mpow(w, -al - 1.0) * ps / tf;
            o[5] = a * sig * (-mlog(w)) * decay;
            o[6] = T(0.0);
            return;
        }
        case 3: {
            T a = mexp(p[0]), ph = t - p[1], tm = mexp(p[2]);
            T ps = sp64_t(ph);
            T sp = mexp(ph) / (1.0 + mexp(ph));
            T f = 1.0 / (1.0 + mexp(-p[3]));
            T eni = mexp(-ps / 8.8), eco = mexp(-ps / 111.3);
            T heat = f * eni + (1.0 - f) * eco;
            T x = ps / tm;
            T ex2 = mexp(-x * x);
            T trap = 1.0 - ex2;
            o[0] = a * heat * trap;
            T dheat = -f * eni / 8.8 - (1.0 - f) * eco / 111.3;
            T dtrap = 2.0 * ps * ex2 / (tm * tm);
            o[1] = a * (-sp) * (dheat * trap + heat * dtrap);
            o[2] = -2.0 * a * heat * ex2 * x * x;
            o[3] = a * trap * (eni - eco) * f * (1.0 - f);
            o[4] = T(0.0);
            return;
        }
        case 4: {
            T a = mexp(p[0]), ph = t - p[1], tsd = mexp(p[2]), td = mexp(p[3]);
            T ps = sp64_t(ph);
            T sp = mexp(ph) / (1.0 + mexp(ph));
            T w = 1.0 + ps / tsd;
            T sd = 1.0 / (w * w);
            T x = ps / td;
            T ex2 = mexp(-x * x);
            T trap = 1.0 - ex2;
            o[0] = a * sd * trap;
            T w3 = 1.0 / (w * w * w);
            o[1] = a * (-sp) * ((-2.0 * w3 / tsd) * trap + sd * (2.0 * ps * ex2 / (td * td)));
            o[2] = a * trap * 2.0 * ps * w3 / tsd;
            o[3] = -2.0 * a * sd * ex2 * x * x;
            o[4] = T(0.0);
            return;
        }
        case 5: {
            T a = mexp(p[0]), ph = t - p[1], n = p[2], ttr = mexp(p[3]);
            T sig5 = 1.0 / (1.0 + mexp(-ph * 5.0));
            T ps = sp64_t(ph);
            T sp = mexp(ph) / (1.0 + mexp(ph));
            T cooling = mpow(ps, -n);
            T r = ps / ttr;
            T cutoff = mexp(-r * r);
            T base = cooling * cutoff;
            T flux = a * sig5 * base;
            o[0] = flux;
            o[1] = a * base * (-5.0 * sig5 * (1.0 - sig5) + sig5 * sp * (n / ps + 2.0 * ps / (ttr * ttr)));
            o[2] = -flux * mlog(ps);
            o[3] = flux * 2.0 * r * r;
            o[4] = T(0.0);
            return;
        }
        default: {
            T a = mexp(p[0]), ph = t - p[1], tb = mexp(p[2]), a1 = p[3], a2 = p[4];
            T ps = sp64_t(ph);
            T sp = mexp(ph) / (1.0 + mexp(ph));
            T lr = mlog(ps / tb);
            T u1 = mexp(2.0 * a1 * lr), u2 = mexp(2.0 * a2 * lr);
            T u = u1 + u2;
            T um15 = mpow(u, -1.5);
            o[0] = a * mpow(u, -0.5);
            T du_dps = (2.0 * a1 * u1 + 2.0 * a2 * u2) / ps;
            o[1] = a * (-0.5) * um15 * du_dps * (-sp);
            o[2] = a * (-0.5) * um15 * (-(2.0 * a1 * u1 + 2.0 * a2 * u2));
            o[3] = a * (-0.5) * um15 * 2.0 * lr * u1;
            o[4] = a * (-0.5) * um15 * 2.0 * lr * u2;
            o[5] = T(0.0);
            return;
        }
    }
}
__device__ inline void model_grad_f64(int m, const double* p, double t, double* o) { model_grad_t<double>(m, p, t, o); }

// Hoisted FP64 evaluator: the per-parameter-vector constants (exponentials of
// the log parameters, reciprocals) are formed once in init(); value() and
// value_grad() then spend only the per-observation transcendentals.  Same
// formulas as eval_model_f64 / model_grad_f64 (dividing by tau and
// multiplying by 1/tau differ by at most one rounding).
struct Model64 {
    int m;
    double c[12];
    __device__ void init(int model, const double* p) {
        m = model;
        switch (m) {
            case 0: c[0] = exp(p[0]); c[1] = p[1]; c[2] = p[2]; c[3] = 1.0 / exp(p[3]); c[4] = 1.0 / exp(p[4]); break;
            case 1: c[0] = exp(p[0]); c[1] = p[1]; c[2] = exp(p[2]); c[3] = p[3]; c[4] = 1.0 / exp(p[4]);
                    c[5] = 1.0 / exp(p[5]); c[6] = 1.0 - p[1] * exp(p[2]); break;
            case 2: c[0] = exp(p[0]); c[1] = p[1]; c[2] = p[2]; c[3] = 1.0 / exp(p[3]); c[4] = 1.0 / exp(p[4]);
                    c[5] = p[5]; break;
            case 3: c[0] = exp(p[0]); c[1] = p[1]; c[2] = 1.0 / exp(p[2]); c[3] = 1.0 / (1.0 + exp(-p[3])); break;
            case 4: c[0] = exp(p[0]); c[1] = p[1]; c[2] = 1.0 / exp(p[2]); c[3] = 1.0 / exp(p[3]); break;
            case 5: c[0] = exp(p[0]); c[1] = p[1]; c[2] = p[2]; c[3] = 1.0 / exp(p[3]); break;
            default: c[0] = exp(p[0]); c[1] = p[1]; c[2] = p[2]; c[3] = p[3]; c[4] = p[4]; break;
        }
    }
    // init() from precomputed ep[k] = exp(p[k]) and rp[k] = 1.0 / exp(p[k])
    // (the same constants, bit for bit)
    __device__ void init_pre(int model, const double* p, const double* ep, const double* rp) {
        m = model;
        switch (m) {
            case 0: c[0] = ep[0]; c[1] = p[1]; c[2] = p[2]; c[3] = rp[3]; c[4] = rp[4]; break;
            case 1: c[0] = ep[0]; c[1] = p[1]; c[2] = ep[2]; c[3] = p[3]; c[4] = rp[4];
                    c[5] = rp[5]; c[6] = 1.0 - p[1] * ep[2]; break;
            case 2: c[0] = ep[0]; c[1] = p[1]; c[2] = p[2]; c[3] = rp[3]; c[4] = rp[4]; c[5] = p[5]; break;
            case 3: c[0] = ep[0]; c[1] = p[1]; c[2] = rp[2]; c[3] = 1.0 / (1.0 + exp(-p[3])); break;
            case 4: c[0] = ep[0]; c[1] = p[1]; c[2] = rp[2]; c[3] = rp[3]; break;
            case 5: c[0] = ep[0]; c[1] = p[1]; c[2] = p[2]; c[3] = rp[3]; break;
            default: c[0] = ep[0]; c[1] = p[1]; c[2] = p[2]; c[3] = p[3]; c[4] = p[4]; break;
        }
    }
    // prediction; with g != nullptr also d pred / d theta (sigma_extra slot 0)
    __device__ double eval(double t, double* g) const {
        switch (m) {
            case 0: {
                double a = c[0], dt = t - c[2], itr = c[3], itf = c[4];
                double sig = 1.0 / (1.0 + exp(-dt * itr));
                double base = a * exp(-dt * itf) * sig;
                if (g) {
                    g[0] = base; g[1] = 1.0;
                    g[2] = base * (itf - (1.0 - sig) * itr);
                    g[3] = -base * (1.0 - sig) * dt * itr;
                    g[4] = base * dt * itf;
                    g[5] = 0.0;
                }
                return base + c[1];
            }
            case 1: {
                double a = c[0], beta = c[1], gamma = c[2], ph = t - c[3], itr = c[4], itf = c[5], omb = c[6];
                double sig = 1.0 / (1.0 + exp(-ph * itr));
                double w = 1.0 / (1.0 + exp(-10.0 * (ph - gamma)));
                double pl = 1.0 - beta * ph;
                double ed = exp((gamma - ph) * itf);
                double pr = omb * ed;
                double piece = (1.0 - w) * pl + w * pr;
                if (g) {
                    const double k = 10.0;
                    g[0] = a * sig * piece;
                    g[1] = a * sig * ((1.0 - w) * (-ph) + w * (-gamma * ed));
                    g[2] = a * sig * ((-k * w * (1.0 - w) * gamma) * (pr - pl) + w * (ed * (-beta + omb * itf) * gamma));
                    double dpdt0 = (-(k * w * (1.0 - w))) * (pr - pl) + (1.0 - w) * beta + w * (omb * ed * itf);
                    g[3] = a * ((-(sig * (1.0 - sig) * itr)) * piece + sig * dpdt0);
                    g[4] = a * piece * sig * (1.0 - sig) * (-ph * itr);
                    g[5] = a * sig * w * (pr * (ph - gamma) * itf);
                    g[6] = 0.0;
                }
                return a * sig * piece;
            }
            case 2: {
                double a = c[0], ph = t - c[2], itr = c[3], itf = c[4], al = c[5];
                double sig = 1.0 / (1.0 + exp(-ph * itr));
                double eph = exp(ph);
                double ps = log(1.0 + eph) + 1e-6;
                double w = 1.0 + ps * itf;
                double lw = log(w);
                double decay = exp(-al * lw);
                if (g) {
                    double sp = eph / (1.0 + eph);
                    double wm1 = decay / w;
                    g[0] = a * sig * decay; g[1] = 1.0;
                    g[2] = a * ((-sig * (1.0 - sig) * itr) * decay + sig * (al * wm1 * sp * itf));
                    g[3] = a * decay * (-sig * (1.0 - sig) * ph * itr);
                    g[4] = a * sig * al * wm1 * ps * itf;
                    g[5] = a * sig * (-lw) * decay;
                    g[6] = 0.0;
                }
                return a * sig * decay + c[1];
            }
            case 3: {
                double a = c[0], ph = t - c[1], itm = c[2], f = c[3];
                double eph = exp(ph);
                double ps = log(1.0 + eph) + 1e-6;
                double eni = exp(-ps / 8.8), eco = exp(-ps / 111.3);
                double heat = f * eni + (1.0 - f) * eco;
                double x = ps * itm;
                double ex2 = exp(-x * x);
                double trap = 1.0 - ex2;
                if (g) {
                    double sp = eph / (1.0 + eph);
                    g[0] = a * heat * trap;
                    double dheat = -f * eni / 8.8 - (1.0 - f) * eco / 111.3;
                    double dtrap = 2.0 * ps * ex2 * itm * itm;
                    g[1] = a * (-sp) * (dheat * trap + heat * dtrap);
                    g[2] = -2.0 * a * heat * ex2 * x * x;
                    g[3] = a * trap * (eni - eco) * f * (1.0 - f);
                    g[4] = 0.0;
                }
                return a * heat * trap;
            }
            case 4: {
                double a = c[0], ph = t - c[1], itsd = c[2], itd = c[3];
                double eph = exp(ph);
                double ps = log(1.0 + eph) + 1e-6;
                double w = 1.0 + ps * itsd;
                double sd = 1.0 / (w * w);
                double x = ps * itd;
                double ex2 = exp(-x * x);
                double trap = 1.0 - ex2;
                if (g) {
                    double sp = eph / (1.0 + eph);
                    double w3 = sd / w;
                    g[0] = a * sd * trap;
                    g[1] = a * (-sp) * ((-2.0 * w3 * itsd) * trap + sd * (2.0 * ps * ex2 * itd * itd));
                    g[2] = a * trap * 2.0 * ps * w3 * itsd;
                    g[3] = -2.0 * a * sd * ex2 * x * x;
                    g[4] = 0.0;
                }
                return a * sd * trap;
            }
            case 5: {
                double a = c[0], ph = t - c[1], n = c[2], ittr = c[3];
                double sig5 = 1.0 / (1.0 + exp(-ph * 5.0));
                double eph = exp(ph);
                double ps = log(1.0 + eph) + 1e-6;
                double lps = log(ps);
                double r = ps * ittr;
                double base = exp(-n * lps) * exp(-r * r);
                double flux = a * sig5 * base;
                if (g) {
                    double sp = eph / (1.0 + eph);
                    g[0] = flux;
                    g[1] = a * base * (-5.0 * sig5 * (1.0 - sig5) + sig5 * sp * (n / ps + 2.0 * ps * ittr * ittr));
                    g[2] = -flux * lps;
                    g[3] = flux * 2.0 * r * r;
                    g[4] = 0.0;
                }
                return flux;
            }
            default: {
                double a = c[0], ph = t - c[1], ltb = c[2], a1 = c[3], a2 = c[4];
                double eph = exp(ph);
                double ps = log(1.0 + eph) + 1e-6;
                double lr = log(ps) - ltb;
                double u1 = exp(2.0 * a1 * lr), u2 = exp(2.0 * a2 * lr);
                double u = u1 + u2;
                double iu = 1.0 / sqrt(u);
                if (g) {
                    double sp = eph / (1.0 + eph);
                    double um15 = iu / u;
                    g[0] = a * iu;
                    g[1] = a * (-0.5) * um15 * ((2.0 * a1 * u1 + 2.0 * a2 * u2) / ps) * (-sp);
                    g[2] = a * (-0.5) * um15 * (-(2.0 * a1 * u1 + 2.0 * a2 * u2));
                    g[3] = a * (-0.5) * um15 * 2.0 * lr * u1;
                    g[4] = a * (-0.5) * um15 * 2.0 * lr * u2;
                    g[5] = 0.0;
                }
                return a * iu;
            }
        }
    }
};

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

// log_normal_cdf on a second-order Taylor number (dual64.cuh): the same A&S
// expression, branches and floor as log_normal_cdf_f64, carrying its first
// and second derivatives (c1, 2 c2) for the analytic Laplace Hessian.
__device__ __forceinline__ Jet2 log_normal_cdf_jet(Jet2 x) {
    if (x.c0 > 8.0) return jet(0.0);
    if (x.c0 < -30.0) return -0.5 * x * x - 0.5 * log(2.0 * 3.14159265358979323846) - mlog(-x);
    const Jet2 z = -x * 0.70710678118654752440;
    const Jet2 t = 1.0 / (1.0 + 0.3275911 * mabs(z));
    const Jet2 poly = t * (0.254829592 + t * (-0.284496736 + t * (1.421413741 + t * (-1.453152027 + t * 1.061405429))));
    const Jet2 e = poly * mexp(-z * z);
    const Jet2 phi = z.c0 >= 0.0 ? 0.5 * e : 1.0 - 0.5 * e;
    return phi.c0 > 1e-300 ? mlog(phi) : jet(log(1e-300));
}

// Upper-limit term of the cost and its gradient factor at z = (u - pred) /
// sigma, sharing one evaluation of the A&S erf pieces (t, the polynomial and
// e^(-z^2/2)) between log_normal_cdf (the cost, src/parametric.rs:882-901)
// and the gradient's Gaussian pdf / CDF ratio (PsoCost::gradient, :1420-1431).
// The CDF keeps the reference's form 0.5 * (1 + erf), so it rounds to exactly
// 0 (floored at 1e-300) for z below ~-8.3 as the reference's does.
__device__ __forceinline__ double upper_cost_ratio(double z, bool want_ratio, double& ratio) {
    const double a = fabs(z) * 0.70710678118654752440;
    const double t = 1.0 / (1.0 + 0.3275911 * a);
    const double poly = t * (0.254829592 + t * (-0.284496736 + t * (1.421413741 + t * (-1.453152027 + t * 1.061405429))));
    const double e = exp(-a * a);
    const double pe = poly * e;
    if (want_ratio) {
        double v = 1.0 - pe;
        double cdf = 0.5 * (1.0 + (z >= 0.0 ? v : -v));
        ratio = (e * 0.39894228040143267794) / fmax(cdf, 1e-300);
    }
    if (z > 8.0) return 0.0;
    if (z < -30.0) return -0.5 * z * z - 0.5 * log(2.0 * 3.14159265358979323846) - log(-z);
    double phi = z <= 0.0 ? 0.5 * pe : 1.0 - 0.5 * pe;
    return log(fmax(phi, 1e-300));
}

// MetzgerKN sweep (metzger_kn_eval_batch, src/parametric.rs:544-648) over a
// band whose times are sorted ascending: integrates the ODE on the 200-point
// log grid and calls visit(j, l) with the unnormalised luminosity
// interpolated at every observation j >= j_start (the observations with
// t - t0 <= 0 come first and predict 0; they are not visited).  Returns
// false when the reference returns all zeros before integrating
// (phase_max <= 0.01); l_peak is the grid maximum the predictions are
// divided by.
template <class V>
__device__ __forceinline__ bool metzger_sweep64(const double* p, const double* times, int n, V& visit,
                                                int& j_start, double& l_peak) {
    const double MSUN = 1.989e33, C = 2.998e10, SPD = 86400.0, PI = 3.14159265358979323846;
    double m_ej = pow(10.0, p[0]) * MSUN, v_ej = pow(10.0, p[1]) * C, kappa_r = pow(10.0, p[2]), t0 = p[3];
    double phase_max = 0.01;
    for (int i = 0; i < n; i++) phase_max = fmax(phase_max, times[i] - t0);
    j_start = n;
    l_peak = -INFINITY;
    if (phase_max <= 0.01) return false;
    const int NG = 200;
    double lmin = log(0.01), lmax = log(phase_max * 1.05);
    double e0 = 0.5 * m_ej * v_ej * v_ej;
    double e_th = e0 / 1e40, e_kin = e0 / 1e40, v = v_ej;
    double gt0 = exp(lmin);
    double r = gt0 * SPD * v;
    double prev_t = gt0, prev_l = 0.0;
    double t_day = gt0;
    int j = 0;
    while (j < n && times[j] - t0 <= 0.0) j++;
    j_start = j;
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
            while (j < n && times[j] - t0 <= t_day) { visit(j, l_rad); j++; }
        } else {
            while (j < n) {
                double ph = times[j] - t0;
                if (ph > t_day) break;
                double frac = (ph - prev_t) / (t_day - prev_t);
                visit(j, prev_l + frac * (l_rad - prev_l));
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
    while (j < n) { visit(j, prev_l); j++; }
    return true;
}

// MetzgerKN at one observation as the reference's GPU cost and SVI kernels
// evaluate it (cuda/models_device.h:376-456, cuda/models.cu:429-511): its
// own 100-point log grid from 0.01 d to 1.05 x the observation's phase
// (at least 0.02 d), the same explicit-Euler thermal / kinetic energy ODE as
// the band sweep, the luminosity interpolated at the phase and divided by the
// grid's running maximum; 0 before t0 or for a non-positive / non-finite
// maximum.  This is a different model evaluation from the band sweep above
// (whole-band grid, band peak) and from the CPU path; the operations keep the
// reference kernel's order so that FP64 rounding matches it.
__device__ inline double metzger_at_obs_f64(const double* p, double t) {
    const double MSUN = 1.989e33, C = 2.998e10, SPD = 86400.0, PI = 3.14159265358979323846;
    const double m_ej = pow(10.0, p[0]) * MSUN, v_ej = pow(10.0, p[1]) * C, kappa_r = pow(10.0, p[2]);
    const double phase = t - p[3];
    if (phase <= 0.0) return 0.0;
    const double phase_max = fmax(phase * 1.05, 0.02);
    const int NG = 100;
    const double lmin = log(0.01), lmax = log(phase_max);
    const double xn0 = 1.0 - 2.0 * 0.1;
    const double xr = 1.0 - xn0;
    const double e0 = 0.5 * m_ej * v_ej * v_ej;
    double e_th = e0 / 1e40, e_kin = e0 / 1e40, v = v_ej;
    const double gt0 = exp(lmin);
    double r = gt0 * SPD * v;
    double l_peak = 0.0, l_at = 0.0, prev_t = gt0, prev_l = 0.0;
    for (int i = 0; i < NG; i++) {
        const double t_day = exp(lmin + (lmax - lmin) * (double)i / (double)(NG - 1));
        const double t_sec = t_day * SPD;
        const double ef = 0.34 * pow(t_day, 0.74);
        const double eth = 0.36 * (exp(-0.56 * t_day) + (ef > 1e-10 ? log(1.0 + ef) / ef : 1.0));
        const double xn = xn0 * exp(-t_sec / 900.0);
        const double tt = fmax(0.5 - atan((t_sec - 1.3) / 0.11) / PI, 1e-30);
        const double eps_rp = 2e18 * eth * pow(tt, 1.3);
        const double l_heat = m_ej * (3.2e14 * xn + eps_rp) / 1e40;
        const double kappa_eff = 0.4 * (xn0 - xn) + kappa_r * xr;
        const double t_diff = 3.0 * kappa_eff * m_ej / (4.0 * PI * C * v * t_sec) + r / C;
        const double l_rad = (e_th > 0.0 && t_diff > 0.0) ? e_th / t_diff : 0.0;
        if (l_rad > l_peak) l_peak = l_rad;
        if (i > 0 && phase >= prev_t && phase <= t_day)
            l_at = prev_l + (phase - prev_t) / (t_day - prev_t) * (l_rad - prev_l);
        if (i == NG - 1 && phase >= t_day) l_at = l_rad;
        if (i == 0 && phase <= t_day) l_at = l_rad;
        prev_t = t_day;
        prev_l = l_rad;
        const double l_pdv = r > 0.0 ? e_th * v / r : 0.0;
        if (i < NG - 1) {
            const double t_next = exp(lmin + (lmax - lmin) * (double)(i + 1) / (double)(NG - 1));
            const double dts = (t_next - t_day) * SPD;
            e_th += (l_heat - l_pdv - l_rad) * dts;
            if (e_th < 0.0) e_th = 0.0;
            e_kin += l_pdv * dts;
            v = sqrt(2.0 * e_kin * 1e40 / m_ej);
            if (v > C) v = C;
            r += v * dts;
        }
    }
    if (l_peak <= 0.0 || !isfinite(l_peak)) return 0.0;
    return l_at / l_peak;
}

// MetzgerKN predictions of the band (metzger_kn_eval_batch): the sweep's
// interpolants divided by l_peak; all zeros when the reference returns
// zeros (phase_max <= 0.01, or a non-positive / non-finite peak).
__device__ inline void metzger_f64(const double* p, const double* times, int n, double* out) {
    for (int i = 0; i < n; i++) out[i] = 0.0;
    struct Store {
        double* out;
        __device__ void operator()(int j, double l) { out[j] = l; }
    } st{out};
    int j_start;
    double l_peak;
    if (!metzger_sweep64(p, times, n, st, j_start, l_peak)) return;
    if (l_peak <= 0.0 || !isfinite(l_peak)) {
        for (int i = 0; i < n; i++) out[i] = 0.0;
        return;
    }
    for (int i = j_start; i < n; i++) out[i] /= l_peak;
}

}  // namespace lcf
