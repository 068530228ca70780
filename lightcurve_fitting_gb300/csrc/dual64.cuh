// dual64.cuh — forward-mode differentiation in FP64 for the Laplace Hessian.
//
// Dual: a value and one directional derivative, (v, d) = f + f' e with
// e^2 = 0.  The analytic model gradient (models_f64.cuh, model_grad_t),
// evaluated on Duals whose parameter k carries d = 1, gives the gradient and
// its derivative along parameter k: one column of the second derivatives of
// the prediction (forward mode over the gradient).
//
// Jet2: a truncated Taylor series to second order, c0 + c1 e + c2 e^2, for a
// scalar function's first and second derivatives at a point (f' = c1,
// f'' = 2 c2): the upper-limit term's log-CDF.
//
// The scalar functions the model formulas use are called through mexp /
// mlog / mpow, overloaded for double (the library functions themselves, so
// that the double instantiations compute exactly what they did), Dual and
// Jet2.
#pragma once

#include <math.h>

namespace lcf {

__device__ __forceinline__ double mexp(double x) { return exp(x); }
__device__ __forceinline__ double mlog(double x) { return log(x); }
__device__ __forceinline__ double mpow(double x, double y) { return pow(x, y); }
__device__ __forceinline__ double mval(double x) { return x; }

struct Dual {
    double v, d;
    Dual() = default;
    __device__ __forceinline__ Dual(double x, double dx = 0.0) : v(x), d(dx) {}
};
__device__ __forceinline__ Dual dual(double v, double d = 0.0) { return Dual(v, d); }
__device__ __forceinline__ double mval(Dual x) { return x.v; }
__device__ __forceinline__ Dual operator-(Dual a) { return dual(-a.v, -a.d); }
__device__ __forceinline__ Dual operator+(Dual a, Dual b) { return dual(a.v + b.v, a.d + b.d); }
__device__ __forceinline__ Dual operator-(Dual a, Dual b) { return dual(a.v - b.v, a.d - b.d); }
__device__ __forceinline__ Dual operator*(Dual a, Dual b) { return dual(a.v * b.v, a.d * b.v + a.v * b.d); }
__device__ __forceinline__ Dual operator/(Dual a, Dual b) {
    const double q = a.v / b.v;
    return dual(q, (a.d - q * b.d) / b.v);
}
__device__ __forceinline__ Dual operator+(Dual a, double b) { return dual(a.v + b, a.d); }
__device__ __forceinline__ Dual operator+(double a, Dual b) { return dual(a + b.v, b.d); }
__device__ __forceinline__ Dual operator-(Dual a, double b) { return dual(a.v - b, a.d); }
__device__ __forceinline__ Dual operator-(double a, Dual b) { return dual(a - b.v, -b.d); }
__device__ __forceinline__ Dual operator*(Dual a, double b) { return dual(a.v * b, a.d * b); }
__device__ __forceinline__ Dual operator*(double a, Dual b) { return dual(a * b.v, a * b.d); }
__device__ __forceinline__ Dual operator/(Dual a, double b) { return dual(a.v / b, a.d / b); }
__device__ __forceinline__ Dual operator/(double a, Dual b) {
    const double q = a / b.v;
    return dual(q, -q * b.d / b.v);
}
__device__ __forceinline__ Dual mexp(Dual a) {
    const double e = exp(a.v);
    return dual(e, e * a.d);
}
__device__ __forceinline__ Dual mlog(Dual a) { return dual(log(a.v), a.d / a.v); }
__device__ __forceinline__ Dual mpow(Dual a, double y) {
    const double p = pow(a.v, y);
    return dual(p, y * pow(a.v, y - 1.0) * a.d);
}
__device__ __forceinline__ Dual mpow(Dual a, Dual y) {
    const double p = pow(a.v, y.v);
    return dual(p, p * (y.d * log(a.v) + y.v * a.d / a.v));
}

struct Jet2 {
    double c0, c1, c2;
    Jet2() = default;
    __device__ __forceinline__ Jet2(double x, double x1 = 0.0, double x2 = 0.0) : c0(x), c1(x1), c2(x2) {}
};
__device__ __forceinline__ Jet2 jet(double c0, double c1 = 0.0, double c2 = 0.0) { return Jet2(c0, c1, c2); }
__device__ __forceinline__ double mval(Jet2 x) { return x.c0; }
__device__ __forceinline__ Jet2 operator-(Jet2 a) { return jet(-a.c0, -a.c1, -a.c2); }
__device__ __forceinline__ Jet2 operator+(Jet2 a, Jet2 b) { return jet(a.c0 + b.c0, a.c1 + b.c1, a.c2 + b.c2); }
__device__ __forceinline__ Jet2 operator-(Jet2 a, Jet2 b) { return jet(a.c0 - b.c0, a.c1 - b.c1, a.c2 - b.c2); }
__device__ __forceinline__ Jet2 operator*(Jet2 a, Jet2 b) {
    return jet(a.c0 * b.c0, a.c0 * b.c1 + a.c1 * b.c0, a.c0 * b.c2 + a.c1 * b.c1 + a.c2 * b.c0);
}
__device__ __forceinline__ Jet2 operator/(Jet2 a, Jet2 b) {
    const double q0 = a.c0 / b.c0;
    const double q1 = (a.c1 - q0 * b.c1) / b.c0;
    return jet(q0, q1, (a.c2 - q0 * b.c2 - q1 * b.c1) / b.c0);
}
__device__ __forceinline__ Jet2 operator+(Jet2 a, double b) { return jet(a.c0 + b, a.c1, a.c2); }
__device__ __forceinline__ Jet2 operator+(double a, Jet2 b) { return jet(a + b.c0, b.c1, b.c2); }
__device__ __forceinline__ Jet2 operator-(Jet2 a, double b) { return jet(a.c0 - b, a.c1, a.c2); }
__device__ __forceinline__ Jet2 operator-(double a, Jet2 b) { return jet(a - b.c0, -b.c1, -b.c2); }
__device__ __forceinline__ Jet2 operator*(Jet2 a, double b) { return jet(a.c0 * b, a.c1 * b, a.c2 * b); }
__device__ __forceinline__ Jet2 operator*(double a, Jet2 b) { return jet(a * b.c0, a * b.c1, a * b.c2); }
__device__ __forceinline__ Jet2 operator/(double a, Jet2 b) { return jet(a) / b; }
__device__ __forceinline__ Jet2 mexp(Jet2 a) {
    const double e = exp(a.c0);
    return jet(e, e * a.c1, e * (a.c2 + 0.5 * a.c1 * a.c1));
}
__device__ __forceinline__ Jet2 mlog(Jet2 a) {
    const double u1 = a.c1 / a.c0, u2 = a.c2 / a.c0;
    return jet(log(a.c0), u1, u2 - 0.5 * u1 * u1);
}
__device__ __forceinline__ Jet2 mabs(Jet2 a) { return a.c0 < 0.0 ? -a : a; }

}  // namespace lcf
