// TEST INFRASTRUCTURE ONLY.  Host-side harness that compiles the reference's
// own device model header (cuda/models_device.h of boom-astro/lightcurve-fitting)
// as plain C++ so that its FP64 model evaluations, analytic gradients,
// log-normal CDF and erf approximation can be sampled on the CPU.  The header
// is included from the reference checkout at build time (path given by the
// Makefile); nothing from it is copied into this repository.  The outputs are
// written as golden vectors by tests/golden/make_golden.py and pin the oracle.
#define __device__
#define __forceinline__ inline
#include <cmath>
using std::isfinite;
#include REF_MODELS_DEVICE_H

extern "C" {
double ref_eval(int model_id, const double* p, double t) { return lc_eval_model_at(model_id, p, t); }
int ref_grad(int model_id, const double* p, double t, double* out) { return lc_eval_model_grad(model_id, p, t, out) ? 1 : 0; }
double ref_log_normal_cdf(double x) { return lc_log_normal_cdf_d(x); }
double ref_erf_approx(double x) { return lc_erf_approx(x); }
}
