// likelihood.cu — the likelihood API: FP32 PsoCost::cost_from_slice of
// parameter vectors on one band (lcf_band_cost through launch_band_cost, and
// the allocation-free lcf_band_cost_static), through the per-lane particle
// cost the swarm uses (swarm_cost.cuh).  This unit is compiled with the
// accurate single-precision library forms of exp, log and division (the
// swarm units use the fast forms), so the API holds FP32 accuracy: 1e-5 of
// the FP64 cost for costs below 1e6.
#include <cuda_runtime.h>

#include <mutex>

#include "lcf_internal.cuh"
#include "swarm_cost.cuh"

namespace lcf {

// Batched likelihood of parameter vectors on one band, through the same
// per-lane cost function the PSO kernel uses (lane = parameter vector).
__device__ __forceinline__ void band_cost_body(int model, const float4* obs, int n, float t_last, const double* params,
                                               int n_eval, int with_prior, double* costs, float* scratch) {
    int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    int e = warp * 32 + lane;
    if (warp * 32 >= n_eval) return;
    TaskCtx t;
    t.kind = model;
    t.model = model;
    t.np = n_params_of(model);
    t.D = t.np;
    t.t0i = t0_idx_of(model);
    t.flags = with_prior ? TASK_PRIOR : 0;
    t.n = n;
    t.t0_fixed = 0.0f;
    t.t_last = t_last;
    t.obs = obs;
    t.mscratch = scratch + (size_t)warp * 32 * (size_t)max(n, 1);
    t.inv_n = 1.0 / (double)max(n, 1);
    float x[MAXP];
    double xd[MAXP];
    for (int j = 0; j < MAXP; j++) {
        xd[j] = (e < n_eval && j < t.np) ? params[(size_t)e * t.np + j] : 0.0;
        x[j] = (float)xd[j];
    }
    double c = particle_cost(t, x, xd);
    if (e < n_eval) costs[e] = c;
}

__global__ void band_cost_kernel(int model, const float4* obs, int n, float t_last, const double* params, int n_eval,
                                 int with_prior, double* costs, float* scratch) {
    band_cost_body(model, obs, n, t_last, params, n_eval, with_prior, costs, scratch);
}

void launch_band_cost(int model, const float4* obs, int n, float t_last, const double* params, int n_eval,
                      int with_prior, double* costs, float* scratch, cudaStream_t s) {
    if (n_eval <= 0) return;
    int warps = (n_eval + 31) / 32;
    band_cost_kernel<<<(warps * 32 + 127) / 128, 128, 0, s>>>(model, obs, n, t_last, params, n_eval, with_prior,
                                                              costs, scratch);
}


// ---------------------------------------------------------------------------
// Allocation-free likelihood: lcf_band_cost_static (declared in include/lcf.h).
//
// For callers that cannot call cudaMalloc.  Its scratch — the band's sorted
// FP32 records, its last time, and the MetzgerKN per-lane interpolation
// buffer — lives in the file-scope array below, sized for at most
// STATIC_MAX_OBS observations and STATIC_MAX_EVAL parameter vectors per call
// (4.03 MiB, held by every GPU that loads the library until the process
// exits).  Every value a call reads from the array is first written by that
// same call, so nothing has to be cleared between calls; the array keeps the
// last call's contents.  All calls share the one array, so calls that overlap
// on the GPU (different streams, or host threads without ordering) race.
// ---------------------------------------------------------------------------
constexpr int STATIC_MAX_OBS = 2048;
constexpr int STATIC_MAX_EVAL = 512;
constexpr size_t STATIC_REC_FLOATS = (size_t)STATIC_MAX_OBS * 4 + 4;  // records, then t_last (16-B padded)
constexpr size_t STATIC_SCRATCH_FLOATS = STATIC_REC_FLOATS + (size_t)STATIC_MAX_EVAL * STATIC_MAX_OBS;
static __device__ __align__(256) float g_band_cost_scratch[STATIC_SCRATCH_FLOATS];

// One block: time-sorted FP32 records of the caller's band and its last time
// into the static array (same records as lcf_band_cost builds on the host).
// Observation i goes to slot rank(i) = the number of observations before it
// in a strict total order: times ascending, NaN times after all others, ties
// in input order.  The ranks are therefore a permutation of 0..n-1 and every
// record slot the cost kernel reads is written by this call.
__global__ void static_prep_kernel(const double* t, const double* f, const double* var, const uint8_t* up,
                                   const double* uf, int n, float* scratch) {
    float4* rec = reinterpret_cast<float4*>(scratch);
    __shared__ double smax[256];
    double mx = -INFINITY;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        double ti = t[i];
        mx = fmax(mx, ti);
        const bool ni = isnan(ti);
        int pos = 0;
        for (int j = 0; j < n; j++) {
            double tj = t[j];
            const bool nj = isnan(tj);
            const bool before = ni ? (!nj || j < i) : (!nj && (tj < ti || (tj == ti && j < i)));
            pos += before ? 1 : 0;
        }
        float th = (float)ti;
        bool u = up[i] != 0;
        rec[pos] = make_float4(th, (float)(ti - (double)th), (float)(u ? uf[i] : f[i]), u ? -(float)var[i] : (float)var[i]);
    }
    smax[threadIdx.x] = mx;
    __syncthreads();
    for (int s2 = blockDim.x / 2; s2 > 0; s2 >>= 1) {
        if (threadIdx.x < s2) smax[threadIdx.x] = fmax(smax[threadIdx.x], smax[threadIdx.x + s2]);
        __syncthreads();
    }
    if (threadIdx.x == 0) scratch[(size_t)STATIC_MAX_OBS * 4] = (float)smax[0];
}

__global__ void band_cost_static_kernel(int model, int n, const double* params, int n_eval, int with_prior,
                                        double* costs, float* scratch) {
    const float4* rec = reinterpret_cast<const float4*>(scratch);
    float t_last = scratch[(size_t)STATIC_MAX_OBS * 4];
    band_cost_body(model, rec, n, t_last, params, n_eval, with_prior, costs, scratch + STATIC_REC_FLOATS);
}

// Device address of the static array, looked up once per device.
static std::mutex g_static_mu;
static float* g_static_ptr[64] = {nullptr};

}  // namespace lcf


extern "C" int lcf_band_cost_static(int device, int model, const double* times, const double* flux,
                                    const double* obs_var, const uint8_t* is_upper, const double* upper_flux,
                                    int n_obs, const double* params, int n_eval, int with_prior, double* costs,
                                    void* stream) {
    using namespace lcf;
    if (device < 0 || device >= 64 || model < 0 || model > 7 || n_obs < 1 || n_eval < 0) return LCF_E_INVALID;
    if (n_obs > STATIC_MAX_OBS || n_eval > STATIC_MAX_EVAL) return LCF_E_CAPACITY;
    if (!times || !flux || !obs_var || !is_upper || !upper_flux || (n_eval > 0 && (!params || !costs)))
        return LCF_E_INVALID;
    if (n_eval == 0) return LCF_OK;
    int prev = -1;
    if (cudaGetDevice(&prev) != cudaSuccess) return LCF_E_CUDA;
    if (prev != device && cudaSetDevice(device) != cudaSuccess) return LCF_E_CUDA;
    float* scratch = nullptr;
    {
        // set-up, once per device, with that device current
        std::lock_guard<std::mutex> lock(g_static_mu);
        if (!g_static_ptr[device]) {
            void* ptr = nullptr;
            if (cudaGetSymbolAddress(&ptr, g_band_cost_scratch) != cudaSuccess || !ptr) {
                if (prev != device) cudaSetDevice(prev);
                return LCF_E_CUDA;
            }
            g_static_ptr[device] = reinterpret_cast<float*>(ptr);
        }
        scratch = g_static_ptr[device];
    }
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    static_prep_kernel<<<1, 256, 0, s>>>(times, flux, obs_var, is_upper, upper_flux, n_obs, scratch);
    int warps = (n_eval + 31) / 32;
    band_cost_static_kernel<<<(warps * 32 + 127) / 128, 128, 0, s>>>(model, n_obs, params, n_eval, with_prior, costs,
                                                                      scratch);
    cudaError_t e = cudaGetLastError();
    if (prev != device) cudaSetDevice(prev);
    return e == cudaSuccess ? LCF_OK : LCF_E_CUDA;
}
