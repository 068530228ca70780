// lcf_internal.cuh — shared declarations of liblcf_gb300: model tables,
// device data layout, task and result records, and the launch wrappers each
// translation unit exports to the host orchestrator (host.cpp).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "lcf.h"

namespace lcf {

// ---------------------------------------------------------------------------
// Model tables (src/parametric.rs:124-162, :1541-1621, :2072-2115).
// Model ids: 0 Bazin, 1 Villar, 2 Tde, 3 Arnett, 4 Magnetar, 5 ShockCooling,
// 6 Afterglow, 7 MetzgerKN.  Task kinds 8..11 are MultiBazin with K = 1..4.
// ---------------------------------------------------------------------------
enum : int { BAZIN = 0, VILLAR = 1, TDE = 2, ARNETT = 3, MAGNETAR = 4, SHOCK = 5, AFTERGLOW = 6, METZGER = 7 };
enum : int { KIND_MB1 = 8 };  // kind = KIND_MB1 + (K - 1)

constexpr int NP = 30;          // particles, src/parametric.rs:1974-1987
constexpr int MAX_ITERS = 60;
constexpr int STALL_ITERS = 12;
constexpr int MAXP = LCF_MAX_PARAMS;
constexpr int MB_MAXP = LCF_MB_MAX_PARAMS;
// Length of the per-seed uniform-draw table: the longest PSO run (18
// dimensions) consumes 30*2*18 initial draws plus 60*30*2*18 in its iterations.
constexpr int DRAWS_PER_SEED = 66000;
// SVI reparameterisation noise table: 1000 steps x 4 samples x up to 7 params.
constexpr int SVI_STEPS = 1000;
constexpr int SVI_SAMPLES = 4;
constexpr double SVI_LR = 0.01;
// Joint multi-band Villar fit (joint.cu): at most 6 bands per source, so
// 42 joint parameters.
constexpr int J_MAX_BANDS = 6;
constexpr int J_MAX_D = 7 * J_MAX_BANDS;
// Per-particle arrays of the joint swarm's state: position, velocity and
// personal best as double-float pairs, and the trial position.
constexpr int JOINT_STATE_ARRAYS = 7;

__host__ __device__ constexpr int n_params_of(int m) {
    return m == BAZIN ? 6 : m == VILLAR ? 7 : m == TDE ? 7 : m == ARNETT ? 5 : m == MAGNETAR ? 5 : m == SHOCK ? 5
         : m == AFTERGLOW ? 6 : 5;
}
__host__ __device__ constexpr int se_idx_of(int m) {
    return m == BAZIN ? 5 : m == VILLAR ? 6 : m == TDE ? 6 : m == ARNETT ? 4 : m == MAGNETAR ? 4 : m == SHOCK ? 4
         : m == AFTERGLOW ? 5 : 4;
}
__host__ __device__ constexpr int t0_idx_of(int m) {
    return m == BAZIN ? 2 : m == VILLAR ? 3 : m == TDE ? 2 : m == ARNETT ? 1 : m == MAGNETAR ? 1 : m == SHOCK ? 1
         : m == AFTERGLOW ? 1 : 3;
}

// pso_bounds, src/parametric.rs:1541-1579 (row = model id)
static __device__ __constant__ double c_lo[8][MAXP] = {
    {-3.0, -0.3, -100.0, -2.0, -2.0, -5.0, 0.0},
    {-1.5, -0.02, 1.0, -60.0, -1.0, 1.0, -6.0},
    {-3.0, -1.0, -100.0, -2.0, -1.0, 0.5, -5.0},
    {-3.0, -100.0, 0.5, -3.0, -5.0, 0.0, 0.0},
    {-3.0, -100.0, 0.0, 0.5, -5.0, 0.0, 0.0},
    {-3.0, -100.0, 0.1, -1.0, -5.0, 0.0, 0.0},
    {-3.0, -100.0, -2.0, -2.0, 0.5, -5.0, 0.0},
    {-3.0, -2.0, -1.0, -2.0, -5.0, 0.0, 0.0}};
static __device__ __constant__ double c_hi[8][MAXP] = {
    {3.0, 0.3, 100.0, 5.0, 6.0, 0.0, 0.0},
    {1.5, 0.05, 5.0, 40.0, 3.0, 5.5, 0.0},
    {3.0, 1.0, 100.0, 5.0, 6.0, 4.0, 0.0},
    {3.0, 100.0, 4.5, 3.0, 0.0, 0.0, 0.0},
    {3.0, 100.0, 6.0, 4.5, 0.0, 0.0, 0.0},
    {3.0, 100.0, 3.0, 4.0, 0.0, 0.0, 0.0},
    {3.0, 100.0, 6.0, 3.0, 5.0, 0.0, 0.0},
    {-0.5, -0.5, 2.0, 1.0, 0.0, 0.0, 0.0}};

#define LCF_LN10 2.302585092994045684
// population_priors (center, width), src/parametric.rs:1588-1621
static __device__ __constant__ double c_pop_c[8][MAXP] = {
    {0.0, 0.0, 0.0, 1.5, 3.0, -3.0, 0.0},
    {-0.009 * LCF_LN10, 0.009, 1.327 * LCF_LN10, -12.0, 0.360 * LCF_LN10, 1.454 * LCF_LN10, -1.033 * LCF_LN10},
    {0, 0, 0, 0, 0, 0, 0}, {0, 0, 0, 0, 0, 0, 0}, {0, 0, 0, 0, 0, 0, 0},
    {0, 0, 0, 0, 0, 0, 0}, {0, 0, 0, 0, 0, 0, 0}, {0, 0, 0, 0, 0, 0, 0}};
static __device__ __constant__ double c_pop_w[8][MAXP] = {
    {2.0, 0.2, 30.0, 2.5, 2.5, 2.0, 0.0},
    {0.10 * LCF_LN10, 0.010, 0.40 * LCF_LN10, 15.0, 0.35 * LCF_LN10, 0.40 * LCF_LN10, 0.50 * LCF_LN10},
    {5, 5, 5, 5, 5, 5, 5}, {5, 5, 5, 5, 5, 0, 0}, {5, 5, 5, 5, 5, 0, 0},
    {5, 5, 5, 5, 5, 0, 0}, {5, 5, 5, 5, 5, 5, 0}, {5, 5, 5, 5, 5, 0, 0}};
// 1 / width of the population priors (0 where the width is 0)
static __device__ __constant__ double c_pop_iw[8][MAXP] = {
    {1.0 / 2.0, 1.0 / 0.2, 1.0 / 30.0, 1.0 / 2.5, 1.0 / 2.5, 1.0 / 2.0, 0.0},
    {1.0 / (0.10 * LCF_LN10), 1.0 / 0.010, 1.0 / (0.40 * LCF_LN10), 1.0 / 15.0, 1.0 / (0.35 * LCF_LN10),
     1.0 / (0.40 * LCF_LN10), 1.0 / (0.50 * LCF_LN10)},
    {0.2, 0.2, 0.2, 0.2, 0.2, 0.2, 0.2}, {0.2, 0.2, 0.2, 0.2, 0.2, 0, 0}, {0.2, 0.2, 0.2, 0.2, 0.2, 0, 0},
    {0.2, 0.2, 0.2, 0.2, 0.2, 0, 0}, {0.2, 0.2, 0.2, 0.2, 0.2, 0.2, 0}, {0.2, 0.2, 0.2, 0.2, 0.2, 0, 0}};
// prior_params (center, width), src/parametric.rs:2072-2115
static __device__ __constant__ double c_pri_c[8][MAXP] = {
    {0, 0, 0, 0, 0, 0, 0},
    {0, 0, 0, 0, 0, 0, 0},
    {0, 0, 0, 0, 0, 1.67, 0},
    {0, 0, 2.3, 0, 0, 0, 0},
    {0, 0, 3.0, 2.3, 0, 0, 0},
    {0, 0, 0.5, 1.0, 0, 0, 0},
    {0, 0, 1.0, 0.8, 2.0, 0, 0},
    {-1.75, -1.25, 0.5, -0.5, 0.0, 0, 0}};
static __device__ __constant__ double c_pri_w[8][MAXP] = {
    {2, 2, 2, 2, 2, 2, 0},
    {2, 2, 2, 2, 2, 2, 2},
    {2, 2, 2, 2, 2, 1.0, 2},
    {2, 2, 1.0, 2, 2, 0, 0},
    {2, 2, 1.5, 1.0, 2, 0, 0},
    {2, 2, 1.0, 2.0, 2, 0, 0},
    {2, 2, 2.0, 1.0, 1.0, 2, 0},
    {1.25, 0.75, 1.5, 1.5, 2.0, 0, 0}};
// model order of pso_model_select, src/parametric.rs:2002-2011
static __device__ __constant__ int c_select_order[8] = {BAZIN, ARNETT, TDE, AFTERGLOW, VILLAR, MAGNETAR, SHOCK, METZGER};

// ---------------------------------------------------------------------------
// Device data layout (all arrays in HBM, sized for the batch)
// ---------------------------------------------------------------------------
// One observation of a peak-normalised band, as staged for the FP32 kernels:
//   x = time (FP32 high part), y = time low part (t - x),
//   z = flux / peak for detections, 3*err/peak (the upper limit) for upper
//       limits,
//   w = obs_var = (err/peak)^2 + 1e-10, negated for upper limits.
// Observations are stored sorted by time within each band (16 B each; the
// 16-byte granule is what the TMA bulk copy into shared memory needs).
struct BandStats {
    int64_t off;        // first observation (into the observation arrays)
    int32_t n;          // observations
    int32_t valid;      // 1 if the reference would fit this band
    double peak;        // peak raw flux
    double t_first;     // min time
    double t_last;      // max time
    double t_peak;      // time of the first maximum detection flux (original order)
    double t_peak_all;  // time of the first maximum flux over all observations
    int32_t source;
    int32_t rank;       // position after the by-count sort inside the source
    int32_t joint;      // 1: the band belongs to a source of the joint multi-band fit
    int32_t pad;
};

// A PSO task: one swarm run.
struct PsoTask {
    int32_t band;
    int16_t kind;       // model id, or KIND_MB1 + K - 1
    int8_t restart;     // 0, 1, 2 -> seed 42, 137, 271
    uint8_t flags;      // TASK_*
    int32_t out;        // result slot
    int32_t aux;        // seed-particle slot (MultiBazin seeded restart) or -1
    double t0_fixed;    // profile t0 search: value t0 is held at
};
enum : uint8_t {
    TASK_PRIOR = 1,       // add the population prior
    TASK_T0_BOUNDS = 2,   // data-informed t0 bounds (pso_fit_single_model)
    TASK_SEEDED = 4,      // first particle is a seed particle
    TASK_T0_FIXED = 8,    // t0 removed from the search (profile_t0_search)
    TASK_RANK0 = 16,      // run only if the band is its source's rank-0 band with n >= 5
};

// Result of one PSO run.
struct PsoResult {
    double cost;
    int32_t iters;
    int32_t evals;
    float params[MB_MAXP];
    float params_lo[MB_MAXP];
    float pad[2];
};
// Parameter j of a swarm result.  The exact-trajectory swarms (every swarm
// but MetzgerKN's) store each component as a double-float pair, params[j] +
// params_lo[j], and mark it with pad[0] == 1; MetzgerKN's stores FP32.
__host__ __device__ inline double pso_param(const PsoResult& R, int j) {
    return R.pad[0] == 1.0f ? (double)R.params[j] + (double)R.params_lo[j] : (double)R.params[j];
}

// Result of one joint multi-band swarm run (one source, one restart).
struct JointResult {
    double cost;
    int32_t iters;
    int32_t evals;
    float params[J_MAX_D];     // the best position as double-float pairs,
    float params_lo[J_MAX_D];  // params[j] + params_lo[j]
};

// Per (band, model) polished fit.
struct ModelFit {
    double cost;
    double params[MAXP];
};

// Per band selected fit and final outputs (device side, FP64).
struct BandOut {
    int32_t model;
    int32_t svi_steps;
    double pso_cost;
    double pso_params[MAXP];
    double mu[MAXP];
    double log_sigma[MAXP];
    double elbo;
    double mag_chi2;
    double per_chi2[8];
};

// MultiBazin state per band (only rank-0 bands).
struct MbState {
    int32_t best_k;
    int32_t done;       // early stop reached
    int32_t k_done;     // last K fitted
    int32_t pad;
    double best_cost, best_bic;
    double per_k_cost[LCF_MB_MAX_K];
    double per_k_bic[LCF_MB_MAX_K];
    double best_params[MB_MAXP];
    double prev_params[MB_MAXP];
    double seed[MB_MAXP];
};

// Device counters shared by the kernels of one fit.
struct Counters {
    int32_t task_head[8];       // dynamic work queues (one per PSO launch slot)
    int32_t task_count[8];      // tasks appended by device task builders
    unsigned long long particle_obs_evals;
    unsigned long long ode_steps;
    unsigned long long slot0_evals[12];      // particle x observation evaluations of the first PSO launch, by kind
    unsigned long long slot0_particles[12];  // particle evaluations of the first PSO launch, by kind
    unsigned long long lb_polishes, lb_iters, lb_evals, lb_obs_evals;  // L-BFGS work
    unsigned long long lb_obs_evals_by_model[8];  // observation x (cost + gradient) evaluations, by model
    unsigned long long lb_fp64_obs_evals_by_model[8];  // of which in FP64 (ff range fallback)
    int32_t sort_hist[8][256];  // per slot: key histogram, then offsets, of the device task sort
    int32_t band_hist[16];      // bands by selected model: histogram, then offsets (band_order)
    int32_t polish_hist[256];   // bands by length: histogram, then offsets (polish_order)
    int32_t lb_next[8];         // per model: next index of the polish queue (eight lanes a band)
    int32_t lb_next_long[8];    // per model: next index of its long bands (a warp a band)
    int32_t error;              // first error code raised on the device
    int32_t joint_head;         // next (source, restart) task of the joint multi-band swarm
};

struct DeviceBatch {
    // raw inputs (FP64, caller layout)
    const double* times;
    const double* flux;
    const double* err;
    const int64_t* band_off;
    const int32_t* src_off;
    int n_sources, n_bands;
    int64_t n_obs;
    // prepared
    BandStats* stats;
    float4* obs;            // [n_obs] sorted FP32 records
    double* t64;            // [n_obs] sorted FP64 copies for the FP64 stages
    double* f64;            // flux / peak
    double* fe64;           // err / peak
    double* var64;          // obs_var
    double* uf64;           // upper flux
    double* mag64;          // observed magnitude
    uint8_t* up;            // is_upper
    // the same observations as double-float pairs for the polish (ff.cuh),
    // each band's detections first, then its upper limits (each in time
    // order): ffa = (t hi, t lo, y hi, y lo), y = flux / peak, or the upper
    // flux for an upper limit; ffb = obs_var (hi, lo), negated for upper limits
    float4* ffa;
    float2* ffb;
    // tables
    const float* draws;     // [3][DRAWS_PER_SEED] uniforms of seeds 42, 137, 271
    const double* draws64;  // the same uniforms in FP64 (swarm initialisation)
    const float2* draws15;  // 1.5 x those uniforms (FP64 products) as double-float pairs
    const double* svi_eps;  // [3][SVI_STEPS][SVI_SAMPLES][7] noise for 5, 6, 7 params (FP64, the reference's draws)
    const double* svi_adam_bc;  // [2][SVI_STEPS] Adam's bias corrections 1 / (1 - b1^t), 1 / (1 - b2^t)
    // results
    PsoResult* pso_res;     // per task slot
    ModelFit* fits;         // [n_bands * 8]
    BandOut* out;           // [n_bands]
    MbState* mb;            // [n_bands]
    PsoTask* tasks[8];      // per launch slot
    int task_cap[8];
    PsoTask* task_sorted;   // device-built task lists of slots 1..3 after the sort
    PsoTask* task_sorted_mb;  // the same for slots 4..6 (the MultiBazin branch, which may run concurrently)
    int32_t* band_order;    // [n_bands] bands grouped by selected model (MetzgerKN first), for the
                            // per-band uncertainty and refinement kernels
    int32_t* polish_order;  // [n_bands] bands longest first: the polish's queue order
    int lb_grid;            // blocks of the persistent polish grid
    int lb_n_long;          // bands of LB_LONG_OBS observations or more (the first of polish_order)
    Counters* ctr;
    float* scratch;         // MetzgerKN per-warp scratch: [warps][n_max][32]
    int64_t scratch_per_warp;
    double* scratch64;      // FP64 scratch, 5 values per observation
    float* scratch_svi;     // MetzgerKN SVI scratch, 20 values per observation
    double* t0_state;       // per band: t0_min, t0_max, best t0 of the profile search
    int64_t t0_slot_base;   // first PsoResult slot of the t0 search region
    int64_t mb_slot_base;   // first PsoResult slot of the MultiBazin region
    int smem_obs;           // observations staged per warp in the PSO kernel
    int wait_polls;         // bound of the staging copy's barrier wait, in polls (lcf_set_wait_bound)
    // joint multi-band fit
    const uint8_t* joint_flag;   // per source: 1 if fitted jointly
    const int32_t* joint_src;    // the jointly fitted sources
    int n_joint;
    JointResult* joint_res;      // [n_joint][3]
    const float2* joint_draws15;  // [3][joint_draws_per_seed] 1.5 u of seeds 42, 137, 271 as double-float
    const double* joint_draws64;  // [3][joint_init_per_seed] the first uniforms (initialisation) in FP64
    int64_t joint_draws_per_seed;
    int64_t joint_init_per_seed;
    float* joint_state;          // [joint_grid][JOINT_STATE_ARRAYS][joint_max_d][200] swarm state
    int joint_grid;              // blocks of the persistent joint swarm
    int joint_max_obs;           // most observations of a joint source
    int joint_max_d;             // most joint parameters of a joint source
};

// ---------------------------------------------------------------------------
// Launch wrappers (defined in the .cu files, called by host.cpp)
// ---------------------------------------------------------------------------
// pso.cu
void launch_prep(const DeviceBatch& d, cudaStream_t s);
// Run the PSO tasks of `slot` (count = n_host if >= 0, else the device
// counter of the slot).  `max_dim` selects the kernel instantiation.
// `minb`: the register budget of the 7-dimension swarm (resident 256-thread
// blocks per SM it is built for: 2 or 3); the other swarms are built for 2.
void launch_pso(const DeviceBatch& d, int slot, const PsoTask* tasks, int n_host, int max_dim, int grid, int block,
                cudaStream_t s, int minb = 2);
// Sort the device-built task list of `slot` into `out` (d.task_sorted, or
// d.task_sorted_mb for the MultiBazin branch): MetzgerKN first, then by
// kind, longest bands first within a kind.
void launch_task_sort(const DeviceBatch& d, int slot, PsoTask* out, cudaStream_t s);
size_t pso_smem_bytes(int block, int smem_obs, int max_dim = 7);
int pso_blocks_per_sm(int block, size_t smem, int minb);
int pso_init_attributes(const int* blocks, const int* smem_obs, int n);
int pso_stage_obs(int block, int smem_obs, int max_dim);
void launch_t0_build(const DeviceBatch& d, int slot, int fine, cudaStream_t s);
void launch_t0_pick(const DeviceBatch& d, int slot, int fine, cudaStream_t s);
void launch_gate_build(const DeviceBatch& d, int slot, cudaStream_t s);
void launch_mb_pick(const DeviceBatch& d, int k, cudaStream_t s);
void launch_mb_build(const DeviceBatch& d, int slot, int k, cudaStream_t s);
// polish.cu
void launch_lbfgs(const DeviceBatch& d, int model_mask, cudaStream_t s);
// Bands of at least this many observations are polished by a whole warp.
constexpr int LB_LONG_OBS = 256;
// the polish queue's band order (three launches); before the first launch_lbfgs
void launch_polish_order(const DeviceBatch& d, cudaStream_t s);
// blocks of the persistent polish grid on `num_sms` SMs
int lbfgs_grid(int num_sms);
void launch_select(const DeviceBatch& d, int fit_all, int forced, cudaStream_t s);
void launch_svi(const DeviceBatch& d, cudaStream_t s);
// one SVI step's ELBO estimate and gradient at given variational parameters
// (lcf_svi_elbo_grad); scratch = 5 n floats per point
void launch_svi_grad(int model, const float4* obs, int n, float t_last, const double* init, const double* vpar,
                     int n_points, const double* eps, int n_samples, double* elbo, double* grad, int* flags,
                     float* scratch, cudaStream_t s);
// plain.cu (the plain FP64 form)
void launch_plain_pso(const DeviceBatch& d, int m, int gate, double* mscr, cudaStream_t s);
void launch_plain_lbfgs(const DeviceBatch& d, int m, cudaStream_t s);
void launch_plain_svi(const DeviceBatch& d, int m, double* mscr, cudaStream_t s);
// joint.cu
int launch_joint(const DeviceBatch& d, cudaStream_t s);
size_t joint_smem_bytes(int max_obs, int max_d);
// finalize.cu
void launch_laplace(const DeviceBatch& d, cudaStream_t s);
// bands grouped by selected model into d.band_order (three launches)
void launch_band_order(const DeviceBatch& d, cudaStream_t s);
void launch_refine(const DeviceBatch& d, cudaStream_t s);
double probe_fp32_tflops(int num_sms);
// polish.cu: FP64 peaks: out[m] = observation-term evaluations per second of
// the polish's FP64 cost+gradient term for model m (0..6) at full occupancy,
// out[7] = 0 (MetzgerKN is not polished), out[8] = FP64 TFLOP/s of DFMA chains
int probe_fp64_peaks(int num_sms, double* out9);
int probe_ff(int num_sms, double* out80);
double probe_mufu_gops(int num_sms);
void launch_band_cost(int model, const float4* obs, int n, float t_last, const double* params, int n_eval,
                      int with_prior, double* costs, float* scratch, cudaStream_t s);

// Host-side generation of the RNG tables (host.cpp)
void make_draw_tables(float* draws, double* draws64, float2* draws15, double* svi_eps);
void make_joint_draws(float2* draws15, double* draws64, int64_t per_seed, int64_t init_per_seed);
int joint_grid(int max_obs, int max_d, int num_sms);

}  // namespace lcf
