/*
 * lcf.h — C ABI of the GB300 (sm_103a) parametric light-curve fitting library
 * (liblcf_gb300.so).
 *
 * Two groups of entry points:
 *
 *  1. The fused batch fit.  One call runs, for every band of every source,
 *     what the reference's per-band `fit_parametric_model` does
 *     (src/parametric.rs:3563-3739): PSO model selection over the eight flux
 *     models with three restarts, bounded L-BFGS polish and BIC selection,
 *     then SVI or Laplace uncertainty, the t0 / all-parameter profile
 *     refinements, the magnitude-space chi2 and the MultiBazin fit of the
 *     most populated band.  It replaces the reference's host-driven PSO loop
 *     (src/gpu_cuda.rs:368-637), its GPU SVI driver (src/gpu_cuda.rs:1315-1422)
 *     and the CPU finalisation (src/parametric.rs:3126-3553) with one
 *     device-resident pipeline.
 *
 *  2. Drop-in exports with the exact names and signatures the reference's
 *     Rust host binds (src/gpu_cuda.rs:31-40 and :102-164), and the
 *     semantics of the reference kernels behind them, so that an
 *     unmodified `GpuContext` links against this library instead of the
 *     reference's `liblightcurve_cuda.a` (build.rs:14-18).  They take device
 *     pointers and launch on the legacy default stream, as the reference's do.
 *
 * Conventions of the fused API:
 *   - every function returns an int status: 0 = success, <0 = error code
 *     (LCF_E_*); the message is available from lcf_last_error();
 *   - inputs and outputs are caller-owned host arrays in FP64 (the reference's
 *     arithmetic type) unless stated otherwise;
 *   - one context per host thread; a context owns its stream, its device
 *     buffers and its captured CUDA graph.
 *
 * Model ids follow the reference (src/gpu_types.rs:51-62,
 * src/parametric.rs:3279-3288): 0 Bazin, 1 Villar, 2 Tde, 3 Arnett,
 * 4 Magnetar, 5 ShockCooling, 6 Afterglow, 7 MetzgerKN.
 */
#ifndef LCF_H
#define LCF_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LCF_N_MODELS 8
#define LCF_MAX_PARAMS 7          /* Villar / Tde */
#define LCF_MB_MAX_K 4            /* MULTI_BAZIN_MAX_K, src/parametric.rs:915 */
#define LCF_MB_MAX_PARAMS 18      /* 4*K + 2 at K = 4 */

/* status codes */
#define LCF_OK 0
#define LCF_E_INVALID (-1)        /* bad argument (sizes, offsets, options) */
#define LCF_E_CUDA (-2)           /* a CUDA runtime call failed */
#define LCF_E_NOMEM (-3)          /* device or pinned allocation failed */
#define LCF_E_TIMEOUT (-4)        /* a bounded device wait expired */
#define LCF_E_UNSUPPORTED (-5)    /* option combination not built */
#define LCF_E_CAPACITY (-6)       /* a size beyond a fixed capacity (lcf_band_cost_static) */

/* UncertaintyMethod, src/parametric.rs:13-21 */
#define LCF_METHOD_SVI 0
#define LCF_METHOD_LAPLACE 1

/*
 * Batch of sources in CSR form.  Source s owns bands
 * [source_band_offsets[s], source_band_offsets[s+1]); band b owns
 * observations [band_obs_offsets[b], band_obs_offsets[b+1]).  `times`,
 * `flux` and `flux_err` are one band's `BandData{times, values, errors}`
 * (src/common.rs:11-15) concatenated: times relative to the source's first
 * observation, flux and errors in linear flux units.  Band order within a
 * source is the caller's; the fit ranks bands by observation count,
 * descending, with ties kept in caller order (the reference sorts a HashMap's
 * iteration order, src/parametric.rs:3632).
 */
typedef struct lcf_bands_csr {
    int32_t n_sources;
    int32_t n_bands;
    const int32_t* source_band_offsets; /* [n_sources + 1] */
    const int64_t* band_obs_offsets;    /* [n_bands + 1]   */
    const double* times;                /* [n_obs] */
    const double* flux;                 /* [n_obs] */
    const double* flux_err;             /* [n_obs] */
} lcf_bands_csr;

typedef struct lcf_fit_options {
    int32_t fit_all_models;   /* fit_parametric_model(.., fit_all_models, ..) */
    int32_t method;           /* LCF_METHOD_SVI or LCF_METHOD_LAPLACE */
    int32_t forced_model;     /* -1: model selection; else the model id */
    int32_t run_multi_bazin;  /* 1: fit MultiBazin on each source's rank-0 band (reference behaviour) */
    int32_t joint_multiband;  /* 1: fit_parametric's dispatch (src/parametric.rs:3742-3761): with
                               * fit_all_models == 0 and forced_model == -1, a source with >= 2 non-empty
                               * bands gets the joint multi-band Villar fit (fit_parametric_multiband,
                               * :3763-4131); 0: fit_parametric_model for every source */
} lcf_fit_options;

/*
 * Per-band outputs (caller-allocated, indexed by the caller's band index b).
 * A band the reference would skip (no data, or peak flux <= 0) has
 * model[b] = -1 and rank[b] = -1.  Parameter rows are padded to
 * LCF_MAX_PARAMS with NaN.  NaN stands for the reference's `None`
 * (`finite_or_none`, src/common.rs:463).
 */
typedef struct lcf_fit_outputs {
    int32_t* model;             /* [n_bands] selected model id */
    int32_t* rank;              /* [n_bands] position after the by-count sort */
    int32_t* n_obs;             /* [n_bands] */
    double* pso_params;         /* [n_bands * 7] */
    double* pso_chi2;           /* [n_bands] */
    double* svi_mu;             /* [n_bands * 7] */
    double* svi_log_sigma;      /* [n_bands * 7] */
    double* svi_elbo;           /* [n_bands] */
    double* mag_chi2;           /* [n_bands] */
    double* per_model_chi2;     /* [n_bands * 8], by model id; NaN = None or not fitted */
    double* per_model_params;   /* [n_bands * 8 * 7]; filled when fit_all_models */
    int32_t* mb_best_k;         /* [n_bands]; 0 = no MultiBazin result */
    double* mb_params;          /* [n_bands * 18] */
    double* mb_cost;            /* [n_bands] */
    double* mb_bic;             /* [n_bands] */
    double* mb_per_k_cost;      /* [n_bands * 4] */
    double* mb_per_k_bic;       /* [n_bands * 4] */
} lcf_fit_outputs;

/* Timing and work counters of the last fit, filled by lcf_last_stats(). */
typedef struct lcf_fit_stats {
    double ms_total;            /* device time of the whole pipeline (CUDA events) */
    double ms_pso;              /* model-selection PSO launch */
    double ms_lbfgs;            /* restart reduce + L-BFGS polish + BIC select */
    double ms_t0_search;        /* SVI-mode profile t0 search (two PSO launches) */
    double ms_uncertainty;      /* SVI or Laplace */
    double ms_refine;           /* profile refinements + mag chi2 */
    double ms_multi_bazin;      /* MultiBazin K = 2..4 launches (on their own stream when branched) */
    double particle_obs_evals;  /* device-counted particle x observation evaluations in PSO launches */
    double ode_steps;           /* device-counted MetzgerKN Euler steps in PSO launches */
    int64_t pso_tasks;          /* PSO runs executed */
    int64_t kernel_launches;    /* kernels launched by the last fit */
    double h2d_bytes;           /* host -> device bytes moved by the last lcf_fit_parametric_batch */
    double d2h_bytes;           /* device -> host bytes moved by the last output download */
    double pso0_evals_by_kind[12];      /* particle x observation evaluations of the model-selection PSO launch, by task kind */
    double pso0_particles_by_kind[12];  /* particle evaluations of that launch, by task kind (kinds 8..11: MultiBazin K = 1..4) */
    double lbfgs_polishes;      /* L-BFGS polishes run (one per band and polished model) */
    double lbfgs_iters;         /* their L-BFGS iterations */
    double lbfgs_evals;         /* their cost + gradient evaluations */
    double lbfgs_obs_evals;     /* observation x (cost + gradient) evaluations */
    double lbfgs_obs_evals_by_model[8];  /* the same, by model (MetzgerKN: 0, not polished) */
    double ms_joint;            /* joint multi-band swarm + pick (fit_parametric's multi-band branch) */
    double lbfgs_fp64_obs_evals_by_model[8];  /* polish observation terms evaluated in FP64 (range fallback) */
} lcf_fit_stats;

typedef struct lcf_ctx lcf_ctx;

/* Context management.  The context binds `device` and creates its stream. */
int lcf_ctx_create(int device, lcf_ctx** out);
void lcf_ctx_destroy(lcf_ctx* ctx);
const char* lcf_last_error(const lcf_ctx* ctx);  /* never NULL */
int lcf_last_stats(const lcf_ctx* ctx, lcf_fit_stats* out);

/*
 * Fused batch fit of host-resident data: copies the CSR into pinned staging,
 * then to the device, runs the pipeline and copies the outputs back.
 * Replaces, per band, fit_parametric_model(bands, fit_all_models, method,
 * forced_model) (src/parametric.rs:3563-3739).
 */
int lcf_fit_parametric_batch(lcf_ctx* ctx, const lcf_bands_csr* bands,
                             const lcf_fit_options* opts, lcf_fit_outputs* out);

/*
 * Asynchronous form of lcf_fit_parametric_batch: the inputs are copied into
 * the context's pinned staging before the call returns (the caller may reuse
 * them), the pipeline and the output copies are queued on the context's
 * stream, and the call returns without waiting.  The outputs are written
 * into `out`'s arrays, which must stay valid, by lcf_wait().  Until then
 * every other call that queues work on the context returns LCF_E_INVALID.
 * The reference's GpuContext calls are synchronous; this is the boundary's
 * async variant.
 */
int lcf_fit_parametric_batch_async(lcf_ctx* ctx, const lcf_bands_csr* bands,
                                   const lcf_fit_options* opts, lcf_fit_outputs* out);

/*
 * Waits up to timeout_ms milliseconds (< 0: without limit) for the pending
 * asynchronous fit.  Returns LCF_OK once it has finished and its outputs and
 * statistics are written; LCF_E_TIMEOUT while it is still running (it stays
 * pending: call again); the fit's own error otherwise.  With no fit pending
 * it returns LCF_OK at once.  lcf_fit_parametric_batch is the asynchronous
 * call followed by lcf_wait(ctx, -1).
 */
int lcf_wait(lcf_ctx* ctx, int timeout_ms);

/*
 * Same pipeline on data that is already resident on the device: the three
 * observation arrays and two offset arrays are device pointers, the outputs
 * stay on the device in the context's buffers.  Used to time the kernels
 * without host transfers; lcf_download_outputs() copies them out.
 */
int lcf_fit_parametric_device(lcf_ctx* ctx, const lcf_bands_csr* dev_bands,
                              const lcf_fit_options* opts);
int lcf_download_outputs(lcf_ctx* ctx, lcf_fit_outputs* out);

/*
 * Selected swarm results supplied by the caller, one row per CSR band: the
 * fields of the reference's GpuPsoBandResult (src/parametric.rs:3101-3114)
 * that the finalisation reads, and optionally uncertainty outputs computed
 * elsewhere (the reference's GPU SVI, src/gpu_cuda.rs:1315-1422).
 *   model:          [n_bands] model id 0..7, or -1 to skip the band
 *                   (an empty pso_params in the reference)
 *   pso_params:     [n_bands * 7], the first n_params(model) are read
 *   pso_cost:       [n_bands] or NULL (NaN), copied to pso_chi2
 *   per_model_chi2: [n_bands * 8] or NULL (NaN), copied through
 *   svi_mu, svi_log_sigma: [n_bands * 7] or NULL; svi_elbo: [n_bands] or
 *                   NULL.  With svi_mu and svi_log_sigma given the
 *                   uncertainty stage is not run (the *_with_gpu_svi forms).
 */
typedef struct lcf_pso_selection {
    const int32_t* model;
    const double* pso_params;
    const double* pso_cost;
    const double* per_model_chi2;
    const double* svi_mu;
    const double* svi_log_sigma;
    const double* svi_elbo;
} lcf_pso_selection;

/*
 * Batched finalisation of externally selected fits on the GPU, per band:
 *   finalize_parametric_from_gpu (src/parametric.rs:3126-3257): SVI from
 *     pso_params (1000 steps, 4 samples, lr 0.01) or Laplace at pso_params
 *     (`method`), then profile_t0_refine, profile_refine_all and the
 *     magnitude chi2;
 *   finalize_parametric_with_gpu_svi (:3298-3421) and
 *   finalize_all_models_with_gpu_svi (:3429-3553): the same from the
 *     supplied svi_mu / svi_log_sigma / svi_elbo, without the uncertainty
 *     stage (`method` is then ignored).
 * The band preparation is fit_parametric_model's (:3581-3632); a band it
 * skips gets model -1.  Outputs as lcf_fit_parametric_batch's; rank is the
 * band's position in the by-count order, per_model_params and MultiBazin
 * come back NaN / 0 (the caller holds its own).  A (band, model) pair list,
 * as finalize_all_models_with_gpu_svi takes, is a CSR with the band repeated.
 */
int lcf_finalize_batch(lcf_ctx* ctx, const lcf_bands_csr* bands, const lcf_pso_selection* sel,
                       int method, lcf_fit_outputs* out);

/*
 * The plain FP64 GPU form of the same fit, the baseline the fused pipeline is
 * measured against: PSO model selection (one thread per particle, FP64,
 * observations from global memory, synchronous global best), L-BFGS polish,
 * BIC selection and SVI, one kernel launch per model per stage and no CUDA
 * graph.  It omits the profile t0 search, the refinements, the magnitude chi2
 * and MultiBazin (those outputs come back NaN / 0).  SVI only
 * (LCF_E_UNSUPPORTED for Laplace).  Device pointers as in
 * lcf_fit_parametric_device; outputs via lcf_download_outputs.  It is the
 * straightforward rendering of the reference's CPU algorithm on the GPU
 * (src/parametric.rs:1646-2066, 2215-2454, driven the way the reference's
 * GPU host drives its per-particle kernels, src/gpu_cuda.rs:368-567).
 */
int lcf_fit_plain_device(lcf_ctx* ctx, const lcf_bands_csr* dev_bands,
                         const lcf_fit_options* opts);

/* The context's CUDA stream (a cudaStream_t), for callers that time with events. */
void* lcf_ctx_stream(lcf_ctx* ctx);

/* Replay the stage sequence from a CUDA graph captured per batch layout
 * (default 1), or launch the kernels one by one (0). */
int lcf_set_graph(lcf_ctx* ctx, int enabled);

/* Bound of the swarm kernel's one device wait (the barrier of the TMA bulk
 * copy that stages a band in shared memory), in polls; default 2^24, 0 makes
 * every staged band's wait expire at once.  No counterpart in the reference,
 * whose swarms run on the host.  On expiry a warp records LCF_E_TIMEOUT, lets
 * the copy it issued land (a second wait, bounded at 2^24 polls) and takes no
 * further tasks; the fit returns LCF_E_TIMEOUT and the context stays usable.
 * For tests of that path; a fit never needs it otherwise. */
int lcf_set_wait_bound(lcf_ctx* ctx, int polls);

/* Stage concurrency: MultiBazin K = 2..4 (fit_multi_bazin's greedy loop)
 * depends only on the band preparation and its K = 1 swarms, so the fit can
 * run it on a second stream beside the later stages.  mode 0: the stages
 * run in sequence; 1 (default): the branch forks after the model-selection
 * swarm launch and runs beside the polish; 2: it forks after the polish and
 * BIC selection.  The results are the same under every mode. */
int lcf_set_multi_bazin_branch(lcf_ctx* ctx, int mode);

/*
 * Launch autotuner of the swarm kernel (no counterpart in the reference,
 * whose CPU swarms have no launch shape).  Candidate c has a block size and
 * a staging depth (observations a warp stages in shared memory; longer bands
 * are read from global memory); every candidate gives bit-identical results.
 * A context tunes online per shape bucket of the batch (ceil log2 of the
 * band count, and of the 90th-percentile band length / 32): the first fits
 * of a new bucket run the candidates in turn, timed by their swarm stages,
 * and later fits of the bucket use the fastest.
 *   lcf_set_autotune: mode 1 = online tuning (default), 0 = candidate 0;
 *       forced_candidate >= 0 pins that candidate (-1: none).
 *   lcf_autotune_candidates: out[3c..3c+2] = block, staging depth, resident
 *       blocks per SM of candidate c; returns the number of candidates.
 *   lcf_autotune_table: per bucket seen, 6 doubles (bucket, chosen candidate
 *       or -1 while exploring, next candidate to explore, stage ms of each
 *       candidate); returns the number of buckets (rows beyond max_rows are
 *       not written).
 *   lcf_autotune_load: installs rows of that form as explored buckets (the
 *       table of an earlier context, to skip exploration).
 *   lcf_last_launch: out = candidate, block, staging depth, bucket of the
 *       last fused fit.
 */
int lcf_set_autotune(lcf_ctx* ctx, int mode, int forced_candidate);
int lcf_autotune_candidates(const lcf_ctx* ctx, int* out9);
int lcf_autotune_table(const lcf_ctx* ctx, double* rows, int max_rows);
int lcf_autotune_load(lcf_ctx* ctx, const double* rows, int n_rows);
int lcf_last_launch(const lcf_ctx* ctx, int* out4);

/* Measured pipe peaks of the context's GPU: out[0] = FP32 FMA TFLOP/s,
 * out[1] = SFU (MUFU ex2) Gop/s, from dependent-chain probe kernels over a
 * full grid.  The roofline denominators of the fused kernels, which are
 * bound by these two pipes rather than by HBM or the tensor cores. */
int lcf_probe_peaks(lcf_ctx* ctx, double* out2);

/* FP64 ceilings of the L-BFGS polish, which is bound by the FP64 pipe:
 * out[m] (m = 0..6) = evaluations per second of the polish's own FP64
 * observation term (value, gradient and cost of one observation of model m)
 * streamed at full occupancy over a resident band; out[7] = 0 (MetzgerKN is
 * not polished); out[8] = FP64 TFLOP/s of independent DFMA chains. */
int lcf_probe_fp64(lcf_ctx* ctx, double* out9);

/* The polish's double-float observation term (its arithmetic wherever the
 * exponents stay inside FP32's range): out[m] (m = 0..6) = its evaluations
 * per second, streamed as lcf_probe_fp64 streams the FP64 term; out[7 + m] =
 * the largest disagreement with the FP64 term over 256 parameter points of
 * model m inside the PSO box (|ff - FP64| / sum of the terms' magnitudes,
 * floored for a gradient component at 1e-10 of the whole gradient's, over the
 * cost and the gradient components; gradients over the detections);
 * out[14 + 8 m + c] = the same per component (c = 0: cost, 1 + k: gradient
 * component k); out[70 + m] = the
 * points of the 256 that the range check keeps in double-float; out[77] =
 * points where exactly one of the two terms was non-finite. */
int lcf_probe_ff(lcf_ctx* ctx, double* out80);

/* Diagnostic: raw swarm results of the last fit, 21 doubles per result slot
 * (cost, iterations, particle evaluations, 18 parameters; the swarms of the
 * models other than MetzgerKN report their best position at double-float
 * precision and, in model selection, an FP32 estimate of its cost).  Slots
 * [0, 24 n_bands) hold (band * 8 + model) * 3 + restart of the model
 * selection, [24 n_bands, 32 n_bands) the profile-t0 runs, [32 n_bands,
 * 44 n_bands) the MultiBazin runs.  A slot that did not run has cost NaN. */
int lcf_debug_swarm_results(lcf_ctx* ctx, double* out, int64_t max_rows);

/*
 * Batched likelihood: cost of `n_eval` parameter vectors of one model on one
 * band, exactly PsoCost::cost_from_slice (src/parametric.rs:1303-1370):
 * per-observation Gaussian / upper-limit negative log-likelihood over the
 * band, divided by n, plus the population prior / n^2 when with_prior != 0.
 * The band arrays are host FP64 (already peak-normalised, as BandFitData);
 * evaluation runs in the fused kernel's FP32 arithmetic.  `params` is
 * [n_eval * n_params(model)].
 */
int lcf_band_cost(lcf_ctx* ctx, int model, const double* times, const double* flux,
                  const double* obs_var, const uint8_t* is_upper, const double* upper_flux,
                  int n_obs, const double* params, int n_eval, int with_prior,
                  double* costs);

/*
 * SVI ELBO gradient at given variational parameters: for each of `n_points`
 * points, the Monte-Carlo ELBO estimate of one SVI step and its gradient,
 * as svi_fit forms them (src/parametric.rs:2262-2393; the reference GPU
 * kernel's per-step gradient, cuda/svi.cu, bound at src/gpu_cuda.rs:139-164):
 * for each draw eps_s, theta = mu + exp(log_sigma) * eps_s; the log-likelihood
 * of theta over the band and its gradient by the adjoint through the analytic
 * model gradient (MetzgerKN: forward-mode duals through the ODE); the Gaussian
 * prior centred on `prior_init` (the PSO parameters; sigma_extra has its
 * fixed centre); the sample mean, plus the entropy sum(log_sigma) +
 * np/2 ln(2 pi e).  The arithmetic is the SVI kernel's own (FP32 likelihood
 * and adjoint, FP64 bookkeeping).
 *   band: host FP64, peak-normalised, as lcf_band_cost;
 *   prior_init [np]; var_params [n_points][2 np] = (mu, log_sigma);
 *   eps [n_points][n_samples][np] standard-normal draws;
 *   elbo [n_points]; grad [n_points][2 np] = (d/d mu, d/d log_sigma);
 *   flags [n_points]: bit 0 = an upper-limit CDF underflowed (the reference's
 *   gradient is ~1e285 there and its Adam freezes), bit 1 = a MetzgerKN sample
 *   was skipped by the reference's peak-rescale rule.
 */
int lcf_svi_elbo_grad(lcf_ctx* ctx, int model, const double* times, const double* flux,
                      const double* obs_var, const uint8_t* is_upper, const double* upper_flux, int n_obs,
                      const double* prior_init, const double* var_params, int n_points,
                      const double* eps, int n_samples, double* elbo, double* grad, int* flags);

/*
 * Allocation-free variant of lcf_band_cost, for callers that cannot call
 * cudaMalloc: a host framework that owns all device memory through its own
 * pool or budget, or an embedding where the library must not allocate GPU
 * memory of its own.  No counterpart in the reference.
 *
 * All array arguments are device pointers supplied by the caller (the band
 * as in lcf_band_cost, params [n_eval * n_params(model)], costs [n_eval]);
 * the work is enqueued on `stream` (a cudaStream_t of `device`, NULL = the
 * legacy default stream) and the call returns without synchronising.  The
 * library's scratch for it is a fixed static device array, so the call
 * allocates nothing (no cudaMalloc, cudaFree or allocating library routine)
 * and accepts at most 2048 observations and 512 parameter vectors per call
 * (LCF_E_CAPACITY beyond that).  The array's device address is looked up
 * with cudaGetSymbolAddress on the first call on each device: make that
 * first call before any stream capture.  Every call on a device shares the
 * array and leaves its contents behind; each call writes everything it reads,
 * and calls that overlap on the GPU race.
 */
int lcf_band_cost_static(int device, int model, const double* times, const double* flux,
                         const double* obs_var, const uint8_t* is_upper, const double* upper_flux,
                         int n_obs, const double* params, int n_eval, int with_prior, double* costs,
                         void* stream);

/* ---------------------------------------------------------------------------
 * Reference drop-in exports (device pointers, default stream, void return;
 * errors surface through cudaGetLastError as in the reference).
 * ------------------------------------------------------------------------- */

/* cuda/models.cu launch_* eval wrappers, bound at src/gpu_cuda.rs:31-40:
 * out[d * n_times + t] = model(params[d * n_params ..], times[t]), FP64. */
void launch_bazin(const double* p, const double* t, double* o, int nd, int nt, int np, int grid, int block);
void launch_villar(const double* p, const double* t, double* o, int nd, int nt, int np, int grid, int block);
void launch_tde(const double* p, const double* t, double* o, int nd, int nt, int np, int grid, int block);
void launch_arnett(const double* p, const double* t, double* o, int nd, int nt, int np, int grid, int block);
void launch_magnetar(const double* p, const double* t, double* o, int nd, int nt, int np, int grid, int block);
void launch_shock_cooling(const double* p, const double* t, double* o, int nd, int nt, int np, int grid, int block);
void launch_afterglow(const double* p, const double* t, double* o, int nd, int nt, int np, int grid, int block);
/* MetzgerKN over the whole times array per draw, as metzger_kn_eval_batch
 * (src/parametric.rs:544-648). */
void launch_metzger_kn(const double* p, const double* t, double* o, int nd, int nt, int np, int grid, int block);

/* launch_batch_pso_cost, bound at src/gpu_cuda.rs:102-118 (kernel
 * cuda/models.cu:516-584): costs[s * n_particles + k] = sum over the
 * source's observations of (pred - y)^2 / v + ln v (detections) or
 * -ln Phi((u - pred) / sqrt v) (upper limits), v = obs_var + sigma_extra^2,
 * divided by n, for positions [s][k][n_params]; sigma_extra is the last
 * parameter; 1e99 for a source with no observations or a non-finite
 * prediction.  As in the reference kernel (and unlike the CPU path's PsoCost)
 * there is no prior, no Villar constraint and no MetzgerKN peak rescale, and
 * MetzgerKN (model 7) is evaluated per observation on its own 100-point ODE
 * grid (cuda/models_device.h:376-456).  `grid` and `block` are accepted and
 * ignored (the launch shape is this library's). */
void launch_batch_pso_cost(const double* all_times, const double* all_flux,
                           const double* all_obs_var, const int* all_is_upper,
                           const double* all_upper_flux, const int* source_offsets,
                           const double* positions, double* costs, int n_sources,
                           int n_particles, int n_params, int model_id, int grid, int block);

/* launch_batch_pso_cost_multi_bazin, bound at src/gpu_cuda.rs:120-135
 * (kernel cuda/models.cu:318-362): the same cost for MultiBazin, the sum of
 * K = source_k[s] Bazin components (log A, t0, log tau_rise, log tau_fall
 * each) plus the baseline B (position 4K) and log sigma_extra (4K + 1);
 * rows padded to n_params = 4 max_K + 2. */
void launch_batch_pso_cost_multi_bazin(const double* all_times, const double* all_flux,
                                       const double* all_obs_var, const int* all_is_upper,
                                       const double* all_upper_flux, const int* source_offsets,
                                       const double* positions, double* costs, const int* source_k,
                                       int n_sources, int n_particles, int n_params, int grid, int block);

/* launch_batch_svi_fit, bound at src/gpu_cuda.rs:139-164 (kernel
 * cuda/svi.cu:48-367): the reference GPU's SVI of each source from
 * pso_params [n_sources * max_params], with model_ids, n_params_arr and
 * se_idx_arr per source and Gaussian priors prior_centers / prior_widths
 * [n_sources * max_params]; outputs out_mu, out_log_sigma
 * [n_sources * max_params] (padded with 0) and out_elbo [n_sources].  Its
 * semantics are that kernel's, not the CPU path's svi_fit: noise from
 * xorshift64 seeded 42 + source * 123456789, MetzgerKN per observation with a
 * forward-difference gradient, early stop after >= 50 steps on a 20-step
 * stall, log sigma reported without the ln 4 inflation; a source without
 * observations gets out_elbo = -1e99 and nothing else. */
void launch_batch_svi_fit(const double* all_times, const double* all_flux,
                          const double* all_obs_var, const int* all_is_upper,
                          const double* all_upper_flux, const int* source_offsets,
                          const double* pso_params, const int* model_ids, const int* n_params_arr,
                          const int* se_idx_arr, const double* prior_centers, const double* prior_widths,
                          double* out_mu, double* out_log_sigma, double* out_elbo, int n_sources,
                          int max_params, int n_steps, int n_samples, double lr, int grid, int block);

#ifdef __cplusplus
}
#endif

#endif /* LCF_H */
