// host.cu — context, device memory, the stage sequence of the fused fit,
// CUDA-graph capture, and the C ABI of include/lcf.h.
//
// Stage sequence of one fit (all on the context's stream, captured once per
// batch layout into a CUDA graph and replayed):
//   prep          normalise bands, FP32 records, stats, rank inside source
//   pso[0]        3 restarts x 8 models per band + MultiBazin K = 1
//   lbfgs         best restart + bounded L-BFGS per (band, model)
//   select        BIC model selection
//   (gate)        fit_all_models == false: Bazin first, the 7 others only
//                 for bands whose Bazin cost is >= 2 (device-built tasks)
//   t0 search     SVI mode, rank-0 bands: 5 coarse + 3 fine PSO runs
//   svi | laplace
//   refine        profile t0 + all-parameter refinement + mag chi2
//   MultiBazin    K = 2, 3, 4 (device-built tasks, early stop)
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <chrono>
#include <string>
#include <thread>
#include <vector>

#include "lcf.h"
#include "lcf_internal.cuh"

using namespace lcf;

namespace lcf {

// xoshiro256++ seeded by SplitMix64 (rand 0.9 SmallRng::seed_from_u64)
struct Xoshiro {
    uint64_t s[4];
    explicit Xoshiro(uint64_t seed) {
        uint64_t st = seed;
        for (int i = 0; i < 4; i++) {
            st += 0x9e3779b97f4a7c15ULL;
            uint64_t z = st;
            z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
            z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
            s[i] = z ^ (z >> 31);
        }
    }
    static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
    uint64_t next() {
        uint64_t r = rotl(s[0] + s[3], 23) + s[0];
        uint64_t t = s[1] << 17;
        s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3]; s[2] ^= t;
        s[3] = rotl(s[3], 45);
        return r;
    }
    double f64() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
};

void make_draw_tables(float* draws, double* draws64, float2* draws15, double* svi_eps) {
    const uint64_t seeds[3] = {42, 137, 271};
    for (int k = 0; k < 3; k++) {
        Xoshiro r(seeds[k]);
        for (int i = 0; i < DRAWS_PER_SEED; i++) {
            const size_t q = (size_t)k * DRAWS_PER_SEED + i;
            const double u = r.f64();
            draws[q] = (float)u;
            draws64[q] = u;
            // c1 * r and c2 * r of the velocity update (c1 = c2 = 1.5), the
            // FP64 product as a double-float pair
            const double cu = 1.5 * u;
            const float hi = (float)cu;
            draws15[q] = make_float2(hi, (float)(cu - (double)hi));
        }
    }
    // svi_fit, src/parametric.rs:2282-2288: SmallRng(42); per step, sample
    // and parameter: u1 = max(U, 1e-10), u2 = U, eps = sqrt(-2 ln u1) cos(2 pi u2)
    for (int np = 5; np <= 7; np++) {
        Xoshiro r(42);
        double* tab = svi_eps + (size_t)(np - 5) * SVI_STEPS * SVI_SAMPLES * 7;
        for (int s = 0; s < SVI_STEPS; s++)
            for (int k = 0; k < SVI_SAMPLES; k++)
                for (int j = 0; j < 7; j++) {
                    double v = 0.0;
                    if (j < np) {
                        double u1 = std::fmax(r.f64(), 1e-10);
                        double u2 = r.f64();
                        v = std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * 3.14159265358979323846 * u2);
                    }
                    tab[((size_t)s * SVI_SAMPLES + k) * 7 + j] = v;
                }
    }
}

// The same three streams, longer: the joint multi-band swarm (200 particles,
// up to 42 dimensions, 1500 iterations) draws up to ~25 M uniforms per seed.
// Its exact-trajectory swarm reads each draw as the FP64 product 1.5 u in a
// double-float pair, and the first init_per_seed draws (the initialisation)
// as FP64 uniforms.
void make_joint_draws(float2* draws15, double* draws64, int64_t per_seed, int64_t init_per_seed) {
    const uint64_t seeds[3] = {42, 137, 271};
    for (int k = 0; k < 3; k++) {
        Xoshiro r(seeds[k]);
        float2* out = draws15 + (size_t)k * per_seed;
        double* init = draws64 + (size_t)k * init_per_seed;
        for (int64_t i = 0; i < per_seed; i++) {
            const double u = r.f64();
            if (i < init_per_seed) init[i] = u;
            const double cu = 1.5 * u;
            const float hi = (float)cu;
            out[i] = make_float2(hi, (float)(cu - (double)hi));
        }
    }
}

}  // namespace lcf

// ---------------------------------------------------------------------------
// Context
// ---------------------------------------------------------------------------
enum { N_EVENTS = 11 };

struct DevArr {
    void* p = nullptr;
    size_t bytes = 0;
};

// ---------------------------------------------------------------------------
// Launch autotuner.  The swarm kernel's launch shape (threads per block, and
// with it the resident blocks per SM) and its staging depth (observations a
// warp stages in shared memory; longer bands are read from global memory)
// are chosen per shape bucket of the batch: log2 of the band count and of
// the 90th-percentile band length.  A context tunes online: the first fits of
// a new bucket run the candidates in turn, each timed by the stage events of
// the fit (model-selection swarm + t0 search + MultiBazin), and later fits of
// that bucket use the fastest.  The candidates change only where a warp reads
// its band from and which warp runs which swarm, so every candidate gives
// bit-identical results and an exploring fit is ordinary work.
// ---------------------------------------------------------------------------
struct TuneCand {
    int block, smem_obs;
    int minb;  // register budget of the model-selection swarm (blocks per SM)
};
// (256, 512, 2): 16 warps per SM, bands <= 512 staged (the default);
// (256, 256, 3): a shallower stage, and the model-selection swarm at 24 warps
//   per SM on the three-block register budget (the later swarms, fewer and
//   longer tasks, keep the two-block build);
// (128, 1024, 2): bands <= 1024 staged at 12 warps per SM (long-band batches)
static const TuneCand TUNE_CAND[] = {{256, 512, 2}, {256, 256, 3}, {128, 1024, 2}};
constexpr int N_TUNE = 3;
struct TuneEntry {
    uint32_t bucket = 0;
    int next = 0;     // next candidate to explore (N_TUNE: done)
    int best = -1;    // chosen candidate once explored
    double ms[N_TUNE] = {0.0, 0.0, 0.0};
};

struct lcf_ctx {
    int device = 0;
    int num_sms = 0;
    int pso_block = 256;
    int pso_blocks_per_sm = 1;   // the model-selection swarm's
    int pso_rest_per_sm = 1;     // the t0-search, gate and MultiBazin swarms'
    int pso_minb = 2;
    int smem_obs = 512;
    // autotuner state
    int tune_mode = 1;       // 1: online tuning per shape bucket, 0: candidate 0
    int tune_forced = -1;    // >= 0: always this candidate
    int cand_bps[N_TUNE] = {1, 1, 1};       // blocks per SM, model-selection swarm
    int cand_bps_rest[N_TUNE] = {1, 1, 1};  // blocks per SM, the other swarms
    int max_pso_warps_per_sm = 1;
    int lb_grid = 1;          // blocks of the persistent polish grid
    int lb_n_long = 0;        // bands polished by a whole warp (LB_LONG_OBS observations or more)
    int cfg = 0;             // candidate of the current fit
    bool exploring = false;
    uint32_t bucket = 0;
    std::vector<TuneEntry> tune;
    cudaStream_t stream = nullptr;
    // MultiBazin K = 2..4 branch: its own stream, forked from and joined to
    // the main stage sequence (mb_branch: 0 = no branch, the stages run in
    // sequence; 1 = fork after the model-selection swarm launch; 2 = fork
    // after the polish and BIC selection)
    cudaStream_t stream_mb = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    int mb_branch = 1;
    bool mb_timed = false;   // the last enqueued sequence recorded ev[9], ev[10]
    bool mb_branched = false;  // ... and ran MultiBazin on its branch
    std::string err;
    lcf_fit_stats stats{};
    cudaEvent_t ev[N_EVENTS]{};
    // tables
    float* d_draws = nullptr;
    double* d_draws64 = nullptr;
    float2* d_draws15 = nullptr;
    double* d_eps = nullptr;
    // device buffers (capacity-sized)
    DevArr times, flux, ferr, boff, soff, stats_b, obs, t64, f64, fe64, var64, uf64, mag64, up, ffa, ffb, res, fits, out, mb,
        ctr, scratch, scratch64, scratch_svi, t0state, tasks[7], task_sorted, task_sorted_mb, band_order, polish_order, joint_flag, joint_src,
        joint_res, joint_draws15, joint_draws64, joint_state;
    int64_t joint_per_seed = 0;   // draws per seed held in joint_draws15
    int64_t joint_init_per_seed = 0;
    int joint_grid = 0;
    int n_joint = 0, joint_max_obs = 0, joint_max_d = 0;
    int64_t task_cap[7] = {0, 0, 0, 0, 0, 0, 0};
    // pinned staging
    DevArr h_in, h_out, h_sel, h_ctr;
    // lcf_fit_parametric_batch_async: the fit waiting for lcf_wait()
    bool pending = false;
    lcf_fit_outputs pending_out{};
    size_t pending_in_bytes = 0;
    cudaEvent_t ev_done = nullptr;
    // band-cost scratch
    DevArr bc_obs, bc_params, bc_costs, bc_scratch;
    // ELBO-gradient check buffers
    DevArr sg_in, sg_out, sg_scratch;
    // plain FP64 form: MetzgerKN prediction rows (96 per observation)
    DevArr plain_scr;
    // layout cache
    std::vector<int64_t> h_boff;
    std::vector<int32_t> h_soff;
    std::vector<PsoTask> h_tasks0;
    uint64_t layout_key = 0;
    int n_tasks0 = 0;
    int64_t n_max = 0;
    // graph
    cudaGraphExec_t graph = nullptr;
    uint64_t graph_key = 0;
    bool use_graph = true;
    int wait_polls = 1 << 24;  // bound of the staging barrier wait (lcf_set_wait_bound)
    bool capturing = false;   // enqueue_pipeline is recording into a graph
    DeviceBatch db{};
    int n_sources = 0, n_bands = 0;
    int64_t n_obs = 0;
    lcf_fit_options opts{};
    int64_t launches = 0;
};

static int set_err(lcf_ctx* c, int code, const std::string& msg) {
    if (c) c->err = msg;
    return code;
}
#define CK(call)                                                                                         \
    do {                                                                                                 \
        cudaError_t e_ = (call);                                                                         \
        if (e_ != cudaSuccess)                                                                           \
            return set_err(ctx, LCF_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));        \
    } while (0)

static int grow(lcf_ctx* ctx, DevArr& a, size_t bytes) {
    if (bytes == 0) bytes = 16;
    if (a.bytes >= bytes) return 0;
    if (a.p) cudaFree(a.p);
    a.p = nullptr;
    a.bytes = 0;
    size_t want = bytes + bytes / 4;
    cudaError_t e = cudaMalloc(&a.p, want);
    if (e != cudaSuccess) {
        a.p = nullptr;
        return set_err(ctx, LCF_E_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    }
    a.bytes = want;
    if (ctx->graph) {
        cudaGraphExecDestroy(ctx->graph);
        ctx->graph = nullptr;
        ctx->graph_key = 0;
    }
    return 0;
}
static int grow_pinned(lcf_ctx* ctx, DevArr& a, size_t bytes) {
    if (bytes == 0) bytes = 16;
    if (a.bytes >= bytes) return 0;
    if (a.p) cudaFreeHost(a.p);
    a.p = nullptr;
    a.bytes = 0;
    size_t want = bytes + bytes / 4;
    cudaError_t e = cudaMallocHost(&a.p, want);
    if (e != cudaSuccess) {
        a.p = nullptr;
        return set_err(ctx, LCF_E_NOMEM, std::string("cudaMallocHost: ") + cudaGetErrorString(e));
    }
    a.bytes = want;
    return 0;
}
static void free_arr(DevArr& a) {
    if (a.p) cudaFree(a.p);
    a = DevArr();
}

extern "C" int lcf_ctx_create(int device, lcf_ctx** out) {
    if (!out) return LCF_E_INVALID;
    *out = nullptr;
    lcf_ctx* ctx = new (std::nothrow) lcf_ctx();
    if (!ctx) return LCF_E_NOMEM;
    ctx->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) {
        delete ctx;
        return LCF_E_CUDA;
    }
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) {
        delete ctx;
        return LCF_E_CUDA;
    }
    ctx->num_sms = prop.multiProcessorCount;
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete ctx;
        return LCF_E_CUDA;
    }
    for (int i = 0; i < N_EVENTS; i++) cudaEventCreate(&ctx->ev[i]);
    if (cudaStreamCreateWithFlags(&ctx->stream_mb, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_done, cudaEventDisableTiming) != cudaSuccess) {
        lcf_ctx_destroy(ctx);
        return LCF_E_CUDA;
    }
    // each instantiation accepts the largest candidate's dynamic shared memory
    {
        int blocks[N_TUNE], obs[N_TUNE];
        for (int c = 0; c < N_TUNE; c++) { blocks[c] = TUNE_CAND[c].block; obs[c] = TUNE_CAND[c].smem_obs; }
        if (pso_init_attributes(blocks, obs, N_TUNE) != 0) {
            lcf_ctx_destroy(ctx);
            return LCF_E_CUDA;
        }
    }
    // occupancy of the 7-dimension instantiations decides each candidate's
    // persistent grids
    for (int c = 0; c < N_TUNE; c++) {
        size_t smem = pso_smem_bytes(TUNE_CAND[c].block, TUNE_CAND[c].smem_obs);
        ctx->cand_bps[c] = std::max(1, pso_blocks_per_sm(TUNE_CAND[c].block, smem, TUNE_CAND[c].minb));
        ctx->cand_bps_rest[c] = std::max(1, pso_blocks_per_sm(TUNE_CAND[c].block, smem, 2));
        int bps = std::max(ctx->cand_bps[c], ctx->cand_bps_rest[c]);
        ctx->max_pso_warps_per_sm = std::max(ctx->max_pso_warps_per_sm, bps * TUNE_CAND[c].block / 32);
    }
    ctx->pso_blocks_per_sm = ctx->cand_bps[0];
    ctx->pso_rest_per_sm = ctx->cand_bps_rest[0];
    ctx->lb_grid = lbfgs_grid(ctx->num_sms);
    // RNG tables
    std::vector<float> draws((size_t)3 * DRAWS_PER_SEED);
    // the SVI noise, then Adam's bias corrections 1 / (1 - 0.9^t) and
    // 1 / (1 - 0.999^t) for t = 1 .. SVI_STEPS (the powers by the repeated FP64
    // products Adam's recurrence forms)
    std::vector<double> eps((size_t)3 * SVI_STEPS * SVI_SAMPLES * 7 + 2 * SVI_STEPS);
    std::vector<double> draws64(draws.size());
    std::vector<float2> draws15(draws.size());
    make_draw_tables(draws.data(), draws64.data(), draws15.data(), eps.data());
    {
        double* bc = eps.data() + (size_t)3 * SVI_STEPS * SVI_SAMPLES * 7;
        double b1t = 1.0, b2t = 1.0;
        for (int t = 0; t < SVI_STEPS; t++) {
            b1t *= 0.9;
            b2t *= 0.999;
            bc[t] = 1.0 / (1.0 - b1t);
            bc[SVI_STEPS + t] = 1.0 / (1.0 - b2t);
        }
    }
    if (cudaMalloc(&ctx->d_draws, draws.size() * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&ctx->d_draws64, draws64.size() * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&ctx->d_draws15, draws15.size() * sizeof(float2)) != cudaSuccess ||
        cudaMalloc(&ctx->d_eps, eps.size() * sizeof(double)) != cudaSuccess) {
        lcf_ctx_destroy(ctx);
        return LCF_E_NOMEM;
    }
    cudaMemcpy(ctx->d_draws, draws.data(), draws.size() * sizeof(float), cudaMemcpyHostToDevice);
    cudaMemcpy(ctx->d_draws64, draws64.data(), draws64.size() * sizeof(double), cudaMemcpyHostToDevice);
    cudaMemcpy(ctx->d_draws15, draws15.data(), draws15.size() * sizeof(float2), cudaMemcpyHostToDevice);
    cudaMemcpy(ctx->d_eps, eps.data(), eps.size() * sizeof(double), cudaMemcpyHostToDevice);
    *out = ctx;
    return LCF_OK;
}

extern "C" void lcf_ctx_destroy(lcf_ctx* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->graph) cudaGraphExecDestroy(ctx->graph);
    DevArr* all[] = {&ctx->times, &ctx->flux, &ctx->ferr, &ctx->boff, &ctx->soff, &ctx->stats_b, &ctx->obs,
                     &ctx->t64, &ctx->f64, &ctx->fe64, &ctx->var64, &ctx->uf64, &ctx->mag64, &ctx->up, &ctx->ffa, &ctx->ffb, &ctx->res,
                     &ctx->fits, &ctx->out, &ctx->mb, &ctx->ctr, &ctx->scratch, &ctx->scratch64, &ctx->scratch_svi,
                     &ctx->t0state, &ctx->task_sorted, &ctx->task_sorted_mb, &ctx->band_order, &ctx->polish_order, &ctx->joint_flag,
                     &ctx->joint_src, &ctx->joint_res,
                     &ctx->joint_draws15, &ctx->joint_draws64, &ctx->joint_state,
                     &ctx->bc_obs, &ctx->bc_params, &ctx->bc_costs, &ctx->bc_scratch, &ctx->plain_scr,
                     &ctx->sg_in, &ctx->sg_out, &ctx->sg_scratch};
    for (DevArr* a : all) free_arr(*a);
    for (auto& a : ctx->tasks) free_arr(a);
    if (ctx->h_in.p) cudaFreeHost(ctx->h_in.p);
    if (ctx->h_out.p) cudaFreeHost(ctx->h_out.p);
    if (ctx->h_sel.p) cudaFreeHost(ctx->h_sel.p);
    if (ctx->h_ctr.p) cudaFreeHost(ctx->h_ctr.p);
    if (ctx->ev_done) cudaEventDestroy(ctx->ev_done);
    if (ctx->d_draws) cudaFree(ctx->d_draws);
    if (ctx->d_draws64) cudaFree(ctx->d_draws64);
    if (ctx->d_draws15) cudaFree(ctx->d_draws15);
    if (ctx->d_eps) cudaFree(ctx->d_eps);
    for (int i = 0; i < N_EVENTS; i++)
        if (ctx->ev[i]) cudaEventDestroy(ctx->ev[i]);
    if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
    if (ctx->ev_join) cudaEventDestroy(ctx->ev_join);
    if (ctx->stream_mb) cudaStreamDestroy(ctx->stream_mb);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

extern "C" const char* lcf_last_error(const lcf_ctx* ctx) {
    if (!ctx) return "null context";
    return ctx->err.c_str();
}

extern "C" int lcf_last_stats(const lcf_ctx* ctx, lcf_fit_stats* out) {
    if (!ctx || !out) return LCF_E_INVALID;
    *out = ctx->stats;
    return LCF_OK;
}

extern "C" void* lcf_ctx_stream(lcf_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

// ---------------------------------------------------------------------------
// Layout: validation, capacity, stage-1 task list
// ---------------------------------------------------------------------------
static int validate_layout(lcf_ctx* ctx, int n_sources, int n_bands, const int32_t* soff, const int64_t* boff) {
    if (n_sources < 0 || n_bands < 0) return set_err(ctx, LCF_E_INVALID, "negative source or band count");
    if (soff[0] != 0 || soff[n_sources] != n_bands)
        return set_err(ctx, LCF_E_INVALID, "source_band_offsets must start at 0 and end at n_bands");
    for (int s = 0; s < n_sources; s++)
        if (soff[s + 1] < soff[s]) return set_err(ctx, LCF_E_INVALID, "source_band_offsets not monotone");
    if (boff[0] != 0) return set_err(ctx, LCF_E_INVALID, "band_obs_offsets must start at 0");
    for (int b = 0; b < n_bands; b++) {
        if (boff[b + 1] < boff[b]) return set_err(ctx, LCF_E_INVALID, "band_obs_offsets not monotone");
        if (boff[b + 1] - boff[b] > (1 << 24)) return set_err(ctx, LCF_E_INVALID, "band longer than 2^24 points");
    }
    return 0;
}

static uint64_t hash_layout(const std::vector<int64_t>& boff, const std::vector<int32_t>& soff,
                            const lcf_fit_options& o) {
    uint64_t h = 1469598103934665603ULL;
    auto mix = [&](uint64_t v) { h = (h ^ v) * 1099511628211ULL; };
    for (int64_t v : boff) mix((uint64_t)v);
    mix(0xabcdefULL);
    for (int32_t v : soff) mix((uint64_t)(uint32_t)v);
    mix((uint64_t)o.fit_all_models);
    mix((uint64_t)o.method + 7);
    mix((uint64_t)(o.forced_model + 100));
    mix((uint64_t)o.run_multi_bazin + 11);
    mix((uint64_t)o.joint_multiband + 13);
    return h;
}

// Estimated cost of a PSO task, in observation evaluations, for the
// longest-first order of the work queue.
static double task_cost(int kind, int n) {
    if (kind == METZGER) return 330.0 + 0.8 * n;
    if (kind >= KIND_MB1) return 0.9 * n * (kind - KIND_MB1 + 1);
    return (double)n;
}

// Shape bucket of a batch: ceil(log2) of the band count, and of the
// 90th-percentile band length over 32 (0: <= 32 ... 7: > 2048).
static uint32_t shape_bucket(const std::vector<int64_t>& boff, int n_bands) {
    std::vector<int64_t> n((size_t)std::max(n_bands, 1), 0);
    for (int b = 0; b < n_bands; b++) n[b] = boff[b + 1] - boff[b];
    size_t k = (n.size() * 9) / 10;
    if (k >= n.size()) k = n.size() - 1;
    std::nth_element(n.begin(), n.begin() + k, n.end());
    int64_t p90 = n[k];
    uint32_t lb = 0;
    while (lb < 7 && ((int64_t)32 << lb) < p90) lb++;
    uint32_t nb = 0;
    while (nb < 31 && ((int64_t)1 << nb) < (int64_t)n_bands) nb++;
    return (nb << 4) | lb;
}

// Candidate for the next fused fit: forced, the bucket's next unexplored
// candidate, or its chosen one.
static void choose_launch(lcf_ctx* ctx) {
    int c = 0;
    ctx->exploring = false;
    if (ctx->tune_forced >= 0) {
        c = ctx->tune_forced;
    } else if (ctx->tune_mode) {
        TuneEntry* e = nullptr;
        for (auto& t : ctx->tune)
            if (t.bucket == ctx->bucket) e = &t;
        if (!e) {
            ctx->tune.push_back(TuneEntry());
            e = &ctx->tune.back();
            e->bucket = ctx->bucket;
        }
        if (e->next < N_TUNE) {
            c = e->next;
            ctx->exploring = true;
        } else {
            c = e->best;
        }
    }
    ctx->cfg = c;
    ctx->pso_block = TUNE_CAND[c].block;
    ctx->smem_obs = TUNE_CAND[c].smem_obs;
    ctx->pso_blocks_per_sm = ctx->cand_bps[c];
    ctx->pso_rest_per_sm = ctx->cand_bps_rest[c];
    ctx->pso_minb = TUNE_CAND[c].minb;
    ctx->db.smem_obs = ctx->smem_obs;
}

// After an exploring fit: the candidate's time, and the choice once all ran.
static void record_launch(lcf_ctx* ctx) {
    if (!ctx->exploring) return;
    for (auto& e : ctx->tune) {
        if (e.bucket != ctx->bucket || e.next >= N_TUNE || e.next != ctx->cfg) continue;
        // the swarm stages; with the MultiBazin branch running beside the polish
        // its span measures the overlap, not the swarms, so the whole fit is timed
        e.ms[e.next] = ctx->mb_branched ? ctx->stats.ms_total
                                        : ctx->stats.ms_pso + ctx->stats.ms_t0_search + ctx->stats.ms_multi_bazin;
        e.next++;
        if (e.next == N_TUNE) {
            e.best = 0;
            for (int c = 1; c < N_TUNE; c++)
                if (e.ms[c] < e.ms[e.best]) e.best = c;
        }
    }
    ctx->exploring = false;
}

static int prepare_layout(lcf_ctx* ctx, int n_sources, int n_bands, int64_t n_obs, const lcf_fit_options& o) {
    uint64_t key = hash_layout(ctx->h_boff, ctx->h_soff, o);
    bool same = key == ctx->layout_key && ctx->n_bands == n_bands && ctx->n_obs == n_obs;
    ctx->n_sources = n_sources;
    ctx->n_bands = n_bands;
    ctx->n_obs = n_obs;
    ctx->opts = o;
    int64_t n_max = 1;
    int n_long = 0;
    for (int b = 0; b < n_bands; b++) {
        const int64_t nb_obs = ctx->h_boff[b + 1] - ctx->h_boff[b];
        n_max = std::max<int64_t>(n_max, nb_obs);
        n_long += nb_obs >= LB_LONG_OBS ? 1 : 0;
    }
    ctx->n_max = n_max;
    ctx->lb_n_long = n_long;
    // capacity
    size_t nb = (size_t)std::max(n_bands, 1), no = (size_t)std::max<int64_t>(n_obs, 1);
    int rc = 0;
    rc |= grow(ctx, ctx->times, no * 8);
    rc |= grow(ctx, ctx->flux, no * 8);
    rc |= grow(ctx, ctx->ferr, no * 8);
    rc |= grow(ctx, ctx->boff, (nb + 1) * 8);
    rc |= grow(ctx, ctx->soff, ((size_t)n_sources + 1) * 4);
    rc |= grow(ctx, ctx->stats_b, nb * sizeof(BandStats));
    rc |= grow(ctx, ctx->obs, no * sizeof(float4));
    rc |= grow(ctx, ctx->t64, no * 8);
    rc |= grow(ctx, ctx->f64, no * 8);
    rc |= grow(ctx, ctx->fe64, no * 8);
    rc |= grow(ctx, ctx->var64, no * 8);
    rc |= grow(ctx, ctx->uf64, no * 8);
    rc |= grow(ctx, ctx->mag64, no * 8);
    rc |= grow(ctx, ctx->up, no);
    rc |= grow(ctx, ctx->ffa, no * sizeof(float4));
    rc |= grow(ctx, ctx->ffb, no * sizeof(float2));
    rc |= grow(ctx, ctx->res, nb * 44 * sizeof(PsoResult));
    rc |= grow(ctx, ctx->fits, nb * 8 * sizeof(ModelFit));
    rc |= grow(ctx, ctx->out, nb * sizeof(BandOut));
    rc |= grow(ctx, ctx->mb, nb * sizeof(MbState));
    rc |= grow(ctx, ctx->ctr, sizeof(Counters));
    rc |= grow(ctx, ctx->scratch64, no * 5 * 8);
    rc |= grow(ctx, ctx->scratch_svi, no * 20 * sizeof(float));
    rc |= grow(ctx, ctx->t0state, nb * 3 * 8);
    // MetzgerKN scratch of every resident swarm warp under any candidate
    size_t warps = (size_t)ctx->num_sms * ctx->max_pso_warps_per_sm;
    rc |= grow(ctx, ctx->scratch, warps * 32 * (size_t)n_max * sizeof(float));
    const int64_t caps[7] = {(int64_t)nb * 26, (int64_t)nb * 21, (int64_t)nb * 5, (int64_t)nb * 3, (int64_t)nb * 3,
                             (int64_t)nb * 3, (int64_t)nb * 3};
    for (int s = 0; s < 7; s++) {
        rc |= grow(ctx, ctx->tasks[s], (size_t)caps[s] * sizeof(PsoTask));
        ctx->task_cap[s] = caps[s];
    }
    rc |= grow(ctx, ctx->task_sorted, (size_t)nb * 21 * sizeof(PsoTask));     // slots 1..3
    rc |= grow(ctx, ctx->task_sorted_mb, (size_t)nb * 3 * sizeof(PsoTask));   // slots 4..6 (MultiBazin branch)
    rc |= grow(ctx, ctx->band_order, nb * sizeof(int32_t));
    rc |= grow(ctx, ctx->polish_order, nb * sizeof(int32_t));
    if (rc) return rc;
    // stage-1 task list (bands, models, restarts; MultiBazin K = 1), longest first
    if (!same) {
        // fit_parametric's dispatch (src/parametric.rs:3742-3761): the sources
        // with >= 2 non-empty bands get the joint multi-band fit
        std::vector<uint8_t> jflag((size_t)std::max(n_sources, 1), 0);
        std::vector<int32_t> jsrc;
        int jmax_obs = 0, jmax_nb = 0;
        if (o.joint_multiband && !o.fit_all_models && o.forced_model < 0) {
            for (int sidx = 0; sidx < n_sources; sidx++) {
                int nwd = 0;
                int64_t tot = 0;
                for (int b = ctx->h_soff[sidx]; b < ctx->h_soff[sidx + 1]; b++) {
                    int64_t n = ctx->h_boff[b + 1] - ctx->h_boff[b];
                    if (n > 0) { nwd++; tot += n; }
                }
                if (nwd < 2) continue;
                if (nwd > J_MAX_BANDS)
                    return set_err(ctx, LCF_E_UNSUPPORTED, "joint multi-band fit: at most 6 bands with data per source");
                jflag[sidx] = 1;
                jsrc.push_back(sidx);
                jmax_obs = std::max<int>(jmax_obs, (int)tot);
                jmax_nb = std::max(jmax_nb, nwd);
            }
        }
        ctx->n_joint = (int)jsrc.size();
        ctx->joint_max_obs = jmax_obs;
        ctx->joint_max_d = 7 * jmax_nb;
        if (ctx->n_joint > 0) {
            int dev = ctx->device, optin = 0;
            cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
            if (joint_smem_bytes(jmax_obs, ctx->joint_max_d) > (size_t)optin)
                return set_err(ctx, LCF_E_UNSUPPORTED, "joint multi-band fit: a source's observations exceed shared memory");
            int rc2 = 0;
            rc2 |= grow(ctx, ctx->joint_flag, (size_t)std::max(n_sources, 1));
            rc2 |= grow(ctx, ctx->joint_src, jsrc.size() * sizeof(int32_t));
            rc2 |= grow(ctx, ctx->joint_res, jsrc.size() * 3 * sizeof(JointResult));
            // the persistent swarm's grid and its blocks' state
            ctx->joint_grid = joint_grid(jmax_obs, ctx->joint_max_d, ctx->num_sms);
            rc2 |= grow(ctx, ctx->joint_state,
                        (size_t)ctx->joint_grid * JOINT_STATE_ARRAYS * ctx->joint_max_d * 200 * sizeof(float));
            // draws per seed: init (2 D P) + 1500 iterations x 2 D P
            int64_t need = (int64_t)3002 * ctx->joint_max_d * 200;
            int64_t need_init = (int64_t)2 * ctx->joint_max_d * 200;
            if (need > ctx->joint_per_seed) {
                rc2 |= grow(ctx, ctx->joint_draws15, (size_t)need * 3 * sizeof(float2));
                rc2 |= grow(ctx, ctx->joint_draws64, (size_t)need_init * 3 * sizeof(double));
                if (!rc2) {
                    std::vector<float2> h15((size_t)need * 3);
                    std::vector<double> h64((size_t)need_init * 3);
                    make_joint_draws(h15.data(), h64.data(), need, need_init);
                    CK(cudaMemcpy(ctx->joint_draws15.p, h15.data(), h15.size() * sizeof(float2),
                                  cudaMemcpyHostToDevice));
                    CK(cudaMemcpy(ctx->joint_draws64.p, h64.data(), h64.size() * sizeof(double),
                                  cudaMemcpyHostToDevice));
                    ctx->joint_per_seed = need;
                    ctx->joint_init_per_seed = need_init;
                }
            }
            if (rc2) return rc2;
            CK(cudaMemcpyAsync(ctx->joint_flag.p, jflag.data(), (size_t)n_sources, cudaMemcpyHostToDevice, ctx->stream));
            CK(cudaMemcpyAsync(ctx->joint_src.p, jsrc.data(), jsrc.size() * sizeof(int32_t), cudaMemcpyHostToDevice,
                               ctx->stream));
            CK(cudaStreamSynchronize(ctx->stream));
        }
        std::vector<PsoTask>& T = ctx->h_tasks0;
        T.clear();
        int64_t mb_base = (int64_t)n_bands * 32;
        for (int b = 0; b < n_bands; b++) {
            int n = (int)(ctx->h_boff[b + 1] - ctx->h_boff[b]);
            if (n <= 0) continue;
            int sidx = (int)(std::upper_bound(ctx->h_soff.begin(), ctx->h_soff.end(), b) - ctx->h_soff.begin()) - 1;
            const bool joint = ctx->n_joint > 0 && jflag[sidx];
            int models[8], nm = 0;
            if (joint) nm = 0;  // fitted by the joint multi-band swarm
            else if (o.forced_model >= 0) models[nm++] = o.forced_model;
            else if (o.fit_all_models) for (int m = 0; m < 8; m++) models[nm++] = m;
            else models[nm++] = BAZIN;
            for (int i = 0; i < nm; i++)
                for (int r = 0; r < 3; r++) {
                    PsoTask t;
                    t.band = b;
                    t.kind = (int16_t)models[i];
                    t.restart = (int8_t)r;
                    t.flags = TASK_PRIOR | TASK_T0_BOUNDS | (r > 0 ? TASK_SEEDED : 0);
                    t.out = (b * 8 + models[i]) * 3 + r;
                    t.aux = -1;
                    t.t0_fixed = 0.0;
                    T.push_back(t);
                }
            if (o.run_multi_bazin && n >= 5)
                for (int r = 0; r < 3; r += 2) {
                    PsoTask t;
                    t.band = b;
                    t.kind = (int16_t)KIND_MB1;
                    t.restart = (int8_t)r;
                    t.flags = TASK_RANK0;
                    t.out = (int)(mb_base + ((int64_t)b * 4) * 3 + r);
                    t.aux = -1;
                    t.t0_fixed = 0.0;
                    T.push_back(t);
                }
        }
        // Queue order: grouped by task kind so that the warps resident on an
        // SM at any moment run the same model's code (one kind's loop stays in
        // the instruction cache), the costliest kind (MetzgerKN) first, and
        // longest bands first within a kind (longest-processing-time order).
        std::vector<double> key(T.size());
        for (size_t i = 0; i < T.size(); i++)
            key[i] = task_cost(T[i].kind, (int)(ctx->h_boff[T[i].band + 1] - ctx->h_boff[T[i].band]));
        auto group = [](int kind) { return kind == METZGER ? 0 : 1 + kind; };
        std::vector<size_t> ord(T.size());
        for (size_t i = 0; i < ord.size(); i++) ord[i] = i;
        std::stable_sort(ord.begin(), ord.end(), [&](size_t a, size_t b) {
            int ga = group(T[a].kind), gb = group(T[b].kind);
            if (ga != gb) return ga < gb;
            return key[a] > key[b];
        });
        std::vector<PsoTask> S(T.size());
        for (size_t i = 0; i < ord.size(); i++) S[i] = T[ord[i]];
        T.swap(S);
        ctx->n_tasks0 = (int)T.size();
        CK(cudaMemcpyAsync(ctx->tasks[0].p, T.data(), T.size() * sizeof(PsoTask), cudaMemcpyHostToDevice,
                           ctx->stream));
        ctx->layout_key = hash_layout(ctx->h_boff, ctx->h_soff, o);
        ctx->bucket = shape_bucket(ctx->h_boff, n_bands);
        if (ctx->graph) {
            cudaGraphExecDestroy(ctx->graph);
            ctx->graph = nullptr;
            ctx->graph_key = 0;
        }
    }
    // device batch view
    DeviceBatch& d = ctx->db;
    d.times = (const double*)ctx->times.p;
    d.flux = (const double*)ctx->flux.p;
    d.err = (const double*)ctx->ferr.p;
    d.band_off = (const int64_t*)ctx->boff.p;
    d.src_off = (const int32_t*)ctx->soff.p;
    d.n_sources = n_sources;
    d.n_bands = n_bands;
    d.n_obs = n_obs;
    d.stats = (BandStats*)ctx->stats_b.p;
    d.obs = (float4*)ctx->obs.p;
    d.t64 = (double*)ctx->t64.p;
    d.f64 = (double*)ctx->f64.p;
    d.fe64 = (double*)ctx->fe64.p;
    d.var64 = (double*)ctx->var64.p;
    d.uf64 = (double*)ctx->uf64.p;
    d.mag64 = (double*)ctx->mag64.p;
    d.up = (uint8_t*)ctx->up.p;
    d.ffa = (float4*)ctx->ffa.p;
    d.ffb = (float2*)ctx->ffb.p;
    d.draws = ctx->d_draws;
    d.draws64 = ctx->d_draws64;
    d.draws15 = ctx->d_draws15;
    d.svi_eps = ctx->d_eps;
    d.svi_adam_bc = ctx->d_eps + (size_t)3 * SVI_STEPS * SVI_SAMPLES * 7;
    d.pso_res = (PsoResult*)ctx->res.p;
    d.fits = (ModelFit*)ctx->fits.p;
    d.out = (BandOut*)ctx->out.p;
    d.mb = (MbState*)ctx->mb.p;
    for (int s = 0; s < 7; s++) {
        d.tasks[s] = (PsoTask*)ctx->tasks[s].p;
        d.task_cap[s] = (int)ctx->task_cap[s];
    }
    d.tasks[7] = nullptr;
    d.task_cap[7] = 0;
    d.task_sorted = (PsoTask*)ctx->task_sorted.p;
    d.task_sorted_mb = (PsoTask*)ctx->task_sorted_mb.p;
    d.band_order = (int32_t*)ctx->band_order.p;
    d.polish_order = (int32_t*)ctx->polish_order.p;
    d.lb_grid = ctx->lb_grid;
    d.lb_n_long = ctx->lb_n_long;
    d.n_joint = ctx->n_joint;
    d.joint_flag = ctx->n_joint > 0 ? (const uint8_t*)ctx->joint_flag.p : nullptr;
    d.joint_src = (const int32_t*)ctx->joint_src.p;
    d.joint_res = (JointResult*)ctx->joint_res.p;
    d.joint_draws15 = (const float2*)ctx->joint_draws15.p;
    d.joint_draws64 = (const double*)ctx->joint_draws64.p;
    d.joint_draws_per_seed = ctx->joint_per_seed;
    d.joint_init_per_seed = ctx->joint_init_per_seed;
    d.joint_state = (float*)ctx->joint_state.p;
    d.joint_grid = ctx->joint_grid;
    d.joint_max_obs = ctx->joint_max_obs;
    d.joint_max_d = ctx->joint_max_d;
    d.ctr = (Counters*)ctx->ctr.p;
    d.scratch = (float*)ctx->scratch.p;
    d.scratch_per_warp = 32 * n_max;
    d.scratch64 = (double*)ctx->scratch64.p;
    d.scratch_svi = (float*)ctx->scratch_svi.p;
    d.t0_state = (double*)ctx->t0state.p;
    d.t0_slot_base = (int64_t)n_bands * 24;
    d.mb_slot_base = (int64_t)n_bands * 32;
    d.smem_obs = ctx->smem_obs;
    d.wait_polls = ctx->wait_polls;
    return 0;
}

// ---------------------------------------------------------------------------
// Stage sequence
// ---------------------------------------------------------------------------
// A stage-timing event: an external event node while the stage sequence is
// captured into the graph (so that replays record it), a plain record when
// the kernels are launched one by one (the external flag is only valid
// during capture).
static void stage_event(lcf_ctx* ctx, cudaEvent_t e, cudaStream_t q) {
    if (ctx->capturing) cudaEventRecordWithFlags(e, q, cudaEventRecordExternal);
    else cudaEventRecord(e, q);
}

static void enqueue_pipeline(lcf_ctx* ctx) {
    const DeviceBatch& d = ctx->db;
    const lcf_fit_options& o = ctx->opts;
    cudaStream_t s = ctx->stream;
    int grid0 = ctx->num_sms * ctx->pso_blocks_per_sm;
    int grid = ctx->num_sms * ctx->pso_rest_per_sm;
    int block = ctx->pso_block;
    int64_t L = 0;
    stage_event(ctx, ctx->ev[0], s);
    cudaMemsetAsync(ctx->res.p, 0xff, (size_t)std::max(ctx->n_bands, 1) * 44 * sizeof(PsoResult), s);
    cudaMemsetAsync(ctx->ctr.p, 0, sizeof(Counters), s);
    cudaMemsetAsync(ctx->fits.p, 0xff, (size_t)std::max(ctx->n_bands, 1) * 8 * sizeof(ModelFit), s);
    launch_prep(d, s); L++;
    stage_event(ctx, ctx->ev[1], s);
    launch_pso(d, 0, d.tasks[0], ctx->n_tasks0, 7, grid0, block, s, ctx->pso_minb); L++;
    stage_event(ctx, ctx->ev[2], s);
    // MultiBazin K = 2..4 (fit_multi_bazin's greedy loop) needs only the band
    // preparation and its K = 1 swarms of the launch above, so it can run on
    // a branch beside the polish / selection / t0 / uncertainty / refinement
    // stages and fill their tails; it owns slots 4..6, its own sorted task
    // list and no state the main sequence reads
    auto enqueue_mb = [&](cudaStream_t q) {
        stage_event(ctx, ctx->ev[9], q);
        launch_mb_pick(d, 1, q); L++;
        for (int k = 2; k <= 4; k++) {
            launch_mb_build(d, 2 + k, k, q); L++;
            launch_task_sort(d, 2 + k, d.task_sorted_mb, q); L += 3;
            launch_pso(d, 2 + k, d.task_sorted_mb, -1, 4 * k + 2, grid, block, q); L++;
            launch_mb_pick(d, k, q); L++;
        }
        stage_event(ctx, ctx->ev[10], q);
    };
    const int branch = o.run_multi_bazin ? ctx->mb_branch : 0;
    auto fork_mb = [&]() {
        cudaEventRecord(ctx->ev_fork, s);
        cudaStreamWaitEvent(ctx->stream_mb, ctx->ev_fork, 0);
        enqueue_mb(ctx->stream_mb);
        cudaEventRecord(ctx->ev_join, ctx->stream_mb);
    };
    if (branch == 1) fork_mb();
    int gated = (o.forced_model < 0 && !o.fit_all_models);
    launch_polish_order(d, s); L += 3;
    launch_lbfgs(d, gated ? 1 : 0xff, s); L++;
    if (gated) {
        launch_gate_build(d, 1, s); L++;
        launch_task_sort(d, 1, d.task_sorted, s); L += 3;
        launch_pso(d, 1, d.task_sorted, -1, 7, grid, block, s); L++;
        launch_lbfgs(d, 0xfe, s); L++;
    }
    launch_select(d, o.fit_all_models, o.forced_model, s); L++;
    stage_event(ctx, ctx->ev[3], s);
    if (branch == 2) fork_mb();
    if (d.n_joint > 0 && launch_joint(d, s) == 0) L += 2;
    stage_event(ctx, ctx->ev[8], s);
    if (o.method == LCF_METHOD_SVI) {
        launch_t0_build(d, 2, 0, s); L++;
        launch_task_sort(d, 2, d.task_sorted, s); L += 3;
        launch_pso(d, 2, d.task_sorted, -1, 7, grid, block, s); L++;
        launch_t0_pick(d, 2, 0, s); L++;
        launch_t0_build(d, 3, 1, s); L++;
        launch_task_sort(d, 3, d.task_sorted, s); L += 3;
        launch_pso(d, 3, d.task_sorted, -1, 7, grid, block, s); L++;
        launch_t0_pick(d, 3, 1, s); L++;
    }
    stage_event(ctx, ctx->ev[4], s);
    launch_band_order(d, s); L += 3;
    if (o.method == LCF_METHOD_SVI) launch_svi(d, s);
    else launch_laplace(d, s);
    L++;
    stage_event(ctx, ctx->ev[5], s);
    launch_refine(d, s); L++;
    stage_event(ctx, ctx->ev[6], s);
    if (o.run_multi_bazin && branch == 0) enqueue_mb(s);
    if (branch) cudaStreamWaitEvent(s, ctx->ev_join, 0);
    stage_event(ctx, ctx->ev[7], s);
    ctx->launches = L;
}

static int run_pipeline(lcf_ctx* ctx) {
    cudaGetLastError();  // a failed query elsewhere in the process must not be reported as ours
    // set per fit (a graph replay does not run enqueue_pipeline)
    ctx->mb_timed = ctx->opts.run_multi_bazin != 0;
    ctx->mb_branched = ctx->mb_timed && ctx->mb_branch != 0;
    uint64_t gkey = ctx->layout_key ^ ((uint64_t)(uintptr_t)ctx->db.times * 31) ^ ((uint64_t)ctx->n_obs << 7) ^
                    ((uint64_t)(ctx->cfg + 1) << 56) ^ ((uint64_t)(ctx->mb_branch + 1) << 52);
    if (ctx->use_graph) {
        if (!ctx->graph || ctx->graph_key != gkey) {
            if (ctx->graph) {
                cudaGraphExecDestroy(ctx->graph);
                ctx->graph = nullptr;
            }
            cudaGraph_t g;
            CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
            ctx->capturing = true;
            enqueue_pipeline(ctx);
            ctx->capturing = false;
            CK(cudaStreamEndCapture(ctx->stream, &g));
            cudaError_t e = cudaGraphInstantiate(&ctx->graph, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) {
                ctx->graph = nullptr;
                return set_err(ctx, LCF_E_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
            }
            ctx->graph_key = gkey;
        }
        CK(cudaGraphLaunch(ctx->graph, ctx->stream));
    } else {
        enqueue_pipeline(ctx);
        CK(cudaGetLastError());
    }
    return 0;
}

// The plain FP64 form (plain.cu): same inputs and outputs, one launch per
// model per stage, no graph.  Stage events: 0 start, 1 prep, 2 PSO,
// 3 L-BFGS + selection, 5 SVI (4, 6, 7 coincide with their neighbours).
static void enqueue_plain(lcf_ctx* ctx) {
    const DeviceBatch& d = ctx->db;
    const lcf_fit_options& o = ctx->opts;
    cudaStream_t s = ctx->stream;
    double* scr = (double*)ctx->plain_scr.p;
    int64_t L = 0;
    ctx->mb_timed = false;
    cudaEventRecord(ctx->ev[0], s);
    cudaMemsetAsync(ctx->res.p, 0xff, (size_t)std::max(ctx->n_bands, 1) * 44 * sizeof(PsoResult), s);
    cudaMemsetAsync(ctx->ctr.p, 0, sizeof(Counters), s);
    cudaMemsetAsync(ctx->fits.p, 0xff, (size_t)std::max(ctx->n_bands, 1) * 8 * sizeof(ModelFit), s);
    launch_prep(d, s); L++;
    cudaEventRecord(ctx->ev[1], s);
    static const int order[8] = {BAZIN, ARNETT, TDE, AFTERGLOW, VILLAR, MAGNETAR, SHOCK, METZGER};
    if (o.forced_model >= 0) {
        launch_plain_pso(d, o.forced_model, 0, scr, s); L++;
        cudaEventRecord(ctx->ev[2], s);
        launch_plain_lbfgs(d, o.forced_model, s); L++;
    } else if (!o.fit_all_models) {
        launch_plain_pso(d, BAZIN, 0, scr, s); L++;
        launch_plain_lbfgs(d, BAZIN, s); L++;
        for (int k = 1; k < 8; k++) { launch_plain_pso(d, order[k], 1, scr, s); L++; }
        cudaEventRecord(ctx->ev[2], s);
        for (int k = 1; k < 8; k++) { launch_plain_lbfgs(d, order[k], s); L++; }
    } else {
        for (int k = 0; k < 8; k++) { launch_plain_pso(d, order[k], 0, scr, s); L++; }
        cudaEventRecord(ctx->ev[2], s);
        for (int k = 0; k < 8; k++) { launch_plain_lbfgs(d, order[k], s); L++; }
    }
    launch_select(d, o.fit_all_models, o.forced_model, s); L++;
    cudaEventRecord(ctx->ev[3], s);
    cudaEventRecord(ctx->ev[4], s);
    for (int m = 0; m < 8; m++) { launch_plain_svi(d, m, scr, s); L++; }
    cudaEventRecord(ctx->ev[5], s);
    cudaEventRecord(ctx->ev[6], s);
    cudaEventRecord(ctx->ev[7], s);
    ctx->launches = L;
}

// Stage times (from the stage events) and device counters of the fit that
// just completed; LCF_E_TIMEOUT when a bounded device wait expired in it.
static int stats_from_counters(lcf_ctx* ctx, const Counters& c) {
    float ms[8] = {0};
    for (int i = 1; i < 8; i++)
        if (cudaEventElapsedTime(&ms[i], ctx->ev[i - 1], ctx->ev[i]) != cudaSuccess) ms[i] = 0.0f;
    float tot = 0;
    if (cudaEventElapsedTime(&tot, ctx->ev[0], ctx->ev[7]) != cudaSuccess) tot = 0.0f;
    cudaGetLastError();
    lcf_fit_stats& st = ctx->stats;
    st.ms_total = tot;
    st.ms_pso = ms[2];
    st.ms_lbfgs = ms[3];
    float mj = 0.0f, mt0 = 0.0f;
    if (cudaEventElapsedTime(&mj, ctx->ev[3], ctx->ev[8]) != cudaSuccess) mj = 0.0f;
    if (cudaEventElapsedTime(&mt0, ctx->ev[8], ctx->ev[4]) != cudaSuccess) mt0 = 0.0f;
    st.ms_joint = mj;
    st.ms_t0_search = mt0;
    st.ms_uncertainty = ms[5];
    st.ms_refine = ms[6];
    float mmb = 0.0f;
    if (!ctx->mb_timed || cudaEventElapsedTime(&mmb, ctx->ev[9], ctx->ev[10]) != cudaSuccess) mmb = 0.0f;
    cudaGetLastError();
    st.ms_multi_bazin = mmb;
    st.particle_obs_evals = (double)c.particle_obs_evals;
    st.ode_steps = (double)c.ode_steps;
    st.pso_tasks = ctx->n_tasks0;
    st.kernel_launches = ctx->launches;
    st.lbfgs_polishes = (double)c.lb_polishes;
    st.lbfgs_iters = (double)c.lb_iters;
    st.lbfgs_evals = (double)c.lb_evals;
    st.lbfgs_obs_evals = (double)c.lb_obs_evals;
    for (int m = 0; m < 8; m++) st.lbfgs_obs_evals_by_model[m] = (double)c.lb_obs_evals_by_model[m];
    for (int m = 0; m < 8; m++) st.lbfgs_fp64_obs_evals_by_model[m] = (double)c.lb_fp64_obs_evals_by_model[m];
    for (int k = 0; k < 12; k++) {
        st.pso0_evals_by_kind[k] = (double)c.slot0_evals[k];
        st.pso0_particles_by_kind[k] = (double)c.slot0_particles[k];
    }
    if (c.error) return set_err(ctx, c.error, "a bounded device wait expired");
    return 0;
}

static int finish_stats(lcf_ctx* ctx) {
    CK(cudaStreamSynchronize(ctx->stream));
    CK(cudaGetLastError());
    Counters c;
    CK(cudaMemcpy(&c, ctx->ctr.p, sizeof(Counters), cudaMemcpyDeviceToHost));
    return stats_from_counters(ctx, c);
}

// ---------------------------------------------------------------------------
// Output unpacking
// ---------------------------------------------------------------------------
// Queues the copies of the device results into the pinned output buffer
// (lcf_fit_outputs order is filled from there by fill_outputs).
static int enqueue_download(lcf_ctx* ctx) {
    int nb = ctx->n_bands;
    size_t bytes = (size_t)nb * (sizeof(BandOut) + sizeof(BandStats) + sizeof(MbState) +
                                 (ctx->opts.fit_all_models ? 8 * sizeof(ModelFit) : 0));
    ctx->stats.d2h_bytes = (double)(nb > 0 ? (size_t)nb * (sizeof(BandOut) + sizeof(BandStats) +
                                                          (ctx->opts.run_multi_bazin ? sizeof(MbState) : 0) +
                                                          (ctx->opts.fit_all_models ? 8 * sizeof(ModelFit) : 0))
                                           : 0);
    if (grow_pinned(ctx, ctx->h_out, bytes)) return LCF_E_NOMEM;
    char* hp = (char*)ctx->h_out.p;
    BandOut* ho = (BandOut*)hp;
    BandStats* hs = (BandStats*)(hp + (size_t)nb * sizeof(BandOut));
    MbState* hm = (MbState*)((char*)hs + (size_t)nb * sizeof(BandStats));
    ModelFit* hf = (ModelFit*)((char*)hm + (size_t)nb * sizeof(MbState));
    if (nb > 0) {
        CK(cudaMemcpyAsync(ho, ctx->out.p, (size_t)nb * sizeof(BandOut), cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaMemcpyAsync(hs, ctx->stats_b.p, (size_t)nb * sizeof(BandStats), cudaMemcpyDeviceToHost, ctx->stream));
        if (ctx->opts.run_multi_bazin)
            CK(cudaMemcpyAsync(hm, ctx->mb.p, (size_t)nb * sizeof(MbState), cudaMemcpyDeviceToHost, ctx->stream));
        if (ctx->opts.fit_all_models)
            CK(cudaMemcpyAsync(hf, ctx->fits.p, (size_t)nb * 8 * sizeof(ModelFit), cudaMemcpyDeviceToHost,
                               ctx->stream));
    }
    return 0;
}

// The caller's output arrays from the pinned output buffer (after the copies
// of enqueue_download have completed).
static void fill_outputs(lcf_ctx* ctx, lcf_fit_outputs* out) {
    int nb = ctx->n_bands;
    char* hp = (char*)ctx->h_out.p;
    BandOut* ho = (BandOut*)hp;
    BandStats* hs = (BandStats*)(hp + (size_t)nb * sizeof(BandOut));
    MbState* hm = (MbState*)((char*)hs + (size_t)nb * sizeof(BandStats));
    ModelFit* hf = (ModelFit*)((char*)hm + (size_t)nb * sizeof(MbState));
    const double nan = std::nan("");
    for (int b = 0; b < nb; b++) {
        const BandStats& st = hs[b];
        const BandOut& o = ho[b];
        bool ok = st.valid && o.model >= 0;
        out->model[b] = ok ? o.model : -1;
        out->rank[b] = ok ? st.rank : -1;
        out->n_obs[b] = ok ? st.n : 0;
        int np = ok ? n_params_of(o.model) : 0;
        for (int j = 0; j < MAXP; j++) {
            out->pso_params[b * 7 + j] = j < np ? o.pso_params[j] : nan;
            out->svi_mu[b * 7 + j] = j < np ? o.mu[j] : nan;
            out->svi_log_sigma[b * 7 + j] = j < np ? o.log_sigma[j] : nan;
        }
        out->pso_chi2[b] = ok && std::isfinite(o.pso_cost) ? o.pso_cost : nan;
        out->svi_elbo[b] = ok && std::isfinite(o.elbo) ? o.elbo : nan;
        out->mag_chi2[b] = ok && std::isfinite(o.mag_chi2) ? o.mag_chi2 : nan;
        for (int m = 0; m < 8; m++) {
            out->per_model_chi2[b * 8 + m] = ok ? o.per_chi2[m] : nan;
            // fits are reset to NaN before each run: a NaN cost means "not fitted"
            bool have = ok && ctx->opts.fit_all_models && !std::isnan(hf[b * 8 + m].cost);
            int npm = n_params_of(m);
            for (int j = 0; j < 7; j++)
                out->per_model_params[(b * 8 + m) * 7 + j] = (have && j < npm) ? hf[b * 8 + m].params[j] : nan;
        }
        out->mb_best_k[b] = 0;
        for (int j = 0; j < LCF_MB_MAX_PARAMS; j++) out->mb_params[b * 18 + j] = nan;
        out->mb_cost[b] = nan;
        out->mb_bic[b] = nan;
        for (int k = 0; k < 4; k++) {
            out->mb_per_k_cost[b * 4 + k] = nan;
            out->mb_per_k_bic[b * 4 + k] = nan;
        }
        if (ok && ctx->opts.run_multi_bazin && st.rank == 0 && st.n >= 5) {
            const MbState& S = hm[b];
            out->mb_best_k[b] = S.best_k;
            for (int j = 0; j < LCF_MB_MAX_PARAMS; j++) out->mb_params[b * 18 + j] = S.best_params[j];
            out->mb_cost[b] = S.best_cost;
            out->mb_bic[b] = S.best_bic;
            for (int k = 0; k < 4; k++) {
                out->mb_per_k_cost[b * 4 + k] = S.per_k_cost[k];
                out->mb_per_k_bic[b * 4 + k] = S.per_k_bic[k];
            }
        }
    }
}

static int unpack_outputs(lcf_ctx* ctx, lcf_fit_outputs* out) {
    if (int rc = enqueue_download(ctx)) return rc;
    if (ctx->n_bands > 0) CK(cudaStreamSynchronize(ctx->stream));
    fill_outputs(ctx, out);
    return 0;
}

static int check_opts(lcf_ctx* ctx, const lcf_fit_options* o) {
    if (!o) return set_err(ctx, LCF_E_INVALID, "null options");
    if (o->method != LCF_METHOD_SVI && o->method != LCF_METHOD_LAPLACE)
        return set_err(ctx, LCF_E_INVALID, "method must be LCF_METHOD_SVI or LCF_METHOD_LAPLACE");
    if (o->forced_model < -1 || o->forced_model > 7) return set_err(ctx, LCF_E_INVALID, "forced_model out of range");
    return 0;
}

// Validates a host CSR, prepares the layout for options `o` and queues the
// copies of its observations and offsets to the device through pinned
// staging; *in_bytes = the bytes copied.
static int stage_host_batch(lcf_ctx* ctx, const lcf_bands_csr* in, const lcf_fit_options& o, size_t* in_bytes) {
    int ns = in->n_sources, nb = in->n_bands;
    if (ns < 0 || nb < 0 || !in->source_band_offsets || (nb > 0 && !in->band_obs_offsets))
        return set_err(ctx, LCF_E_INVALID, "bad CSR header");
    if (int rc = validate_layout(ctx, ns, nb, in->source_band_offsets, in->band_obs_offsets)) return rc;
    int64_t n_obs = nb > 0 ? in->band_obs_offsets[nb] : 0;
    if (n_obs > 0 && (!in->times || !in->flux || !in->flux_err)) return set_err(ctx, LCF_E_INVALID, "null data array");
    ctx->h_boff.assign(in->band_obs_offsets, in->band_obs_offsets + nb + 1);
    ctx->h_soff.assign(in->source_band_offsets, in->source_band_offsets + ns + 1);
    if (int rc = prepare_layout(ctx, ns, nb, n_obs, o)) return rc;
    size_t bytes = (size_t)n_obs * 24 + (size_t)(nb + 1) * 8 + (size_t)(ns + 1) * 4;
    if (grow_pinned(ctx, ctx->h_in, bytes)) return LCF_E_NOMEM;
    char* hp = (char*)ctx->h_in.p;
    std::memcpy(hp, in->times, (size_t)n_obs * 8);
    std::memcpy(hp + (size_t)n_obs * 8, in->flux, (size_t)n_obs * 8);
    std::memcpy(hp + (size_t)n_obs * 16, in->flux_err, (size_t)n_obs * 8);
    std::memcpy(hp + (size_t)n_obs * 24, in->band_obs_offsets, (size_t)(nb + 1) * 8);
    std::memcpy(hp + (size_t)n_obs * 24 + (size_t)(nb + 1) * 8, in->source_band_offsets, (size_t)(ns + 1) * 4);
    cudaStream_t s = ctx->stream;
    if (n_obs > 0) {
        CK(cudaMemcpyAsync(ctx->times.p, hp, (size_t)n_obs * 8, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(ctx->flux.p, hp + (size_t)n_obs * 8, (size_t)n_obs * 8, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(ctx->ferr.p, hp + (size_t)n_obs * 16, (size_t)n_obs * 8, cudaMemcpyHostToDevice, s));
    }
    CK(cudaMemcpyAsync(ctx->boff.p, hp + (size_t)n_obs * 24, (size_t)(nb + 1) * 8, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(ctx->soff.p, hp + (size_t)n_obs * 24 + (size_t)(nb + 1) * 8, (size_t)(ns + 1) * 4,
                       cudaMemcpyHostToDevice, s));
    *in_bytes = bytes;
    return 0;
}

// Rejects a call that would enqueue work behind an asynchronous fit still
// waiting for lcf_wait().
static int busy(lcf_ctx* ctx) {
    return ctx->pending ? set_err(ctx, LCF_E_INVALID, "an asynchronous fit is pending: call lcf_wait first") : 0;
}

extern "C" int lcf_fit_parametric_batch_async(lcf_ctx* ctx, const lcf_bands_csr* in, const lcf_fit_options* o,
                                              lcf_fit_outputs* out) {
    if (!ctx) return LCF_E_INVALID;
    if (int rc = busy(ctx)) return rc;
    if (!in || !out) return set_err(ctx, LCF_E_INVALID, "null argument");
    if (int rc = check_opts(ctx, o)) return rc;
    CK(cudaSetDevice(ctx->device));
    size_t in_bytes = 0;
    if (int rc = stage_host_batch(ctx, in, *o, &in_bytes)) return rc;
    if (in->n_bands == 0) return 0;
    choose_launch(ctx);
    if (int rc = run_pipeline(ctx)) return rc;
    if (grow_pinned(ctx, ctx->h_ctr, sizeof(Counters))) return LCF_E_NOMEM;
    CK(cudaMemcpyAsync(ctx->h_ctr.p, ctx->ctr.p, sizeof(Counters), cudaMemcpyDeviceToHost, ctx->stream));
    if (int rc = enqueue_download(ctx)) return rc;
    CK(cudaEventRecord(ctx->ev_done, ctx->stream));
    ctx->pending = true;
    ctx->pending_out = *out;
    ctx->pending_in_bytes = in_bytes;
    return 0;
}

extern "C" int lcf_wait(lcf_ctx* ctx, int timeout_ms) {
    if (!ctx) return LCF_E_INVALID;
    if (!ctx->pending) return 0;
    CK(cudaSetDevice(ctx->device));
    const auto t0 = std::chrono::steady_clock::now();
    while (true) {
        cudaError_t e = cudaEventQuery(ctx->ev_done);
        if (e == cudaSuccess) break;
        if (e != cudaErrorNotReady) {
            ctx->pending = false;
            return set_err(ctx, LCF_E_CUDA, std::string("cudaEventQuery: ") + cudaGetErrorString(e));
        }
        if (timeout_ms >= 0 &&
            std::chrono::steady_clock::now() - t0 >= std::chrono::milliseconds(timeout_ms))
            return set_err(ctx, LCF_E_TIMEOUT, "the asynchronous fit has not finished yet");
        std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
    ctx->pending = false;
    CK(cudaGetLastError());
    Counters c;
    std::memcpy(&c, ctx->h_ctr.p, sizeof(Counters));
    const int rc = stats_from_counters(ctx, c);
    record_launch(ctx);
    ctx->stats.h2d_bytes = (double)ctx->pending_in_bytes;
    fill_outputs(ctx, &ctx->pending_out);
    return rc;
}

extern "C" int lcf_fit_parametric_batch(lcf_ctx* ctx, const lcf_bands_csr* in, const lcf_fit_options* o,
                                        lcf_fit_outputs* out) {
    if (int rc = lcf_fit_parametric_batch_async(ctx, in, o, out)) return rc;
    return lcf_wait(ctx, -1);
}

// ---------------------------------------------------------------------------
// Batched finalisation of caller-selected fits (lcf_finalize_batch): band
// preparation, then the uncertainty stage unless its outputs are supplied,
// then the refinements and the magnitude chi2 -- the per-band kernels of the
// fused pipeline, fed from the caller's selection instead of the swarms.
// Stage events as in the fused pipeline (the swarm and polish stages empty).
// ---------------------------------------------------------------------------
static void enqueue_finalize(lcf_ctx* ctx, bool given, size_t sel_bytes) {
    const DeviceBatch& d = ctx->db;
    cudaStream_t s = ctx->stream;
    int64_t L = 0;
    ctx->mb_timed = false;
    cudaEventRecord(ctx->ev[0], s);
    cudaMemsetAsync(ctx->ctr.p, 0, sizeof(Counters), s);
    launch_prep(d, s); L++;
    // the caller's selection rows (pinned staging)
    cudaMemcpyAsync(ctx->out.p, (char*)ctx->h_sel.p, sel_bytes, cudaMemcpyHostToDevice, s);
    cudaEventRecord(ctx->ev[1], s);
    cudaEventRecord(ctx->ev[2], s);
    cudaEventRecord(ctx->ev[3], s);
    cudaEventRecord(ctx->ev[8], s);
    launch_band_order(d, s); L += 3;
    cudaEventRecord(ctx->ev[4], s);
    if (!given) {
        if (ctx->opts.method == LCF_METHOD_SVI) launch_svi(d, s);
        else launch_laplace(d, s);
        L++;
    }
    cudaEventRecord(ctx->ev[5], s);
    launch_refine(d, s); L++;
    cudaEventRecord(ctx->ev[6], s);
    cudaEventRecord(ctx->ev[7], s);
    ctx->launches = L;
}

extern "C" int lcf_finalize_batch(lcf_ctx* ctx, const lcf_bands_csr* in, const lcf_pso_selection* sel, int method,
                                  lcf_fit_outputs* out) {
    if (!ctx) return LCF_E_INVALID;
    if (int rc = busy(ctx)) return rc;
    if (!in || !sel || !out) return set_err(ctx, LCF_E_INVALID, "null argument");
    const bool given = sel->svi_mu != nullptr || sel->svi_log_sigma != nullptr;
    if (given && !(sel->svi_mu && sel->svi_log_sigma))
        return set_err(ctx, LCF_E_INVALID, "svi_mu and svi_log_sigma are given together");
    if (!given && method != LCF_METHOD_SVI && method != LCF_METHOD_LAPLACE)
        return set_err(ctx, LCF_E_INVALID, "method must be LCF_METHOD_SVI or LCF_METHOD_LAPLACE");
    const int nb = in->n_bands;
    if (nb > 0 && (!sel->model || !sel->pso_params)) return set_err(ctx, LCF_E_INVALID, "null selection array");
    for (int b = 0; b < nb; b++)
        if (sel->model[b] < -1 || sel->model[b] > 7) return set_err(ctx, LCF_E_INVALID, "selection model out of range");
    CK(cudaSetDevice(ctx->device));
    lcf_fit_options o;
    o.fit_all_models = 0;
    o.method = given ? LCF_METHOD_SVI : method;
    o.forced_model = -1;
    o.run_multi_bazin = 0;
    o.joint_multiband = 0;
    size_t in_bytes = 0;
    if (int rc = stage_host_batch(ctx, in, o, &in_bytes)) return rc;
    if (nb == 0) return 0;
    // the per-band selection rows, in the device layout of the selected fit
    const size_t sel_bytes = (size_t)nb * sizeof(BandOut);
    if (grow_pinned(ctx, ctx->h_sel, sel_bytes)) return LCF_E_NOMEM;
    BandOut* rows = (BandOut*)ctx->h_sel.p;
    const double nan = std::nan("");
    for (int b = 0; b < nb; b++) {
        BandOut& r = rows[b];
        const int m = sel->model[b];
        const int np = m >= 0 ? n_params_of(m) : 0;
        r.model = m;
        r.svi_steps = 0;
        r.pso_cost = sel->pso_cost ? sel->pso_cost[b] : nan;
        for (int j = 0; j < MAXP; j++) {
            r.pso_params[j] = j < np ? sel->pso_params[b * 7 + j] : nan;
            r.mu[j] = given && j < np ? sel->svi_mu[b * 7 + j] : nan;
            r.log_sigma[j] = given && j < np ? sel->svi_log_sigma[b * 7 + j] : nan;
        }
        r.elbo = given && sel->svi_elbo ? sel->svi_elbo[b] : nan;
        r.mag_chi2 = nan;
        for (int k = 0; k < 8; k++) r.per_chi2[k] = sel->per_model_chi2 ? sel->per_model_chi2[b * 8 + k] : nan;
    }
    cudaGetLastError();
    enqueue_finalize(ctx, given, sel_bytes);
    CK(cudaGetLastError());
    if (int rc = finish_stats(ctx)) return rc;
    ctx->stats.pso_tasks = 0;
    ctx->stats.h2d_bytes = (double)(in_bytes + sel_bytes);
    return unpack_outputs(ctx, out);
}

extern "C" int lcf_fit_parametric_device(lcf_ctx* ctx, const lcf_bands_csr* dev, const lcf_fit_options* o) {
    if (!ctx) return LCF_E_INVALID;
    if (int rc = busy(ctx)) return rc;
    if (!dev) return set_err(ctx, LCF_E_INVALID, "null argument");
    if (int rc = check_opts(ctx, o)) return rc;
    CK(cudaSetDevice(ctx->device));
    int ns = dev->n_sources, nb = dev->n_bands;
    if (ns < 0 || nb < 0) return set_err(ctx, LCF_E_INVALID, "bad CSR header");
    // the offsets drive the host-side task list: read them back
    std::vector<int64_t> boff((size_t)nb + 1);
    std::vector<int32_t> soff((size_t)ns + 1);
    CK(cudaMemcpy(boff.data(), dev->band_obs_offsets, boff.size() * 8, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(soff.data(), dev->source_band_offsets, soff.size() * 4, cudaMemcpyDeviceToHost));
    if (int rc = validate_layout(ctx, ns, nb, soff.data(), boff.data())) return rc;
    ctx->h_boff.swap(boff);
    ctx->h_soff.swap(soff);
    int64_t n_obs = ctx->h_boff[nb];
    if (int rc = prepare_layout(ctx, ns, nb, n_obs, *o)) return rc;
    // point the batch at the caller's device arrays
    ctx->db.times = dev->times;
    ctx->db.flux = dev->flux;
    ctx->db.err = dev->flux_err;
    ctx->db.band_off = dev->band_obs_offsets;
    ctx->db.src_off = dev->source_band_offsets;
    if (nb == 0) return 0;
    choose_launch(ctx);
    if (int rc = run_pipeline(ctx)) return rc;
    if (int rc = finish_stats(ctx)) return rc;
    record_launch(ctx);
    return 0;
}

extern "C" int lcf_fit_plain_device(lcf_ctx* ctx, const lcf_bands_csr* dev, const lcf_fit_options* o) {
    if (!ctx) return LCF_E_INVALID;
    if (int rc = busy(ctx)) return rc;
    if (!dev) return set_err(ctx, LCF_E_INVALID, "null argument");
    if (int rc = check_opts(ctx, o)) return rc;
    if (o->method != LCF_METHOD_SVI) return set_err(ctx, LCF_E_UNSUPPORTED, "the plain form runs SVI only");
    CK(cudaSetDevice(ctx->device));
    int ns = dev->n_sources, nb = dev->n_bands;
    if (ns < 0 || nb < 0) return set_err(ctx, LCF_E_INVALID, "bad CSR header");
    std::vector<int64_t> boff((size_t)nb + 1);
    std::vector<int32_t> soff((size_t)ns + 1);
    CK(cudaMemcpy(boff.data(), dev->band_obs_offsets, boff.size() * 8, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(soff.data(), dev->source_band_offsets, soff.size() * 4, cudaMemcpyDeviceToHost));
    if (int rc = validate_layout(ctx, ns, nb, soff.data(), boff.data())) return rc;
    ctx->h_boff.swap(boff);
    ctx->h_soff.swap(soff);
    int64_t n_obs = ctx->h_boff[nb];
    lcf_fit_options po = *o;
    po.run_multi_bazin = 0;  // not part of the plain form
    if (int rc = prepare_layout(ctx, ns, nb, n_obs, po)) return rc;
    if (int rc = grow(ctx, ctx->plain_scr, (size_t)std::max<int64_t>(n_obs, 1) * 96 * sizeof(double))) return rc;
    ctx->db.times = dev->times;
    ctx->db.flux = dev->flux;
    ctx->db.err = dev->flux_err;
    ctx->db.band_off = dev->band_obs_offsets;
    ctx->db.src_off = dev->source_band_offsets;
    if (nb == 0) return 0;
    cudaGetLastError();
    enqueue_plain(ctx);
    CK(cudaGetLastError());
    return finish_stats(ctx);
}

extern "C" int lcf_set_multi_bazin_branch(lcf_ctx* ctx, int mode) {
    if (!ctx) return LCF_E_INVALID;
    if (mode < 0 || mode > 2) return set_err(ctx, LCF_E_INVALID, "MultiBazin branch mode must be 0, 1 or 2");
    ctx->mb_branch = mode;
    return 0;
}

extern "C" int lcf_set_autotune(lcf_ctx* ctx, int mode, int forced_candidate) {
    if (!ctx) return LCF_E_INVALID;
    if ((mode != 0 && mode != 1) || forced_candidate < -1 || forced_candidate >= N_TUNE)
        return set_err(ctx, LCF_E_INVALID, "autotune mode must be 0 or 1 and the candidate -1 .. 2");
    ctx->tune_mode = mode;
    ctx->tune_forced = forced_candidate;
    return 0;
}

extern "C" int lcf_autotune_candidates(const lcf_ctx* ctx, int* out9) {
    if (!ctx || !out9) return LCF_E_INVALID;
    for (int c = 0; c < N_TUNE; c++) {
        out9[3 * c] = TUNE_CAND[c].block;
        out9[3 * c + 1] = TUNE_CAND[c].smem_obs;
        out9[3 * c + 2] = ctx->cand_bps[c];
    }
    return N_TUNE;
}

extern "C" int lcf_autotune_table(const lcf_ctx* ctx, double* rows, int max_rows) {
    if (!ctx || (max_rows > 0 && !rows)) return LCF_E_INVALID;
    int n = 0;
    for (const auto& e : ctx->tune) {
        if (n >= max_rows) break;
        double* r = rows + (size_t)n * 6;
        r[0] = (double)e.bucket;
        r[1] = (double)e.best;
        r[2] = (double)e.next;
        for (int c = 0; c < N_TUNE; c++) r[3 + c] = e.ms[c];
        n++;
    }
    return (int)ctx->tune.size();
}

extern "C" int lcf_autotune_load(lcf_ctx* ctx, const double* rows, int n_rows) {
    if (!ctx || n_rows < 0 || (n_rows > 0 && !rows)) return LCF_E_INVALID;
    for (int i = 0; i < n_rows; i++) {
        const double* r = rows + (size_t)i * 6;
        int best = (int)r[1];
        if (r[0] < 0.0 || r[0] > 4294967295.0 || best < 0 || best >= N_TUNE)
            return set_err(ctx, LCF_E_INVALID, "autotune row: bad bucket or candidate");
        TuneEntry e;
        e.bucket = (uint32_t)r[0];
        e.best = best;
        e.next = N_TUNE;
        for (int c = 0; c < N_TUNE; c++) e.ms[c] = r[3 + c];
        bool found = false;
        for (auto& t : ctx->tune)
            if (t.bucket == e.bucket) { t = e; found = true; }
        if (!found) ctx->tune.push_back(e);
    }
    return 0;
}

extern "C" int lcf_last_launch(const lcf_ctx* ctx, int* out4) {
    if (!ctx || !out4) return LCF_E_INVALID;
    out4[0] = ctx->cfg;
    out4[1] = ctx->pso_block;
    out4[2] = ctx->smem_obs;
    out4[3] = (int)ctx->bucket;
    return 0;
}

extern "C" int lcf_download_outputs(lcf_ctx* ctx, lcf_fit_outputs* out) {
    if (!ctx || !out) return LCF_E_INVALID;
    if (int rc = busy(ctx)) return rc;
    return unpack_outputs(ctx, out);
}

// ---------------------------------------------------------------------------
// Batched likelihood on one band (PsoCost::cost_from_slice)
// ---------------------------------------------------------------------------
// FP32 observation records of one peak-normalised band, sorted by time
// (stable), as prep_kernel builds them for a fit; returns the last time.
// NaN times sort after all others (in input order), the order
// lcf_band_cost_static's device ranking uses.
static double band_records(const double* times, const double* flux, const double* obs_var, const uint8_t* is_upper,
                           const double* upper_flux, int n_obs, std::vector<float4>& rec) {
    std::vector<int> ord(n_obs);
    for (int i = 0; i < n_obs; i++) ord[i] = i;
    std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) {
        const bool na = std::isnan(times[a]), nb = std::isnan(times[b]);
        if (na || nb) return !na && nb;
        return times[a] < times[b];
    });
    rec.assign(std::max(n_obs, 1), make_float4(0.0f, 0.0f, 0.0f, 0.0f));
    double t_last = -INFINITY;
    for (int k = 0; k < n_obs; k++) {
        int i = ord[k];
        double t = times[i];
        t_last = std::fmax(t_last, t);
        float th = (float)t;
        bool up = is_upper[i] != 0;
        rec[k] = make_float4(th, (float)(t - (double)th), (float)(up ? upper_flux[i] : flux[i]),
                             up ? -(float)obs_var[i] : (float)obs_var[i]);
    }
    return t_last;
}

extern "C" int lcf_band_cost(lcf_ctx* ctx, int model, const double* times, const double* flux, const double* obs_var,
                             const uint8_t* is_upper, const double* upper_flux, int n_obs, const double* params,
                             int n_eval, int with_prior, double* costs) {
    if (!ctx) return LCF_E_INVALID;
    if (int rc = busy(ctx)) return rc;
    if (model < 0 || model > 7 || n_obs < 0 || n_eval < 0) return set_err(ctx, LCF_E_INVALID, "bad argument");
    if (n_eval == 0) return 0;
    CK(cudaSetDevice(ctx->device));
    std::vector<float4> rec;
    double t_last = band_records(times, flux, obs_var, is_upper, upper_flux, n_obs, rec);
    int np = n_params_of(model);
    int rc = 0;
    rc |= grow(ctx, ctx->bc_obs, rec.size() * sizeof(float4));
    rc |= grow(ctx, ctx->bc_params, (size_t)n_eval * np * 8);
    rc |= grow(ctx, ctx->bc_costs, (size_t)n_eval * 8);
    rc |= grow(ctx, ctx->bc_scratch, (size_t)((n_eval + 31) / 32) * 32 * (size_t)std::max(n_obs, 1) * 4);
    if (rc) return rc;
    cudaStream_t s = ctx->stream;
    CK(cudaMemcpyAsync(ctx->bc_obs.p, rec.data(), rec.size() * sizeof(float4), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(ctx->bc_params.p, params, (size_t)n_eval * np * 8, cudaMemcpyHostToDevice, s));
    launch_band_cost(model, (const float4*)ctx->bc_obs.p, n_obs, (float)t_last, (const double*)ctx->bc_params.p,
                     n_eval, with_prior, (double*)ctx->bc_costs.p, (float*)ctx->bc_scratch.p, s);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(costs, ctx->bc_costs.p, (size_t)n_eval * 8, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return 0;
}

extern "C" int lcf_svi_elbo_grad(lcf_ctx* ctx, int model, const double* times, const double* flux,
                                 const double* obs_var, const uint8_t* is_upper, const double* upper_flux, int n_obs,
                                 const double* prior_init, const double* var_params, int n_points, const double* eps,
                                 int n_samples, double* elbo, double* grad, int* flags) {
    if (!ctx) return LCF_E_INVALID;
    if (int rc = busy(ctx)) return rc;
    if (model < 0 || model > 7 || n_obs < 1 || n_points < 0 || n_samples < 1)
        return set_err(ctx, LCF_E_INVALID, "bad argument");
    if (!times || !flux || !obs_var || !is_upper || !upper_flux || !prior_init)
        return set_err(ctx, LCF_E_INVALID, "null band or prior pointer");
    if (n_points == 0) return 0;
    if (!var_params || !eps || !elbo || !grad || !flags) return set_err(ctx, LCF_E_INVALID, "null point pointer");
    CK(cudaSetDevice(ctx->device));
    std::vector<float4> rec;
    double t_last = band_records(times, flux, obs_var, is_upper, upper_flux, n_obs, rec);
    const int np = n_params_of(model);
    const size_t n_vp = (size_t)n_points * 2 * np, n_eps = (size_t)n_points * n_samples * np;
    int rc = 0;
    rc |= grow(ctx, ctx->bc_obs, rec.size() * sizeof(float4));
    rc |= grow(ctx, ctx->sg_in, (np + n_vp + n_eps) * 8);
    rc |= grow(ctx, ctx->sg_out, (n_points + n_vp) * 8 + (size_t)n_points * 4);
    rc |= grow(ctx, ctx->sg_scratch, (size_t)n_points * 5 * n_obs * 4);
    if (rc) return rc;
    cudaStream_t s = ctx->stream;
    double* din = (double*)ctx->sg_in.p;
    double* dout = (double*)ctx->sg_out.p;
    int* dflags = (int*)(dout + n_points + n_vp);
    CK(cudaMemcpyAsync(ctx->bc_obs.p, rec.data(), rec.size() * sizeof(float4), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(din, prior_init, (size_t)np * 8, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(din + np, var_params, n_vp * 8, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(din + np + n_vp, eps, n_eps * 8, cudaMemcpyHostToDevice, s));
    launch_svi_grad(model, (const float4*)ctx->bc_obs.p, n_obs, (float)t_last, din, din + np, n_points,
                    din + np + n_vp, n_samples, dout, dout + n_points, dflags, (float*)ctx->sg_scratch.p, s);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(elbo, dout, (size_t)n_points * 8, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(grad, dout + n_points, n_vp * 8, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(flags, dflags, (size_t)n_points * 4, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return 0;
}

extern "C" int lcf_debug_swarm_results(lcf_ctx* ctx, double* out, int64_t max_rows) {
    if (!ctx || !out) return LCF_E_INVALID;
    int64_t rows = std::min<int64_t>(max_rows, (int64_t)ctx->n_bands * 44);
    std::vector<PsoResult> h((size_t)std::max<int64_t>(rows, 1));
    if (rows > 0) CK(cudaMemcpy(h.data(), ctx->res.p, (size_t)rows * sizeof(PsoResult), cudaMemcpyDeviceToHost));
    for (int64_t r = 0; r < rows; r++) {
        double* o = out + r * 21;
        o[0] = h[r].iters < 0 ? std::nan("") : h[r].cost;
        o[1] = h[r].iters;
        o[2] = h[r].evals;
        for (int j = 0; j < MB_MAXP; j++)
            o[3 + j] = pso_param(h[r], j);
    }
    return 0;
}

extern "C" int lcf_probe_peaks(lcf_ctx* ctx, double* out2) {
    if (!ctx || !out2) return LCF_E_INVALID;
    CK(cudaSetDevice(ctx->device));
    CK(cudaDeviceSynchronize());
    out2[0] = probe_fp32_tflops(ctx->num_sms);
    out2[1] = probe_mufu_gops(ctx->num_sms);
    CK(cudaGetLastError());
    return 0;
}

extern "C" int lcf_probe_fp64(lcf_ctx* ctx, double* out9) {
    if (!ctx || !out9) return LCF_E_INVALID;
    CK(cudaSetDevice(ctx->device));
    CK(cudaDeviceSynchronize());
    if (probe_fp64_peaks(ctx->num_sms, out9)) return set_err(ctx, LCF_E_CUDA, "FP64 probe failed");
    return 0;
}

extern "C" int lcf_probe_ff(lcf_ctx* ctx, double* out80) {
    if (!ctx || !out80) return LCF_E_INVALID;
    CK(cudaSetDevice(ctx->device));
    CK(cudaDeviceSynchronize());
    for (int i = 0; i < 80; i++) out80[i] = 0.0;
    if (probe_ff(ctx->num_sms, out80)) return set_err(ctx, LCF_E_CUDA, "double-float probe failed");
    return 0;
}

// Switch CUDA-graph replay of the stage sequence on or off (on by default).
extern "C" int lcf_set_graph(lcf_ctx* ctx, int enabled) {
    if (!ctx) return LCF_E_INVALID;
    ctx->use_graph = enabled != 0;
    return 0;
}

extern "C" int lcf_set_wait_bound(lcf_ctx* ctx, int polls) {
    if (!ctx || polls < 0) return LCF_E_INVALID;
    ctx->wait_polls = polls;
    ctx->db.wait_polls = polls;
    ctx->graph_key = 0;  // the bound is a kernel argument: capture the graph again
    return LCF_OK;
}
