/*
 * nnet_gb300 — C ABI of the GB300 (sm_103a) nuclear-burn library.
 *
 * Drop-in replacement for the GPU side of SPH-EXA-nnet's per-particle burn path.  All
 * entry points take plain pointers and sizes; device arrays are caller-owned and stay
 * in place (Y, T and dt are updated in place, as in the reference).  Calls that take a
 * stream are asynchronous with respect to the host unless stated otherwise.
 *
 * Reference interfaces replaced (file:line in SPH-EXA-nnet):
 *   nnet::parallel::computeNuclearReactions<use_gpu=true>
 *                       include/nnet/parallel/parallel_nuclear_net.hpp:86-142
 *   nnet::parallel::cudaComputeNuclearReactions
 *                       include/nnet/parallel/CUDA/parallel_nuclear_net.cuh:70-75, .cu:115-163
 *   nnet::parallel::computeHelmEOS<use_gpu=true> / cudaComputeHelmholtz
 *                       include/nnet/parallel/parallel_nuclear_net.hpp:191-231,
 *                       include/nnet/parallel/CUDA/parallel_nuclear_net.cuh:77-79, .cu:216-226
 *   helmholtz::constants::readCPUTable / copyTableToGPU
 *                       include/nnet/parameterization/eos/helmholtz.cpp:89-218
 *   net87::electrons::constants::copyTableToGPU, nnet::moveToGpu(ReactionList)
 *                       include/nnet/parameterization/net87/net87.cpp:89-99,
 *                       include/nnet/CUDA/nuclear_net.cuh:61-72
 */
#ifndef NNET_GB300_H
#define NNET_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NNET_MAX_SPECIES 87

/* Return codes of every entry point. */
enum nnet_error
{
    NNET_SUCCESS         = 0,
    NNET_ERR_INVALID     = -1, /* bad argument (null pointer, unknown network, size) */
    NNET_ERR_CUDA        = -2, /* a CUDA runtime call failed; see nnet_last_error_message */
    NNET_ERR_NO_TABLE    = -3, /* Helmholtz EOS requested before a table was loaded */
    NNET_ERR_TOO_LARGE   = -4, /* request exceeds a fixed capacity */
    NNET_ERR_FILE        = -5, /* table file missing or malformed */
    NNET_ERR_ABORTED     = -6, /* nnet_get_stats: the last launch hit its time limit (time_limit_seconds) */
};

/* Per-particle outcome written to nnet_burn_args.status (int32 per particle). */
enum nnet_particle_status
{
    NNET_PARTICLE_OK       = 0, /* burned to hydro_dt */
    NNET_PARTICLE_SKIPPED  = 1, /* rho <= 1e5 or T <= 1e8: left untouched (parallel_nuclear_net_impl.cpp:83) */
    NNET_PARTICLE_LIVELOCK = 2, /* the substep loop entered a cycle: rejected attempts returned to
                                   an attempt-start state already seen (the same Newton temperature,
                                   dt equal within a relative 2^-20), so the reference would retry
                                   them forever (nuclear_net.hpp:745-748 with :899-904); Y and T
                                   are those of the last accepted substep */
    NNET_PARTICLE_MAXITER  = 3, /* Newton-iteration budget exhausted */
    NNET_PARTICLE_ZERO_DT  = 4, /* timestep underflowed to 0 (the reference throws, nuclear_net.hpp:533-549) */
    NNET_PARTICLE_ABORTED  = 5, /* the launch reached nnet_burn_args.time_limit_seconds (no reference
                                   counterpart): a particle in progress keeps its last accepted substep
                                   (Y, T) and its current timestep proposal; a particle not yet started
                                   keeps its input state */
    NNET_NUM_PARTICLE_STATUS = 6
};

enum nnet_network
{
    NNET_NET14 = 14, /* 14-isotope alpha chain, 29 reactions  (net14.hpp:69-134) */
    NNET_NET86 = 86, /* 86 isotopes, 309 reactions              (net86.hpp:95-192) */
    NNET_NET87 = 87, /* net86 + electrons, 311 reactions        (net87.hpp:88-98) */
};

enum nnet_eos
{
    NNET_EOS_IDEAL_GAS = 0, /* IdealGasFunctor(mu)             (ideal_gas.hpp:46-83) */
    NNET_EOS_HELMHOLTZ = 1, /* HelmholtzFunctor(Z of network)  (helmholtz.hpp:150-226) */
};

/* Linear-solver form of the Newton step. */
enum nnet_solver
{
    NNET_SOLVER_DENSE_FP64  = 0, /* plain form: dense Gaussian elimination in the reference's
                                    operation order (eigen.hpp:178-223), one thread per particle */
    NNET_SOLVER_SPARSE_FP64 = 1, /* fill-reducing sparse LU in FP64 */
    NNET_SOLVER_MIXED       = 2, /* sparse LU factored in FP32, FP64 residual, iterative refinement */
};

/* How the sparse and mixed solvers map particles onto the GPU (no reference counterpart;
 * the dense solver always runs one thread per particle, like the reference's kernel). */
enum nnet_layout
{
    NNET_LAYOUT_AUTO    = 0, /* library choice (currently: batched warps) */
    NNET_LAYOUT_THREAD  = 1, /* one thread per particle, Newton system in strided global scratch */
    NNET_LAYOUT_WARP    = 2, /* one warp per particle, Newton system in shared memory */
    NNET_LAYOUT_BATCHED = 3, /* 32 particles per warp in lockstep: per-particle scalar work one
                                lane per particle, each Newton system by the whole warp */
};

typedef struct nnet_context* nnet_handle;

/* Burn statistics accumulated over one nnet_burn call (device-side counters). */
typedef struct
{
    unsigned long long newton_iterations;
    unsigned long long substeps;
    unsigned long long status_count[NNET_NUM_PARTICLE_STATUS]; /* indexed by nnet_particle_status */
    unsigned long long refinement_steps; /* NNET_SOLVER_MIXED: FP64-residual refinement steps */
    unsigned long long fp64_fallbacks;   /* NNET_SOLVER_MIXED: systems re-solved in FP64 */
} nnet_stats;

/* Arguments of nnet_burn.  All arrays are DEVICE pointers of num_particles entries. */
typedef struct
{
    int           network;      /* nnet_network */
    int           eos;          /* nnet_eos */
    double        ideal_gas_mu; /* mean molecular weight for NNET_EOS_IDEAL_GAS */
    int           solver;       /* nnet_solver */
    size_t        num_particles;
    double* const* Y;           /* host array of `network` device pointers, Y[species][particle]
                                   (the reference's per-species field vectors) */
    double*       T;            /* temperature, in/out */
    const double* rho;          /* density at the end of the hydro step */
    const double* rho_m1;       /* density at the previous step (may be NULL) */
    double*       dt;           /* carried nuclear timestep, in/out */
    double        hydro_dt;     /* integration time of this call */
    double        previous_dt;  /* previous hydro step, for drho/dt */
    int           use_drhodt;   /* drho/dt = (rho - rho_m1)/previous_dt where rho_m1 != 0,
                                   as the CUDA driver does (parallel_nuclear_net.cu:80-82) */
    long long     max_newton_iterations; /* per particle; <= 0 selects 100000 */
    int32_t*      status;       /* optional, nnet_particle_status per particle */
    int32_t*      substeps;     /* optional, accepted substeps per particle */
    int32_t*      iterations;   /* optional, Newton iterations per particle */

    /* Launch watchdog (no reference counterpart).  > 0: after this many seconds of GPU time the
     * launch takes no further Newton iteration; unfinished particles end with
     * NNET_PARTICLE_ABORTED and nnet_get_stats returns NNET_ERR_ABORTED.  <= 0: no limit. */
    double        time_limit_seconds;

    /* Post-burn steps, applied after each particle's burn (no reference counterpart unless noted).
     * The reference only clips abundances at 1e-16 (nuclear_net.hpp:760) and accepts a substep
     * after 11 Newton iterations whether or not the abundances converged (:763-764), so
     * sum_i X_i drifts from 1; these steps report and remove the drift. */
    int           normalize_mass; /* nonzero: Y_i <- Y_i / sum_j A_j Y_j for every particle not
                                     skipped, so sum_i X_i = 1 to rounding (X_i = A_i Y_i; the net87
                                     electron entry has A = 0) */
    double*       mass_drift;     /* optional, per particle: sum_i A_i Y_i - 1 of the burned state,
                                     before normalisation (skipped particles: of their input state) */
    /* optional, all five or none: the post-burn Helmholtz EOS at the final (Y, T, rho) of every
     * particle, over the network's charges (computeHelmEOS, parallel_nuclear_net.hpp:191-261; needs
     * a loaded table).  The batched layout evaluates it as each particle retires; the other layouts
     * in one pass after the burn. */
    double*       u;
    double*       cv;
    double*       p;
    double*       c;
    double*       dpdT;

    /* Optional device array of num_particles particle indices, a permutation (no reference
     * counterpart): the work queue hands out particle order[k] k-th.  Per-particle results do
     * not depend on it; only the launch's schedule does.  NULL: index order. */
    const uint32_t* order;
} nnet_burn_args;

/* Create a context on `device` (network tables uploaded, no Helmholtz table yet). */
int nnet_create(int device, nnet_handle* out);
/* Release every device buffer held by the context. */
int nnet_destroy(nnet_handle h);

/* Load the Helmholtz free-energy table from host memory: 21 arrays of 541 x 201 doubles in
 * the reference's quantity order f fd ft fdd ftt fdt fddt fdtt fddtt dpdf dpdfd dpdft
 * dpdfdt ef efd eft efdt xf xfd xft xfdt, each row-major [density][temperature].
 * Synchronous.  Replaces readCPUTable + copyTableToGPU (helmholtz.cpp:89-218). */
int nnet_load_helmholtz_table(nnet_handle h, const double* table);
/* Same, from a file: the reference's text layout helm_table.dat (helmholtz.cpp:100-137, an
 * optional STR( ... ) wrapper is accepted), or the 21 x 541 x 201 little-endian doubles of
 * nnet_load_helmholtz_table written as raw bytes. */
int nnet_load_helmholtz_table_file(nnet_handle h, const char* path);

/* Burn num_particles particles over hydro_dt on `stream` (a cudaStream_t, 0 = legacy
 * default stream).  Asynchronous; the per-call statistics become readable with
 * nnet_get_stats after the stream has reached this point. */
int nnet_burn(nnet_handle h, const nnet_burn_args* args, void* stream);
/* One persistent launch over up to three sub-batches of different networks (same EOS and
 * solver): warps (batched layout; threads for the dense solver or the thread layout) drain
 * the net86, net87 and net14 work queues in that order, so the costliest particles start
 * first.  Same semantics and, per layout, the same results per particle as nnet_burn. */
int nnet_burn_batch(nnet_handle h, const nnet_burn_args* batches, int count, void* stream);
/* Copy the statistics of the last nnet_burn issued on this handle (synchronises the
 * stream of that call).  Returns NNET_ERR_ABORTED, with the statistics filled in, when that
 * launch stopped at its time limit. */
int nnet_get_stats(nnet_handle h, nnet_stats* out);

/* Post-burn Helmholtz EOS over a batch (computeHelmEOS, parallel_nuclear_net.hpp:191-231):
 * writes u, cv, p, c, dpdT per particle.  Z has `num_species` host doubles; Y is a host
 * array of device pointers.  Asynchronous on `stream`. */
int nnet_helmholtz_eos(nnet_handle h, size_t num_particles, int num_species, const double* Z,
                       const double* T, const double* rho, double* const* Y, double* u, double* cv,
                       double* p, double* c, double* dpdT, void* stream);

/* ---------------------------------------------------------------- burn server
 * Continuous batching of burn requests on one GPU (no reference counterpart: the
 * reference burns one caller-provided batch per blocking call).  Requests are admitted
 * FIFO while their device footprint fits `hbm_budget_bytes` and a workspace is free; the
 * state of an admitted request stays on the device until it completes; admitted requests
 * run concurrently as time slices of `slice_iterations` Newton iterations per particle,
 * so requests arriving while others run start as soon as memory frees up.  Slicing does
 * not change any particle's arithmetic: results equal an unsliced nnet_burn bit for bit. */
typedef struct nnet_server_s* nnet_server;

typedef struct
{
    double    hbm_budget_bytes;        /* device bytes of admitted request state; <= 0: 150e9 */
    int       solver;                  /* nnet_solver */
    long long slice_iterations;        /* Newton iterations per particle per slice; <= 0: 64 */
    int       max_concurrent_requests; /* resident requests (1..64), one workspace each */
} nnet_server_config;

typedef struct
{
    int           network, eos;
    double        ideal_gas_mu;
    size_t        num_particles;
    double*       Y;      /* HOST, species-major [network][num_particles]; overwritten with results */
    double*       T;      /* HOST, in/out */
    const double* rho;    /* HOST */
    double*       dt;     /* HOST, in/out */
    int32_t*      status; /* HOST, optional: nnet_particle_status per particle */
    double        hydro_dt;
    long long     max_newton_iterations; /* <= 0 selects 100000 */
} nnet_request;

typedef struct
{
    unsigned long long completed_requests;
    double             completed_particles;
    double             span_seconds;  /* first submission to last completion */
    double             latency_p50, latency_p95, latency_p99, latency_max; /* seconds */
    unsigned long long slices;        /* kernel launches issued */
} nnet_server_stats;

int nnet_server_create(nnet_handle h, const nnet_server_config* cfg, nnet_server* out);
/* Queue a request (host buffers must stay valid until nnet_server_wait returns). */
int nnet_server_submit(nnet_server s, const nnet_request* r, uint64_t* id);
/* done = 1 when the results are in the host buffers, -1 on failure, 0 otherwise. */
int nnet_server_query(nnet_server s, uint64_t id, int* done);
/* Block until request `id` completed; latency = completion - submission (seconds). */
int nnet_server_wait(nnet_server s, uint64_t id, double* latency_seconds);
int nnet_server_get_stats(nnet_server s, nnet_server_stats* out);
/* Finish every queued request, then release the server. */
int nnet_server_destroy(nnet_server s);

/* Operation counts of one Newton-iteration linear solve of `network` with `solver`
 * (no reference counterpart; used for roofline accounting): multiply-adds of the
 * factorisation and of one pair of triangular solves, and the stored factor entries. */
int nnet_solver_info(int network, int solver, long long* factor_fma, long long* solve_fma, int* factor_entries);
/* Measured FP64 fused-multiply-add throughput of `device` in TFLOP/s (2 flops per FMA)
 * with a dependency-free probe kernel (no reference counterpart; roofline denominator). */
int nnet_measure_fp64_peak(int device, double* tflops);

/* nnet_burn for callers that cannot allocate device memory during a time step (codes whose
 * device memory all belongs to their own arena allocator, or that cannot afford the device-wide
 * synchronisation a cudaMalloc may cause).  No counterpart in the reference.  Same arguments
 * and results as nnet_burn with the batched layout; sparse and mixed solvers only.  Allocates
 * nothing: its slot scratch (7.2 MiB, 4096 particle slots) and counters are fixed arrays that
 * every GPU loading the library holds until exit; the grid is capped to them, so any number of
 * particles is accepted.  The first call on a handle looks the arrays' device addresses up and
 * keeps them in the handle (make it before any stream capture).  Calls share the arrays: calls
 * that overlap on the GPU race, and nnet_get_stats does not report these calls. */
int nnet_burn_noalloc(nnet_handle h, const nnet_burn_args* args, void* stream);

/* Visiting order for nnet_burn_args.order with the costliest particles first (no reference
 * counterpart): a permutation of [0, num_particles) sorted by decreasing floor(log2(cost[i]))
 * (costs <= 1 last), from device arrays `cost` (int32, e.g. the previous burn's iterations)
 * into `order` (uint32).  Asynchronous on `stream`; the order within a power-of-two cost class is
 * unspecified.  The first call on a handle allocates 512 bytes of counters. */
int nnet_cost_order(nnet_handle h, size_t num_particles, const int32_t* cost, uint32_t* order, void* stream);

/* Batched layout: particles in flight per warp, 1..32 (default 32; no reference counterpart,
 * chosen by the autotuner).  Fewer slots shorten each particle's time per Newton iteration
 * (the warp serves fewer systems per round) at the price of less sharing of the per-particle
 * scalar work. */
int nnet_set_batch_slots(nnet_handle h, int slots);

/* Batched layout: rebalance the running particles over the warps once the work queue has
 * drained (default on; no reference counterpart).  A warp holding more than its share,
 * ceil(running particles / warps), hands the extra particles to warps holding fewer, each at
 * its next attempt boundary with everything that attempt depends on, so results are the same
 * bit for bit; the heaviest particles then run spread over the grid instead of queueing behind
 * one another in a few warps.  Uses 4 hand-off records (112 bytes each) per slot of the grid. */
int nnet_set_rebalance(nnet_handle h, int on);

/* Select the particle layout of the sparse and mixed solvers for later nnet_burn calls on
 * `h` (nnet_layout; no reference counterpart: chosen by the autotuner). */
int nnet_set_layout(nnet_handle h, int layout);

/* Number of species / reactions of a network, 0 on success. */
int nnet_network_info(int network, int* num_species, int* num_reactions);
/* Human-readable description of the last error on this thread. */
const char* nnet_last_error_message(void);

#ifdef __cplusplus
}
#endif

#endif /* NNET_GB300_H */
