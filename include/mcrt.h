/*
 * mcrt.h - C ABI of libmcrt, a GB300 (sm_103a) engine for polarised Monte Carlo
 * radiative transfer with coherent backscattering (CB).
 *
 * It is a drop-in for the GPU branch of the reference package's driver
 * `simulate(cfg, g, I0; use_gpu)` (MonteCarloRadiativeTransfer.jl,
 * src/MonteCarloRadiativeTransfer.jl:26-85): the package keeps its Config, scatterer and
 * geometry types and its run_rt entry point, and ccalls this library where the
 * reference launches its CUDA.jl kernel (src/MonteCarloRadiativeTransfer.jl:36-56).
 *
 * Conventions
 *   - Every call returns an int status (MCRT_OK = 0); mcrt_last_error() gives a
 *     message for the calling thread's last failure.
 *   - All arrays are plain host pointers owned by the caller; the library copies what
 *     it keeps. Tally outputs use the reference's Julia column-major layouts:
 *     Irt[4, Ntheta, Nphi] and Icb[4, Ntheta_b, Nphi_b], i.e. element (s, j1, j2) at
 *     s + 4*(j1 + Ntheta*j2), zero-based here.
 *   - Invalid geometry or configuration returns MCRT_EINVAL with the reference's
 *     validate() messages (src/geometries/plane.jl:52-62, sphere.jl:35-37), where a
 *     Julia caller rethrows ArgumentError.
 *   - There is no CPU fallback: without a usable CUDA device the compute calls return
 *     MCRT_ENODEV.
 */
#ifndef MCRT_H
#define MCRT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MCRT_ABI_VERSION 1

enum mcrt_status_code {
  MCRT_OK = 0,
  MCRT_EINVAL = 1,    /* bad argument; message via mcrt_last_error() */
  MCRT_ENOMEM = 2,    /* device or host allocation failed */
  MCRT_ECUDA = 3,     /* CUDA runtime error */
  MCRT_ENONCONV = 4,  /* a capped device loop gave up (see mcrt_stats.status_flags) */
  MCRT_ETIMEDOUT = 5, /* a wait ran out of time */
  MCRT_EBUSY = 6,     /* admission refused: over the memory cap or out of slots */
  MCRT_ENOTFOUND = 7, /* unknown ticket */
  MCRT_ENODEV = 8     /* no CUDA device */
};

enum mcrt_scatterer_kind { MCRT_RAYLEIGH = 0, MCRT_MIE = 1 };
enum mcrt_geometry_kind { MCRT_PLANE = 0, MCRT_SPHERE = 1 };
enum mcrt_precision { MCRT_FP32 = 0, MCRT_FP64 = 1 };
enum mcrt_kernel_kind {
  MCRT_KERNEL_PERSISTENT = 0, /* event-batched persistent kernel (the fast path) */
  MCRT_KERNEL_PLAIN = 1       /* one thread per ray, the structure of src/gpu.jl:177-296 */
};
enum mcrt_rng_mode {
  MCRT_RNG_PHILOX = 0,           /* Philox4x32-10 keyed by (seed, instance) */
  MCRT_RNG_STRATIFIED_DEPTH = 1  /* test mode: first-collision depth draw = (i+0.5)/N */
};
/* Bits of mcrt_stats.status_flags */
enum mcrt_status_flags {
  MCRT_FLAG_REJECT_LIMIT = 1, /* a rejection loop (src/gpu.jl:215-256) hit its cap */
  MCRT_FLAG_KEPLER_CAP = 2,   /* kepler_solver (src/utils.jl:243-261) hit its cap */
  MCRT_FLAG_NONFINITE = 4     /* a non-finite photon weight was dropped */
};

typedef struct mcrt_ctx mcrt_ctx;
typedef struct mcrt_scatterer mcrt_scatterer;
typedef struct mcrt_solve mcrt_solve;
typedef struct mcrt_batch mcrt_batch;
typedef struct mcrt_server mcrt_server;

/* Scatterer: RayleighScatterer (src/scatterers/rayleigh.jl:3-6) or the tables of
 * MieScatterer (src/scatterers/mie.jl:3-15). Mie tables are stored on the device in
 * FP32 (both precisions read the same stored values). */
typedef struct {
  int kind;        /* mcrt_scatterer_kind */
  double omega;    /* single-scattering albedo */
  double kl;       /* mean free path (the CB phase scale, src/gpu.jl:102) */
  int n_theta;     /* Mie: table length on the uniform grid 0..pi */
  const double *F11, *F12, *F33, *F34; /* Mie: n_theta each */
  const double *S11, *S22;             /* Mie: 2*n_theta each, interleaved (re, im) */
  int random_points;                   /* Mie: csrn has random_points + 1 entries */
  const double* csrn;                  /* Mie: inverse CDF of cos(theta) */
} mcrt_scatterer_desc;

/* Config (src/config.jl:55-124); the trigonometric and weight arrays are passed in. */
typedef struct {
  int64_t number_of_rays;
  double minimum_intensity;
  int64_t maximum_scattering_times;
  int64_t maximum_threads; /* used by the plain kernel only, as in the reference */
  int compute_cb;
  double tau0;
  int n_phi;
  const double *cos_phi, *sin_phi;
  int n_theta;
  const double *cos_theta, *sin_theta, *inorm;
  int n_theta_b;
  const double *cos_theta_b, *sin_theta_b;
  int n_phi_b;
  const double *cos_phi_b, *sin_phi_b;
} mcrt_config;

/* Layer (src/geometries/plane.jl:6-21); for a sphere the single layer's tau is the
 * optical radius (src/geometries/sphere.jl:6-21). */
typedef struct {
  double tau;
  double omega;
  int infinite; /* plane only: a semi-infinite last layer (d < 0) */
  const mcrt_scatterer* scatterer;
} mcrt_layer;

typedef struct {
  int kind;            /* mcrt_geometry_kind */
  double theta, phi;   /* plane incidence angles; ignored for a sphere (pi, 0) */
  int n_layers;        /* sphere: 1 */
  const mcrt_layer* layers;
} mcrt_geometry;

/* Launch options; zero-initialised means: FP32, persistent kernel, Philox, autotuned. */
typedef struct {
  int precision;        /* mcrt_precision */
  int kernel;           /* mcrt_kernel_kind */
  uint64_t seed;
  uint32_t instance;    /* Philox key word (one per simulate call of a run_rt) */
  int rng_mode;         /* mcrt_rng_mode */
  int64_t photon_begin; /* first photon index (sub-runs continue a stream) */
  int block_size;       /* persistent: 0 = autotuned; FP32 256, 512, 768 (or 128); FP64 128, 256 */
  int blocks_per_sm;    /* persistent: 0 = autotuned (or the most that fit) */
  int plain_threads;    /* plain: 0 = min(maximum_threads, number_of_rays) */
  int table_staging;    /* persistent: 0 = autotuned, 1 = shared memory, 2 = global memory (L1) */
  int64_t max_attempts; /* cap of every rejection loop; 0 = 2^20. A loop that reaches it ends its
                           photon and sets MCRT_FLAG_REJECT_LIMIT (the call returns MCRT_ENONCONV). */
} mcrt_run_opts;

/* Diagnostics returned beside the tallies (all raw sums over the photons run). */
typedef struct {
  double cb_peak_sum;    /* per-photon sum of its CB peak (s11 at theta_b = 0) */
  double cb_peak_sumsq;  /* per-photon sum of squares of the same */
  double photons;
  double events;         /* scattering events */
  double attempts;       /* rejection-loop attempts */
  double rt_evals;       /* RT peel-off bin evaluations */
  double cb1_evals;      /* CB single-scattering bin evaluations */
  double cbn_evals;      /* CB reciprocal-path bin evaluations */
  double kernel_ms;      /* device time of the transport launch (CUDA events) */
  int status_flags;      /* mcrt_status_flags */
  int block_size, blocks; /* launch shape that ran */
} mcrt_stats;

/* ------------------------------------------------------------------ basics */
int mcrt_abi_version(void);
const char* mcrt_last_error(void);
/* Number of CUDA devices visible (0 without a GPU); never fails. */
int mcrt_device_count(void);

/* Context bound to one device: streams, autotuner cache, scratch pools. */
int mcrt_ctx_create(int device, mcrt_ctx** out);
int mcrt_ctx_destroy(mcrt_ctx* ctx);

/* Uploads the scatterer (replaces the adapt(CuArray, ...) of
 * src/MonteCarloRadiativeTransfer.jl:92-99,194-199). */
int mcrt_scatterer_create(mcrt_ctx* ctx, const mcrt_scatterer_desc* desc, mcrt_scatterer** out);
int mcrt_scatterer_destroy(mcrt_scatterer* s);
/* Single-scattering albedo and mean free path of a scatterer (for scatterers whose
 * tables were made on the device). */
int mcrt_scatterer_params(const mcrt_scatterer* s, double* omega, double* kl);

/* Host-side table producer for MieScatterer(r, m, lambda, nu; Ntheta, random_points)
 * (src/scatterers/mie.jl:36-44, bhmie :129-216, calculate_csrn src/utils.jl:263-287).
 * Outputs: omega, kl; F11,F12,F33,F34 (n_theta each); S11,S22 (2*n_theta, re/im);
 * csrn (random_points+1); q[5] = (q_ext, q_sca, q_abs, q_back, asymm). No GPU needed. */
int mcrt_mie_tables(double r, double m_re, double m_im, double lambda, double nu, int n_theta,
                    int random_points, double* omega, double* kl, double* F11, double* F12,
                    double* F33, double* F34, double* S11, double* S22, double* csrn, double* q);

/* The same table producer on the device, for n scatterers in one launch (one thread
 * block each): MieScatterer(r[i], m_re[i] + i m_im[i], lambda[i], nu[i]; n_theta,
 * random_points) becomes out[i], a scatterer whose FP32 tables are written on the
 * device and never pass through host memory (for a serving stream in which requests
 * bring new size parameters and refractive indices). tables (optional, host) receives
 * per scatterer 7 + 8*n_theta + random_points + 1 doubles: omega, kl, q[5] (as in
 * mcrt_mie_tables), F11, F12, F33, F34, S11 (re/im), S22 (re/im), csrn. */
int mcrt_mie_scatterers_create(mcrt_ctx* ctx, int n, const double* r, const double* m_re, const double* m_im,
                               const double* lambda, const double* nu, int n_theta, int random_points,
                               mcrt_scatterer** out, double* tables);

/* ------------------------------------------------------------------ simulate */
/* The drop-in for simulate(cfg, g, I0; use_gpu=true): runs cfg.number_of_rays photons
 * and returns A_out = (Adt, Aabs, Aref, Atrans, Arem), Irt and Icb, all divided by
 * number_of_rays as src/MonteCarloRadiativeTransfer.jl:78-84 does. Icb_ladder
 * (optional, Ntheta_b*Nphi_b) is the incoherent s11 counterpart of Icb; stats is
 * optional. Synchronous, like the reference (which syncs at :51-56). */
int mcrt_simulate(mcrt_ctx* ctx, const mcrt_config* cfg, const mcrt_geometry* g,
                  const double I0[4], const mcrt_run_opts* opts, double A_out[5], double* Irt,
                  double* Icb, double* Icb_ladder, mcrt_stats* stats);

/* ------------------------------------------------------------------ resident solves */
/* A solve keeps its inputs (bin tables, instance descriptor) and its FP64 tallies
 * resident in device memory, so it can be run repeatedly without host traffic. */
int mcrt_solve_create(mcrt_ctx* ctx, const mcrt_config* cfg, const mcrt_geometry* g,
                      const double I0[4], const mcrt_run_opts* opts, mcrt_solve** out);
/* Zeroes the tallies and launches the transport of n_photons photons starting at
 * photon index photon_begin, asynchronously on the context's stream. */
int mcrt_solve_launch(mcrt_solve* s, int64_t photon_begin, int64_t n_photons);
/* Waits for the solve and copies raw (undivided) sums to the host; any pointer may be
 * NULL. */
int mcrt_solve_read(mcrt_solve* s, double A_out[5], double* Irt, double* Icb, double* Icb_ladder,
                    mcrt_stats* stats);
int mcrt_solve_destroy(mcrt_solve* s);

/* ------------------------------------------------------------------ batched launch */
/* Many independent simulate() instances (each with its own geometry, scatterers,
 * incident Stokes vector, seed and photon budget) run in one persistent launch from
 * per-instance work queues. Instances of one batch share the config's bin grids. */
typedef struct {
  const mcrt_geometry* geometry;
  double I0[4];
  uint64_t seed;
  uint32_t instance;
  int64_t n_photons;
} mcrt_instance;

int mcrt_batch_create(mcrt_ctx* ctx, const mcrt_config* cfg, const mcrt_instance* inst,
                      int n_inst, const mcrt_run_opts* opts, mcrt_batch** out);
int mcrt_batch_launch(mcrt_batch* b);
/* Per-instance raw sums for instance i (any output pointer may be NULL). */
int mcrt_batch_read(mcrt_batch* b, int i, double A_out[5], double* Irt, double* Icb,
                    double* Icb_ladder, mcrt_stats* stats);
/* Device time of the last launch and the total photons it ran. */
int mcrt_batch_timing(mcrt_batch* b, double* kernel_ms, double* photons);
int mcrt_batch_destroy(mcrt_batch* b);

/* ------------------------------------------------------------------ run_rt */
/* run_rt(cfg, g) of src/MonteCarloRadiativeTransfer.jl:87-291: the Mueller matrices of
 * the reflected (RT) and coherently backscattered (CB) light. The reference calls
 * simulate once per incident polarisation state (plane.jl:70-75: 6 states; sphere.jl:
 * 49-52: 2 states); here the states run as one batched launch (state i with Philox
 * instance opts->instance + i, the same stream as an mcrt_simulate with that instance)
 * and a device epilogue assembles the matrices from the device tallies.
 * Outputs (caller-allocated host memory), element s_ab at index 4(a-1)+(b-1):
 *   plane:  M_rt[16][Nphi][Ntheta], M_cb[16][Nphi_b][Ntheta_b] (the reference's
 *           DataFrame rows, theta fastest);
 *   sphere: M_rt[16][Ntheta], M_cb[16][Ntheta_b].
 *   energy[5] = {direct transmission, absorption, reflection, transmission (0 for a
 *   sphere), remaining}: the G sums that the reference logs (MonteCarloRadiativeTransfer.jl
 *   :113-118 and :161-165 for a sphere, :217-223 and :250-255 for a plane).
 * stats (optional) sums the states' counters. Persistent kernel only. */
int mcrt_run_rt(mcrt_ctx* ctx, const mcrt_config* cfg, const mcrt_geometry* g, const mcrt_run_opts* opts,
                double* M_rt, double* M_cb, double energy[5], mcrt_stats* stats);

/* ------------------------------------------------------------------ serving loop */
/* A continuous-batching request loop in front of the persistent kernel. Requests (each
 * a simulate() instance with its own config, geometry, scatterers, I0, seed and photon
 * budget) are admitted while the resident device footprint (the request's Mie tables,
 * bin tables and tallies) stays under memory_cap_bytes and fewer than max_active are
 * resident; their state stays on the device until they finish. A worker thread runs
 * waves: each wave is one persistent launch in which every active request processes up
 * to its share of wave_photons photons, replayed from a captured CUDA graph; requests
 * that arrive while a wave runs join a following wave, so their work overlaps others'
 * on the device. Each request's photons are fixed by its (seed, instance) streams and
 * photon indices, so its result does not depend on what it ran beside. */
typedef struct {
  double memory_cap_bytes; /* admission cap on the resident footprint (0 = 20e9) */
  int max_active;          /* most requests resident at once (0 = 256) */
  int64_t wave_photons;    /* photons per wave, shared by the active requests (0 = 1<<20) */
  int64_t min_quantum;     /* at least this many photons per request per wave (0 = 4096) */
  int precision;           /* mcrt_precision */
  int use_graphs;          /* 0 = direct launches, 1 = replay captured CUDA graphs */
  double wave_work;        /* 0: photon quanta (above). > 0: bin evaluations per wave shared
                            * equally by the active requests, each request's photon quantum
                            * being its share over its cost per photon (estimated before its
                            * first wave, measured after each); measured slower on the mixed
                            * stream than photon quanta, kept as an option */
} mcrt_server_opts;

typedef struct {
  const mcrt_config* config;
  const mcrt_geometry* geometry;
  double I0[4];
  uint64_t seed;
  uint32_t instance;
  int64_t n_photons;
} mcrt_request;

typedef struct {
  double submitted_s, admitted_s, completed_s; /* on the server's monotonic clock */
  double footprint_bytes;
  int64_t photons;
  int waves;      /* waves the request took part in */
  int status_flags;
} mcrt_ticket_info;

int mcrt_server_create(mcrt_ctx* ctx, const mcrt_server_opts* opts, mcrt_server** out);
/* Copies the request (the scatterers must outlive it) and queues it; returns a ticket. */
int mcrt_server_submit(mcrt_server* s, const mcrt_request* r, uint64_t* ticket);
/* MCRT_OK once the ticket's result is ready, MCRT_ETIMEDOUT if not within timeout_ms. */
int mcrt_server_wait(mcrt_server* s, uint64_t ticket, double timeout_ms);
/* The result divided by the request's photon count (as mcrt_simulate returns it), then
 * releases the ticket; any output pointer may be NULL. */
int mcrt_server_result(mcrt_server* s, uint64_t ticket, double A_out[5], double* Irt, double* Icb,
                       double* Icb_ladder, mcrt_ticket_info* info);
/* out[0..7] = completed, photons completed, waves, busy seconds, peak resident bytes,
 * resident bytes, pending, active. */
int mcrt_server_stats(mcrt_server* s, double out[8]);
int mcrt_server_destroy(mcrt_server* s);

/* ------------------------------------------------------------------ no device allocation */
/* Size of the device array that mcrt_simulate_noalloc works in (24 MiB). */
#define MCRT_NOALLOC_SCRATCH_BYTES (24u << 20)

/* mcrt_simulate without device allocation. No counterpart in the reference.
 *
 * Same arguments, outputs and results as mcrt_simulate on the persistent kernel, for
 * callers that must not allocate device memory when they call: for example a host
 * application whose device memory is entirely reserved by its own allocator at start
 * up, or a loop that is not allowed to allocate once it runs. It calls no cudaMalloc,
 * cudaFree or other device allocator. Everything the call needs on the device besides
 * the caller's scatterers (created beforehand with mcrt_scatterer_create) lives in one
 * file-scope device array of MCRT_NOALLOC_SCRATCH_BYTES bytes, which every GPU that
 * loads the library holds until the process exits: the instance descriptor, the bin
 * tables, the tallies, the work counters and the photon-state pool.
 *
 * - The array is created on a device, and the kernels this call launches are loaded
 *   there, when the first context on that device is created (mcrt_ctx_create looks up
 *   the array's device address with that device current). A caller that reserves the
 *   device's memory itself creates its context, and its scatterers, before it does.
 * - It runs one block per SM (256 threads in FP32, 128 in FP64, Mie tables staged in
 *   shared memory), so it is slower than mcrt_simulate. In opts, block_size must be 0
 *   or that size, blocks_per_sm 0 or 1, table_staging 0 or 1, and kernel the persistent
 *   one; other values are rejected with MCRT_EINVAL.
 * - A config whose bin tables and tallies do not fit in the array beside the
 *   photon-state pool is rejected with MCRT_EINVAL and a message giving both sizes.
 * - Every call reuses the same array: each call clears the tallies and counters it
 *   needs before its launch, and calls that overlap on the GPU (from several threads or
 *   contexts on one device) race on the array and must be serialised by the caller. */
int mcrt_simulate_noalloc(mcrt_ctx* ctx, const mcrt_config* cfg, const mcrt_geometry* g,
                          const double I0[4], const mcrt_run_opts* opts, double A_out[5],
                          double* Irt, double* Icb, double* Icb_ladder, mcrt_stats* stats);

/* ------------------------------------------------------------------ measurement */
/* Measured FP32 FMA throughput of this device (TFLOP/s, FMA = 2 flops) from a short
 * dependent-FMA microbenchmark; used as the roofline peak of the transport kernel. */
int mcrt_measure_fp32_peak(mcrt_ctx* ctx, double* tflops);

#ifdef __cplusplus
}
#endif

#endif /* MCRT_H */
