/*
 * swept1d -- GB300 (sm_103a) swept-rule and classic solvers for the 1D heat
 * (FTCS), Kuramoto-Sivashinsky and Euler/Sod problems.  C ABI.
 *
 * The reference (Niemeyer-Research-Group/1DSweptCUDA) has no library: its
 * public surface is three programs, SweptSource/{Heat,KS,Euler}1D_SweptShared.cu,
 * built as bin/<Problem><Single|Double>Out and driven by argv
 * (`nx tpb dt tf freq alg solution.dat [timing.txt]`).  Each entry point below
 * replaces one piece of those programs; the citation is on each declaration.
 * bin/<Problem><Precision>Out of this project is a thin main() over
 * sw_cli_main().
 *
 * Conventions
 *  - Every function returns SW_OK (0) or a negative SW_ERR_* code; nothing
 *    throws across the ABI.  sw_strerror() names a code, sw_ctx_last_error()
 *    gives the message of the last failure on a context.
 *  - Host state layout (ic_host / final_host / snapshots): REAL[nx] for Heat
 *    and KS; REAL[3*nx] of (rho, rho*u, E) per cell for Euler -- the layout of
 *    the reference's REAL / REALthree host arrays.  REAL is float when
 *    precision == 4, double when precision == 8.
 *  - Device state layout (sw_run_device): REAL[nx] for Heat/KS; for Euler
 *    REAL[4*nx] of (rho, rho*u, E, pad) per cell (a double4/float4 array).
 *  - A context owns one CUDA stream and the device work buffers; it is
 *    reusable across runs and is not thread-safe (one host thread at a time).
 */
#ifndef SWEPT1D_H
#define SWEPT1D_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SW_ABI_VERSION 1

/* ---------------------------------------------------------------- codes */
enum sw_status {
    SW_OK = 0,
    SW_ERR_ARG = -1,         /* null pointer or unknown enum value */
    SW_ERR_SIZE = -2,        /* nx / tpb rule broken (Heat1D_SweptShared.cu:735-740) */
    SW_ERR_UNSTABLE = -3,    /* Euler dt/dx > 0.21 (Euler1D_SweptShared.cu:1168-1172) */
    SW_ERR_CUDA = -4,        /* a CUDA call or kernel failed */
    SW_ERR_NOMEM = -5,       /* device or pinned host allocation failed */
    SW_ERR_IO = -6,          /* output file could not be opened or written */
    SW_ERR_TIMEOUT = -7,     /* a kernel's bounded wait (inter-block flags, a bulk copy) ran out; state not valid */
    SW_ERR_UNSUPPORTED = -8, /* valid request this library does not provide */
    SW_ERR_CALLBACK = -9,    /* the snapshot callback asked to stop */
    SW_ERR_USAGE = -10       /* too few command-line arguments (argc < 8) */
};

enum sw_problem { SW_HEAT = 0, SW_KS = 1, SW_EULER = 2 };

/* alg: the reference's 6th argument (Heat1D_SweptShared.cu:717) */
enum sw_alg {
    SW_ALG_CLASSIC = 0,  /* one launch per (sub-)step, ping-pong arrays */
    SW_ALG_SWEPT = 1,    /* shared-memory swept rule: up-triangle, diamonds, down-triangle */
    SW_ALG_VARIANT = 2,  /* GPU-only variant: persistent swept kernel (Heat, Euler);
                            KS: 32-point warp nodes, the reference's register path cycle */
    SW_ALG_SELFTEST = 3  /* KS only: warp-node kernels vs shared kernels (KS1D_SweptShared.cu:681-751) */
};

enum sw_bc {
    SW_BC_DEFAULT = 0,   /* the reference's: Heat mirror, KS periodic, Euler Dirichlet */
    SW_BC_MIRROR = 1,    /* insulated ends (Heat) */
    SW_BC_PERIODIC = 2,  /* periodic (Heat, KS) */
    SW_BC_DIRICHLET = 3  /* cells 0 and nx-1 held at the boundary states (Euler) */
};

enum sw_time_mode {
    SW_TIME_REFERENCE = 0, /* the reference wrappers' t_eq bookkeeping from dt, tf, freq */
    SW_TIME_STEPS = 1      /* exactly n_steps time steps (swept finishes the remainder classically) */
};

/* sw_config.flags */
enum sw_flag {
    /* KS: divide by 4 dx, dx^2 and dx^4 instead of multiplying by their
     * reciprocals -- the reference's DIVISE build (KS1D_SweptShared.cu:111-132,
     * 904-914), kept for its divide-vs-multiply timing study.  At a power-of-two
     * dx (the reference's 0.5) both forms give the same bits. */
    SW_FLAG_KS_DIVIDE = 1,
    /* The hybrid variant (the reference's alg 2 for Heat and Euler,
     * Heat1D_SweptShared.cu:410-468,550-644; Euler1D_SweptShared.cu:761-835,
     * 935-1050): in every phase-1 pass the tile that straddles the domain's
     * ends is computed on the host CPU while the GPU computes the others; its
     * two slots go down and back by copies on the run's stream.  Same results
     * bit for bit.  With alg 1 (any problem) or alg 2 (Heat, Euler; then run as
     * alg 1 with the host tile, as the reference's alg 2 is); not with
     * SW_FLAG_KS_DIVIDE.  The sw_run / sw_run_device runs only. */
    SW_FLAG_HOST_TILE = 2
};

/* ------------------------------------------------------------ run config */
typedef struct sw_config {
    int32_t problem;     /* enum sw_problem */
    int32_t precision;   /* 4 = float (Single), 8 = double (Double) */
    int32_t alg;         /* enum sw_alg */
    int32_t bc;          /* enum sw_bc */
    int64_t nx;          /* spatial points (argv[1]) */
    int32_t tpb;         /* points per swept node (argv[2]; the reference runs a thread per point) */
    int32_t time_mode;   /* enum sw_time_mode */
    double dt;           /* time step (argv[3]) */
    double tf;           /* finish time as given (argv[4]); the library applies tf - dt/4 like main() */
    double freq;         /* output interval (argv[5]); <= 0 or >= tf: no intermediate snapshots */
    int64_t n_steps;     /* SW_TIME_STEPS only */
    /* physics; 0 selects the reference's constant */
    double dx;           /* Heat 0.001, KS 0.5, Euler 1/(nx-2) */
    double alpha;        /* Heat diffusivity 8.418e-5 */
    double gamma;        /* Euler heat-capacity ratio 1.4 */
    double left[3];      /* Euler left state (rho, u, p); all 0 = Sod (1, 0, 1) */
    double right[3];     /* Euler right state (rho, u, p); all 0 = Sod (0.125, 0, 0.1) */
    int32_t threads;     /* threads per swept tile: 0 = the library's default for the tile width (on
                            a domain of >= 1024 tiles one block may then hold several tiles); a
                            multiple of 32 up to min(tpb, 512) (Euler 256), else the default */
    int32_t flags;       /* enum sw_flag bits; 0 = none */
} sw_config;

/* Derived constants, rounded to the run's precision exactly as the
 * reference's main() rounds them (Heat1D_SweptShared.cu:719-728,
 * KS1D_SweptShared.cu:917-926, Euler1D_SweptShared.cu:1127-1154). */
typedef struct sw_constants {
    double fourier, fourier_two;                  /* Heat */
    double dx_times4, dx2, dx4, dt, dt_half;      /* KS (reciprocals; the divisors under SW_FLAG_KS_DIVIDE) */
    double gam, mgam, dt_dx;                      /* Euler */
    double bd[6];                                 /* Euler boundary states (rho, rho u, E) x 2 */
    double lx, dx;                                /* domain length and spacing as the .dat header prints them */
} sw_constants;

typedef struct sw_result {
    double t_final;     /* simulated time reached, as the reference wrappers return it (t_eq) */
    int64_t n_steps;    /* time steps actually advanced */
    double elapsed_ms;  /* event time around the whole run: allocation, copies, stepping, snapshots */
    double us_per_step; /* elapsed_ms*1e3 / (t_final/dt): the reference's timing-file figure */
    double kernel_ms;   /* device time of the stepping launches alone */
    int64_t launches;   /* kernel launches issued */
    int32_t snapshots;  /* intermediate snapshots delivered */
    int32_t tile;       /* tile width used by the swept / variant path */
} sw_result;

/* Intermediate output, called with the host state at each output time
 * (replaces the in-wrapper .dat row writes, Heat1D_SweptShared.cu:497-509,
 * 660-678).  Return 0 to continue, non-zero to stop the run. */
typedef int (*sw_snapshot_fn)(void *user, double t, const void *state_host, int64_t nx);

typedef struct sw_ctx sw_ctx;

/* ---------------------------------------------------------- entry points */
int sw_abi_version(void);
const char *sw_strerror(int code);

/* Create / destroy a context on a CUDA device (replaces cudaSetDevice(GPUNUM)
 * and the per-run cudaMalloc/cudaFree pairs, Heat1D_SweptShared.cu:709,
 * 530-536, 688-692). */
int sw_ctx_create(int device, sw_ctx **out);
int sw_ctx_destroy(sw_ctx *ctx);
const char *sw_ctx_last_error(const sw_ctx *ctx);

/* Fill a config with the reference's defaults for a problem/precision. */
int sw_config_init(sw_config *cfg, int problem, int precision);

/* main()'s input checks (Heat1D_SweptShared.cu:735-740, KS1D_SweptShared.cu:897-902,
 * Euler1D_SweptShared.cu:1161-1172). */
int sw_validate(const sw_config *cfg);

/* The derived constants (main(), see sw_constants). */
int sw_constants_of(const sw_config *cfg, sw_constants *out);

/* The reference's initial condition, initFun (Heat1D_SweptShared.cu:60-66,751-754;
 * KS1D_SweptShared.cu:67-72,945; Euler1D_SweptShared.cu:1179). */
int sw_initial_condition(const sw_config *cfg, void *ic_host);

/* One run from a host initial condition to a host final state: replaces
 * classicWrapper / sweptWrapper (Heat1D_SweptShared.cu:470-695,
 * KS1D_SweptShared.cu:595-864, Euler1D_SweptShared.cu:837-1110).
 * cb may be NULL. */
int sw_run(sw_ctx *ctx, const sw_config *cfg, const void *ic_host, void *final_host,
           sw_snapshot_fn cb, void *user, sw_result *out);

/* The same run on a device-resident state (updated in place, device layout),
 * enqueued on `stream` (a cudaStream_t; NULL = the context's stream).  No
 * snapshots; returns when the run has completed. */
int sw_run_device(sw_ctx *ctx, const sw_config *cfg, void *state_dev, void *stream, sw_result *out);

/* One pass of the swept decomposition (the reference's upTriangle,
 * wholeDiamond / splitDiamond or downTriangle launch; Heat1D_SweptShared.cu:
 * 147-408, KS1D_SweptShared.cu:209-394, Euler1D_SweptShared.cu:437-746) over
 * all tiles of the domain, enqueued on `stream` (NULL = the context's), not
 * waited for.  cfg->alg must be SW_ALG_SWEPT; the tile width is cfg->tpb,
 * the threads per tile cfg->threads.  mode 0 = up-triangle (phase must be
 * 0): state -> slots; 1 = diamond: slots -> slots; 2 = down-triangle: slots
 * -> state.  Phase 0 tiles start at t*tpb, phase 1 tiles at t*tpb + tpb/2
 * (mod nx); diamonds alternate phases 1, 0, 1, ... after the up-triangle.
 *
 * slots_dev holds 2*nx cells (device layout) of edge slots, one of tpb cells
 * per half-tile: half-tile h (cells [h*tpb/2, (h+1)*tpb/2)) owns slot cells
 * [h*tpb, (h+1)*tpb).  A phase-1 pass reads and writes slot 0 only through
 * the last tile, the one whose cells wrap from nx-1 to 0, and in the
 * down-triangle that tile writes state cells [0, tpb/2).  A periodic domain
 * split into parts that run their passes as periodic domains of their own
 * therefore needs only that slot (before and after each phase-1 pass) and
 * those cells (after a phase-1 down-triangle) moved between neighbours; the
 * package's split.py does this across devices or processes.  The kernels'
 * bounded waits (on their bulk copies) are not reported by this call, which
 * does not wait for them; sw_run_device reports them as SW_ERR_TIMEOUT. */
int sw_swept_pass(sw_ctx *ctx, const sw_config *cfg, int32_t mode, int32_t phase, void *state_dev, void *slots_dev,
                  void *stream);

/* What a run would do, without a device: the time bookkeeping of
 * classicWrapper / sweptWrapper (Heat1D_SweptShared.cu:483-510,541-682;
 * KS1D_SweptShared.cu:609-631,676-851; Euler1D_SweptShared.cu:855-888,924-1100).
 * Fills the final t_eq, the time steps advanced and the snapshot count; if
 * snap_t / snap_steps are non-NULL, up to `cap` snapshot times and the step
 * count at each are written. */
typedef struct sw_plan_info {
    double t_final;
    int64_t n_steps;
    int32_t n_snapshots;
    int32_t tile;        /* swept / variant tile width (0 for classic) */
    int64_t launches;    /* kernel launches the run will issue (launch-per-pass paths) */
} sw_plan_info;
int sw_plan(const sw_config *cfg, sw_plan_info *out, double *snap_t, int64_t *snap_steps, int32_t cap);

/* ---------------------------------------------------------- ensembles
 * No counterpart in the reference, which solves one domain per program run:
 * many independent domains of uneven length advanced together, in one launch
 * per swept pass (alg 1) or one persistent cooperative launch (alg 2), the
 * whole sequence captured in a CUDA graph and replayed while the shape is
 * unchanged.  cfg->time_mode must be SW_TIME_STEPS; cfg->nx is ignored, the
 * domain lengths are nx[0..n_domains-1]; cfg->tpb is the tile width (it must
 * divide every domain; 0 = take the autotuner's choice) and cfg->threads the
 * threads per block.  State: the domains concatenated in order, in the host
 * (sw_run_batch) or device (sw_run_batch_device) layout. */
typedef struct sw_tuning {
    int32_t tile;                 /* chosen tile width; a swept cycle is tile/(R*S) time steps */
    int32_t threads;              /* chosen threads per block */
    double cell_updates_per_s;    /* measured rate of the choice */
    int32_t n_candidates;
    int32_t cand_tile[48];
    int32_t cand_threads[48];
    double cand_rate[48];
} sw_tuning;

int sw_run_batch(sw_ctx *ctx, const sw_config *cfg, int32_t n_domains, const int64_t *nx, const void *ic_host,
                 void *final_host, sw_result *out);
int sw_run_batch_device(sw_ctx *ctx, const sw_config *cfg, int32_t n_domains, const int64_t *nx, void *state_dev,
                        void *stream, sw_result *out);
/* Autotuner: times every valid (tile width, threads per block) pair on a
 * sample of the ensemble (every k-th domain, at least 2^22 cells where there
 * are that many) for the same number of time steps, and returns the fastest.
 * The choice is remembered by the context for this ensemble shape. */
int sw_query_tuning(sw_ctx *ctx, const sw_config *cfg, int32_t n_domains, const int64_t *nx, sw_tuning *out);

/* ------------------------------------------------------------ KS closure
 * No counterpart in the reference (the learned extension): a 3-layer 1D
 * convolution, 1 -> 32 -> 32 -> 1 channels, kernel 5, GELU, circular padding
 * per domain, that corrects a 4x-coarsened KS step:
 *     u(t + dt) = coarse KS step(u(t)) + f(u(t)).
 * Parameters are SW_CLOSURE_PARAMS FP32 values laid out
 *     w1[32][5] b1[32] | w2[32][32][5] b2[32] | w3[32][5] b3[1] | s[1]
 * (w[out][in][tap], tap t multiplies u[x + t - 2]); f(u) = s * net(u), the
 * output scale s is chosen by the caller (e.g. the spread of the training
 * targets) and never trained.  Weights are rounded to BF16 for the forward
 * pass; the 32 -> 32 layer runs on the tensor cores (BF16 x BF16,
 * FP32 accumulation), forward and backward.  Every array argument is a
 * device pointer; states are float32 domains of n cells (n a multiple of
 * 128) stored one after another.  The calls run on the context's stream,
 * after the work already queued on the legacy default stream, and return
 * when done. */
#define SW_CLOSURE_PARAMS 5506
/* delta = f(u) for n_dom domains. */
int sw_closure_infer(sw_ctx *ctx, const float *theta, const float *u, float *delta, int32_t n_dom, int64_t n);
/* n_steps coarse KS steps (coarse: problem SW_KS, precision 4, its dt and dx)
 * fused with the closure (use_closure = 0: the plain coarse step, theta may
 * then be NULL), in place. */
int sw_closure_step(sw_ctx *ctx, const sw_config *coarse, const float *theta, float *u, int32_t n_dom, int64_t n,
                    int64_t n_steps, int32_t use_closure, sw_result *out);
/* Loss L = mean over points of (net(u) - target / s)^2 over the n_dom domains
 * (rows[d] selects the sample for domain d when rows is non-NULL) and its
 * gradient: grad_and_loss[0..SW_CLOSURE_PARAMS-1] = dL/dtheta (0 for s),
 * [SW_CLOSURE_PARAMS] = L. */
int sw_closure_grad(sw_ctx *ctx, const float *theta, const float *u, const float *target, const int64_t *rows,
                    int32_t n_dom, int64_t n, float *grad_and_loss);
/* One Adam step (beta1 0.9, beta2 0.999, eps 1e-8) on the FP32 parameters; m, v zero at step 1. */
int sw_closure_adam(sw_ctx *ctx, float *theta, const float *grad, float *m, float *v, int32_t step, float lr);
/* `steps` Adam steps on minibatches of `batch` samples drawn (seeded) from
 * n_samples (input, target) pairs of n cells; loss_host (optional, host,
 * `steps` floats) receives the loss of each step. */
int sw_closure_train(sw_ctx *ctx, float *theta, const float *inputs, const float *targets, int64_t n_samples,
                     int64_t n, int32_t batch, int32_t steps, float lr, uint64_t seed, float *loss_host);
/* The certified coarse run of an ensemble (no counterpart in the reference):
 * n_dom domains of n_fine FP64 cells at t0 (fine0, device) are coarse-grained
 * by `factor` into u_out (n_dom x n_fine/factor FP32, device) and advanced
 * coarse_steps coarse steps (`coarse`: KS FP32; each coarse step is `factor`
 * steps of `fine`, a KS FP64 swept config) segment by segment.  The judge is
 * the fine solver on a second context, `judge`: it advances the exact fine
 * state of the sample d = shadow_offset, shadow_offset + shadow_every, ...
 * ahead of each segment.  In the first segment both the closure-corrected
 * and the plain coarse step advance the sample and the one nearer the
 * coarse-grained shadow (mean relative L2 error) advances the ensemble; after
 * that the ensemble runs the pick while the other variant runs on the sample,
 * and the pick switches when the other ends a segment nearer.  The sample's
 * mean relative L2 error is the certificate: when it passes tau, or its last
 * growth extrapolated linearly to the end passes tau, every domain is solved
 * by the fine solver from fine0 instead (info->fallback = 1), so u_out is
 * then the coarse-grained fine solution.  log_out (optional, host) receives
 * up to log_cap rows of (coarse steps done, variant 0 plain / 1 closure,
 * certificate, the other variant's error). */
typedef struct sw_adaptive_info {
    int32_t closure_segments;   /* segments the ensemble ran with the closure */
    int32_t plain_segments;     /* segments it ran with the plain coarse step */
    int32_t fallback;           /* 1: the fine solver's answer was returned */
    int32_t n_shadow;           /* domains in the judge's sample */
    int32_t n_log;              /* rows written to log_out */
    double shadow_mean_rel_l2;  /* the last kept segment's certificate */
    double shadow_max_rel_l2;   /* the sample's largest error then */
} sw_adaptive_info;
int sw_closure_adaptive(sw_ctx *ctx, sw_ctx *judge, const sw_config *coarse, const sw_config *fine,
                        const float *theta, const double *fine0, int32_t n_dom, int64_t n_fine, int32_t factor,
                        int64_t coarse_steps, int64_t segment, double tau, int32_t shadow_every,
                        int32_t shadow_offset, float *u_out, sw_adaptive_info *info, double *log_out,
                        int32_t log_cap);
/* Cell averages of `factor` consecutive fine FP64 cells into FP32 coarse cells. */
int sw_coarse_grain(sw_ctx *ctx, const double *fine, float *coarse, int64_t n_coarse_total, int32_t factor);

/* ------------------------------------------------ no-allocation entry point
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory when they step the solver: codes that size all GPU memory once at
 * start-up and own it through their own arena or pool, and code that runs
 * where cudaMalloc is not allowed or would stall the device (a real-time
 * loop, a region another library has locked down).  sw_run_device needs a
 * context whose buffers grow on demand; this call needs none.
 *
 * It runs the swept path (cfg->alg must be SW_ALG_SWEPT, cfg->time_mode
 * SW_TIME_STEPS) on the caller's device-resident state (device layout, see
 * sw_run_device), enqueued on `stream` (a cudaStream_t, NULL = legacy default
 * stream), and returns without waiting.  Its scratch -- the edge slots, two
 * cells per cell, and one work row for the classic remainder steps, so three
 * times the state's bytes -- is a fixed device array of
 * SW_NOALLOC_SCRATCH_BYTES (24 MiB) inside the library, held by every GPU that
 * loads it until the process exits; larger states return SW_ERR_SIZE
 * (e.g. up to nx = 2^20 for FP64 Heat/KS, 2^18 for FP64 Euler).  It calls no
 * cudaMalloc, cudaFree or other allocating routine.
 *
 * state_dev must be device memory of the CUDA device that is current when
 * the call is made (the array used is that device's); anything else returns
 * SW_ERR_ARG.  The array's device address is looked up (cudaGetSymbolAddress)
 * on every call made outside stream capture, so a device reset by the host
 * application is picked up by the next such call; a call inside a capture
 * reuses the address found by the last call outside one, so make the first
 * call on a device, and the first after a device reset, before any stream
 * capture.  Every call on a device shares the one array and leaves its
 * contents behind (nothing in it needs to start at zero); calls that overlap
 * on the GPU -- on different streams, or from different host threads -- race
 * on it, so order them on one stream. */
#define SW_NOALLOC_SCRATCH_BYTES (24u * 1024u * 1024u)
int sw_run_device_noalloc(const sw_config *cfg, void *state_dev, void *stream);

/* Failure-path check (no reference counterpart): runs the persistent kernels'
 * bounded wait on a flag that nothing sets, with a limit of limit_ns
 * (1e6..1e10 ns).  Returns SW_ERR_TIMEOUT once the wait has run out, with the
 * wait's duration in *waited_ms (may be NULL); the context stays usable. */
int sw_wait_probe(sw_ctx *ctx, int64_t limit_ns, double *waited_ms);

/* Measurement aid (no reference counterpart): the FP64 pipe's issue rates
 * of the context's device, in operations per second, measured with a full
 * grid of independent fma / add / multiply chains (about 0.3 s).  The swept
 * and classic FP64 kernels are bound by this pipe, not by HBM; their roofs
 * are these rates times each stencil's operation counts. */
int sw_fp64_rates(sw_ctx *ctx, double *fma_per_s, double *add_per_s, double *mul_per_s);

/* The whole program: argv exactly as bin/<Problem><Precision>Out takes it
 * (replaces main(), Heat1D_SweptShared.cu:697-836, KS1D_SweptShared.cu:866-1029,
 * Euler1D_SweptShared.cu:1112-1287).  Writes solution.dat and appends the
 * timing row like the reference.  Returns 0 or a negative code. */
int sw_cli_main(int problem, int precision, int argc, char **argv);

#ifdef __cplusplus
}
#endif
#endif /* SWEPT1D_H */
