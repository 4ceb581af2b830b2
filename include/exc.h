/*
 * exc.h -- C ABI of libexc, the GB300 (sm_103a) implementation of the
 * DNS-aided LES hot path of agdestein/ExactClosure.jl.
 *
 * The reference is a Julia module (src/N.jl, `module NavierStokes`) whose
 * operators take tuples of CuArrays; this ABI is what a `ccall` from that
 * module binds.  Every entry point returns an int status (EXC_OK == 0);
 * nothing throws across the boundary; exc_last_error() gives the message of
 * the last failure on the calling thread.
 *
 * Conventions
 *   - `precision` is EXC_F64 or EXC_F32 and fixes the word type of every
 *     field argument (double or float).
 *   - Scalar fields are n^3 words, x fastest (the reference's column-major
 *     Field, src/N.jl:34-42); vector fields are three such arrays, component
 *     slowest (the tuple of src/N.jl:45).  Operator-level pointers are DEVICE
 *     pointers owned by the caller; `stream` is a cudaStream_t (NULL = the
 *     legacy default stream).
 *   - Tensor arguments hold 6 symmetric components in the reference's order
 *     (s11, s22, s33, s12, s23, s31; src/N.jl:94-104) or 9 non-symmetric
 *     ones in the order (s11, s21, s31, s12, s22, s32, s13, s23, s33)
 *     (src/N.jl:181), each an n^3 (or n_les^3) array.
 *   - Grid sizes: n = 2^a 3^b 5^c 7^d 11^e 13^f 17^g, a >= 1, 4 <= n <= 1024; an LES ratio c must
 *     divide n and n/c must itself be a supported size for LES projection.
 *   - Case-level host pointers are borrowed for the duration of the call.
 *   - A handle is not re-entrant; distinct handles may be used from
 *     distinct threads.
 */
#ifndef EXC_H
#define EXC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum exc_status {
  EXC_OK = 0,
  EXC_ERR_ARG = 1,       /* null pointer, bad enum or out-of-range scalar */
  EXC_ERR_SHAPE = 2,     /* unsupported grid size */
  EXC_ERR_RATIO = 3,     /* filter ratio does not divide the grid */
  EXC_ERR_OOM = 4,       /* device or pinned allocation failed */
  EXC_ERR_CUDA = 5,      /* CUDA runtime error */
  EXC_ERR_NONFINITE = 6, /* a non-finite velocity was detected */
  EXC_ERR_TIMEOUT = 7,   /* a bounded device-side wait ran out */
  EXC_ERR_STATE = 8      /* call made in the wrong state */
};

enum exc_precision { EXC_F64 = 0, EXC_F32 = 1 };
enum exc_filter_kind { EXC_FILTER_VOLUME = 0, EXC_FILTER_FACE = 1 };

/* Message of the last failed call on this thread (never NULL). */
const char* exc_last_error(void);
/* ABI version (major*100 + minor). */
int exc_version(void);

/* ======================================================================
 * Operator level (device pointers owned by the caller)
 * ====================================================================== */

/* du = doadd*du - div sigma(u): `stresstensor` + `tensordivergence!`
 * (src/N.jl:94-160).  u, du: vector fields on the n^3 grid of side l. */
int exc_tensordivergence(int precision, int n, double l, double visc,
                         const void* u, void* du, int doadd, void* stream);

/* du = doadd*du - sum_j delta_j s_ij for an explicit tensor s:
 * `tensordivergence!` with 6 symmetric components (nsym == 6) or
 * `tensordivergence_nonsym!` with 9 components (nsym == 9)
 * (src/N.jl:120-200).  s: nsym n^3 arrays, contiguous. */
int exc_tensordivergence_tensor(int precision, int n, double l, int nsym,
                                const void* s, void* du, int doadd, void* stream);

/* The 6 components of the staggered stress (src/N.jl:94-118), materialised. */
int exc_stresstensor(int precision, int n, double l, double visc,
                     const void* u, void* s6, void* stream);

/* d = div u at cell centres (`divergence!`, src/N.jl:222-238). */
int exc_divergence(int precision, int n, double l, const void* u, void* d, void* stream);

/* u -= grad p (`pressuregradient!`, src/N.jl:240-254). */
int exc_pressuregradient(int precision, int n, double l, void* u, const void* p, void* stream);

/* FFT Poisson solver bound to one grid (`poissonsolver`, src/N.jl:202-220).
 * Owns its spectral work array and twiddle tables. */
typedef struct exc_poisson exc_poisson;
int exc_poisson_create(int precision, int n, double l, exc_poisson** out);
int exc_poisson_destroy(exc_poisson* ps);
/* Device faults recorded by kernels since the last call (and cleared): bit 0
 * = a wait for a TMA plane of the FP32 RHS sweep gave up after its poll
 * limit (the copy never completed; that sweep's output is not valid); bit 1
 * = a wait for the tensor-core (tcgen05) convolution of the learned closure
 * gave up (that convolution's output is not valid).  0 in normal operation. */
int exc_device_faults(int* flags);
/* Synchronise `stream` (null: the legacy default stream), then read and
 * clear the device fault flags like exc_device_faults; returns
 * EXC_ERR_TIMEOUT when any is set (a bounded device wait gave up: the output
 * of that kernel is not valid), EXC_OK otherwise.  No counterpart in the
 * reference. */
int exc_device_sync(void* stream, int* flags);
/* Wait drill, for testing the give-up path of the bounded device waits (no
 * counterpart in the reference; 0, the default, is normal operation).  Bit 0:
 * the RHS sweep's tiles that take their planes by TMA issue no copy; bit 1:
 * the tensor-core convolution of the learned closure issues no copy.  The
 * waits for those copies then give up after 64 polls with nothing in flight,
 * set their fault bit and the kernels finish (their outputs are not valid);
 * the context stays usable.  Process-wide; launches made while it is set are
 * affected. */
int exc_debug_wait_drill(int flags);

/* FFT engine of a solver (no counterpart in the reference).  0 (the
 * default): in FP64 on grids n = 128, 192, 256, 384, 512, 1024 a
 * mixed-precision solve (three FP32 register-pass solves refined by residuals
 * formed in FP64: the pressure agrees with the FP64 FFT solve to FP64
 * rounding); otherwise register-resident two-level passes where the grid has
 * a plan (n = 32, 48, 64, 96, 128, 192, 256 and, in FP32, 384, 512, 1024),
 * shared-memory Stockham passes for the rest.  1 = FP64/FP32 Stockham passes
 * for every grid.  2 = register passes where planned, else Stockham, in the
 * solver's own precision throughout.  Results agree to round-off; the
 * autotuner of the serving form picks per grid. */
int exc_poisson_set_engine(exc_poisson* ps, int engine);
/* p with L_h p = d, mean(p) = 0 (src/N.jl:262-301).  d and p may alias. */
int exc_poisson_solve(exc_poisson* ps, const void* d, void* p, void* stream);
/* In-place projection u <- u - grad L^-1 div u (`project!`, src/N.jl:256-307).
 * p_out (n^3, may be NULL) receives the pressure. */
int exc_project(exc_poisson* ps, void* u, void* p_out, void* stream);

/* exc_project without any device allocation.  No counterpart in the
 * reference: it exists for callers that cannot call cudaMalloc (a host whose
 * device memory belongs to its own pool, a loop under a fixed memory budget,
 * code that cannot afford the synchronisation cudaFree implies).  Its work
 * array lives in one static 4 MiB device array that every GPU loading the
 * library holds until exit, so grids are limited to n <= 72 (EXC_F64) and
 * n <= 96 (EXC_F32); larger n returns EXC_ERR_SHAPE.  Every call looks the
 * array's device address up in the current context (cudaGetSymbolAddress, a
 * host call), so a device reset or a new primary context is handled; the
 * first call on a device also sets the library's kernel attributes and should
 * come before any stream capture.  All calls share the array: calls that
 * overlap on the GPU race. */
int exc_project_noalloc(int precision, int n, double l, void* u, void* p_out, void* stream);

/* max_i |x_i| over `count` words, written as a double to *out_dev (device). */
int exc_max_abs(int precision, size_t count, const void* x, double* out_dev, void* stream);

/* dt = min(cfl*h/max|u|, cfl*h^2/visc/6) (`propose_timestep`,
 * src/N.jl:348-356); synchronises `stream` and returns dt on the host. */
int exc_propose_timestep(int precision, int n, double l, double visc, double cfl,
                         const void* u, double* dt_host, void* stream);

/* Discrete filter + coarse-grain of a vector field from n^3 to (n/ratio)^3:
 * kind VOLUME is `lazycoarsegrain(faces[i], lazyfilter(u_i, GDH))`
 * (src/N.jl:1228-1237 without the projection), kind FACE the face average.
 * fdelta (host, odd length nfdelta, may be NULL) is the optional Gaussian
 * FDelta of `get_kernels` (src/N.jl:1008-1020), convolved into the box. */
int exc_filter(int precision, int n, int ratio, int kind, const double* fdelta, int nfdelta,
               const void* u, void* ubar, void* stream);

/* Face-filtered total flux rDHi (src/N.jl:1038-1073): the 9 components of
 * r = sigma(u) + p*I (`get_r`, src/N.jl:1022-1036) filtered with GDHi[j]
 * and coarse-grained at LES centres/edges; output r9: 9 (n/ratio)^3 arrays. */
int exc_closure_flux(int precision, int n, int ratio, double l, double visc,
                     const double* fdelta, int nfdelta,
                     const void* u, const void* p, void* r9, void* stream);

/* Volume-filtered DNS stress sigmaDH at LES centres/edges (`get_sigmaDH`,
 * src/N.jl:1088-1115); output s6: 6 (n/ratio)^3 arrays. */
int exc_filtered_stress(int precision, int n, int ratio, double l, double visc,
                        const double* fdelta, int nfdelta,
                        const void* u, void* s6, void* stream);

/* ======================================================================
 * Case level: a DNS with attached LES grids, RK4 with the exact closure
 * evaluated at every stage (the `dnsaid_project` loop, src/N.jl:1239-1332,
 * with RK4 stages in place of forward Euler).  Device memory is owned by the
 * case.  Host arrays are float64 in the field layout above.
 * ====================================================================== */

#define EXC_MAX_LES 4

typedef struct {
  int ratio; /* n / n_les */
  int kind;  /* exc_filter_kind */
} exc_les_desc;

typedef struct {
  int n;          /* DNS cells per side */
  double l;       /* domain side */
  double visc;    /* kinematic viscosity */
  double cfl;     /* CFL factor of propose_timestep */
  int precision;  /* exc_precision of stencil, filter and RK stages */
  int nles;       /* number of attached LES grids (0..EXC_MAX_LES) */
  exc_les_desc les[EXC_MAX_LES];
} exc_case_desc;

typedef struct exc_case exc_case;

/* `stream` (cudaStream_t, may be NULL) is bound to the case for life.  A case
 * with LES grids also runs the LES work of each RK stage on a stream of its own
 * (created here), forked from and joined back into `stream` inside every step:
 * work the caller orders on `stream` sees complete steps. */
int exc_case_create(const exc_case_desc* desc, void* stream, exc_case** out);
int exc_case_destroy(exc_case* cs);

/* Solenoidal random field with E(k) ~ k^4 exp(-2 (k/kpeak)^2) normalised to
 * `energy` (`randomfield` + `peak_profile`, src/N.jl:366-476) from the
 * project's counter-based normal generator with `seed`; resets the LES
 * states to the filtered DNS and the clock to 0. */
int exc_case_init_random(exc_case* cs, double kpeak, double energy, uint64_t seed);

/* Copy the DNS velocity in (3 n^3 doubles) and reset LES states and clock. */
int exc_case_set_velocity(exc_case* cs, const double* host_u);
int exc_case_get_velocity(exc_case* cs, double* host_u);

/* LES field `which`: 0 = filtered DNS target, 1 = exact-closure LES,
 * 2 = no-model LES, 3 = last exact closure m (stage 1 of the last step),
 * 4 = learned-closure LES (exc_case_attach_net), 5 = the filtered DNS at
 * stage 1 of the last step (the input that goes with 3);
 * 3 (n/ratio)^3 doubles. */
int exc_case_get_les(exc_case* cs, int les_index, int which, double* host_v);

/* Restart every LES state of every LES grid from the filtered DNS
 * (`apply_DHpi`, src/N.jl:1228-1237) and the clock from 0. */
int exc_case_reset_les(exc_case* cs);

/* Relative L2 error (compute_errors) of one LES state against the filtered
 * DNS: which = 1 exact closure, 2 no model, 4 learned closure. */
int exc_case_les_error(exc_case* cs, int les_index, int which, double* err);

/* Device-to-device copy of the pair (filtered DNS, exact closure m) at stage
 * 1 of the last step, 3 (n/ratio)^3 words each in the case precision: the
 * training data of the learned closure (what the reference's driver stores
 * with JLD2, dns_aid.jl:87-103, kept on the device here). */
int exc_case_snapshot(exc_case* cs, int les_index, void* dev_u, void* dev_m);

/* Advance `nsteps` RK4 steps.  dt_fixed > 0 uses that step, otherwise
 * propose_timestep on the device every step (no host synchronisation). */
int exc_case_step(exc_case* cs, int nsteps, double dt_fixed);

/* Relative L2 errors of the exact and no-model LES against the filtered DNS
 * (`compute_errors`, src/N.jl:1334-1349): err[0] exact, err[1] no-model. */
int exc_case_errors(exc_case* cs, int les_index, double* err2);

/* Simulated time and the last dt (host; synchronises the case stream). */
int exc_case_time(exc_case* cs, double* t, double* last_dt);

/* Mean kinetic energy of the DNS (FP64 reduction). */
int exc_case_energy(exc_case* cs, double* energy);

/* Viscous dissipation visc/N sum_ij (delta_j u_i)^2 of the DNS (FP64): the
 * energy drained by the viscous part of `stress` (src/N.jl:106-118) for a
 * divergence-free field (the reference computes it with Turbulox,
 * dns_aid.jl:92-94). */
int exc_case_dissipation(exc_case* cs, double* eps);

/* Shell spectrum E(k), k = 1..nshell (`spectrum`, src/N.jl:576-590),
 * nshell = div(2*div(n,2), 3); FP64. */
int exc_case_spectrum(exc_case* cs, double* host_e, int nshell);

/* Device pointer of an internal field (0 = DNS velocity) for zero-copy
 * callers; valid until the case is destroyed. */
int exc_case_device_ptr(exc_case* cs, int which, void** ptr);

/* Number of kernel launches in one captured RK4 step (valid after the first
 * exc_case_step). */
int exc_case_launches_per_step(exc_case* cs, int* count);

/* Synchronise the case stream; returns EXC_ERR_NONFINITE if a non-finite
 * velocity was flagged during the last steps. */
int exc_case_sync(exc_case* cs);

/* ======================================================================
 * Serving form (no counterpart in the reference, whose driver runs one
 * solve at a time): continuous batching of independent periodic NS solves of
 * mixed grid sizes.  Requests queue on the host; each tick admits every
 * queued request for which a slot of its grid size is free or a new batch of
 * slots fits the memory budget (a share of the free device memory at
 * creation), advances every active solve by one RK4 step, and retires the
 * solves that reached their step count.  Same-size solves are batched slot
 * after slot and stepped by one captured CUDA graph per size whose kernels
 * cover every slot; all state stays in device memory between steps.
 * ====================================================================== */

typedef struct exc_server exc_server;

typedef struct {
  int precision;       /* EXC_F32 (the served form) or EXC_F64 */
  double mem_fraction; /* share of the free device memory the server may hold, (0, 0.95] */
  double max_bytes;    /* absolute cap on that budget in bytes (0: none) */
  int slots_per_chunk; /* same-size solves per batch (0: by grid size) */
  int autotune;        /* nonzero: time FFT tile shapes per grid size before capture */
} exc_server_desc;

typedef struct {
  int n;               /* grid cells per side */
  double l, visc, cfl; /* domain side, viscosity, CFL factor */
  double kpeak, energy; /* initial spectrum peak and kinetic energy (randomfield) */
  uint64_t seed;       /* initial-field seed */
  int nsteps;          /* RK4 steps to run */
  double* result_host; /* optional: receives the final velocity, 3 n^3 doubles */
} exc_solve_req;

typedef struct {
  int64_t id;
  int n, nsteps;
  double t_submit, t_admit, t_finish; /* seconds since creation; t_finish from the device clock */
  double energy;       /* final mean kinetic energy (FP64 reduction) */
  double sim_time;     /* simulated time reached */
} exc_solve_result;

typedef struct {
  int chunks, slots, active, queued, kernels_per_tick;
  double bytes_used, bytes_budget, ticks, clock;
} exc_server_info;

int exc_server_create(const exc_server_desc* desc, exc_server** out);
int exc_server_destroy(exc_server* sv);
/* Admission bound (no counterpart in the reference): a queued request is
 * admitted only while fewer than max_active_per_size solves of its grid size
 * run (0 = no bound, the default); requests are taken in arrival order among
 * those eligible.  Trades aggregate throughput for lower median latency. */
int exc_server_set_admission(exc_server* sv, int max_active_per_size);
/* Queue a solve; *id identifies its result. */
int exc_server_submit(exc_server* sv, const exc_solve_req* req, int64_t* id);
/* One non-blocking pass of the host side: collect every batch whose device
 * loop has ended (its retired solves become results), admit queued requests
 * into free slots of idle batches or new batches, and relaunch every idle
 * batch that has work.  A batch's stepping runs on the device: a captured
 * graph whose WHILE node repeats two RK4 steps of all its slots while any has
 * steps left (a few milliseconds of work per launch at most); the device
 * counts each solve's steps, retires it at its own step count and records its
 * finish time, energy and simulated time.  *active: admitted, unreported
 * solves; *queued: waiting requests. */
int exc_server_tick(exc_server* sv, int* active, int* queued);
/* Up to `max` results of finished solves whose device work has completed. */
int exc_server_poll(exc_server* sv, exc_solve_result* out, int max, int* count);
/* Tick until every submitted solve has finished; synchronises the device. */
int exc_server_drain(exc_server* sv);
int exc_server_stats(exc_server* sv, exc_server_info* st);
/* FFT engine and tile shape the autotuner chose for (precision, n, slots per
 * batch): engine 0 = register-resident passes (col_w = kx columns per column
 * tile, x_rows = rows per x-pass CTA of its plan), 1 = Stockham passes with
 * the tuned col_w and x_rows. */
int exc_server_tuning(int precision, int n, int slots, int* engine, int* col_w, int* x_rows);

/* ======================================================================
 * Learned closure (no counterpart in the reference): a 3-D convolutional
 * net on the LES grid with periodic 3x3x3 kernels, channels 3 -> 32 -> 32 -> 3
 * and GELU after the first two layers, trained on (filtered velocity, exact
 * closure) pairs.  BF16 weights and activations, FP32 accumulation on the
 * tensor cores; FP32 master weights and Adam moments.  Fields are device
 * arrays [batch][3][n^3] of the given precision; the net sees u/in_scale and
 * predicts m/out_scale.  Parameters are one FP32 vector in the padded layout
 * [W1 b1 W2 b2 W3 b3], W_l[tap][KP_l][NP_l] with (KP, NP) = (16, 32),
 * (32, 32), (32, 16) and tap = (dz+1)*9 + (dy+1)*3 + (dx+1).
 * ====================================================================== */

typedef struct exc_net exc_net;

int exc_net_create(uint64_t seed, exc_net** out);
int exc_net_destroy(exc_net* net);
int exc_net_param_count(void);
int exc_net_set_scales(exc_net* net, double in_scale, double out_scale);
int exc_net_get_params(exc_net* net, float* host, int count);
/* Convolution engine: 0 (default) = tcgen05 tensor-core kernels (tensor
 * memory accumulators) on 64^3 grids and mma.sync kernels elsewhere; 1 =
 * mma.sync kernels everywhere.  Both sum the same BF16 products in FP32. */
int exc_net_set_conv_engine(exc_net* net, int engine);
/* Also resets the Adam state. */
int exc_net_set_params(exc_net* net, const float* host, int count);
/* m = net(u) */
int exc_net_forward(exc_net* net, int precision, int batch, int n, const void* u, void* m, void* stream);
/* Gradients of the MSE loss mean((net(u) - m/out_scale)^2) (host copy in
 * the parameter layout when grad_host != NULL) and the loss. */
int exc_net_gradients(exc_net* net, int precision, int batch, int n, const void* u, const void* m,
                      float* grad_host, double* loss_host, void* stream);
/* One Adam step (b1 0.9, b2 0.999, eps 1e-8) on that loss; returns the loss
 * before the update. */
int exc_net_train_step(exc_net* net, int precision, int batch, int n, const void* u, const void* m, double lr,
                       double* loss_host, void* stream);

/* Drive a third LES state of LES grid `les_index` with the learned closure,
 * k = P_H(RHS_H(v) + net(v)), starting from the exact-closure state (NULL
 * detaches).  exc_case_get_les(which = 4) reads it. */
int exc_case_attach_net(exc_case* cs, int les_index, exc_net* net);
/* No-model fallback of the learned-closure LES of `les_index` (no
 * counterpart in the reference): before every step the state's kinetic
 * energy E = 1/2 sum v^2 / (n/ratio)^3 is checked on the device; when it is
 * not finite or leaves [e_lo, e_hi] the state goes back to the last one
 * inside the band and the LES continues without the net's term (no model)
 * from then on.  Default band [0, inf): non-finite states only.  Attaching a
 * net or exc_case_reset_les disengages it. */
int exc_case_set_fallback(exc_case* cs, int les_index, double e_lo, double e_hi);
/* Whether that fallback has engaged (1) or not (0). */
int exc_case_fallback(exc_case* cs, int les_index, int* engaged);

/* ======================================================================
 * The reference's driver `dnsaid_project` (src/N.jl:1239-1332): a forward
 * Euler warm-up of the DNS, then the DNS and five LES stepped in lockstep
 * with the DNS time step -- no model (`step_forwardeuler!`), classic
 * (`step_ΔHπ_classic!`), classic+flux, classic+flux+div (the exact closure)
 * and its symmetrised form (src/N.jl:1137-1226).  FP64.  The ratio must be
 * odd (the classic closure's fine-grid top hat) and n/ratio an FFT size.
 * ====================================================================== */

typedef struct exc_dnsaid exc_dnsaid;

typedef struct {
  int n;                  /* DNS cells per side */
  double l;
  double visc;
  int ratio;              /* n / n_les, odd */
  const double* fdelta;   /* optional Gaussian FDelta (odd length) or NULL */
  int nfdelta;
} exc_dnsaid_desc;

/* Initial spectrum of exc_dnsaid_init_random: `peak_profile` with k0 = param
 * (src/N.jl:366) or the power law (k > 0) k^param of dnsaid_project
 * (src/N.jl:1245). */
enum exc_profile { EXC_PROFILE_PEAK = 0, EXC_PROFILE_POWER = 1 };

int exc_dnsaid_create(const exc_dnsaid_desc* desc, void* stream, exc_dnsaid** out);
int exc_dnsaid_destroy(exc_dnsaid* d);
/* `randomfield(profile, ...)` (src/N.jl:394-476) with the project's seeded
 * generator. */
int exc_dnsaid_init_random(exc_dnsaid* d, int profile, double param, double energy, uint64_t seed);
int exc_dnsaid_set_velocity(exc_dnsaid* d, const double* host);
int exc_dnsaid_get_velocity(exc_dnsaid* d, double* host);
/* The warm-up loop (src/N.jl:1264-1276): step_forwardeuler! until t reaches
 * twarm (at most max_steps steps when > 0). */
int exc_dnsaid_warmup(exc_dnsaid* d, double twarm, double cfl, int max_steps, int* steps);
/* Switch the handle (before exc_dnsaid_start) to the paper's volume-average
 * driver `dns_aid_volavg` (src/NavierStokes.jl:141-304): four LES -- no
 * model, classic (divergence of the volume-filtered flux minus
 * sigma_H(fu) + p_H I), swap (the face-filtered flux instead) and the swap
 * flux's symmetric part -- each stepped v += dt P(RHS_H(v)) + dt dsigma, then
 * projected when doproject != 0; the target fu is the volume-filtered DNS,
 * projected when doproject.  The paper module's Turbulox filters are the
 * reference's own GDH (volume) and GDHi (face) filters of src/N.jl. */
int exc_dnsaid_set_paper(exc_dnsaid* d, int doproject);
/* Switch the handle (before exc_dnsaid_start) to the paper's surface-average
 * driver `dns_aid_surface` (src/NavierStokes.jl:306-468): the target fiu is
 * the face-filtered DNS (`surfacefilter!(fiu, u, c)`, never projected); four
 * LES -- no model, classic (divergence of the surface-filtered flux r_ij,
 * point-sampled along i and boxed along the other axes, minus
 * sigma_H(fiu) + p_H I), swap (the surface-filtered flux on the diagonal and
 * the line-filtered flux, point-sampled along i and j, off it) and the swap
 * flux's symmetric part -- each stepped like the volume driver's.  The
 * Turbulox filters are restated from their finite-volume meaning; the swap
 * closure is exact off the diagonal only (the normal flux term of a face
 * average is a fine-grid difference across the face). */
int exc_dnsaid_set_surface(exc_dnsaid* d, int doproject);
/* LES initial states: all five = apply_ΔHπ(u) (src/N.jl:1278-1287), or the
 * four paper LES = fu; t = 0. */
int exc_dnsaid_start(exc_dnsaid* d);
/* The lockstep loop (src/N.jl:1289-1323) until t reaches tstop (at most
 * max_steps steps when > 0). */
int exc_dnsaid_step(exc_dnsaid* d, double tstop, double cfl, int max_steps, int* steps);
int exc_dnsaid_time(exc_dnsaid* d, double* t, int* steps);
/* host (3 n_les^3): 0 = apply_ΔHπ of the current DNS (`u_les`), 1 u_nomo,
 * 2 u_c, 3 u_cf, 4 u_cfd, 5 u_cfd_symm; paper driver: 0 = fu, 1 nomodel,
 * 2 classic, 3 swapfil, 4 swapfil_symm. */
int exc_dnsaid_get(exc_dnsaid* d, int which, double* host);
/* `compute_errors` (src/N.jl:1334-1349) of the five LES against u_les (the
 * paper driver: of its four LES against fu, out[4] = 0). */
int exc_dnsaid_errors(exc_dnsaid* d, double out[5]);
/* The paper drivers' relerr (src/NavierStokes.jl:292-296, 456-460): out[k] =
 * |v_k - fu| / |fu| over all three components for the four LES (nomodel,
 * classic, swapfil, swapfil_symm), reduced on the device in FP64. */
int exc_dnsaid_relerr(exc_dnsaid* d, double out[4]);

/* ======================================================================
 * 1-D Burgers, batched over samples (module `Burgers`, src/Burgers.jl)
 *
 * A handle holds `nsample` independent periodic samples of `nh` cells on
 * [0, l], FP64, laid out [nsample][nh] x fastest (the reference's
 * zeros(nh, nsample) matrices, src/Burgers.jl:273-307).  Velocities sit on
 * the right cell faces.  Every sample advances with its own time step, as in
 * the reference's per-sample loop (src/Burgers.jl:307).  One LES grid of nH
 * cells (nh/nH odd) can be attached; it carries the four LES of
 * `dns_aided_les` and a Smagorinsky LES.
 * ====================================================================== */

typedef struct exc_burgers exc_burgers;

typedef struct {
  int nh;        /* DNS cells per sample (the shared-memory resident limit is about 13,900) */
  int nsample;   /* independent samples */
  double l;      /* domain length (2 pi in the reference's setup) */
  double visc;
} exc_burgers_desc;

enum exc_burgers_filter { EXC_BURGERS_GAUSSIAN = 0, EXC_BURGERS_TOPHAT = 1 };
enum exc_burgers_scheme { EXC_BURGERS_EULER = 0, EXC_BURGERS_RK4 = 1 };
/* Fields of exc_burgers_get_les, the `fields` of dns_aided_les
 * (src/Burgers.jl:272-306) on the LES grid. */
enum exc_burgers_field {
  EXC_BURGERS_DNS_FIL = 0,  /* filtered DNS (computed from the current DNS) */
  EXC_BURGERS_NOMODEL = 1,
  EXC_BURGERS_CLASS_M = 2,  /* classic: vsu - sVU */
  EXC_BURGERS_CLASS_P = 3,  /* classic + flux: vsu - svu */
  EXC_BURGERS_SWAPFIL = 4,  /* classic + flux + div (exact): fsu - svu */
  EXC_BURGERS_SMAG = 5      /* Smagorinsky LES (exc_burgers_smagorinsky_solve) */
};

/* LES filter kernels of one grid: `gaussian_weights`/`tophat_weights`
 * (src/Burgers.jl:146-162) and `build_doublekernel` (src/Burgers.jl:218-233).
 * wl gets 2*Rl+1 weights, wd 2*Rd+1 (either may be NULL to query R). */
int exc_burgers_kernels(int nh, int nH, double l, double delta_ratio, int filter, int* Rl, double* wl, int* Rd,
                        double* wd);
int exc_burgers_create(const exc_burgers_desc* desc, void* stream, exc_burgers** out);
int exc_burgers_destroy(exc_burgers* b);
/* `randomfield` with `bump_profile` (src/Burgers.jl:192-202); sample s uses
 * the phase stream seed + s.  Also records the initial field and resets the
 * per-sample clocks. */
int exc_burgers_init_random(exc_burgers* b, double kpeak, double energy, uint64_t seed);
/* host: [nsample][nh]; records the initial field and resets the clocks. */
int exc_burgers_set_velocity(exc_burgers* b, const double* host);
/* initial != 0 reads the recorded initial field (`ustart`). */
int exc_burgers_get_velocity(exc_burgers* b, int initial, double* host);
/* Back to the recorded initial field with the clocks at zero. */
int exc_burgers_restart(exc_burgers* b);
/* Per-sample time and step count (either pointer may be NULL). */
int exc_burgers_time(exc_burgers* b, double* t, int* steps);
/* Attach an LES grid of nH cells (nH == 0 detaches) with LES filter width
 * delta_ratio * H; its four LES start from the double-filtered current DNS
 * (src/Burgers.jl:366-379). */
int exc_burgers_les_setup(exc_burgers* b, int nH, double delta_ratio, int filter);
/* Advance every sample until its time reaches tstop, at most max_steps
 * steps this call (<= 0 or above 1,000,000: 1,000,000), with dt = min(cfl * cfl(u), tstop - t).
 * With an LES grid: `dns_aided_les` (src/Burgers.jl:350-445, forward
 * Euler); without: the DNS of `create_dns` with `timestep!` (EULER) or
 * `rk4_timestep!` (RK4) (src/Burgers.jl:112-142, :522-545).  steps_max
 * (may be NULL) gets the largest per-sample step count so far. */
int exc_burgers_advance(exc_burgers* b, double tstop, double cfl, int scheme, int max_steps, int* steps_max);
/* host: [nsample][nH] of the selected field. */
int exc_burgers_get_les(exc_burgers* b, int which, double* host);
/* The double-filtered DNS on the DNS grid, `dns_ref_fil`, host [nsample][nh]. */
int exc_burgers_filtered(exc_burgers* b, double* host_fine);
/* `compute_errors` (src/Burgers.jl:909-916): norm(x - dns_fil)/norm(dns_fil)
 * over all samples for nomodel, class_m, class_p, swapfil, smag (NaN when no
 * Smagorinsky solve ran). */
int exc_burgers_errors(exc_burgers* b, double out[5]);
/* Closure terms of the current DNS: terms [nsample][5][nH] = fsu, vsu, vu,
 * sVU, svu (src/Burgers.jl:397-412); diss [nsample][3][nH] =
 * delta_stag(vu) * sigma for classic, classic+flux, exact
 * (`compute_dissipation`, src/Burgers.jl:447-520); fractions = the mean
 * shares of |classic|, |flux|, |div| (`compute_fractions`,
 * src/Burgers.jl:1022-1116).  Any output may be NULL. */
int exc_burgers_closure_terms(exc_burgers* b, double* terms, double* diss, double fractions[3]);
/* `smagorinsky_fields` (src/Burgers.jl:547-688) on the current DNS and the
 * coefficient fits theta^2 = -<S,T>/<S,S> (smagorinsky.jl:32-45):
 * theta2[0] classic, theta2[1] discrete.  fields (may be NULL):
 * [nsample][4][nh] = Sh, Th, SH, TH. */
int exc_burgers_smagorinsky_fit(exc_burgers* b, double theta2[2], double* fields);
/* `solve_smagorinsky` (src/Burgers.jl:690-786) from the recorded initial
 * field (restart != 0) or continuing the previous call, C = theta^2
 * (Delta^2 + H^2). */
int exc_burgers_smagorinsky_solve(exc_burgers* b, double theta, double tstop, double cfl, int max_steps,
                                  int restart, int* steps_max);
/* Device pointers: 0 = velocity, 1 = initial velocity, 2 = LES states
 * [nsample][4][nH]. */
int exc_burgers_device_ptr(exc_burgers* b, int which, void** ptr);

#ifdef __cplusplus
}
#endif

#endif /* EXC_H */
