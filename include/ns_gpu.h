/*
 * ns_gpu.h -- thin C-ABI over the sm_103a kernels of the pseudospectral step.
 *
 * Plain pointers and sizes only; no CUDA or framework types cross this
 * boundary.  Host arrays use the reference solver's layouts
 * (src/spectral/ns_spectral_solver.h:22-68 of DiogoRibeiro7/navier-stokes-solvers):
 *   real fields      double[ny][nx]             (idx = j*nx + i)
 *   spectral fields  double complex[nky][nkx]   (interleaved re,im; nkx = nx/2+1, nky = ny)
 *
 * Every function returns an ns_gpu_status (0 = success).  Errors are never
 * silent: a failing call returns non-zero and records a message retrievable
 * with ns_gpu_last_error().  There is no CPU fallback: without a CUDA device
 * ns_gpu_create fails with NS_GPU_ERR_NO_DEVICE.
 *
 * Each entry point names the reference routine whose work it performs
 * (file:line in the reference project).  The drop-in implementation of the
 * reference header (include/ns_spectral_solver.h) is written on top of this
 * layer; an FFI binding (ctypes, cgo, JNI) can bind either.
 */
#ifndef NS_GPU_H
#define NS_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ns_gpu ns_gpu;

typedef enum {
    NS_GPU_OK = 0,
    NS_GPU_ERR_INVALID = 1,     /* bad argument (size, NULL pointer, range) */
    NS_GPU_ERR_NO_DEVICE = 2,   /* no CUDA device / driver */
    NS_GPU_ERR_CUDA = 3,        /* a CUDA runtime call failed */
    NS_GPU_ERR_ALLOC = 4,       /* device allocation failed */
    NS_GPU_ERR_DIVERGED = 5     /* non-finite values detected in the state */
} ns_gpu_status;

enum { NS_GPU_FP64 = 0, NS_GPU_FP32 = 1 };

/* Solver parameters.  Fields mirror NSSpectralData scalars and
 * NSSpectralHyperviscosityConfig (src/spectral/ns_spectral_solver.h:8-29)
 * plus the forcing extension. */
typedef struct {
    double Re;                 /* Reynolds number, nu = 1/Re */
    double cfl_factor;         /* CFL safety factor (reference default 0.3) */
    int adaptive_dt;           /* 1: dt from the reference CFL rule at every step, on the device */
    double dt;                 /* fixed dt when adaptive_dt == 0 */
    /* hyperviscosity and selective frequency damping (hyperviscosity.c:15-178) */
    int hv_enabled;
    double hv_coefficient;
    int hv_order;
    double hv_cutoff_ratio;
    int sfd_enabled;
    double sfd_strength;
    double sfd_timescale;
    /* white-in-time forcing on the shell kmin <= |k| <= kmax with energy
     * injection rate epsilon (Philox4x64-10 counter RNG keyed by seed; the
     * counter is the physical mode (kx, ky) and the forcing step, so every grid
     * that resolves the shell draws the same noise for the same step) */
    int forcing_enabled;
    double forcing_kmin;
    double forcing_kmax;
    double forcing_epsilon;
    uint64_t forcing_seed;
    /* time scheme: NS_GPU_RK4 (the reference's classical RK4,
     * spectral_time_integration.c:34-106) or NS_GPU_IFRK4 (integrating-factor
     * RK4: viscous and hyperviscous decay exp(-(k^2/Re + w) t) integrated
     * exactly, the Jacobian and SFD relaxation explicit; no reference counterpart) */
    int scheme;
    /* forcing draws per step (0 or 1: one): a step of M draws adds
     * sigma sqrt(dt/M) (xi_c + ... + xi_{c+M-1}) and advances the forcing counter
     * by M, so a coarse step of M fine steps receives exactly the fine run's
     * forcing over those steps */
    int forcing_substeps;
} ns_gpu_params;

enum { NS_GPU_RK4 = 0, NS_GPU_IFRK4 = 1 };

/* ----------------------------------------------------------- lifetime */

/* Replaces the device side of ns_spectral_allocate / initialize_fft_plans
 * (spectral_memory.c:6-68, spectral_initialization.c:57-69).  The reference's
 * FFTW takes any size; here nx and ny lie in [8, 4096] and each transform
 * length (nx/2 for even nx, nx for odd nx; ny) has no prime factor above 31
 * (every 2^a 3^b 5^c 7^d grid qualifies; a prime factor p costs a direct
 * p-point pass).  Power-of-two sides run the radix-16/8/4 kernels, other sides
 * the mixed-radix ones.  Any other size returns NS_GPU_ERR_INVALID with the
 * reason on stderr, as does a grid whose stage kernels would need more shared
 * memory than one CTA has (odd nx above about 2700 in FP64).  precision is
 * NS_GPU_FP64 or NS_GPU_FP32. */
int ns_gpu_create(int nx, int ny, double Lx, double Ly, int precision, ns_gpu **out);
/* Tiling of an instance's stage kernels (no reference counterpart: the
 * reference hands its transforms to FFTW plans, spectral_initialization.c:57-69).
 * Zero fields are chosen by ns_gpu_create's own rule. */
typedef struct {
    int row_radix;         /* complex values per thread of a row transform: 4 or 16 */
    int col_radix;         /* complex values per thread of a column transform: 4 or 16 */
    int rows_per_cta;      /* rows per row-pass CTA: a power of two dividing ny */
    int cols_per_cta;      /* kept columns per column-pass CTA: a power of two, at most 64 */
    int row_field_groups;  /* 1: a thread group per field of a row (the fields' transforms run side
                            * by side), -1: one group per row, 0: automatic */
    int col_field_groups;  /* the same for the column pass (four groups per column block) */
    int register_resident; /* output of ns_gpu_get_tiling: bit 0 (1) the row pass, bit 1 (2) the
                            * column pass runs the register-resident 2048 / 4096 kernels */
} ns_gpu_tiling;
/* ns_gpu_create with a fixed tiling.  Setting row_radix or col_radix selects the
 * generic stage kernels at every size (also at 2048 and 4096); the radix applies
 * to power-of-two transform lengths (others run the mixed-radix bodies).
 * NS_GPU_ERR_INVALID (reason on stderr) when the tiling cannot run: CTAs above
 * 256 (row) / 512 (column) threads, row field groups that are neither whole
 * warps nor a divisor of a warp, column field groups (cols_per_cta times the
 * transform's threads) that are not whole warps, shared memory above the
 * device's limit. */
int ns_gpu_create_tiled(int nx, int ny, double Lx, double Ly, int precision, const ns_gpu_tiling *tiling,
                        ns_gpu **out);
/* The tiling an instance runs with (every field resolved; radix 0 = mixed radix;
 * field groups 1 or -1). */
int ns_gpu_get_tiling(const ns_gpu *g, ns_gpu_tiling *tiling);
/* Per-instance teardown (spectral_memory.c:71-104 without the global fftw_cleanup). */
void ns_gpu_destroy(ns_gpu *g);
const char *ns_gpu_last_error(const ns_gpu *g);
const char *ns_gpu_status_string(int status);
/* kept (dealiased) mode counts: kx columns 0..kx_kept-1, ky rows |band| <= (ky_kept-1)/2 */
int ns_gpu_dims(const ns_gpu *g, int *kx_kept, int *ky_kept);
int ns_gpu_set_params(ns_gpu *g, const ns_gpu_params *p);
int ns_gpu_synchronize(ns_gpu *g);
/* number of kernels this library has launched on the instance's stream */
uint64_t ns_gpu_launch_count(const ns_gpu *g);

/* ------------------------------------------------ geometry and tables */

/* Grid, wavenumbers, k^2 and the 2/3 mask computed on the device and copied
 * to host arrays (spectral_initialization.c:10-50).  Any pointer may be NULL. */
int ns_gpu_geometry(ns_gpu *g, double *x, double *y, double *kx, double *ky, double *k2, int *mask);
/* Hyperviscosity weights (hyperviscosity.c:60-102): computes kmax over all
 * modes on the device, derives the cutoff and inverse bandwidth exactly as the
 * reference, stores the weight table on the device and copies it to
 * weights_out ([nky][nkx], may be NULL).  Uses the hv_* fields of the params. */
int ns_gpu_hv_weights(ns_gpu *g, double *kmax, double *cutoff_wavenumber, double *inv_bandwidth,
                      double *weights_out);

/* ------------------------------------- transforms over host arrays */

/* physical -> spectral: r2c, scale 1/(nx*ny), dealias (spectral_transforms.c:9-22) */
int ns_gpu_forward(ns_gpu *g, const double *field, double *field_hat);
/* spectral -> physical: dealias then unnormalised c2r (spectral_transforms.c:25-32).
 * masked_copy (may be NULL) receives the dealiased input, the reference's
 * nonlinear_hat scratch contents after the call. */
int ns_gpu_inverse(ns_gpu *g, const double *field_hat, double *field, double *masked_copy);
/* zero every mode outside the 2/3 mask, in place (spectral_transforms.c:35-43) */
int ns_gpu_dealias(ns_gpu *g, double *field_hat);
/* psi = -omega/k^2, u_hat = i ky psi, v_hat = -i kx psi (spectral_core.c:8-34) */
int ns_gpu_velocity(ns_gpu *g, const double *omega_hat, double *psi_hat, double *u_hat, double *v_hat);
/* velocity_from_vorticity plus the three masked c2r of u, v, omega
 * (spectral_core.c:37-43).  masked_copy receives the dealiased omega_hat. */
int ns_gpu_derivatives(ns_gpu *g, const double *omega_hat, double *psi_hat, double *u_hat,
                       double *v_hat, double *u, double *v, double *omega, double *masked_copy);
/* N_hat = -mask(r2c(psi_x omega_y - psi_y omega_x))/(nx ny) from omega_hat and the
 * stored psi_hat (spectral_core.c:46-112).  The five physical outputs (may be
 * NULL) receive psi_x, psi_y, omega_x, omega_y and the Jacobian. */
int ns_gpu_nonlinear(ns_gpu *g, const double *omega_hat, const double *psi_hat, double *nonlinear_hat,
                     double *psi_x, double *psi_y, double *omega_x, double *omega_y, double *jacobian);
/* rhs -= w state + s ramp (state - sfd) over all modes (hyperviscosity.c:104-150) */
int ns_gpu_hv_apply(ns_gpu *g, double *rhs_hat, const double *state_hat, const double *sfd_hat);
/* sfd <- (1-a) sfd + a state, a = clamp(dt/tau) (hyperviscosity.c:152-178) */
int ns_gpu_hv_post_step(ns_gpu *g, const double *state_hat, double *sfd_hat, double dt);

enum { NS_GPU_REDUCE_CFL = 0, NS_GPU_REDUCE_ENERGY = 1, NS_GPU_REDUCE_ENSTROPHY = 2 };
/* Reductions over host real arrays with FP64 compensated accumulation:
 * CFL dt from max|u| (spectral_time_integration.c:9-31), energy mean 0.5(u^2+v^2)
 * (spectral_analysis.c:8-19), enstrophy mean 0.5 omega^2 (:22-33). */
int ns_gpu_reduce(ns_gpu *g, int kind, const double *a, const double *b, double *out);
/* Spectral statistics of host spectra: resolution fraction above 0.8 kmax
 * (spectral_analysis.c:36-66), max|omega_hat| and high-mode error (:69-100),
 * shell-binned energy sums and counts of 0.5(|u_hat|^2+|v_hat|^2) over
 * nbins = min(nkx, nky/2) bins (:103-142).  Outputs may be NULL. */
int ns_gpu_spectral_stats(ns_gpu *g, const double *omega_hat, const double *u_hat, const double *v_hat,
                          double *resolution_fraction, double *max_abs, double *spectral_error,
                          double *bin_energy, int *bin_count);
/* Taylor-Green initial fields (spectral_initialization.c:72-95): u, v, omega, p */
int ns_gpu_taylor_green(ns_gpu *g, double *u, double *v, double *omega, double *p);

/* ------------------------------------------------------ stepping */

/* Copy the caller's spectral state to the device.  psi_hat is the stream
 * function used by the first stage (the reference reads the stored psi_hat
 * there, spectral_core.c:51,66,76); NULL means -omega_hat/k^2.  sfd_hat may be
 * NULL when SFD is off.  step0 seeds the forcing counter. */
int ns_gpu_upload_state(ns_gpu *g, const double *omega_hat, const double *psi_hat, const double *sfd_hat,
                        double t, double dt, uint64_t step0);
/* Advance nsteps classical RK4 steps on the device (spectral_time_integration.c:34-106,
 * plus the forcing extension), with device-side CFL dt when adaptive.  A step's
 * launches are captured once as a CUDA graph and replayed until ns_gpu_set_params
 * (or an outside-mode state) changes their arguments. */
int ns_gpu_advance(ns_gpu *g, int nsteps);
/* Copy the device state back in reference layouts; any pointer may be NULL.
 * psi_hat/u_hat/v_hat are recomputed from omega_hat as compute_derivatives does;
 * u, v, omega are the masked inverse transforms. */
int ns_gpu_download_state(ns_gpu *g, double *omega_hat, double *psi_hat, double *u_hat, double *v_hat,
                          double *sfd_hat, double *u, double *v, double *omega, double *t, double *dt);
/* One classical RK4 step over host arrays: ns_gpu_upload_state(omega_hat,
 * psi_hat, sfd_hat, t, dt, step0), ns_gpu_advance(g, 1) and
 * ns_gpu_download_state(omega_hat, psi_hat, u_hat, v_hat, sfd_hat, u, v, omega)
 * in one call (the data movement of ns_spectral_advance_rk4,
 * spectral_time_integration.c:34-106), with the copies overlapped: psi_hat and
 * sfd_hat upload on a second stream beside omega_hat, and the output spectra
 * leave on that stream while the instance stream computes and copies out the
 * physical fields.  Modes outside the 2/3 mask that were zero in the caller's
 * omega_hat and psi_hat are zero after the step, so those two arrays only take
 * their kept modes back (the rest of each array is left as it is, equal to what
 * a full copy would write).  sfd_hat may be NULL (SFD off); u_hat, v_hat, u, v,
 * omega may be NULL.  t_out, dt_out (may be NULL) receive the new time and the
 * step's dt. */
int ns_gpu_step_host(ns_gpu *g, double *omega_hat, double *psi_hat, double *u_hat, double *v_hat, double *sfd_hat,
                     double *u, double *v, double *omega, double t, double dt, uint64_t step0, double *t_out,
                     double *dt_out);
/* Advance nsteps, timing each step with CUDA events on the instance stream.
 * When flush_bytes > 0 a device buffer of that size is overwritten between
 * steps, outside the timed events, so no timed step starts with the previous
 * step's data resident in L2.  total_ms receives the sum of the step times,
 * step_ms (nsteps entries, may be NULL) each step's time. */
int ns_gpu_advance_timed(ns_gpu *g, int nsteps, size_t flush_bytes, double *total_ms, double *step_ms);
/* Same stepping with CUDA events around every kernel launch: kernel_ms[0] and
 * counts[0] total the row (x-pass) kernels, kernel_ms[1] and counts[1] the
 * column (y-pass) kernels. */
int ns_gpu_profile_kernels(ns_gpu *g, int nsteps, size_t flush_bytes, double *kernel_ms, int *counts);
/* Energy, enstrophy (Parseval over the dealiased state, FP64 compensated),
 * and time of the device state. */
int ns_gpu_diagnostics(ns_gpu *g, double *energy, double *enstrophy, double *t, double *dt);
/* Shell-binned energy spectrum of the device state, the reference's
 * ns_spectral_analyze_spectrum (spectral_analysis.c:103-142) without the print:
 * bin b = (int)(|k| + 0.5) < nbins, energy_sum[b] = sum over the modes of the
 * bin of 0.5 (|u_hat|^2 + |v_hat|^2), count[b] = modes of the half spectrum in
 * the bin (dealiased or not, as the reference counts them), energy_mean[b] =
 * energy_sum[b] / count[b] (the reference's printed E(k)).  FP64 sums; any
 * output may be NULL. */
int ns_gpu_energy_spectrum(ns_gpu *g, int nbins, double *energy_sum, double *energy_mean, int *count);
/* Seeded random-phase vorticity with E(k) ~ k^4 exp(-(k/k0)^2) rescaled to the
 * given kinetic energy, written to the device state (no reference counterpart). */
int ns_gpu_init_random_spectrum(ns_gpu *g, uint64_t seed, double k0, double energy);
/* Same field, also copied to a host-layout array omega_hat[nky][nkx]. */
int ns_gpu_random_spectrum_host(ns_gpu *g, uint64_t seed, double k0, double energy, double *omega_hat);

/* ------------------------------------------------ reference forcing stream */

/* ns_forcing_state_init's shell selection (forcing.c:53-103) on the device:
 * weights[idx] = 1 where kmin <= sqrt(k2[idx]) <= kmax; returns the count. */
int ns_gpu_forcing_weights(ns_gpu *g, const double *k2, int n, double kmin, double kmax,
                           double *weights, int *active);
/* ns_forcing_generate (forcing.c:117-184) on the device: reproduces the
 * reference splitmix64 + Box-Muller stream counter-addressably (mode m of a call
 * whose generator state is s uses draws s+(2m+1)G and s+(2m+2)G), OU update for
 * colored noise, global rescale to energy_target.  rng_state is advanced by
 * 2*active draws. */
int ns_gpu_forcing_generate(ns_gpu *g, int n, const double *weights, int active, int colored,
                            double dt, double correlation_time, double energy_target,
                            uint64_t *rng_state, double *colored_state, double *forcing_out);

/* ------------------------------------------- device-resident access */

/* Allocation-free forward transform, for callers that cannot allocate device
 * memory (no counterpart in the reference): r2c of a real field, scaled by
 * 1/(nx*ny), with every mode outside the 2/3 mask set to zero.
 * Frameworks that own every device allocation through their own pool,
 * real-time loops that may not allocate, and processes whose device memory is
 * already fully reserved pass their own input and output and get the transform
 * without any allocation: its scratch lives in a fixed 8 MiB static device array
 * that every GPU loading this library holds until exit.  That limit admits every
 * power-of-two grid up to 1024 x 1024 (FP64; sides in [8, 4096]); a grid whose
 * intermediate (ny x Kx complex doubles plus twiddles) exceeds it is rejected
 * with NS_GPU_ERR_INVALID and a message on stderr.
 *   field      device pointer, double[ny][nx], 16-byte aligned
 *   field_hat  device pointer, double complex[ny][nx/2+1] (interleaved), 16-byte
 *              aligned; receives r2c/(nx*ny) with every mode outside the 2/3
 *              mask set to zero
 *   stream     cudaStream_t to issue on (NULL: the default stream); the call
 *              returns once the work is queued.
 * The first call on a device looks up the scratch address there
 * (cudaGetSymbolAddress with that device current): make it before any stream
 * capture.  All calls share the scratch array, so calls that overlap on the GPU
 * race; serialise them. */
int ns_gpu_forward_noalloc(int nx, int ny, const double *field, double *field_hat, void *stream);

/* Zero-initialised page-locked host memory for arrays that are copied to and
 * from the device every step (the drop-in allocates its host arrays here). */
void *ns_gpu_host_alloc(size_t bytes);
void ns_gpu_host_free(void *ptr);

/* Raw device pointer to the kept-mode vorticity state (layout [kx_kept][ky_kept]
 * complex of the instance precision) for callers that keep data on the GPU. */
void *ns_gpu_state_device_ptr(ns_gpu *g);

/* ----------------------------------------- device-resident physical fields */

/* Physical vorticity of the device state, omega[ny][nx] as float in a caller
 * device buffer (the masked c2r of spectral_transforms.c:25-32 on the state). */
int ns_gpu_vorticity_device(ns_gpu *g, float *omega_dev);
/* omega += delta for a physical float field delta[ny][nx] on the device: the
 * normalised, dealiased forward transform (spectral_transforms.c:9-22) of delta
 * is added to the state's kept modes. */
int ns_gpu_add_vorticity_device(ns_gpu *g, const float *delta_dev);
/* Spectral truncation of a fine state onto a coarser instance of the same box
 * and precision: the coarse kept modes take the fine values of the same (kx, ky)
 * (forward transforms are normalised by 1/(nx ny), so amplitudes carry over);
 * the coarse time and forcing counter are set to the fine ones.  No reference
 * counterpart. */
int ns_gpu_filter_state(ns_gpu *fine, ns_gpu *coarse);

/* ----------------------------------------------------- batched ensembles */

/* Many independent solvers of mixed sizes advanced together by one persistent
 * kernel launch, replayed from a CUDA graph (no reference counterpart: the
 * reference advances one NSSpectralData per ns_spectral_advance_rk4 call,
 * spectral_time_integration.c:34-106).  Each member is an ordinary FP32
 * ns_gpu instance with its own state, parameters, seeds and device-side dt;
 * the ensemble runs the same stage arithmetic as that instance's own
 * ns_gpu_advance, so a member advanced in the ensemble equals the same member
 * advanced alone with the same tiling (ns_gpu_create_for_ensemble). */
typedef struct ns_gpu_ensemble ns_gpu_ensemble;

/* Tiling of the persistent kernel (chosen by ns_gpu_ensemble_autotune). */
typedef struct {
    int threads;    /* threads per CTA: a multiple of 32, at most 256 */
    int row_radix;  /* complex values per thread in the row (x) transforms: 4 or 16 */
    int col_radix;  /* complex values per thread in the column (y) transforms: 4 or 16 */
    int cluster;    /* CTAs of a thread-block cluster that share one large member: 1, 2, 4 or 8 */
} ns_gpu_ensemble_config;

/* Members over ranks (one GPU per rank; no reference counterpart): longest
 * processing time first on the cost n^2 log2(n^2) of member m's side n[m],
 * deterministic, so every rank computes the same split with no exchange.
 * rank_of_member[m] receives the rank of member m; rank_cost (nranks entries,
 * may be NULL) the summed cost per rank.  Host-only: needs no device. */
int ns_ensemble_partition(int nmembers, const int *n, int nranks, int *rank_of_member, double *rank_cost);
/* the cost a member of side n counts for in that partition */
double ns_ensemble_member_cost(int n);

/* A standalone instance whose stage kernels use an ensemble tiling: the
 * sequential reference run of one ensemble member.  nx == ny. */
int ns_gpu_create_for_ensemble(int nx, int ny, double Lx, double Ly, int precision,
                               const ns_gpu_ensemble_config *cfg, ns_gpu **out);
/* nmembers FP32 members of side n[m] (powers of two in [16, 1024]) on
 * [0, L]^2.  Set each member's parameters and initial state through
 * ns_gpu_ensemble_member and the instance API before advancing. */
int ns_gpu_ensemble_create(int nmembers, const int *n, double L, const ns_gpu_ensemble_config *cfg,
                           ns_gpu_ensemble **out);
void ns_gpu_ensemble_destroy(ns_gpu_ensemble *e);
/* The instance of member m (owned by the ensemble; NULL when out of range). */
ns_gpu *ns_gpu_ensemble_member(ns_gpu_ensemble *e, int m);
/* Advance every member nsteps RK4 steps in one persistent launch.  Asynchronous:
 * later calls on a member's instance wait for it. */
int ns_gpu_ensemble_advance(ns_gpu_ensemble *e, int nsteps);
int ns_gpu_ensemble_synchronize(ns_gpu_ensemble *e);
/* reps launches of nsteps steps each, timed with CUDA events on the ensemble
 * stream after one untimed launch; ms_per_rep receives the mean. */
int ns_gpu_ensemble_advance_timed(ns_gpu_ensemble *e, int nsteps, int reps, double *ms_per_rep);
/* Switch the tiling (members' state is kept). */
int ns_gpu_ensemble_reconfigure(ns_gpu_ensemble *e, const ns_gpu_ensemble_config *cfg);
/* Time every valid tiling for steps steps on this ensemble (which advances its
 * members: tune before setting initial conditions), switch to the fastest and
 * append it to the JSON-lines cache at cache_path (may be NULL); a cached entry
 * for the same GPU and member mix is used without timing. */
int ns_gpu_ensemble_autotune(ns_gpu_ensemble *e, int steps, const char *cache_path, ns_gpu_ensemble_config *best,
                             double *best_ms_per_step);
int ns_gpu_ensemble_info(const ns_gpu_ensemble *e, int *grid, int *threads, size_t *smem, int *cluster,
                         uint64_t *launches);
const char *ns_gpu_ensemble_last_error(const ns_gpu_ensemble *e);

/* -------------------------------------------------- learned corrector */

/* A periodic 3x3 CNN that corrects coarse-grid steps (no reference
 * counterpart): 6 layers, 2 -> 64 -> 64 -> 64 -> 64 -> 64 -> 1 channels, GELU
 * between layers, BF16 weights (rounded from an FP32 master copy after every
 * AdamW step), FP32 activations and accumulation, hand-written forward and
 * backward kernels.  Input sample: [2][H][W] float = (coarse omega(t), plain
 * coarse-step increment omega_plain(t+dt) - omega(t)); output [H][W]: the
 * vorticity correction.  Parameters are one flat FP32 vector, per layer l the
 * weights [3 dy + dx][ci][co] then the biases [co]. */
typedef struct ns_cnn ns_cnn;
/* H a multiple of 8, W a multiple of 16; activations for max_batch samples */
int ns_cnn_create(int height, int width, int max_batch, uint64_t seed, ns_cnn **out);
void ns_cnn_destroy(ns_cnn *c);
const char *ns_cnn_last_error(const ns_cnn *c);
int ns_cnn_param_count(const ns_cnn *c, size_t *n);
uint64_t ns_cnn_launch_count(const ns_cnn *c);
int ns_cnn_get_params(ns_cnn *c, float *host);
/* sets the parameters and resets the AdamW moments */
int ns_cnn_set_params(ns_cnn *c, const float *host);
/* network input = (in0 * in_scale0, in1 * in_scale1); target = correction * out_scale */
int ns_cnn_set_normalization(ns_cnn *c, float in_scale0, float in_scale1, float out_scale);
/* training set on the device: inputs [n][2][H][W], targets [n][H][W] (host arrays) */
int ns_cnn_set_dataset(ns_cnn *c, const float *inputs, const float *targets, int n);
/* mean-squared-error loss (normalised units) and its parameter gradient for a host
 * batch, parameters unchanged (gradient checks) */
int ns_cnn_loss_and_grads(ns_cnn *c, const float *inputs, const float *targets, int batch, double *loss, float *grads);
/* corrections [batch][H][W] (physical units) for a host batch */
int ns_cnn_forward_host(ns_cnn *c, const float *inputs, int batch, float *out);
/* iterations AdamW steps (beta 0.9 / 0.999, eps 1e-8, decoupled weight decay) on
 * minibatches drawn from the dataset with a seeded generator; loss_history may be NULL */
int ns_cnn_train(ns_cnn *c, int iterations, int batch, float lr, float weight_decay, uint64_t seed, double *loss_history);
/* The four 64 -> 64 layers run on the tcgen05 tensor cores (BF16 activations and
 * weights, FP32 accumulation in tensor memory) when W is a multiple of 128 (the
 * default there); 0 selects the FP32 SIMT kernels for every layer. */
int ns_cnn_set_tensor_cores(ns_cnn *c, int enable);
/* Failure-detection self-test of the tensor-core layer (W a multiple of 128):
 * every completion wait of that kernel is bounded, and on expiry the kernel
 * records an error, frees its tensor memory and returns instead of waiting
 * forever.  This launch issues no MMA, so each wait runs out after wait_cycles
 * clock cycles (1 .. about 2 s worth); *timed_out receives 1 when the expiry
 * was recorded.  With no tensor-core work in flight the network stays usable.
 * A timeout reported by a real launch (training or inference) instead marks the
 * network unusable: its MMAs may still have been running when the kernel
 * returned, so later tensor-core launches fail until the network is destroyed
 * and recreated. */
int ns_cnn_probe_wait_timeout(ns_cnn *c, long long wait_cycles, int *timed_out);
/* Mean CUDA-event time of one 64 -> 64 hidden layer (the network's dominant
 * kernel) on batch samples, over reps launches after one untimed launch: the
 * training path (FP32 pre-activation and activation plus the BF16 activation),
 * and the inference path (BF16 activation only, as the corrected step runs it). */
int ns_cnn_time_hidden_layer(ns_cnn *c, int batch, int reps, double *ms_per_launch);
int ns_cnn_time_hidden_layer_inference(ns_cnn *c, int batch, int reps, double *ms_per_launch);
/* nsteps corrected steps of an instance on the network's grid: plain RK4 step
 * (ns_gpu_advance), then omega += CNN(omega(t), omega(t+dt) - omega(t)) */
int ns_cnn_correct_step(ns_cnn *c, ns_gpu *g, int nsteps);

#ifdef __cplusplus
}
#endif

#endif /* NS_GPU_H */
