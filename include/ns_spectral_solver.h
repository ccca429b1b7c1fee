/*
 * ns_spectral_solver.h -- drop-in replacement for the reference solver header
 * src/spectral/ns_spectral_solver.h:1-115 (DiogoRibeiro7/navier-stokes-solvers).
 *
 * The 24 functions and the NSSpectralData / NSSpectralHyperviscosityConfig
 * layouts are those of the reference, so existing callers recompile and relink
 * unchanged.  The work of every function runs on the GPU (sm_103a kernels
 * behind include/ns_gpu.h); host arrays stay the source of truth at every call,
 * as in the reference, and are copied to and from the device inside the call.
 *
 * FFTW is not needed: fftw_complex is the C99 double _Complex that the
 * reference gets by including <complex.h> before <fftw3.h> (:5-6), and
 * fftw_plan is an opaque pointer.  The typedefs are identical to FFTW's, so
 * this header may be combined with a real fftw3.h.
 *
 * One field is appended after the reference fields (existing offsets do not
 * move): `gpu`, the per-instance device state.
 *
 * Extensions (no reference counterpart) are declared at the end: FP32
 * instances, multi-step device-resident advance with device-side CFL dt,
 * forcing, seeded random-spectrum initial condition, diagnostics.
 */
#ifndef NS_SPECTRAL_SOLVER_H
#define NS_SPECTRAL_SOLVER_H

#include "common_types.h"
#include <complex.h>

#ifndef FFTW3_H
typedef double _Complex fftw_complex;
typedef struct fftw_plan_s *fftw_plan;
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int enabled;
    double coefficient;
    int order;
    double cutoff_ratio;
    double sfd_strength;
    double sfd_timescale;
    int sfd_enabled;
    double kmax;
    double cutoff_wavenumber;
    double inv_bandwidth;
} NSSpectralHyperviscosityConfig;

struct ns_spectral_gpu;

typedef struct {
    int nx, ny;
    int nkx, nky;
    double Lx, Ly;
    double Re;
    double dt;
    double t;
    double cfl_factor;

    double *NS_RESTRICT u;
    double *NS_RESTRICT v;
    double *NS_RESTRICT p;
    double *NS_RESTRICT omega;
    double *NS_RESTRICT psi;
    double *NS_RESTRICT x;
    double *NS_RESTRICT y;

    fftw_complex *NS_RESTRICT u_hat;
    fftw_complex *NS_RESTRICT v_hat;
    fftw_complex *NS_RESTRICT omega_hat;
    fftw_complex *NS_RESTRICT psi_hat;
    fftw_complex *NS_RESTRICT nonlinear_hat;
    fftw_complex *NS_RESTRICT rk1_hat;
    fftw_complex *NS_RESTRICT rk2_hat;
    fftw_complex *NS_RESTRICT rk3_hat;
    fftw_complex *NS_RESTRICT rk4_hat;
    fftw_complex *NS_RESTRICT omega_tmp_hat;

    double *NS_RESTRICT kx;
    double *NS_RESTRICT ky;
    double *NS_RESTRICT k2;

    fftw_plan forward_plan, backward_plan;

    int *NS_RESTRICT dealias_mask;

    NSSpectralHyperviscosityConfig hyperviscosity;
    double *NS_RESTRICT hyperviscosity_weights;
    fftw_complex *NS_RESTRICT sfd_hat;

    /* appended: device state of this instance (not part of the reference layout) */
    struct ns_spectral_gpu *gpu;
} NSSpectralData;

/* Memory management (spectral_memory.c:6-104).  allocate returns NULL on any
 * failure, including the absence of a CUDA device and a size outside what the
 * device transforms take (nx, ny in [8, 4096], transform lengths nx/2 or odd nx,
 * and ny, free of prime factors above 31; the reason goes to stderr); free is
 * per instance. */
NSSpectralData *ns_spectral_allocate(int nx, int ny, double Lx, double Ly, double Re);
void ns_spectral_free(NSSpectralData *data);

/* Initialization (spectral_initialization.c:10-95) */
void ns_spectral_initialize_grids(NSSpectralData *data);
void ns_spectral_initialize_fft_plans(NSSpectralData *data);
void ns_spectral_initialize_taylor_green(NSSpectralData *data);

/* Transforms (spectral_transforms.c:9-43) */
void ns_spectral_physical_to_spectral(NSSpectralData *data, double *field, fftw_complex *field_hat);
void ns_spectral_spectral_to_physical(NSSpectralData *data, fftw_complex *field_hat, double *field);
void ns_spectral_apply_dealiasing(NSSpectralData *data, fftw_complex *field_hat);

/* Core solver functions (spectral_core.c:8-112) */
void ns_spectral_compute_derivatives(NSSpectralData *data);
void ns_spectral_compute_velocity_from_vorticity(NSSpectralData *data);
void ns_spectral_compute_nonlinear_terms(NSSpectralData *data);

/* Time integration (spectral_time_integration.c:9-106) */
void ns_spectral_advance_rk4(NSSpectralData *data);
double ns_spectral_compute_cfl_timestep(NSSpectralData *data);

/* Analysis (spectral_analysis.c:8-142) */
double ns_spectral_compute_energy(NSSpectralData *data);
double ns_spectral_compute_enstrophy(NSSpectralData *data);
void ns_spectral_analyze_convergence(NSSpectralData *data, int step);
void ns_spectral_analyze_spectrum(NSSpectralData *data);
int ns_spectral_check_resolution(NSSpectralData *data);

/* Hyperviscosity / damping (hyperviscosity.c:15-178) */
void ns_spectral_hyperviscosity_default(NSSpectralHyperviscosityConfig *config);
void ns_spectral_hyperviscosity_set(NSSpectralData *data, const NSSpectralHyperviscosityConfig *config);
void ns_spectral_hyperviscosity_update_weights(NSSpectralData *data);
void ns_spectral_hyperviscosity_apply(NSSpectralData *data, fftw_complex *rhs_hat, const fftw_complex *state_hat);
void ns_spectral_hyperviscosity_post_step(NSSpectralData *data, const fftw_complex *state_hat, double dt);

/* Output (spectral_output.c:4-27) */
void ns_spectral_output_solution(NSSpectralData *data, const char *filename);

/* ------------------------------------------------------------------
 * Extensions (no reference counterpart).  All return a SolverStatus.
 * ------------------------------------------------------------------ */
enum { NS_PRECISION_FP64 = 0, NS_PRECISION_FP32 = 1 };

/* allocate with the arithmetic precision of the device step (FP64 or FP32 bulk) */
NSSpectralData *ns_spectral_allocate_ex(int nx, int ny, double Lx, double Ly, double Re, int precision);
/* Advance nsteps RK4 steps on the device without touching host arrays between
 * steps.  adaptive_dt = 1 recomputes dt at every step from the reference CFL
 * rule (cfl_factor) on the device; 0 uses data->dt.  Host arrays become stale
 * until ns_spectral_gpu_sync_host; any reference-API call syncs them first. */
int ns_spectral_gpu_advance_n(NSSpectralData *data, int nsteps, int adaptive_dt);
/* copy the device state into the host arrays (omega_hat, psi_hat, u_hat, v_hat,
 * sfd_hat, u, v, omega, t, dt) */
int ns_spectral_gpu_sync_host(NSSpectralData *data);
/* white-in-time forcing on kmin <= |k| <= kmax with injection rate epsilon
 * (Philox4x64-10 keyed by seed), applied after each RK4 step */
int ns_spectral_gpu_set_forcing(NSSpectralData *data, int enabled, double kmin, double kmax, double epsilon,
                                unsigned long long seed);
/* time scheme of ns_spectral_advance_rk4 and ns_spectral_gpu_advance_n:
 * NS_SPECTRAL_SCHEME_RK4 (default: the reference's classical RK4) or
 * NS_SPECTRAL_SCHEME_IFRK4 (integrating-factor RK4, viscous and hyperviscous
 * decay integrated exactly; no reference counterpart) */
#define NS_SPECTRAL_SCHEME_RK4 0
#define NS_SPECTRAL_SCHEME_IFRK4 1
int ns_spectral_gpu_set_scheme(NSSpectralData *data, int scheme);
/* Parseval energy and enstrophy of the device state (FP64 compensated);
 * SOLVER_DIVERGED when the state holds non-finite values */
int ns_spectral_gpu_diagnostics(NSSpectralData *data, double *energy, double *enstrophy);
/* seeded random-phase vorticity, E(k) ~ k^4 exp(-(k/k0)^2), kinetic energy `energy`;
 * leaves omega_hat set and refreshes psi_hat, u_hat, v_hat, u, v, omega */
int ns_spectral_initialize_random_spectrum(NSSpectralData *data, unsigned long long seed, double k0, double energy);
/* message of the last failing GPU call of this instance */
const char *ns_spectral_gpu_last_error(const NSSpectralData *data);
/* the C-ABI instance behind this solver (include/ns_gpu.h) */
struct ns_gpu *ns_spectral_gpu_handle(NSSpectralData *data);

#ifdef __cplusplus
}
#endif

#endif /* NS_SPECTRAL_SOLVER_H */
