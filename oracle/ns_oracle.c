/*
 * CPU restatement of the reference's Fourier pseudospectral step (FP64).
 *
 * ORACLE / TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline and reference legs load this library, and only as the
 * checker or the timed CPU baseline; the GPU product never links or calls it.
 *
 * Every function restates one reference function (DiogoRibeiro7/navier-stokes-
 * solvers, paths relative to that project) and cites it.  Arithmetic is written
 * in the same evaluation order as the reference so that, over the same FFT
 * (oracle/fftw_shim.c), the restatement reproduces the reference compiled from
 * its own sources (oracle/_ref/) bit for bit at one thread; tests check that.
 *
 * The state struct has the exact field order of NSSpectralData
 * (src/spectral/ns_spectral_solver.h:8-68) so one ctypes mirror drives the
 * reference build, this restatement and the GPU drop-in alike.
 *
 * Project extensions with no reference counterpart (named nso_ext_*):
 *   - Philox4x64-10 counter RNG (Salmon et al., SC'11, "Parallel Random
 *     Numbers: As Easy as 1, 2, 3"), checked against numpy.random.Philox;
 *   - seeded random-phase initial vorticity with E(k) ~ k^4 exp(-(k/k0)^2);
 *   - white-in-time band-limited forcing with a target injection rate, added
 *     after the RK4 update (Euler-Maruyama splitting);
 *   - an n-step driver with the reference's CFL rule.
 */
#include "fftw3.h"

#include <complex.h>
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

/* include/common_types.h:32-33 */
#define NSO_MIN_DT 1e-8
#define NSO_MAX_DT 0.1

/* src/spectral/ns_spectral_solver.h:8-19 */
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
} nso_hv_config;

/* src/spectral/ns_spectral_solver.h:22-68 (same field order) */
typedef struct {
    int nx, ny;
    int nkx, nky;
    double Lx, Ly;
    double Re;
    double dt;
    double t;
    double cfl_factor;
    double *u, *v, *p, *omega, *psi, *x, *y;
    fftw_complex *u_hat, *v_hat, *omega_hat, *psi_hat, *nonlinear_hat;
    fftw_complex *rk1_hat, *rk2_hat, *rk3_hat, *rk4_hat, *omega_tmp_hat;
    double *kx, *ky, *k2;
    fftw_plan forward_plan, backward_plan;
    int *dealias_mask;
    nso_hv_config hyperviscosity;
    double *hyperviscosity_weights;
    fftw_complex *sfd_hat;
} nso_state;

static int nso_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ---------------------------------------------------------------- memory */

void nso_free(nso_state *s);
void nso_hv_default(nso_hv_config *cfg);

/* src/spectral/spectral_memory.c:6-68: nkx = nx/2+1, dt = 0.01, cfl 0.3,
 * NULL on any allocation failure, HV defaults, zeroed weights and SFD. */
nso_state *nso_allocate(int nx, int ny, double Lx, double Ly, double Re) {
    nso_state *s = (nso_state *)calloc(1, sizeof(nso_state));
    if (!s) return NULL;
    s->nx = nx;
    s->ny = ny;
    s->nkx = nx / 2 + 1;
    s->nky = ny;
    s->Lx = Lx;
    s->Ly = Ly;
    s->Re = Re;
    s->dt = 0.01;
    s->t = 0.0;
    s->cfl_factor = 0.3;
    const size_t nr = (size_t)nx * (size_t)ny;
    const size_t nc = (size_t)s->nkx * (size_t)s->nky;
    double **reals[] = {&s->u, &s->v, &s->p, &s->omega, &s->psi};
    for (size_t i = 0; i < sizeof(reals) / sizeof(reals[0]); ++i) *reals[i] = fftw_alloc_real(nr);
    fftw_complex **cplx[] = {&s->u_hat, &s->v_hat, &s->omega_hat, &s->psi_hat, &s->nonlinear_hat,
                             &s->rk1_hat, &s->rk2_hat, &s->rk3_hat, &s->rk4_hat, &s->omega_tmp_hat,
                             &s->sfd_hat};
    for (size_t i = 0; i < sizeof(cplx) / sizeof(cplx[0]); ++i) *cplx[i] = fftw_alloc_complex(nc);
    s->x = (double *)calloc((size_t)nx, sizeof(double));
    s->y = (double *)calloc((size_t)ny, sizeof(double));
    s->kx = (double *)calloc((size_t)s->nkx, sizeof(double));
    s->ky = (double *)calloc((size_t)s->nky, sizeof(double));
    s->k2 = (double *)calloc(nc, sizeof(double));
    s->dealias_mask = (int *)calloc(nc, sizeof(int));
    s->hyperviscosity_weights = (double *)calloc(nc, sizeof(double));
    int ok = s->x && s->y && s->kx && s->ky && s->k2 && s->dealias_mask && s->hyperviscosity_weights;
    for (size_t i = 0; i < sizeof(reals) / sizeof(reals[0]); ++i) ok = ok && *reals[i];
    for (size_t i = 0; i < sizeof(cplx) / sizeof(cplx[0]); ++i) ok = ok && *cplx[i];
    if (!ok) {
        nso_free(s);
        return NULL;
    }
    nso_hv_default(&s->hyperviscosity);
    return s;
}

/* src/spectral/spectral_memory.c:71-104 (per instance; no global cleanup) */
void nso_free(nso_state *s) {
    if (!s) return;
    if (s->forward_plan) fftw_destroy_plan(s->forward_plan);
    if (s->backward_plan) fftw_destroy_plan(s->backward_plan);
    double *reals[] = {s->u, s->v, s->p, s->omega, s->psi};
    for (size_t i = 0; i < 5; ++i) fftw_free(reals[i]);
    fftw_complex *cplx[] = {s->u_hat, s->v_hat, s->omega_hat, s->psi_hat, s->nonlinear_hat,
                            s->rk1_hat, s->rk2_hat, s->rk3_hat, s->rk4_hat, s->omega_tmp_hat,
                            s->sfd_hat};
    for (size_t i = 0; i < 11; ++i) fftw_free(cplx[i]);
    free(s->x);
    free(s->y);
    free(s->kx);
    free(s->ky);
    free(s->k2);
    free(s->dealias_mask);
    free(s->hyperviscosity_weights);
    free(s);
}

/* ------------------------------------------------------ hyperviscosity */

static double nso_clamp(double v, double lo, double hi) { return v < lo ? lo : (v > hi ? hi : v); }

/* src/spectral/hyperviscosity.c:15-30 */
void nso_hv_default(nso_hv_config *cfg) {
    if (!cfg) return;
    cfg->enabled = 0;
    cfg->coefficient = 0.0;
    cfg->order = 8;
    cfg->cutoff_ratio = 0.65;
    cfg->sfd_strength = 0.0;
    cfg->sfd_timescale = 1.0;
    cfg->sfd_enabled = 0;
    cfg->kmax = 0.0;
    cfg->cutoff_wavenumber = 0.0;
    cfg->inv_bandwidth = 0.0;
}

/* src/spectral/hyperviscosity.c:60-102: kmax over all modes, ramp power law
 * w = c*((|k|-kc)/(kmax-kc))^order above kc = cutoff_ratio*kmax */
void nso_hv_update_weights(nso_state *s) {
    if (!s || !s->hyperviscosity_weights || !s->k2) return;
    const int n = s->nkx * s->nky;
    nso_hv_config *cfg = &s->hyperviscosity;
    double kmax = 0.0;
    for (int i = 0; i < n; ++i) kmax = fmax(kmax, sqrt(s->k2[i]));
    cfg->kmax = kmax;
    const double ratio = nso_clamp(cfg->cutoff_ratio, 0.0, 1.0);
    cfg->cutoff_wavenumber = ratio * kmax;
    const double bw = fmax(kmax - cfg->cutoff_wavenumber, 1e-12);
    cfg->inv_bandwidth = (bw > 0.0) ? 1.0 / bw : 0.0;
    if (!cfg->enabled || cfg->coefficient <= 0.0 || kmax <= 0.0) {
        memset(s->hyperviscosity_weights, 0, sizeof(double) * (size_t)n);
        return;
    }
    const int order = cfg->order > 0 ? cfg->order : 1;
    for (int i = 0; i < n; ++i) {
        const double km = sqrt(s->k2[i]);
        double w = 0.0;
        if (km > cfg->cutoff_wavenumber) w = cfg->coefficient * pow((km - cfg->cutoff_wavenumber) * cfg->inv_bandwidth, order);
        s->hyperviscosity_weights[i] = w;
    }
}

/* src/spectral/hyperviscosity.c:32-58 */
void nso_hv_set(nso_state *s, const nso_hv_config *cfg) {
    if (!s || !cfg) return;
    const size_t n = (size_t)s->nkx * (size_t)s->nky;
    s->hyperviscosity = *cfg;
    if (!s->hyperviscosity.enabled) memset(s->hyperviscosity_weights, 0, n * sizeof(double));
    if (!s->hyperviscosity.sfd_enabled || s->hyperviscosity.sfd_strength <= 0.0) {
        s->hyperviscosity.sfd_enabled = 0;
        s->hyperviscosity.sfd_strength = 0.0;
        memset(s->sfd_hat, 0, n * sizeof(fftw_complex));
    }
    nso_hv_update_weights(s);
    if (s->hyperviscosity.sfd_enabled && s->sfd_hat && s->omega_hat)
        memcpy(s->sfd_hat, s->omega_hat, n * sizeof(fftw_complex));
}

/* src/spectral/hyperviscosity.c:104-150: rhs -= w*state + s*ramp*(state - sfd) */
void nso_hv_apply(nso_state *s, fftw_complex *rhs, const fftw_complex *state) {
    if (!s || !rhs || !state) return;
    const nso_hv_config *cfg = &s->hyperviscosity;
    const int n = s->nkx * s->nky;
    const int visc = cfg->enabled && cfg->coefficient > 0.0;
    const int sfd = cfg->sfd_enabled && cfg->sfd_strength > 0.0;
    const int order = cfg->order > 0 ? cfg->order : 1;
    if (!visc && !sfd) return;
#pragma omp parallel for
    for (int i = 0; i < n; ++i) {
        fftw_complex damp = 0.0;
        if (visc) damp += s->hyperviscosity_weights[i] * state[i];
        if (sfd) {
            double ramp = 0.0;
            if (cfg->inv_bandwidth > 0.0) {
                const double km = sqrt(s->k2[i]);
                if (km > cfg->cutoff_wavenumber)
                    ramp = pow(nso_clamp((km - cfg->cutoff_wavenumber) * cfg->inv_bandwidth, 0.0, 1.0), order);
            }
            const double sw = cfg->sfd_strength * ramp;
            if (sw > 0.0) damp += sw * (state[i] - s->sfd_hat[i]);
        }
        rhs[i] -= damp;
    }
}

/* src/spectral/hyperviscosity.c:152-178: sfd <- (1-a) sfd + a state, a = clamp(dt/tau) */
void nso_hv_post_step(nso_state *s, const fftw_complex *state, double dt) {
    if (!s || !state || dt <= 0.0) return;
    nso_hv_config *cfg = &s->hyperviscosity;
    if (!cfg->sfd_enabled || cfg->sfd_strength <= 0.0 || cfg->sfd_timescale <= 0.0) return;
    double a = dt / cfg->sfd_timescale;
    if (a > 1.0) a = 1.0;
    else if (a < 0.0) a = 0.0;
    const int n = s->nkx * s->nky;
#pragma omp parallel for
    for (int i = 0; i < n; ++i) {
        const fftw_complex prev = s->sfd_hat[i];
        s->sfd_hat[i] = (1.0 - a) * prev + a * state[i];
    }
}

/* ---------------------------------------------------------- initialisation */

/* src/spectral/spectral_initialization.c:10-54: grid, wavenumbers, k^2, 2/3 mask
 * (keep i <= floor(2*nkx/3) and |band| <= floor(2*ny/6)), then HV weights */
void nso_initialize_grids(nso_state *s) {
    const int nx = s->nx, ny = s->ny;
    for (int i = 0; i < nx; ++i) s->x[i] = i * s->Lx / nx;
    for (int j = 0; j < ny; ++j) s->y[j] = j * s->Ly / ny;
    for (int i = 0; i < s->nkx; ++i) s->kx[i] = 2.0 * M_PI * i / s->Lx;
    for (int j = 0; j < s->nky; ++j) s->ky[j] = (j <= ny / 2) ? 2.0 * M_PI * j / s->Ly : 2.0 * M_PI * (j - ny) / s->Ly;
    for (int j = 0; j < s->nky; ++j) {
        for (int i = 0; i < s->nkx; ++i) {
            const int idx = j * s->nkx + i;
            s->k2[idx] = s->kx[i] * s->kx[i] + s->ky[j] * s->ky[j];
            const int band = (j <= ny / 2) ? j : j - ny;
            s->dealias_mask[idx] = (i <= (2 * s->nkx) / 3) && (abs(band) <= (2 * ny) / 6);
        }
    }
    nso_hv_update_weights(s);
}

/* src/spectral/spectral_initialization.c:57-69 */
void nso_initialize_fft_plans(nso_state *s) {
    fftw_init_threads();
    fftw_plan_with_nthreads(nso_threads());
    s->forward_plan = fftw_plan_dft_r2c_2d(s->ny, s->nx, s->omega, s->omega_hat, FFTW_MEASURE);
    s->backward_plan = fftw_plan_dft_c2r_2d(s->ny, s->nx, s->omega_hat, s->omega, FFTW_MEASURE);
}

/* ------------------------------------------------------------- transforms */

/* src/spectral/spectral_transforms.c:35-43 */
void nso_apply_dealiasing(nso_state *s, fftw_complex *f) {
    const int n = s->nkx * s->nky;
#pragma omp parallel for
    for (int i = 0; i < n; ++i)
        if (!s->dealias_mask[i]) f[i] = 0.0;
}

/* src/spectral/spectral_transforms.c:9-22: r2c, scale 1/(nx*ny), mask */
void nso_physical_to_spectral(nso_state *s, double *field, fftw_complex *field_hat) {
    fftw_execute_dft_r2c(s->forward_plan, field, field_hat);
    const double norm = 1.0 / (s->nx * s->ny);
    const int n = s->nkx * s->nky;
#pragma omp parallel for
    for (int i = 0; i < n; ++i) field_hat[i] *= norm;
    nso_apply_dealiasing(s, field_hat);
}

/* src/spectral/spectral_transforms.c:25-32: masked copy into nonlinear_hat, c2r */
void nso_spectral_to_physical(nso_state *s, fftw_complex *field_hat, double *field) {
    const int n = s->nkx * s->nky;
    memcpy(s->nonlinear_hat, field_hat, (size_t)n * sizeof(fftw_complex));
    nso_apply_dealiasing(s, s->nonlinear_hat);
    fftw_execute_dft_c2r(s->backward_plan, s->nonlinear_hat, field);
}

/* src/spectral/spectral_initialization.c:72-95 */
void nso_initialize_taylor_green(nso_state *s) {
    const int nx = s->nx, ny = s->ny;
    for (int j = 0; j < ny; ++j) {
        for (int i = 0; i < nx; ++i) {
            const int idx = j * nx + i;
            const double x = s->x[i], y = s->y[j];
            s->u[idx] = sin(2 * M_PI * x / s->Lx) * cos(2 * M_PI * y / s->Ly);
            s->v[idx] = -cos(2 * M_PI * x / s->Lx) * sin(2 * M_PI * y / s->Ly);
            s->omega[idx] = 2.0 * (2 * M_PI / s->Lx) * cos(2 * M_PI * x / s->Lx) * cos(2 * M_PI * y / s->Ly);
            s->p[idx] = 0.0;
        }
    }
    nso_physical_to_spectral(s, s->omega, s->omega_hat);
    nso_physical_to_spectral(s, s->u, s->u_hat);
    nso_physical_to_spectral(s, s->v, s->v_hat);
}

/* ------------------------------------------------------------------- core */

/* src/spectral/spectral_core.c:8-34: psi = -omega/k^2 (0 where k^2 <= 1e-12),
 * u_hat = i ky psi, v_hat = -i kx psi */
void nso_compute_velocity_from_vorticity(nso_state *s) {
#pragma omp parallel for
    for (int j = 0; j < s->nky; ++j) {
        for (int i = 0; i < s->nkx; ++i) {
            const int idx = j * s->nkx + i;
            if (s->k2[idx] > 1e-12) s->psi_hat[idx] = -s->omega_hat[idx] / s->k2[idx];
            else s->psi_hat[idx] = 0.0;
        }
    }
#pragma omp parallel for
    for (int j = 0; j < s->nky; ++j) {
        for (int i = 0; i < s->nkx; ++i) {
            const int idx = j * s->nkx + i;
            s->u_hat[idx] = I * s->ky[j] * s->psi_hat[idx];
            s->v_hat[idx] = -I * s->kx[i] * s->psi_hat[idx];
        }
    }
}

/* src/spectral/spectral_core.c:37-43 */
void nso_compute_derivatives(nso_state *s) {
    nso_compute_velocity_from_vorticity(s);
    nso_spectral_to_physical(s, s->u_hat, s->u);
    nso_spectral_to_physical(s, s->v_hat, s->v);
    nso_spectral_to_physical(s, s->omega_hat, s->omega);
}

/* scratch = i * k_axis * src, then masked c2r into dst (spectral_core.c:62-99) */
static void nso_derivative_to_physical(nso_state *s, const fftw_complex *src, int axis_y, double *dst) {
    fftw_complex *scratch = s->nonlinear_hat;
#pragma omp parallel for
    for (int j = 0; j < s->nky; ++j) {
        for (int i = 0; i < s->nkx; ++i) {
            const int idx = j * s->nkx + i;
            scratch[idx] = I * (axis_y ? s->ky[j] : s->kx[i]) * src[idx];
        }
    }
    nso_spectral_to_physical(s, scratch, dst);
}

/* src/spectral/spectral_core.c:46-112: N = -mask(r2c(psi_x*omega_y - psi_y*omega_x))/N^2
 * using psi_hat as stored; physical arrays aliased as in the reference (:54-59) */
void nso_compute_nonlinear_terms(nso_state *s) {
    const int nr = s->nx * s->ny;
    const int n = s->nkx * s->nky;
    nso_spectral_to_physical(s, s->psi_hat, s->psi);
    nso_spectral_to_physical(s, s->omega_hat, s->omega);
    double *psi_x = s->u, *psi_y = s->v, *omega_x = s->psi, *omega_y = s->omega, *jac = s->p;
    nso_derivative_to_physical(s, s->psi_hat, 0, psi_x);
    nso_derivative_to_physical(s, s->psi_hat, 1, psi_y);
    nso_derivative_to_physical(s, s->omega_hat, 0, omega_x);
    nso_derivative_to_physical(s, s->omega_hat, 1, omega_y);
#pragma omp parallel for
    for (int k = 0; k < nr; ++k) jac[k] = psi_x[k] * omega_y[k] - psi_y[k] * omega_x[k];
    nso_physical_to_spectral(s, jac, s->nonlinear_hat);
#pragma omp parallel for
    for (int k = 0; k < n; ++k) s->nonlinear_hat[k] = -s->nonlinear_hat[k];
}

/* ------------------------------------------------------- time integration */

/* src/spectral/spectral_time_integration.c:9-31 */
double nso_compute_cfl_timestep(nso_state *s) {
    const int nr = s->nx * s->ny;
    double vmax = 0.0;
#pragma omp parallel for reduction(max : vmax)
    for (int k = 0; k < nr; ++k) {
        const double m = sqrt(s->u[k] * s->u[k] + s->v[k] * s->v[k]);
        if (m > vmax) vmax = m;
    }
    const double dxmin = fmin(s->Lx / s->nx, s->Ly / s->ny);
    const double dt_cfl = s->cfl_factor * dxmin / (vmax + 1e-12);
    const double dt_visc = 0.5 * s->Re * dxmin * dxmin;
    double dt = fmin(dt_cfl, dt_visc);
    dt = fmax(dt, NSO_MIN_DT);
    dt = fmin(dt, NSO_MAX_DT);
    return dt;
}

/* k = N - k^2 * omega / Re, then hyperviscosity (spectral_time_integration.c:50-54) */
static void nso_stage_rhs(nso_state *s, fftw_complex *kout, double inv_re) {
    const int n = s->nkx * s->nky;
#pragma omp parallel for
    for (int k = 0; k < n; ++k) kout[k] = s->nonlinear_hat[k] - s->k2[k] * s->omega_hat[k] * inv_re;
    nso_hv_apply(s, kout, s->omega_hat);
}

/* omega = omega_tmp + c * kin (spectral_time_integration.c:57-60) */
static void nso_stage_state(nso_state *s, const fftw_complex *kin, double c) {
    const int n = s->nkx * s->nky;
#pragma omp parallel for
    for (int k = 0; k < n; ++k) s->omega_hat[k] = s->omega_tmp_hat[k] + c * kin[k];
}

typedef struct {
    int enabled;
    double kmin, kmax;  /* forced shell, inclusive */
    double epsilon;     /* target energy injection rate */
    uint64_t seed;
    uint64_t step;      /* per-step counter for the RNG, advanced by the driver */
} nso_ext_forcing;

static void nso_ext_apply_forcing(nso_state *s, const nso_ext_forcing *f, double dt);

/* src/spectral/spectral_time_integration.c:34-106: classical RK4; the optional
 * forcing hook (project extension) runs after the final update, before the
 * SFD post-step. */
static void nso_advance_rk4_impl(nso_state *s, const nso_ext_forcing *forcing) {
    const int n = s->nkx * s->nky;
    const double dt = s->dt;
    memcpy(s->omega_tmp_hat, s->omega_hat, (size_t)n * sizeof(fftw_complex));
    const double inv_re = 1.0 / s->Re;
    nso_compute_nonlinear_terms(s);
    nso_stage_rhs(s, s->rk1_hat, inv_re);
    nso_stage_state(s, s->rk1_hat, 0.5 * dt);
    nso_compute_derivatives(s);
    nso_compute_nonlinear_terms(s);
    nso_stage_rhs(s, s->rk2_hat, inv_re);
    nso_stage_state(s, s->rk2_hat, 0.5 * dt);
    nso_compute_derivatives(s);
    nso_compute_nonlinear_terms(s);
    nso_stage_rhs(s, s->rk3_hat, inv_re);
    nso_stage_state(s, s->rk3_hat, dt);
    nso_compute_derivatives(s);
    nso_compute_nonlinear_terms(s);
    nso_stage_rhs(s, s->rk4_hat, inv_re);
#pragma omp parallel for
    for (int k = 0; k < n; ++k)
        s->omega_hat[k] = s->omega_tmp_hat[k] +
                          dt / 6.0 * (s->rk1_hat[k] + 2.0 * s->rk2_hat[k] + 2.0 * s->rk3_hat[k] + s->rk4_hat[k]);
    if (forcing && forcing->enabled) nso_ext_apply_forcing(s, forcing, dt);
    nso_hv_post_step(s, s->omega_hat, dt);
    s->t += dt;
    nso_compute_derivatives(s);
}

void nso_advance_rk4(nso_state *s) { nso_advance_rk4_impl(s, NULL); }

/* --------------------------------------------------------------- analysis */

/* src/spectral/spectral_analysis.c:8-19 */
double nso_compute_energy(nso_state *s) {
    const int nr = s->nx * s->ny;
    double e = 0.0;
    for (int k = 0; k < nr; ++k) e += 0.5 * (s->u[k] * s->u[k] + s->v[k] * s->v[k]);
    return e / (s->nx * s->ny);
}

/* src/spectral/spectral_analysis.c:22-33 */
double nso_compute_enstrophy(nso_state *s) {
    const int nr = s->nx * s->ny;
    double z = 0.0;
    for (int k = 0; k < nr; ++k) z += 0.5 * s->omega[k] * s->omega[k];
    return z / (s->nx * s->ny);
}

/* src/spectral/spectral_analysis.c:36-66: fraction of sum |omega_hat|^2 above
 * 0.8*kmax with kmax = sqrt(k2[last]); returns 1 when below 1e-6 */
int nso_check_resolution(nso_state *s, double *fraction_out) {
    const int n = s->nkx * s->nky;
    const double max_k = sqrt(s->k2[n - 1]);
    double hi = 0.0, tot = 0.0;
    for (int idx = 0; idx < n; ++idx) {
        const double m2 = cabs(s->omega_hat[idx]) * cabs(s->omega_hat[idx]);
        tot += m2;
        const double kn = (max_k > 0.0) ? sqrt(s->k2[idx]) / max_k : 0.0;
        if (kn > 0.8) hi += m2;
    }
    const double frac = (tot > 1e-16) ? hi / tot : 0.0;
    if (fraction_out) *fraction_out = frac;
    return frac > 1e-6 ? 0 : 1;
}

/* src/spectral/spectral_analysis.c:69-100 (statistics only, no printing):
 * max|omega_hat| and sqrt(mean |omega_hat|^2 over k^2 > k2[last]/4) */
void nso_convergence_stats(nso_state *s, double *max_abs, double *spectral_error) {
    const int n = s->nkx * s->nky;
    double mx = 0.0, acc = 0.0;
    int cnt = 0;
    for (int idx = 0; idx < n; ++idx) {
        const double m = cabs(s->omega_hat[idx]);
        if (m > mx) mx = m;
        if (s->k2[idx] > 0.25 * s->k2[n - 1]) {
            acc += m * m;
            cnt++;
        }
    }
    *max_abs = mx;
    *spectral_error = cnt > 0 ? sqrt(acc / cnt) : 0.0;
}

/* src/spectral/spectral_analysis.c:103-142 (binning only): bin (int)(|k|+0.5)
 * of 0.5(|u_hat|^2+|v_hat|^2) over the stored half plane, max_k = min(nkx, nky/2);
 * returns the number of bins, energy_k holds the per-bin SUM and count_k the count
 * (the reference prints sum/count). */
int nso_spectrum(nso_state *s, double *energy_k, int *count_k) {
    const int max_k = (int)fmin(s->nkx, s->nky / 2);
    memset(energy_k, 0, sizeof(double) * (size_t)max_k);
    memset(count_k, 0, sizeof(int) * (size_t)max_k);
    for (int j = 0; j < s->nky; ++j) {
        for (int i = 0; i < s->nkx; ++i) {
            const int idx = j * s->nkx + i;
            const int b = (int)(sqrt(s->k2[idx]) + 0.5);
            if (b < max_k) {
                const double u2 = cabs(s->u_hat[idx]) * cabs(s->u_hat[idx]);
                const double v2 = cabs(s->v_hat[idx]) * cabs(s->v_hat[idx]);
                energy_k[b] += 0.5 * (u2 + v2);
                count_k[b]++;
            }
        }
    }
    return max_k;
}

/* ----------------------------------------------------------------- forcing */

/* src/common/forcing.h:7-32 */
typedef struct {
    double kmin;
    double kmax;
    double energy_target;
    double correlation_time;
    unsigned long seed;
    int type; /* 0 white, 1 colored */
} nso_forcing_config;

typedef struct {
    nso_forcing_config config;
    int nkx, nky, spectral_size, active_modes;
    double *weights;
    double complex *colored_state;
    unsigned int have_spare;
    double spare_gaussian;
    unsigned long long rng_state;
} nso_forcing_state;

/* src/common/forcing.c:11-21 */
static uint64_t nso_splitmix64(uint64_t *st) {
    uint64_t z = (*st += UINT64_C(0x9E3779B97F4A7C15));
    z = (z ^ (z >> 30)) * UINT64_C(0xBF58476D1CE4E5B9);
    z = (z ^ (z >> 27)) * UINT64_C(0x94D049BB133111EB);
    return z ^ (z >> 31);
}

/* src/common/forcing.c:18-21: 53-bit uniform in [0,1) */
static double nso_uniform(nso_forcing_state *st) {
    uint64_t bits = nso_splitmix64((uint64_t *)&st->rng_state);
    return (double)(bits >> 11) * (1.0 / 9007199254740992.0);
}

/* src/common/forcing.c:23-39: Box-Muller with a cached spare */
static double nso_gaussian(nso_forcing_state *st) {
    if (st->have_spare) {
        st->have_spare = 0;
        return st->spare_gaussian;
    }
    double u1 = nso_uniform(st);
    double u2 = nso_uniform(st);
    u1 = fmax(u1, DBL_MIN);
    const double r = sqrt(-2.0 * log(u1));
    const double th = 2.0 * M_PI * u2;
    st->spare_gaussian = r * sin(th);
    st->have_spare = 1;
    return r * cos(th);
}

/* src/common/forcing.c:41-51 */
void nso_forcing_config_default(nso_forcing_config *c) {
    if (!c) return;
    c->kmin = 0.0;
    c->kmax = 4.0;
    c->energy_target = 1.0;
    c->correlation_time = 0.5;
    c->seed = 0;
    c->type = 0;
}

void nso_forcing_state_free(nso_forcing_state *st);

/* src/common/forcing.c:53-103: shell kmin <= |k| <= kmax inclusive, seed 0 -> 0x123456789abcdef */
int nso_forcing_state_init(nso_forcing_state *st, const nso_forcing_config *c, const double *k2, int nkx, int nky) {
    if (!st || !c || !k2 || nkx <= 0 || nky <= 0) return -1;
    memset(st, 0, sizeof(*st));
    st->config = *c;
    st->nkx = nkx;
    st->nky = nky;
    st->spectral_size = nkx * nky;
    st->weights = (double *)calloc((size_t)st->spectral_size, sizeof(double));
    if (!st->weights) return -1;
    if (c->type == 1) {
        st->colored_state = (double complex *)calloc((size_t)st->spectral_size, sizeof(double complex));
        if (!st->colored_state) {
            nso_forcing_state_free(st);
            return -1;
        }
    }
    const double kmin = fmax(c->kmin, 0.0);
    const double kmax = fmax(c->kmax, kmin);
    int active = 0;
    for (int idx = 0; idx < st->spectral_size; ++idx) {
        const double km = sqrt(k2[idx]);
        st->weights[idx] = (km >= kmin && km <= kmax) ? 1.0 : 0.0;
        if (st->weights[idx] > 0.0) active++;
    }
    st->active_modes = active;
    st->have_spare = 0;
    st->rng_state = c->seed ? c->seed : UINT64_C(0x123456789abcdef);
    return active == 0 ? -1 : 0;
}

/* src/common/forcing.c:105-115 */
void nso_forcing_state_free(nso_forcing_state *st) {
    if (!st) return;
    free(st->weights);
    st->weights = NULL;
    free(st->colored_state);
    st->colored_state = NULL;
    st->spectral_size = 0;
    st->active_modes = 0;
}

/* src/common/forcing.c:117-184: per active mode g1 + i g2 (white) or OU update
 * (colored), then global rescale so sum w^2 |value|^2 = energy_target */
void nso_forcing_generate(nso_forcing_state *st, double dt, const double *k2, double complex *out) {
    if (!st || !out || !k2) return;
    const int n = st->spectral_size;
    if (n == 0 || st->active_modes == 0) {
        memset(out, 0, (size_t)n * sizeof(double complex));
        return;
    }
    const nso_forcing_config *c = &st->config;
    if (c->energy_target <= 0.0) {
        memset(out, 0, (size_t)n * sizeof(double complex));
        if (st->colored_state) memset(st->colored_state, 0, (size_t)n * sizeof(double complex));
        return;
    }
    const double tau = fmax(c->correlation_time, 1e-6);
    const int colored = (c->type == 1);
    double alpha = 0.0, beta = 1.0;
    if (colored) {
        alpha = exp(-dt / tau);
        beta = sqrt(fmax(1.0 - alpha * alpha, 0.0));
    }
    double total = 0.0;
    for (int idx = 0; idx < n; ++idx) {
        if (st->weights[idx] <= 0.0) {
            out[idx] = 0.0;
            continue;
        }
        const double g1 = nso_gaussian(st);
        const double g2 = nso_gaussian(st);
        const double complex noise = g1 + I * g2;
        double complex val;
        if (colored) {
            st->colored_state[idx] = alpha * st->colored_state[idx] + beta * noise;
            val = st->colored_state[idx];
        } else {
            val = noise;
        }
        out[idx] = st->weights[idx] * val;
        total += pow(st->weights[idx], 2.0) * (creal(val) * creal(val) + cimag(val) * cimag(val));
    }
    total = fmax(total, 1e-16);
    const double scale = sqrt(c->energy_target / total);
    for (int idx = 0; idx < n; ++idx) {
        out[idx] *= scale;
        if (colored) st->colored_state[idx] *= scale;
    }
}

/* ------------------------------------------------- project extensions (ext) */

/* Philox4x64-10 (Salmon et al. 2011): 10 rounds of
 *   (hi0,lo0) = M0*c0, (hi1,lo1) = M1*c2, c = (hi1^c1^k0, lo1, hi0^c3^k1, lo0)
 * with the key bumped by the Weyl constants between rounds. */
static void nso_mulhilo64(uint64_t a, uint64_t b, uint64_t *hi, uint64_t *lo) {
    __uint128_t p = (__uint128_t)a * (__uint128_t)b;
    *hi = (uint64_t)(p >> 64);
    *lo = (uint64_t)p;
}

void nso_ext_philox4x64(const uint64_t ctr_in[4], const uint64_t key_in[2], uint64_t out[4]) {
    uint64_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
    uint64_t k0 = key_in[0], k1 = key_in[1];
    for (int r = 0; r < 10; ++r) {
        if (r > 0) {
            k0 += UINT64_C(0x9E3779B97F4A7C15);
            k1 += UINT64_C(0xBB67AE8584CAA73B);
        }
        uint64_t hi0, lo0, hi1, lo1;
        nso_mulhilo64(UINT64_C(0xD2E7470EE14C6C93), c0, &hi0, &lo0);
        nso_mulhilo64(UINT64_C(0xCA5A826395121157), c2, &hi1, &lo1);
        c0 = hi1 ^ c1 ^ k0;
        c1 = lo1;
        c2 = hi0 ^ c3 ^ k1;
        c3 = lo0;
    }
    out[0] = c0;
    out[1] = c1;
    out[2] = c2;
    out[3] = c3;
}

static double nso_u53(uint64_t b) { return (double)(b >> 11) * (1.0 / 9007199254740992.0); }

/* stream tags in counter word 2 keep the IC and the forcing draws apart */
#define NSO_TAG_IC UINT64_C(0x49430000)
#define NSO_TAG_FORCE UINT64_C(0x464f5243)

/* Random-phase initial vorticity: for every kept mode with |k| > 0,
 * |omega_hat| = sqrt(|k| E(|k|) / pi) with E(k) = k^4 exp(-(k/k0)^2), phase
 * 2*pi*U from Philox(counter = (j*nkx+i, 0, TAG_IC, 0), key = (seed, 0)); the
 * kx = 0 column is made Hermitian (row ny-j is the conjugate of row j); then
 * the field is rescaled so that E = 1/2 sum_full |omega_hat|^2/k^2 = energy.
 * Leaves omega_hat set and refreshes derived fields via compute_derivatives. */
void nso_ext_init_random_spectrum(nso_state *s, uint64_t seed, double k0, double energy) {
    const int nkx = s->nkx, nky = s->nky, ny = s->ny;
    const int n = nkx * nky;
    for (int idx = 0; idx < n; ++idx) s->omega_hat[idx] = 0.0;
    for (int j = 0; j < nky; ++j) {
        for (int i = 0; i < nkx; ++i) {
            const int idx = j * nkx + i;
            if (!s->dealias_mask[idx] || s->k2[idx] <= 1e-12) continue;
            int jsrc = j;
            int flip = 0;
            if (i == 0 && j > ny / 2) {
                jsrc = ny - j;
                flip = 1;
            }
            const uint64_t ctr[4] = {(uint64_t)(jsrc * nkx + i), 0, NSO_TAG_IC, 0};
            const uint64_t key[2] = {seed, 0};
            uint64_t r[4];
            nso_ext_philox4x64(ctr, key, r);
            const double km = sqrt(s->k2[idx]);
            const double ek = km * km * km * km * exp(-(km / k0) * (km / k0));
            const double amp = sqrt(km * ek / M_PI);
            const double th = 2.0 * M_PI * nso_u53(r[0]);
            double complex v = amp * (cos(th) + I * sin(th));
            if (flip) v = conj(v);
            s->omega_hat[idx] = v;
        }
    }
    double e = 0.0;
    for (int j = 0; j < nky; ++j) {
        for (int i = 0; i < nkx; ++i) {
            const int idx = j * nkx + i;
            if (s->k2[idx] <= 1e-12) continue;
            const double w = (i == 0 || 2 * i == s->nx) ? 1.0 : 2.0;
            const double m = cabs(s->omega_hat[idx]);
            e += w * 0.5 * m * m / s->k2[idx];
        }
    }
    const double scale = e > 0.0 ? sqrt(energy / e) : 0.0;
    for (int idx = 0; idx < n; ++idx) s->omega_hat[idx] *= scale;
    nso_compute_derivatives(s);
}

/* sigma^2 = 2 eps / sum_full(1/k^2) over the kept modes of the forced shell */
static double nso_ext_forcing_sigma(const nso_state *s, const nso_ext_forcing *f) {
    double acc = 0.0;
    for (int j = 0; j < s->nky; ++j) {
        for (int i = 0; i < s->nkx; ++i) {
            const int idx = j * s->nkx + i;
            const double km = sqrt(s->k2[idx]);
            if (!s->dealias_mask[idx] || s->k2[idx] <= 1e-12 || km < f->kmin || km > f->kmax) continue;
            const double w = (i == 0) ? 1.0 : 2.0;
            acc += w / s->k2[idx];
        }
    }
    return acc > 0.0 ? sqrt(2.0 * f->epsilon / acc) : 0.0;
}

/* omega_hat += sigma sqrt(dt) xi, xi = (g1 + i g2)/sqrt(2) from Box-Muller on
 * Philox(counter = (mode id, step, TAG_FORCE, 0), key = (seed, 0)) outputs 0,1;
 * mode id = (signed ky) << 32 | kx (the same noise for a physical mode on every
 * grid); kx = 0 rows with ky < 0 take the conjugate of the ky > 0 row. */
static void nso_ext_apply_forcing(nso_state *s, const nso_ext_forcing *f, double dt) {
    const double sigma = nso_ext_forcing_sigma(s, f);
    const double amp = sigma * sqrt(dt);
    const int ny = s->ny;
    for (int j = 0; j < s->nky; ++j) {
        for (int i = 0; i < s->nkx; ++i) {
            const int idx = j * s->nkx + i;
            const double km = sqrt(s->k2[idx]);
            if (!s->dealias_mask[idx] || s->k2[idx] <= 1e-12 || km < f->kmin || km > f->kmax) continue;
            int ky = (j <= ny / 2) ? j : j - ny, flip = 0;
            if (i == 0 && ky < 0) {
                ky = -ky;
                flip = 1;
            }
            const uint64_t id = ((uint64_t)(uint32_t)ky << 32) | (uint32_t)i;
            const uint64_t ctr[4] = {id, f->step, NSO_TAG_FORCE, 0};
            const uint64_t key[2] = {f->seed, 0};
            uint64_t r[4];
            nso_ext_philox4x64(ctr, key, r);
            double u1 = nso_u53(r[0]);
            const double u2 = nso_u53(r[1]);
            u1 = fmax(u1, DBL_MIN);
            const double rad = sqrt(-2.0 * log(u1)) * M_SQRT1_2;
            const double th = 2.0 * M_PI * u2;
            double complex xi = rad * cos(th) + I * (rad * sin(th));
            if (flip) xi = conj(xi);
            s->omega_hat[idx] += amp * xi;
        }
    }
}

/* ------------------------------------------- integrating-factor RK4 (extension)
 * No reference counterpart.  Lawson's integrating-factor RK4 (J. D. Lawson,
 * SIAM J. Numer. Anal. 4 (1967) 372-380): classical RK4 applied to
 * v = exp(-L t) omega_hat, L = -lam, lam = k^2/Re + w (w: hyperviscosity
 * weights when enabled), so the viscous and hyperviscous decay is integrated
 * exactly.  The explicit part is the nonlinear term of the reference stage
 * (spectral_core.c:46-112) minus the SFD relaxation of hyperviscosity.c:132-145.
 * With E1 = exp(-lam h/2) and E2 = E1^2:
 *   a = N(w_n)  u_a = E1 (w_n + h/2 a)       acc = E2 a
 *   b = N(u_a)  u_b = E1 w_n + h/2 b         acc = acc + 2 (E1 b)
 *   c = N(u_b)  u_c = E2 w_n + h (E1 c)      acc = acc + 2 (E1 c)
 *   d = N(u_c)  w_{n+1} = E2 w_n + h/6 (acc + d)
 * Forcing and the SFD post-step follow as in the explicit scheme. */
static void nso_if_rhs(nso_state *s, fftw_complex *kout) {
    const nso_hv_config *cfg = &s->hyperviscosity;
    const int n = s->nkx * s->nky;
    const int sfd = cfg->sfd_enabled && cfg->sfd_strength > 0.0;
    const int order = cfg->order > 0 ? cfg->order : 1;
#pragma omp parallel for
    for (int i = 0; i < n; ++i) {
        fftw_complex k = s->nonlinear_hat[i];
        if (sfd) {
            double ramp = 0.0;
            if (cfg->inv_bandwidth > 0.0) {
                const double km = sqrt(s->k2[i]);
                if (km > cfg->cutoff_wavenumber)
                    ramp = pow(nso_clamp((km - cfg->cutoff_wavenumber) * cfg->inv_bandwidth, 0.0, 1.0), order);
            }
            const double sw = cfg->sfd_strength * ramp;
            if (sw > 0.0) k -= sw * (s->omega_hat[i] - s->sfd_hat[i]);
        }
        kout[i] = k;
    }
}

static void nso_advance_ifrk4_impl(nso_state *s, const nso_ext_forcing *forcing) {
    const int n = s->nkx * s->nky;
    const double h = s->dt;
    const double inv_re = 1.0 / s->Re;
    const int visc = s->hyperviscosity.enabled && s->hyperviscosity.coefficient > 0.0;
    double *e1 = (double *)malloc(sizeof(double) * (size_t)n);
    fftw_complex *acc = s->rk4_hat;
#pragma omp parallel for
    for (int i = 0; i < n; ++i) {
        const double lam = s->k2[i] * inv_re + (visc ? s->hyperviscosity_weights[i] : 0.0);
        e1[i] = exp(-lam * (0.5 * h));
    }
    memcpy(s->omega_tmp_hat, s->omega_hat, (size_t)n * sizeof(fftw_complex));
    nso_compute_nonlinear_terms(s);
    nso_if_rhs(s, s->rk1_hat);
#pragma omp parallel for
    for (int i = 0; i < n; ++i) {
        const double E2 = e1[i] * e1[i];
        acc[i] = E2 * s->rk1_hat[i];
        s->omega_hat[i] = e1[i] * (s->omega_tmp_hat[i] + (0.5 * h) * s->rk1_hat[i]);
    }
    nso_compute_derivatives(s);
    nso_compute_nonlinear_terms(s);
    nso_if_rhs(s, s->rk2_hat);
#pragma omp parallel for
    for (int i = 0; i < n; ++i) {
        acc[i] = acc[i] + 2.0 * (e1[i] * s->rk2_hat[i]);
        s->omega_hat[i] = e1[i] * s->omega_tmp_hat[i] + (0.5 * h) * s->rk2_hat[i];
    }
    nso_compute_derivatives(s);
    nso_compute_nonlinear_terms(s);
    nso_if_rhs(s, s->rk3_hat);
#pragma omp parallel for
    for (int i = 0; i < n; ++i) {
        const double E2 = e1[i] * e1[i];
        acc[i] = acc[i] + 2.0 * (e1[i] * s->rk3_hat[i]);
        s->omega_hat[i] = E2 * s->omega_tmp_hat[i] + h * (e1[i] * s->rk3_hat[i]);
    }
    nso_compute_derivatives(s);
    nso_compute_nonlinear_terms(s);
    nso_if_rhs(s, s->rk2_hat);
#pragma omp parallel for
    for (int i = 0; i < n; ++i) {
        const double E2 = e1[i] * e1[i];
        s->omega_hat[i] = E2 * s->omega_tmp_hat[i] + h / 6.0 * (acc[i] + s->rk2_hat[i]);
    }
    free(e1);
    if (forcing && forcing->enabled) nso_ext_apply_forcing(s, forcing, h);
    nso_hv_post_step(s, s->omega_hat, h);
    s->t += h;
    nso_compute_derivatives(s);
}

/* n-step driver with a choice of scheme (0: the reference RK4, 1: IF-RK4) */
void nso_ext_run_scheme(nso_state *s, int scheme, int nsteps, int adaptive, int forcing_on, double fkmin,
                        double fkmax, double epsilon, uint64_t fseed, uint64_t step0) {
    nso_ext_forcing f;
    f.enabled = forcing_on;
    f.kmin = fkmin;
    f.kmax = fkmax;
    f.epsilon = epsilon;
    f.seed = fseed;
    for (int n = 0; n < nsteps; ++n) {
        if (adaptive) s->dt = nso_compute_cfl_timestep(s);
        f.step = step0 + (uint64_t)n;
        if (scheme == 1) nso_advance_ifrk4_impl(s, forcing_on ? &f : NULL);
        else nso_advance_rk4_impl(s, forcing_on ? &f : NULL);
    }
}

/* n-step driver: optional reference CFL dt per step (the loop of
 * tests/test_taylor_green.c:105-108), optional forcing with a per-step counter */
void nso_ext_run(nso_state *s, int nsteps, int adaptive, int forcing_on, double fkmin, double fkmax,
                 double epsilon, uint64_t fseed, uint64_t step0) {
    nso_ext_forcing f;
    f.enabled = forcing_on;
    f.kmin = fkmin;
    f.kmax = fkmax;
    f.epsilon = epsilon;
    f.seed = fseed;
    for (int n = 0; n < nsteps; ++n) {
        if (adaptive) s->dt = nso_compute_cfl_timestep(s);
        f.step = step0 + (uint64_t)n;
        nso_advance_rk4_impl(s, forcing_on ? &f : NULL);
    }
}

size_t nso_sizeof_state(void) { return sizeof(nso_state); }
size_t nso_sizeof_forcing_state(void) { return sizeof(nso_forcing_state); }
