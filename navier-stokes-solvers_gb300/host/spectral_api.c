/*
 * Drop-in implementation of the reference spectral solver API
 * (src/spectral/ns_spectral_solver.h:71-113) on top of the GPU C-ABI.
 *
 * Host arrays of NSSpectralData are the source of truth at every reference-API
 * call, exactly as in the reference: each call copies the arrays it reads to
 * the device, runs the work there and copies back the arrays the reference
 * function writes.  Nothing is computed on the host except scalar bookkeeping,
 * printing and file output.  Scratch arrays that the reference uses internally
 * (rk1_hat..rk4_hat, omega_tmp_hat) are not refreshed by the GPU step.
 *
 * The extension ns_spectral_gpu_advance_n keeps the state on the device across
 * steps; after it the host arrays are stale until ns_spectral_gpu_sync_host,
 * and every reference-API call performs that sync first.
 */
#include "ns_spectral_solver.h"

#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "ns_gpu.h"
#include "ns_spectral_internal.h"

static void ns_report(NSSpectralData *d, const char *what, int status) {
    fprintf(stderr, "[ns-gb300] %s failed: %s (%s)\n", what, ns_gpu_status_string(status),
            (d && d->gpu && d->gpu->dev) ? ns_gpu_last_error(d->gpu->dev) : "");
}

#define NS_CALL(d, what, expr)                 \
    do {                                       \
        int _st = (expr);                      \
        if (_st != NS_GPU_OK) {                \
            ns_report((d), (what), _st);       \
            return;                            \
        }                                      \
    } while (0)

#define NS_CALL_RET(d, what, expr, ret)        \
    do {                                       \
        int _st = (expr);                      \
        if (_st != NS_GPU_OK) {                \
            ns_report((d), (what), _st);       \
            return (ret);                      \
        }                                      \
    } while (0)

static int ns_status_to_solver(int st) {
    switch (st) {
        case NS_GPU_OK: return SOLVER_SUCCESS;
        case NS_GPU_ERR_INVALID: return SOLVER_INVALID_PARAM;
        case NS_GPU_ERR_ALLOC: return SOLVER_MEM_ERROR;
        case NS_GPU_ERR_DIVERGED: return SOLVER_DIVERGED;
        default: return SOLVER_INVALID_PARAM + 1;
    }
}

static size_t ns_nc(const NSSpectralData *d) { return (size_t)d->nkx * (size_t)d->nky; }
static size_t ns_nr(const NSSpectralData *d) { return (size_t)d->nx * (size_t)d->ny; }

/* device parameters from the struct fields the reference reads */
static int ns_sync_params(NSSpectralData *d, int adaptive) {
    ns_gpu_params p;
    memset(&p, 0, sizeof(p));
    p.Re = d->Re;
    p.cfl_factor = d->cfl_factor;
    p.adaptive_dt = adaptive;
    p.dt = d->dt;
    p.hv_enabled = d->hyperviscosity.enabled;
    p.hv_coefficient = d->hyperviscosity.coefficient;
    p.hv_order = d->hyperviscosity.order;
    p.hv_cutoff_ratio = d->hyperviscosity.cutoff_ratio;
    p.sfd_enabled = d->hyperviscosity.sfd_enabled;
    p.sfd_strength = d->hyperviscosity.sfd_strength;
    p.sfd_timescale = d->hyperviscosity.sfd_timescale;
    p.forcing_enabled = d->gpu->forcing_enabled;
    p.forcing_kmin = d->gpu->forcing_kmin;
    p.forcing_kmax = d->gpu->forcing_kmax;
    p.forcing_epsilon = d->gpu->forcing_epsilon;
    p.forcing_seed = d->gpu->forcing_seed;
    p.scheme = d->gpu->scheme;
    return ns_gpu_set_params(d->gpu->dev, &p);
}

static int ns_sfd_on(const NSSpectralData *d) {
    return d->hyperviscosity.sfd_enabled && d->hyperviscosity.sfd_strength > 0.0;
}

/* bring the host arrays up to date after device-resident steps */
static int ns_host_sync(NSSpectralData *d) {
    if (!d->gpu->host_stale) return NS_GPU_OK;
    double t = d->t, dt = d->dt;
    int st = ns_gpu_download_state(d->gpu->dev, (double *)d->omega_hat, (double *)d->psi_hat, (double *)d->u_hat,
                                   (double *)d->v_hat, ns_sfd_on(d) ? (double *)d->sfd_hat : NULL, d->u, d->v,
                                   d->omega, &t, &dt);
    if (st != NS_GPU_OK) return st;
    d->t = t;
    d->dt = dt;
    d->gpu->host_stale = 0;
    return NS_GPU_OK;
}

/* every reference-API entry point starts here: host arrays become the truth */
static int ns_enter(NSSpectralData *d) {
    if (!d || !d->gpu) return NS_GPU_ERR_INVALID;
    int st = ns_host_sync(d);
    d->gpu->device_current = 0;
    return st;
}

/* ------------------------------------------------------------------ memory */

static void ns_free_arrays(NSSpectralData *d) {
    double *reals[] = {d->u, d->v, d->p, d->omega, d->psi, d->x, d->y, d->kx, d->ky, d->k2, d->hyperviscosity_weights};
    for (size_t i = 0; i < sizeof(reals) / sizeof(reals[0]); ++i) ns_gpu_host_free(reals[i]);
    fftw_complex *cplx[] = {d->u_hat, d->v_hat, d->omega_hat, d->psi_hat, d->nonlinear_hat, d->rk1_hat,
                            d->rk2_hat, d->rk3_hat, d->rk4_hat, d->omega_tmp_hat, d->sfd_hat};
    for (size_t i = 0; i < sizeof(cplx) / sizeof(cplx[0]); ++i) ns_gpu_host_free(cplx[i]);
    ns_gpu_host_free(d->dealias_mask);
}

NSSpectralData *ns_spectral_allocate_ex(int nx, int ny, double Lx, double Ly, double Re, int precision) {
    NSSpectralData *d = (NSSpectralData *)calloc(1, sizeof(NSSpectralData));
    if (!d) return NULL;
    /* spectral_memory.c:10-22 */
    d->nx = nx;
    d->ny = ny;
    d->nkx = nx / 2 + 1;
    d->nky = ny;
    d->Lx = Lx;
    d->Ly = Ly;
    d->Re = Re;
    d->dt = 0.01;
    d->t = 0.0;
    d->cfl_factor = 0.3;
    d->forward_plan = NULL;
    d->backward_plan = NULL;
    d->gpu = (struct ns_spectral_gpu *)calloc(1, sizeof(struct ns_spectral_gpu));
    if (!d->gpu) {
        free(d);
        return NULL;
    }
    d->gpu->precision = precision;
    int st = ns_gpu_create(nx, ny, Lx, Ly, precision == NS_PRECISION_FP32 ? NS_GPU_FP32 : NS_GPU_FP64, &d->gpu->dev);
    if (st != NS_GPU_OK) {
        fprintf(stderr, "[ns-gb300] ns_spectral_allocate(%d, %d): %s\n", nx, ny, ns_gpu_status_string(st));
        free(d->gpu);
        free(d);
        return NULL;
    }
    const size_t nr = ns_nr(d), nc = ns_nc(d);
    d->u = (double *)ns_gpu_host_alloc(nr * sizeof(double));
    d->v = (double *)ns_gpu_host_alloc(nr * sizeof(double));
    d->p = (double *)ns_gpu_host_alloc(nr * sizeof(double));
    d->omega = (double *)ns_gpu_host_alloc(nr * sizeof(double));
    d->psi = (double *)ns_gpu_host_alloc(nr * sizeof(double));
    d->x = (double *)ns_gpu_host_alloc((size_t)nx * sizeof(double));
    d->y = (double *)ns_gpu_host_alloc((size_t)ny * sizeof(double));
    fftw_complex *NS_RESTRICT *cplx[] = {&d->u_hat, &d->v_hat, &d->omega_hat, &d->psi_hat, &d->nonlinear_hat, &d->rk1_hat,
                             &d->rk2_hat, &d->rk3_hat, &d->rk4_hat, &d->omega_tmp_hat, &d->sfd_hat};
    for (size_t i = 0; i < sizeof(cplx) / sizeof(cplx[0]); ++i)
        *cplx[i] = (fftw_complex *)ns_gpu_host_alloc(nc * sizeof(fftw_complex));
    d->kx = (double *)ns_gpu_host_alloc((size_t)d->nkx * sizeof(double));
    d->ky = (double *)ns_gpu_host_alloc((size_t)d->nky * sizeof(double));
    d->k2 = (double *)ns_gpu_host_alloc(nc * sizeof(double));
    d->dealias_mask = (int *)ns_gpu_host_alloc(nc * sizeof(int));
    d->hyperviscosity_weights = (double *)ns_gpu_host_alloc(nc * sizeof(double));
    int ok = d->u && d->v && d->p && d->omega && d->psi && d->x && d->y && d->kx && d->ky && d->k2 &&
             d->dealias_mask && d->hyperviscosity_weights;
    for (size_t i = 0; i < sizeof(cplx) / sizeof(cplx[0]); ++i) ok = ok && *cplx[i];
    if (!ok) {
        fprintf(stderr, "[ns-gb300] ns_spectral_allocate(%d, %d): host allocation failed\n", nx, ny);
        ns_spectral_free(d);
        return NULL;
    }
    ns_spectral_hyperviscosity_default(&d->hyperviscosity);
    return d;
}

NSSpectralData *ns_spectral_allocate(int nx, int ny, double Lx, double Ly, double Re) {
    return ns_spectral_allocate_ex(nx, ny, Lx, Ly, Re, NS_PRECISION_FP64);
}

void ns_spectral_free(NSSpectralData *d) {
    if (!d) return;
    ns_free_arrays(d);
    if (d->gpu) {
        ns_gpu_destroy(d->gpu->dev);
        free(d->gpu);
    }
    free(d);
}

/* ---------------------------------------------------------- initialization */

void ns_spectral_initialize_grids(NSSpectralData *d) {
    NS_CALL(d, "initialize_grids", ns_enter(d));
    NS_CALL(d, "initialize_grids", ns_gpu_geometry(d->gpu->dev, d->x, d->y, d->kx, d->ky, d->k2, d->dealias_mask));
    ns_spectral_hyperviscosity_update_weights(d);
}

void ns_spectral_initialize_fft_plans(NSSpectralData *d) {
    /* the device transforms are planned when the instance is created; the plan
     * fields only need to be non-NULL for callers that test them */
    if (!d || !d->gpu) return;
    d->forward_plan = (fftw_plan)(void *)d->gpu;
    d->backward_plan = (fftw_plan)(void *)d->gpu;
}

void ns_spectral_initialize_taylor_green(NSSpectralData *d) {
    NS_CALL(d, "initialize_taylor_green", ns_enter(d));
    NS_CALL(d, "initialize_taylor_green", ns_gpu_taylor_green(d->gpu->dev, d->u, d->v, d->omega, d->p));
    ns_spectral_physical_to_spectral(d, d->omega, d->omega_hat);
    ns_spectral_physical_to_spectral(d, d->u, d->u_hat);
    ns_spectral_physical_to_spectral(d, d->v, d->v_hat);
}

/* -------------------------------------------------------------- transforms */

void ns_spectral_physical_to_spectral(NSSpectralData *d, double *field, fftw_complex *field_hat) {
    NS_CALL(d, "physical_to_spectral", ns_enter(d));
    NS_CALL(d, "physical_to_spectral", ns_gpu_forward(d->gpu->dev, field, (double *)field_hat));
}

void ns_spectral_spectral_to_physical(NSSpectralData *d, fftw_complex *field_hat, double *field) {
    NS_CALL(d, "spectral_to_physical", ns_enter(d));
    NS_CALL(d, "spectral_to_physical",
            ns_gpu_inverse(d->gpu->dev, (const double *)field_hat, field, (double *)d->nonlinear_hat));
}

void ns_spectral_apply_dealiasing(NSSpectralData *d, fftw_complex *field_hat) {
    NS_CALL(d, "apply_dealiasing", ns_enter(d));
    NS_CALL(d, "apply_dealiasing", ns_gpu_dealias(d->gpu->dev, (double *)field_hat));
}

/* -------------------------------------------------------------------- core */

void ns_spectral_compute_velocity_from_vorticity(NSSpectralData *d) {
    NS_CALL(d, "compute_velocity_from_vorticity", ns_enter(d));
    NS_CALL(d, "compute_velocity_from_vorticity",
            ns_gpu_velocity(d->gpu->dev, (const double *)d->omega_hat, (double *)d->psi_hat, (double *)d->u_hat,
                            (double *)d->v_hat));
}

void ns_spectral_compute_derivatives(NSSpectralData *d) {
    NS_CALL(d, "compute_derivatives", ns_enter(d));
    NS_CALL(d, "compute_derivatives",
            ns_gpu_derivatives(d->gpu->dev, (const double *)d->omega_hat, (double *)d->psi_hat, (double *)d->u_hat,
                               (double *)d->v_hat, d->u, d->v, d->omega, (double *)d->nonlinear_hat));
}

/* physical outputs follow the reference aliasing (spectral_core.c:54-58):
 * u = psi_x, v = psi_y, psi = omega_x, omega = omega_y, p = Jacobian */
void ns_spectral_compute_nonlinear_terms(NSSpectralData *d) {
    NS_CALL(d, "compute_nonlinear_terms", ns_enter(d));
    NS_CALL(d, "compute_nonlinear_terms",
            ns_gpu_nonlinear(d->gpu->dev, (const double *)d->omega_hat, (const double *)d->psi_hat,
                             (double *)d->nonlinear_hat, d->u, d->v, d->psi, d->omega, d->p));
}

/* --------------------------------------------------------- time stepping */

void ns_spectral_advance_rk4(NSSpectralData *d) {
    NS_CALL(d, "advance_rk4", ns_enter(d));
    NS_CALL(d, "advance_rk4", ns_sync_params(d, 0));
    const int sfd = ns_sfd_on(d);
    double t = d->t, dt = d->dt;
    /* upload, one device step and download in one call with overlapped copies */
    NS_CALL(d, "advance_rk4",
            ns_gpu_step_host(d->gpu->dev, (double *)d->omega_hat, (double *)d->psi_hat, (double *)d->u_hat,
                             (double *)d->v_hat, sfd ? (double *)d->sfd_hat : NULL, d->u, d->v, d->omega, d->t, d->dt,
                             d->gpu->step, &t, &dt));
    d->t = t;
    d->gpu->step += 1;
}

double ns_spectral_compute_cfl_timestep(NSSpectralData *d) {
    double dt = d ? d->dt : 0.0;
    NS_CALL_RET(d, "compute_cfl_timestep", ns_enter(d), dt);
    NS_CALL_RET(d, "compute_cfl_timestep", ns_sync_params(d, 0), dt);
    NS_CALL_RET(d, "compute_cfl_timestep", ns_gpu_reduce(d->gpu->dev, NS_GPU_REDUCE_CFL, d->u, d->v, &dt), dt);
    return dt;
}

int ns_spectral_gpu_advance_n(NSSpectralData *d, int nsteps, int adaptive_dt) {
    if (!d || !d->gpu || nsteps < 0) return SOLVER_INVALID_PARAM;
    int st = ns_sync_params(d, adaptive_dt ? 1 : 0);
    if (st != NS_GPU_OK) return ns_status_to_solver(st);
    ns_gpu *g = d->gpu->dev;
    if (!d->gpu->device_current) {
        st = ns_host_sync(d);
        if (st == NS_GPU_OK)
            st = ns_gpu_upload_state(g, (const double *)d->omega_hat, (const double *)d->psi_hat,
                                     ns_sfd_on(d) ? (const double *)d->sfd_hat : NULL, d->t, d->dt, d->gpu->step);
        if (st != NS_GPU_OK) {
            ns_report(d, "gpu_advance_n", st);
            return ns_status_to_solver(st);
        }
        d->gpu->device_current = 1;
    }
    st = ns_gpu_advance(g, nsteps);
    if (st != NS_GPU_OK) {
        ns_report(d, "gpu_advance_n", st);
        return ns_status_to_solver(st);
    }
    d->gpu->step += (unsigned long long)nsteps;
    if (nsteps > 0) d->gpu->host_stale = 1;
    return SOLVER_SUCCESS;
}

int ns_spectral_gpu_sync_host(NSSpectralData *d) {
    if (!d || !d->gpu) return SOLVER_INVALID_PARAM;
    int st = ns_host_sync(d);
    if (st != NS_GPU_OK) ns_report(d, "gpu_sync_host", st);
    /* the caller may now modify the host arrays: the next advance re-uploads */
    d->gpu->device_current = 0;
    return ns_status_to_solver(st);
}

int ns_spectral_gpu_set_forcing(NSSpectralData *d, int enabled, double kmin, double kmax, double epsilon,
                                unsigned long long seed) {
    if (!d || !d->gpu) return SOLVER_INVALID_PARAM;
    if (enabled && (kmin < 0.0 || kmax < kmin || epsilon < 0.0)) return SOLVER_INVALID_PARAM;
    d->gpu->forcing_enabled = enabled;
    d->gpu->forcing_kmin = kmin;
    d->gpu->forcing_kmax = kmax;
    d->gpu->forcing_epsilon = epsilon;
    d->gpu->forcing_seed = seed;
    return ns_status_to_solver(ns_sync_params(d, 0));
}

int ns_spectral_gpu_set_scheme(NSSpectralData *d, int scheme) {
    if (!d || !d->gpu) return SOLVER_INVALID_PARAM;
    if (scheme != NS_SPECTRAL_SCHEME_RK4 && scheme != NS_SPECTRAL_SCHEME_IFRK4) return SOLVER_INVALID_PARAM;
    d->gpu->scheme = scheme;
    return ns_status_to_solver(ns_sync_params(d, 0));
}

int ns_spectral_gpu_diagnostics(NSSpectralData *d, double *energy, double *enstrophy) {
    if (!d || !d->gpu) return SOLVER_INVALID_PARAM;
    /* the host arrays are the state unless device-resident steps are newer */
    if (!d->gpu->host_stale) {
        int st = ns_sync_params(d, 0);
        if (st == NS_GPU_OK)
            st = ns_gpu_upload_state(d->gpu->dev, (const double *)d->omega_hat, (const double *)d->psi_hat,
                                     ns_sfd_on(d) ? (const double *)d->sfd_hat : NULL, d->t, d->dt, d->gpu->step);
        if (st != NS_GPU_OK) return ns_status_to_solver(st);
        d->gpu->device_current = 1;
    }
    double t = 0.0, dt = 0.0;
    return ns_status_to_solver(ns_gpu_diagnostics(d->gpu->dev, energy, enstrophy, &t, &dt));
}

int ns_spectral_initialize_random_spectrum(NSSpectralData *d, unsigned long long seed, double k0, double energy) {
    if (!d || !d->gpu) return SOLVER_INVALID_PARAM;
    int st = ns_enter(d);
    if (st == NS_GPU_OK)
        st = ns_gpu_random_spectrum_host(d->gpu->dev, (uint64_t)seed, k0, energy, (double *)d->omega_hat);
    if (st != NS_GPU_OK) {
        ns_report(d, "initialize_random_spectrum", st);
        return ns_status_to_solver(st);
    }
    ns_spectral_compute_derivatives(d);
    return SOLVER_SUCCESS;
}

const char *ns_spectral_gpu_last_error(const NSSpectralData *d) {
    return (d && d->gpu) ? ns_gpu_last_error(d->gpu->dev) : "no instance";
}

struct ns_gpu *ns_spectral_gpu_handle(NSSpectralData *d) { return (d && d->gpu) ? d->gpu->dev : NULL; }

/* ---------------------------------------------------------------- analysis */

double ns_spectral_compute_energy(NSSpectralData *d) {
    double e = 0.0;
    NS_CALL_RET(d, "compute_energy", ns_enter(d), 0.0);
    NS_CALL_RET(d, "compute_energy", ns_gpu_reduce(d->gpu->dev, NS_GPU_REDUCE_ENERGY, d->u, d->v, &e), 0.0);
    return e;
}

double ns_spectral_compute_enstrophy(NSSpectralData *d) {
    double z = 0.0;
    NS_CALL_RET(d, "compute_enstrophy", ns_enter(d), 0.0);
    NS_CALL_RET(d, "compute_enstrophy", ns_gpu_reduce(d->gpu->dev, NS_GPU_REDUCE_ENSTROPHY, d->omega, NULL, &z), 0.0);
    return z;
}

int ns_spectral_check_resolution(NSSpectralData *d) {
    double frac = 0.0;
    NS_CALL_RET(d, "check_resolution", ns_enter(d), 0);
    NS_CALL_RET(d, "check_resolution",
                ns_gpu_spectral_stats(d->gpu->dev, (const double *)d->omega_hat, NULL, NULL, &frac, NULL, NULL, NULL,
                                      NULL),
                0);
    /* spectral_analysis.c:59-65 */
    if (frac > 1e-6) {
        printf("Warning: %.2e%% of energy in high wavenumbers\n", frac * 100);
        return 0;
    }
    return 1;
}

void ns_spectral_analyze_convergence(NSSpectralData *d, int step) {
    if (step % 10 != 0) return;
    const double energy = ns_spectral_compute_energy(d);
    const double enstrophy = ns_spectral_compute_enstrophy(d);
    double mx = 0.0, err = 0.0;
    NS_CALL(d, "analyze_convergence",
            ns_gpu_spectral_stats(d->gpu->dev, (const double *)d->omega_hat, NULL, NULL, NULL, &mx, &err, NULL, NULL));
    /* spectral_analysis.c:98-99 */
    printf("Step %d: t=%.4f, E=%.6e, \xce\xa9=%.6e, max|\xcf\x89\xcc\x82|=%.2e, err=%.2e, dt=%.2e\n", step, d->t, energy,
           enstrophy, mx, err, d->dt);
}

void ns_spectral_analyze_spectrum(NSSpectralData *d) {
    NS_CALL(d, "analyze_spectrum", ns_enter(d));
    const int max_k = (int)fmin(d->nkx, d->nky / 2);
    double *ek = (double *)calloc((size_t)max_k > 0 ? (size_t)max_k : 1, sizeof(double));
    int *ck = (int *)calloc((size_t)max_k > 0 ? (size_t)max_k : 1, sizeof(int));
    if (!ek || !ck) {
        free(ek);
        free(ck);
        return;
    }
    int st = ns_gpu_spectral_stats(d->gpu->dev, NULL, (const double *)d->u_hat, (const double *)d->v_hat, NULL, NULL,
                                   NULL, ek, ck);
    if (st != NS_GPU_OK) {
        ns_report(d, "analyze_spectrum", st);
        free(ek);
        free(ck);
        return;
    }
    /* spectral_analysis.c:125-139 */
    printf("\nEnergy Spectrum (t=%.4f):\n", d->t);
    printf("k\tE(k)\t\tSlope\n");
    for (int k = 1; k < max_k && ck[k] > 0; k++) {
        ek[k] /= ck[k];
        double slope = 0.0;
        if (k > 1 && ek[k - 1] > 1e-16 && ek[k] > 1e-16) slope = log(ek[k] / ek[k - 1]) / log((double)k / (k - 1));
        if (k <= 10 || k % 5 == 0) printf("%d\t%.2e\t%.2f\n", k, ek[k], slope);
    }
    free(ek);
    free(ck);
}

/* ---------------------------------------------------------- hyperviscosity */

void ns_spectral_hyperviscosity_default(NSSpectralHyperviscosityConfig *c) {
    if (!c) return;
    /* hyperviscosity.c:20-29 */
    c->enabled = 0;
    c->coefficient = 0.0;
    c->order = 8;
    c->cutoff_ratio = 0.65;
    c->sfd_strength = 0.0;
    c->sfd_timescale = 1.0;
    c->sfd_enabled = 0;
    c->kmax = 0.0;
    c->cutoff_wavenumber = 0.0;
    c->inv_bandwidth = 0.0;
}

void ns_spectral_hyperviscosity_update_weights(NSSpectralData *d) {
    if (!d || !d->hyperviscosity_weights || !d->k2) return;
    NS_CALL(d, "hyperviscosity_update_weights", ns_enter(d));
    NS_CALL(d, "hyperviscosity_update_weights", ns_sync_params(d, 0));
    double kmax = 0.0, cutoff = 0.0, inv_bw = 0.0;
    NS_CALL(d, "hyperviscosity_update_weights",
            ns_gpu_hv_weights(d->gpu->dev, &kmax, &cutoff, &inv_bw, d->hyperviscosity_weights));
    d->hyperviscosity.kmax = kmax;
    d->hyperviscosity.cutoff_wavenumber = cutoff;
    d->hyperviscosity.inv_bandwidth = inv_bw;
}

void ns_spectral_hyperviscosity_set(NSSpectralData *d, const NSSpectralHyperviscosityConfig *c) {
    if (!d || !c) return;
    if (ns_enter(d) != NS_GPU_OK) return;
    /* hyperviscosity.c:38-57 */
    const size_t nc = ns_nc(d);
    d->hyperviscosity = *c;
    if (!d->hyperviscosity.enabled) memset(d->hyperviscosity_weights, 0, nc * sizeof(double));
    if (!d->hyperviscosity.sfd_enabled || d->hyperviscosity.sfd_strength <= 0.0) {
        d->hyperviscosity.sfd_enabled = 0;
        d->hyperviscosity.sfd_strength = 0.0;
        memset(d->sfd_hat, 0, nc * sizeof(fftw_complex));
    }
    ns_spectral_hyperviscosity_update_weights(d);
    if (d->hyperviscosity.sfd_enabled && d->sfd_hat && d->omega_hat)
        memcpy(d->sfd_hat, d->omega_hat, nc * sizeof(fftw_complex));
}

void ns_spectral_hyperviscosity_apply(NSSpectralData *d, fftw_complex *rhs_hat, const fftw_complex *state_hat) {
    if (!d || !rhs_hat || !state_hat) return;
    NS_CALL(d, "hyperviscosity_apply", ns_enter(d));
    NS_CALL(d, "hyperviscosity_apply", ns_sync_params(d, 0));
    NS_CALL(d, "hyperviscosity_apply",
            ns_gpu_hv_apply(d->gpu->dev, (double *)rhs_hat, (const double *)state_hat, (const double *)d->sfd_hat));
}

void ns_spectral_hyperviscosity_post_step(NSSpectralData *d, const fftw_complex *state_hat, double dt) {
    if (!d || !state_hat || dt <= 0.0) return;
    NS_CALL(d, "hyperviscosity_post_step", ns_enter(d));
    NS_CALL(d, "hyperviscosity_post_step", ns_sync_params(d, 0));
    NS_CALL(d, "hyperviscosity_post_step",
            ns_gpu_hv_post_step(d->gpu->dev, (const double *)state_hat, (double *)d->sfd_hat, dt));
}

/* ------------------------------------------------------------------ output */

void ns_spectral_output_solution(NSSpectralData *d, const char *filename) {
    FILE *fp = fopen(filename, "w");
    if (!fp) return;
    /* spectral_output.c:10-25: psi refreshed from psi_hat, then one line per point */
    ns_spectral_spectral_to_physical(d, d->psi_hat, d->psi);
    fprintf(fp, "# Spectral Navier-Stokes Solution\n");
    fprintf(fp, "# x y u v omega psi\n");
    for (int j = 0; j < d->ny; j++) {
        for (int i = 0; i < d->nx; i++) {
            const int idx = j * d->nx + i;
            fprintf(fp, "%.8f %.8f %.8e %.8e %.8e %.8e\n", d->x[i], d->y[j], d->u[idx], d->v[idx], d->omega[idx],
                    d->psi[idx]);
        }
        fprintf(fp, "\n");
    }
    fclose(fp);
}
