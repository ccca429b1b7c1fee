/*
 * ns_run -- config-driven runner of the GB300 spectral solver.
 *
 *     ns_run parameters.ini [override.json ...]
 *
 * The reference's drivers hard-code their parameters (src/spectral/main_spectral.c:15-19)
 * although its README advertises a configuration file; this driver reads the
 * reference's ns_config keys (config/parameters.ini: grid.nx, grid.ny, domain.Lx,
 * domain.Ly, fluid.Re, time.dt, time.t_end, forcing.type,
 * spectral.hyperviscosity.coefficient / .order) with later files overriding
 * earlier ones (config_parser.c:543-554), plus keys of its own:
 *
 *   spectral.precision        fp64 (default) | fp32
 *   spectral.hyperviscosity.enabled / .cutoff_ratio / .sfd_strength / .sfd_timescale
 *   ic.type                   taylor_green (default, initialize_taylor_green) | random
 *   ic.seed, ic.k0, ic.energy random-phase spectrum E(k) ~ k^4 exp(-(k/k0)^2)
 *   time.cfl                  > 0: adaptive dt with this CFL factor (else fixed time.dt)
 *   time.steps                step limit (in addition to time.t_end)
 *   forcing.kmin, .kmax, .epsilon, .seed   white-in-time shell forcing (forcing.type = white)
 *   output.dir                directory for files (default .)
 *   output.every              diagnostics line every N steps (default 100)
 *   output.spectrum_every     energy spectrum file every N steps (0: off)
 *   output.checkpoint_every   checkpoint (.npz) every N steps (0: off)
 *   output.solution           1: write solution.dat at the end (default 1)
 *   output.vtk_every          legacy VTK snapshot (u, v, omega) every N steps (0: off),
 *                             in the layout of the reference's ns_vtk_write_spectral_legacy
 *                             (src/output/vtk_writer.c:10-62, 212-227)
 *
 * The state stays on the device between outputs (ns_spectral_gpu_advance_n); t and
 * dt are read from the device state, and the host arrays are brought up to date
 * only where a file needs them (checkpoints, the final solution).  VTK snapshots
 * are written asynchronously: u, v, omega of the device state are copied into one
 * of two host buffer sets and a writer thread formats the file while the solver
 * carries on (the next snapshot into the same set waits for that writer).
 * Diagnostics lines: "step <n> t <t> dt <dt> energy <E> enstrophy <Z>".
 * Exit status: 0 success, 2 configuration error, 3 solver failure.
 */
#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "checkpoint.h"
#include "ns_config.h"
#include "ns_gpu.h"
#include "ns_spectral_solver.h"

static const char *k_prec[] = {"fp64", "fp32"};
static const char *k_ic[] = {"taylor_green", "random"};
static const char *k_forcing[] = {"none", "white", "colored"};

/* one asynchronous VTK snapshot: host copies of the fields and the writer thread */
typedef struct {
    double *u, *v, *w;
    const double *x, *y;
    int nx, ny;
    double t;
    char path[1024];
    pthread_t thread;
    int busy;
    int status;
} vtk_job;

/* legacy structured-grid VTK in the reference's layout: points (x, y, 0),
 * FIELD TIME, VECTORS velocity (u, v, 0), SCALARS vorticity */
static void *vtk_write(void *arg) {
    vtk_job *j = (vtk_job *)arg;
    j->status = -1;
    FILE *fp = fopen(j->path, "w");
    if (!fp) return NULL;
    const int points = j->nx * j->ny;
    fprintf(fp, "# vtk DataFile Version 3.0\n");
    fprintf(fp, "Navier-Stokes Solution t=%.6f\n", j->t);
    fprintf(fp, "ASCII\n");
    fprintf(fp, "DATASET STRUCTURED_GRID\n");
    fprintf(fp, "DIMENSIONS %d %d 1\n", j->nx, j->ny);
    fprintf(fp, "POINTS %d double\n", points);
    for (int y = 0; y < j->ny; ++y)
        for (int x = 0; x < j->nx; ++x) fprintf(fp, "%.9f %.9f 0.0\n", j->x[x], j->y[y]);
    fprintf(fp, "FIELD FieldData 1\n");
    fprintf(fp, "TIME 1 1 double\n%.9f\n", j->t);
    fprintf(fp, "POINT_DATA %d\n", points);
    fprintf(fp, "VECTORS velocity double\n");
    for (int i = 0; i < points; ++i) fprintf(fp, "%.9f %.9f 0.0\n", j->u[i], j->v[i]);
    fprintf(fp, "SCALARS vorticity double 1\n");
    fprintf(fp, "LOOKUP_TABLE default\n");
    for (int i = 0; i < points; ++i) fprintf(fp, "%.9f\n", j->w[i]);
    j->status = (fclose(fp) == 0) ? 0 : -1;
    return NULL;
}

static int vtk_finish(vtk_job *j) {
    if (!j->busy) return 0;
    pthread_join(j->thread, NULL);
    j->busy = 0;
    return j->status;
}

/* copy u, v, omega of the device state into the job's buffers and start its writer */
static int vtk_start(vtk_job *j, NSSpectralData *d, const char *dir, long step) {
    if (vtk_finish(j) != 0) return -1;
    double t = 0.0, dt = 0.0;
    if (ns_gpu_download_state(ns_spectral_gpu_handle(d), NULL, NULL, NULL, NULL, NULL, j->u, j->v, j->w, &t, &dt) != 0)
        return -1;
    j->t = t;
    snprintf(j->path, sizeof(j->path), "%s/solution_%06ld.vtk", dir, step);
    if (pthread_create(&j->thread, NULL, vtk_write, j) != 0) return -1;
    j->busy = 1;
    return 0;
}

static int write_spectrum(NSSpectralData *d, const char *dir, long step) {
    const int nbins = d->nkx < d->nky / 2 ? d->nkx : d->nky / 2;
    double *sum = (double *)calloc((size_t)nbins, sizeof(double));
    double *mean = (double *)calloc((size_t)nbins, sizeof(double));
    int *count = (int *)calloc((size_t)nbins, sizeof(int));
    int st = (sum && mean && count) ? ns_gpu_energy_spectrum(ns_spectral_gpu_handle(d), nbins, sum, mean, count) : -1;
    if (st == 0) {
        char path[1024];
        snprintf(path, sizeof(path), "%s/spectrum_%06ld.dat", dir, step);
        FILE *f = fopen(path, "w");
        if (f) {
            fprintf(f, "# k  E_sum  E_mean  modes   (step %ld, t = %.9g)\n", step, d->t);
            for (int k = 0; k < nbins; ++k) fprintf(f, "%d %.10e %.10e %d\n", k, sum[k], mean[k], count[k]);
            fclose(f);
        } else {
            st = -1;
        }
    }
    free(sum);
    free(mean);
    free(count);
    return st;
}

int main(int argc, char **argv) {
    if (argc < 2) {
        fprintf(stderr, "usage: %s parameters.ini [override.json ...]\n", argv[0]);
        return 2;
    }
    NSConfig cfg;
    ns_config_init(&cfg);
    char err[512];
    if (ns_config_load_files(&cfg, (const char **)(argv + 1), (size_t)(argc - 1), err, sizeof(err)) != 0) {
        fprintf(stderr, "ns_run: %s\n", err);
        ns_config_free(&cfg);
        return 2;
    }
    const NSConfigSchemaEntry schema[] = {
        {"grid.nx", NS_CONFIG_VALUE_INT, 1, 8, 4096, 1, 1, NULL, 0},
        {"grid.ny", NS_CONFIG_VALUE_INT, 1, 8, 4096, 1, 1, NULL, 0},
        {"fluid.Re", NS_CONFIG_VALUE_DOUBLE, 1, 1e-12, 0, 1, 0, NULL, 0},
        {"time.dt", NS_CONFIG_VALUE_DOUBLE, 0, 1e-12, 1.0, 1, 1, NULL, 0},
        {"spectral.precision", NS_CONFIG_VALUE_STRING, 0, 0, 0, 0, 0, k_prec, 2},
        {"ic.type", NS_CONFIG_VALUE_STRING, 0, 0, 0, 0, 0, k_ic, 2},
        {"forcing.type", NS_CONFIG_VALUE_STRING, 0, 0, 0, 0, 0, k_forcing, 3},
    };
    if (ns_config_validate(&cfg, schema, sizeof(schema) / sizeof(schema[0]), err, sizeof(err)) != 0) {
        fprintf(stderr, "ns_run: %s\n", err);
        ns_config_free(&cfg);
        return 2;
    }
    const int nx = ns_config_get_int(&cfg, "grid.nx", 128), ny = ns_config_get_int(&cfg, "grid.ny", 128);
    const double Lx = ns_config_get_double(&cfg, "domain.Lx", 2.0 * M_PI);
    const double Ly = ns_config_get_double(&cfg, "domain.Ly", 2.0 * M_PI);
    const double Re = ns_config_get_double(&cfg, "fluid.Re", 100.0);
    const int fp32 = strcmp(ns_config_get_string(&cfg, "spectral.precision", "fp64"), "fp32") == 0;
    const double t_end = ns_config_get_double(&cfg, "time.t_end", 1.0);
    const long max_steps = ns_config_get_int(&cfg, "time.steps", 0);
    const double cfl = ns_config_get_double(&cfg, "time.cfl", 0.0);
    const char *dir = ns_config_get_string(&cfg, "output.dir", ".");
    const int every = ns_config_get_int(&cfg, "output.every", 100) > 0 ? ns_config_get_int(&cfg, "output.every", 100) : 100;
    const int spec_every = ns_config_get_int(&cfg, "output.spectrum_every", 0);
    const int ck_every = ns_config_get_int(&cfg, "output.checkpoint_every", 0);
    const int vtk_every = ns_config_get_int(&cfg, "output.vtk_every", 0);

    NSSpectralData *d = ns_spectral_allocate_ex(nx, ny, Lx, Ly, Re, fp32 ? NS_PRECISION_FP32 : NS_PRECISION_FP64);
    if (!d) {
        ns_config_free(&cfg);
        return 3;
    }
    ns_spectral_initialize_grids(d);
    ns_spectral_initialize_fft_plans(d);
    d->dt = ns_config_get_double(&cfg, "time.dt", d->dt);
    if (cfl > 0.0) d->cfl_factor = cfl;

    NSSpectralHyperviscosityConfig hv;
    ns_spectral_hyperviscosity_default(&hv);
    const int hv_on = ns_config_has_key(&cfg, "spectral.hyperviscosity.coefficient");
    hv.enabled = ns_config_get_bool(&cfg, "spectral.hyperviscosity.enabled", hv_on);
    hv.coefficient = ns_config_get_double(&cfg, "spectral.hyperviscosity.coefficient", hv.coefficient);
    hv.order = ns_config_get_int(&cfg, "spectral.hyperviscosity.order", hv.order);
    hv.cutoff_ratio = ns_config_get_double(&cfg, "spectral.hyperviscosity.cutoff_ratio", hv.cutoff_ratio);
    hv.sfd_strength = ns_config_get_double(&cfg, "spectral.hyperviscosity.sfd_strength", 0.0);
    hv.sfd_timescale = ns_config_get_double(&cfg, "spectral.hyperviscosity.sfd_timescale", hv.sfd_timescale);
    hv.sfd_enabled = hv.sfd_strength > 0.0;

    if (strcmp(ns_config_get_string(&cfg, "ic.type", "taylor_green"), "random") == 0) {
        if (ns_spectral_initialize_random_spectrum(d, (unsigned long long)ns_config_get_int(&cfg, "ic.seed", 1),
                                                   ns_config_get_double(&cfg, "ic.k0", 8.0),
                                                   ns_config_get_double(&cfg, "ic.energy", 0.5)) != SOLVER_SUCCESS) {
            ns_spectral_free(d);
            ns_config_free(&cfg);
            return 3;
        }
    } else {
        ns_spectral_initialize_taylor_green(d);
    }
    ns_spectral_hyperviscosity_set(d, &hv);  /* after the initial state: SFD starts from it */
    ns_spectral_compute_derivatives(d);      /* psi_hat of the initial state (as performance_benchmark.c:63) */

    if (strcmp(ns_config_get_string(&cfg, "forcing.type", "none"), "none") != 0) {
        if (ns_spectral_gpu_set_forcing(d, 1, ns_config_get_double(&cfg, "forcing.kmin", 4.0),
                                        ns_config_get_double(&cfg, "forcing.kmax", 6.0),
                                        ns_config_get_double(&cfg, "forcing.epsilon", 1e-3),
                                        (unsigned long long)ns_config_get_int(&cfg, "forcing.seed", 1)) != SOLVER_SUCCESS) {
            fprintf(stderr, "ns_run: invalid forcing parameters\n");
            ns_spectral_free(d);
            ns_config_free(&cfg);
            return 2;
        }
    }

    vtk_job vtk[2];
    memset(vtk, 0, sizeof(vtk));
    if (vtk_every > 0) {
        const size_t nr = (size_t)nx * ny * sizeof(double);
        for (int k = 0; k < 2; ++k) {
            vtk[k].u = (double *)ns_gpu_host_alloc(nr);
            vtk[k].v = (double *)ns_gpu_host_alloc(nr);
            vtk[k].w = (double *)ns_gpu_host_alloc(nr);
            vtk[k].x = d->x;
            vtk[k].y = d->y;
            vtk[k].nx = nx;
            vtk[k].ny = ny;
        }
        if (!vtk[0].u || !vtk[0].v || !vtk[0].w || !vtk[1].u || !vtk[1].v || !vtk[1].w) {
            fprintf(stderr, "ns_run: host buffers for VTK output\n");
            ns_spectral_free(d);
            ns_config_free(&cfg);
            return 3;
        }
    }
    long nvtk = 0;

    long step = 0;
    int status = 0;
    double E = 0.0, Z = 0.0;
    ns_spectral_gpu_diagnostics(d, &E, &Z);
    printf("step %ld t %.9g dt %.6g energy %.12e enstrophy %.12e\n", step, d->t, d->dt, E, Z);
    while ((max_steps <= 0 || step < max_steps) && d->t < t_end) {
        /* whole chunks while t_end is far, single steps near it (the reference loop
         * `while (t < t_final)` stops at the first step past t_end) */
        long n = every - step % every;
        if (max_steps > 0 && step + n > max_steps) n = max_steps - step;
        if (d->t + 1.5 * n * d->dt >= t_end) n = 1;
        if (spec_every > 0 && n > spec_every - step % spec_every) n = spec_every - step % spec_every;
        if (ck_every > 0 && n > ck_every - step % ck_every) n = ck_every - step % ck_every;
        if (vtk_every > 0 && n > vtk_every - step % vtk_every) n = vtk_every - step % vtk_every;
        if (ns_spectral_gpu_advance_n(d, (int)n, cfl > 0.0) != SOLVER_SUCCESS) {
            status = 3;
            break;
        }
        step += n;
        {
            /* t and dt of the device state (the host arrays stay stale until a file needs them) */
            double tt = 0.0, dtt = 0.0, e0 = 0.0, z0 = 0.0;
            if (ns_gpu_diagnostics(ns_spectral_gpu_handle(d), &e0, &z0, &tt, &dtt) != 0) {
                status = 3;
                break;
            }
            d->t = tt;
            d->dt = dtt;
        }
        if (step % every == 0 || d->t >= t_end || (max_steps > 0 && step >= max_steps)) {
            if (ns_spectral_gpu_diagnostics(d, &E, &Z) != SOLVER_SUCCESS || !isfinite(E)) {
                status = 3;
                break;
            }
            printf("step %ld t %.9g dt %.6g energy %.12e enstrophy %.12e\n", step, d->t, d->dt, E, Z);
            fflush(stdout);
        }
        if (spec_every > 0 && step % spec_every == 0 && write_spectrum(d, dir, step) != 0) {
            fprintf(stderr, "ns_run: spectrum output failed\n");
            status = 3;
            break;
        }
        if (vtk_every > 0 && step % vtk_every == 0 && vtk_start(&vtk[nvtk++ % 2], d, dir, step) != 0) {
            fprintf(stderr, "ns_run: VTK output failed\n");
            status = 3;
            break;
        }
        if (ck_every > 0 && step % ck_every == 0) {
            char path[1024];
            snprintf(path, sizeof(path), "%s/checkpoint_%06ld.npz", dir, step);
            if (ns_checkpoint_write_spectral(path, d) != 0) {
                fprintf(stderr, "ns_run: checkpoint %s failed\n", path);
                status = 3;
                break;
            }
        }
    }
    for (int k = 0; k < 2; ++k) {
        if (vtk_finish(&vtk[k]) != 0 && status == 0) {
            fprintf(stderr, "ns_run: VTK output failed\n");
            status = 3;
        }
        ns_gpu_host_free(vtk[k].u);
        ns_gpu_host_free(vtk[k].v);
        ns_gpu_host_free(vtk[k].w);
    }
    if (status == 0 && ns_config_get_bool(&cfg, "output.solution", 1)) {
        char path[1024];
        snprintf(path, sizeof(path), "%s/solution.dat", dir);
        ns_spectral_output_solution(d, path);
    }
    if (status != 0) fprintf(stderr, "ns_run: solver failed at step %ld: %s\n", step, ns_spectral_gpu_last_error(d));
    ns_spectral_free(d);
    ns_config_free(&cfg);
    return status;
}
