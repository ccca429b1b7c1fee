/*
 * Drop-in implementation of the reference forcing API (src/common/forcing.c:41-184).
 *
 * The shell selection and the noise generation run on the GPU through a small
 * process-wide utility instance of the C-ABI (the API carries no solver
 * handle).  The struct fields keep the reference meaning: rng_state advances
 * by two splitmix64 draws per active mode and call, have_spare stays 0.
 */
#include "forcing.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "ns_gpu.h"

static ns_gpu *g_util = NULL;

static void ns_forcing_util_release(void) {
    ns_gpu_destroy(g_util);
    g_util = NULL;
}

static ns_gpu *ns_forcing_util(void) {
    if (!g_util) {
        if (ns_gpu_create(8, 8, 1.0, 1.0, NS_GPU_FP64, &g_util) != NS_GPU_OK) {
            fprintf(stderr, "[ns-gb300] forcing: no GPU instance available\n");
            g_util = NULL;
            return NULL;
        }
        atexit(ns_forcing_util_release);
    }
    return g_util;
}

void ns_forcing_config_default(NSForcingConfig *c) {
    if (!c) return;
    /* forcing.c:45-50 */
    c->kmin = 0.0;
    c->kmax = 4.0;
    c->energy_target = 1.0;
    c->correlation_time = 0.5;
    c->seed = 0;
    c->type = NS_FORCING_WHITE_NOISE;
}

int ns_forcing_state_init(NSForcingState *st, const NSForcingConfig *c, const double *k2, int nkx, int nky) {
    if (!st || !c || !k2 || nkx <= 0 || nky <= 0) return -1;
    memset(st, 0, sizeof(*st));
    st->config = *c;
    st->nkx = nkx;
    st->nky = nky;
    st->spectral_size = nkx * nky;
    st->weights = (double *)calloc((size_t)st->spectral_size, sizeof(double));
    if (!st->weights) return -1;
    if (c->type == NS_FORCING_COLORED_NOISE) {
        st->colored_state = (double _Complex *)calloc((size_t)st->spectral_size, sizeof(double _Complex));
        if (!st->colored_state) {
            ns_forcing_state_free(st);
            return -1;
        }
    }
    ns_gpu *g = ns_forcing_util();
    if (!g) {
        ns_forcing_state_free(st);
        return -1;
    }
    /* forcing.c:75-76: kmin clamped at 0, kmax at least kmin */
    const double kmin = fmax(c->kmin, 0.0);
    const double kmax = fmax(c->kmax, kmin);
    int active = 0;
    if (ns_gpu_forcing_weights(g, k2, st->spectral_size, kmin, kmax, st->weights, &active) != NS_GPU_OK) {
        fprintf(stderr, "[ns-gb300] ns_forcing_state_init: %s\n", ns_gpu_last_error(g));
        ns_forcing_state_free(st);
        return -1;
    }
    st->active_modes = active;
    st->have_spare = 0;
    st->rng_state = c->seed ? (unsigned long long)c->seed : 0x123456789abcdefULL;
    return active == 0 ? -1 : 0;
}

void ns_forcing_state_free(NSForcingState *st) {
    if (!st) return;
    free(st->weights);
    st->weights = NULL;
    free(st->colored_state);
    st->colored_state = NULL;
    st->spectral_size = 0;
    st->active_modes = 0;
}

void ns_forcing_generate(NSForcingState *st, double dt, const double *k2, double _Complex *out) {
    if (!st || !out || !k2) return;
    const int n = st->spectral_size;
    if (n == 0) return;
    ns_gpu *g = ns_forcing_util();
    if (!g) return;
    uint64_t rng = (uint64_t)st->rng_state;
    const int colored = (st->config.type == NS_FORCING_COLORED_NOISE);
    int s = ns_gpu_forcing_generate(g, n, st->weights, st->active_modes, colored && st->colored_state, dt,
                                    st->config.correlation_time, st->config.energy_target, &rng,
                                    (double *)st->colored_state, (double *)out);
    if (s != NS_GPU_OK) {
        fprintf(stderr, "[ns-gb300] ns_forcing_generate: %s\n", ns_gpu_last_error(g));
        return;
    }
    if (st->active_modes > 0 && st->config.energy_target > 0.0) {
        st->rng_state = (unsigned long long)rng;
        st->have_spare = 0;
    }
}
