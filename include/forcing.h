/*
 * forcing.h -- drop-in for the reference stochastic forcing API
 * src/common/forcing.h:1-48 (DiogoRibeiro7/navier-stokes-solvers).
 *
 * Same types and functions.  ns_forcing_state_init's shell selection and
 * ns_forcing_generate run on the GPU; generate reproduces the reference
 * splitmix64/Box-Muller stream (forcing.c:11-39) counter-addressably, so the
 * same seed gives the same forcing as the reference up to the last bits of
 * log/sin/cos, and the struct's rng_state advances exactly as the reference's.
 */
#ifndef NS_COMMON_FORCING_H
#define NS_COMMON_FORCING_H

#include "common_types.h"
#include <complex.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    NS_FORCING_WHITE_NOISE = 0,
    NS_FORCING_COLORED_NOISE = 1
} NSForcingType;

typedef struct {
    double kmin;
    double kmax;
    double energy_target;
    double correlation_time;
    unsigned long seed;
    NSForcingType type;
} NSForcingConfig;

typedef struct {
    NSForcingConfig config;
    int nkx;
    int nky;
    int spectral_size;
    int active_modes;
    double *weights;
    double _Complex *colored_state;
    unsigned int have_spare;
    double spare_gaussian;
    unsigned long long rng_state;
} NSForcingState;

void ns_forcing_config_default(NSForcingConfig *config);
int ns_forcing_state_init(NSForcingState *state, const NSForcingConfig *config, const double *k2, int nkx, int nky);
void ns_forcing_state_free(NSForcingState *state);
void ns_forcing_generate(NSForcingState *state, double dt, const double *k2, double _Complex *forcing_out);

#ifdef __cplusplus
}
#endif

#endif /* NS_COMMON_FORCING_H */
