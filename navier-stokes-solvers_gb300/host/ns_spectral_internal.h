/*
 * Private state of the drop-in solver (the appended NSSpectralData::gpu field),
 * shared by the host translation units of the library; not installed.
 */
#ifndef NS_SPECTRAL_INTERNAL_H
#define NS_SPECTRAL_INTERNAL_H

#include "ns_gpu.h"

struct ns_spectral_gpu {
    ns_gpu *dev;
    int precision;
    int host_stale;      /* device state is newer than the host arrays */
    int device_current;  /* device state equals the host arrays (no upload needed) */
    unsigned long long step;
    int forcing_enabled;
    double forcing_kmin, forcing_kmax, forcing_epsilon;
    unsigned long long forcing_seed;
    int scheme;
};

#endif /* NS_SPECTRAL_INTERNAL_H */
