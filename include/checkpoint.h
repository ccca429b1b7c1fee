/*
 * checkpoint.h -- checkpoint / resume of the spectral solver state.
 *
 * Same entry points, attribute names and dataset names as the reference's
 * spectral checkpoint (src/common/checkpoint.h:14-15, checkpoint.c:266-360 of
 * DiogoRibeiro7/navier-stokes-solvers): attributes solver = "spectral", time,
 * dt, Re, nx, ny, Lx, Ly and datasets /fields/{u, v, omega, psi} [ny][nx],
 * /fields/{u_hat, v_hat, omega_hat} [nky][nkx] complex.  The reference writes
 * HDF5; this library writes the same names into an uncompressed NumPy .npz
 * archive (a zip of .npy arrays; numpy.load reads it), entry "<name>.npy" per
 * attribute and "fields/<name>.npy" per dataset, so no HDF5 dependency exists.
 *
 * Beyond the reference's datasets the file also holds what an exact resume
 * needs, which the reference omits: fields/psi_hat (stage 1 of the next step
 * reads the stored psi_hat, spectral_core.c:51,66,76), fields/sfd_hat,
 * cfl_factor, the hyperviscosity configuration, and the GPU extension state
 * (forcing configuration, forcing step counter, time scheme).  A run read back
 * from a checkpoint continues exactly as the uninterrupted run.
 *
 * Both functions return 0 on success and -1 on failure (the reference's
 * convention); read fails when the file's nx, ny differ from the state's.
 * The finite-difference variants of the reference are out of scope.
 */
#ifndef NS_CHECKPOINT_H
#define NS_CHECKPOINT_H

#include "ns_spectral_solver.h"

#ifdef __cplusplus
extern "C" {
#endif

/* src/common/checkpoint.h:14 / checkpoint.c:266-302 */
int ns_checkpoint_write_spectral(const char *filename, const NSSpectralData *state);
/* src/common/checkpoint.h:15 / checkpoint.c:304-360 */
int ns_checkpoint_read_spectral(const char *filename, NSSpectralData *state);

#ifdef __cplusplus
}
#endif

#endif /* NS_CHECKPOINT_H */
