/*
 * Declarations-only FFTW3 API header for the CPU oracle.
 *
 * ORACLE / TEST INFRASTRUCTURE ONLY.  FFTW3 is the reference solver's FFT
 * dependency (call sites: src/spectral/spectral_initialization.c:58-68,
 * src/spectral/spectral_transforms.c:10,31, src/spectral/spectral_memory.c:24-44,74-103;
 * FFTW 3.3.10 per docs/benchmark_results.md:72).  FFTW is not installed on
 * either build machine, so this header declares exactly the 13 symbols the
 * reference uses and oracle/fftw_shim.c implements them from the DFT
 * definition (no FFTW code).
 *
 * Semantics kept from FFTW's published API:
 *   - fftw_plan_dft_r2c_2d(n0, n1, ...) maps real [n0][n1] (row-major) to
 *     complex [n0][n1/2+1]; forward sign e^{-2 pi i jk/n}; unnormalised.
 *   - fftw_plan_dft_c2r_2d is the unnormalised inverse (sign e^{+}); the
 *     imaginary parts of the DC and Nyquist bins of the last dimension are
 *     ignored (Hermitian input assumed).
 *   - fftw_complex is C99 double _Complex when <complex.h> is included first,
 *     which is what src/spectral/ns_spectral_solver.h:5-6 does.
 */
#ifndef FFTW3_H
#define FFTW3_H

#include <stddef.h>
#include <complex.h>

typedef double _Complex fftw_complex;
typedef struct fftw_plan_s *fftw_plan;

#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)

fftw_plan fftw_plan_dft_r2c_2d(int n0, int n1, double *in, fftw_complex *out, unsigned flags);
fftw_plan fftw_plan_dft_c2r_2d(int n0, int n1, fftw_complex *in, double *out, unsigned flags);
void fftw_execute_dft_r2c(const fftw_plan p, double *in, fftw_complex *out);
void fftw_execute_dft_c2r(const fftw_plan p, fftw_complex *in, double *out);
void fftw_destroy_plan(fftw_plan p);
double *fftw_alloc_real(size_t n);
fftw_complex *fftw_alloc_complex(size_t n);
void fftw_free(void *p);
void fftw_cleanup(void);
int fftw_init_threads(void);
void fftw_plan_with_nthreads(int nthreads);
void fftw_cleanup_threads(void);

#endif /* FFTW3_H */
