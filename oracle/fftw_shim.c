/*
 * FFTW3 API shim for the CPU oracle (FP64).
 *
 * ORACLE / TEST INFRASTRUCTURE ONLY.  Used to (a) compile the reference's own
 * spectral sources unmodified into oracle/_ref/, and (b) back the project's C
 * restatement in oracle/ns_oracle.c.  It is never linked into the GPU product.
 *
 * FFTW3 (not vendored by the reference; FFTW 3.3.10 is the version the
 * reference documents in docs/benchmark_results.md:72) is absent here, so the
 * 13 symbols the reference calls are implemented from the DFT definition:
 *
 *   X[k] = sum_n x[n] exp(-2 pi i k n / N)         (forward, unnormalised)
 *   x[n] = sum_k X[k] exp(+2 pi i k n / N)         (backward, unnormalised)
 *
 * Power-of-two lengths use an iterative radix-2 decimation-in-time
 * Cooley-Tukey transform (Cooley & Tukey 1965); other lengths a mixed-radix
 * Stockham transform over their prime factors (each pass a direct p-point sum).  Column transforms run on blocks of columns interleaved so the
 * innermost loop is unit-stride across the block.  The real transforms of
 * length N (even) use the standard half-length packing z[m] = x[2m] + i x[2m+1]
 * with the even/odd split X[k] = E[k] + W^k O[k].  OpenMP threads follow
 * fftw_plan_with_nthreads.
 */
#include "fftw3.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define SHIM_COL_BLOCK 8

static int g_nthreads = 1;

/* cos/sin of 2*pi*k/n, reduced by octant symmetry so that values at exact
 * multiples of pi/4 are exact and the rest are correctly rounded sin/cos of a
 * small argument. */
static void shim_cossin(long k, long n, double *c, double *s) {
    k %= n;
    if (k < 0) k += n;
    if (n % 8 == 0) {
        long q = n / 8;
        long oct = k / q;
        long r = k % q;
        double a = 2.0 * M_PI * (double)r / (double)n;
        double ca = cos(a), sa = sin(a);
        double cb = sin(2.0 * M_PI * (double)(q - r) / (double)n);
        double sb = cos(2.0 * M_PI * (double)(q - r) / (double)n);
        switch (oct) {
            case 0: *c = ca; *s = sa; break;
            case 1: *c = cb; *s = sb; break;           /* angle = pi/2 - b */
            case 2: *c = -sa; *s = ca; break;          /* pi/2 + a */
            case 3: *c = -sb; *s = cb; break;          /* pi - b */
            case 4: *c = -ca; *s = -sa; break;         /* pi + a */
            case 5: *c = -cb; *s = -sb; break;         /* 3pi/2 - b */
            case 6: *c = sa; *s = -ca; break;          /* 3pi/2 + a */
            default: *c = sb; *s = -cb; break;         /* 2pi - b */
        }
        return;
    }
    double a = 2.0 * M_PI * (double)k / (double)n;
    *c = cos(a);
    *s = sin(a);
}

typedef struct {
    int n;
    int pow2;
    int nfac;     /* prime-factor radices of a non-power-of-two length */
    int fac[32];
    int *bitrev;
    double *wr; /* cos(2 pi k/n), k < n */
    double *wi; /* -sin(2 pi k/n): forward twiddle exp(-2 pi i k/n) */
} shim_cfft;

static int shim_is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

static int shim_cfft_init(shim_cfft *f, int n) {
    memset(f, 0, sizeof(*f));
    f->n = n;
    f->pow2 = shim_is_pow2(n);
    f->wr = (double *)malloc(sizeof(double) * (size_t)n);
    f->wi = (double *)malloc(sizeof(double) * (size_t)n);
    if (!f->wr || !f->wi) return -1;
    for (int k = 0; k < n; ++k) {
        double c, s;
        shim_cossin(k, n, &c, &s);
        f->wr[k] = c;
        f->wi[k] = -s;
    }
    if (!f->pow2) {
        int m = n;
        while (m % 4 == 0) { f->fac[f->nfac++] = 4; m /= 4; }
        while (m % 2 == 0) { f->fac[f->nfac++] = 2; m /= 2; }
        for (int p = 3; m > 1; p += 2)
            while (m % p == 0) { f->fac[f->nfac++] = p; m /= p; }
    }
    if (f->pow2) {
        f->bitrev = (int *)malloc(sizeof(int) * (size_t)n);
        if (!f->bitrev) return -1;
        int bits = 0;
        while ((1 << bits) < n) ++bits;
        for (int i = 0; i < n; ++i) {
            int r = 0;
            for (int b = 0; b < bits; ++b) r |= ((i >> b) & 1) << (bits - 1 - b);
            f->bitrev[i] = r;
        }
    }
    return 0;
}

static void shim_cfft_free(shim_cfft *f) {
    free(f->bitrev);
    free(f->wr);
    free(f->wi);
    memset(f, 0, sizeof(*f));
}

/* In-place transform of B interleaved sequences: element (t, b) lives at
 * re[t*B + b], im[t*B + b].  sign = -1 forward, +1 backward.  scratch must
 * hold 2*n*B doubles (used only for non-power-of-two lengths). */
static void shim_cfft_batch(const shim_cfft *f, double *re, double *im, int B, int sign,
                            double *scratch) {
    const int n = f->n;
    if (n == 1) return;
    if (f->pow2) {
        for (int i = 0; i < n; ++i) {
            int r = f->bitrev[i];
            if (r > i) {
                for (int b = 0; b < B; ++b) {
                    double tr = re[i * B + b], ti = im[i * B + b];
                    re[i * B + b] = re[r * B + b];
                    im[i * B + b] = im[r * B + b];
                    re[r * B + b] = tr;
                    im[r * B + b] = ti;
                }
            }
        }
        for (int len = 2; len <= n; len <<= 1) {
            const int half = len >> 1;
            const int step = n / len;
            for (int i0 = 0; i0 < n; i0 += len) {
                for (int j = 0; j < half; ++j) {
                    const double wr = f->wr[j * step];
                    const double wi = (sign < 0) ? f->wi[j * step] : -f->wi[j * step];
                    double *ar = re + (size_t)(i0 + j) * B;
                    double *ai = im + (size_t)(i0 + j) * B;
                    double *br = re + (size_t)(i0 + j + half) * B;
                    double *bi = im + (size_t)(i0 + j + half) * B;
                    for (int b = 0; b < B; ++b) {
                        const double vr = br[b] * wr - bi[b] * wi;
                        const double vi = br[b] * wi + bi[b] * wr;
                        const double ur = ar[b], ui = ai[b];
                        ar[b] = ur + vr;
                        ai[b] = ui + vi;
                        br[b] = ur - vr;
                        bi[b] = ui - vi;
                    }
                }
            }
        }
        return;
    }
    /* other lengths: mixed-radix Stockham autosort (Cooley-Tukey over the prime
     * factors of n, each pass a direct p-point DFT of the twiddled inputs):
     *   butterfly j in [0, n/p), k = j mod Ns:
     *     Y[(j - k) p + k + q Ns] = sum_r X[j + r n/p] W_n^{(k r n/(Ns p)) + (q r mod p) n/p}
     * ping-ponging between the data and the scratch arrays */
    double *sr = re, *si = im;
    double *dr = scratch, *di = scratch + (size_t)n * B;
    int Ns = 1;
    for (int pi = 0; pi < f->nfac; ++pi) {
        const int R = f->fac[pi];
        const int LR = n / R, tstep = n / (Ns * R);
        for (int j = 0; j < LR; ++j) {
            const int k = j % Ns;
            const int base = (j - k) * R + k;
            for (int q = 0; q < R; ++q) {
                double *yr = dr + (size_t)(base + q * Ns) * B;
                double *yi = di + (size_t)(base + q * Ns) * B;
                for (int b = 0; b < B; ++b) {
                    yr[b] = 0.0;
                    yi[b] = 0.0;
                }
                for (int r = 0; r < R; ++r) {
                    const long idx = ((long)tstep * k * r + (long)LR * ((q * r) % R)) % n;
                    const double wr = f->wr[idx];
                    const double wi = (sign < 0) ? f->wi[idx] : -f->wi[idx];
                    const double *xr = sr + (size_t)(j + r * LR) * B;
                    const double *xi = si + (size_t)(j + r * LR) * B;
                    for (int b = 0; b < B; ++b) {
                        yr[b] += xr[b] * wr - xi[b] * wi;
                        yi[b] += xr[b] * wi + xi[b] * wr;
                    }
                }
            }
        }
        double *t = sr; sr = dr; dr = t;
        t = si; si = di; di = t;
        Ns *= R;
    }
    if (sr != re) {
        memcpy(re, sr, sizeof(double) * (size_t)n * B);
        memcpy(im, si, sizeof(double) * (size_t)n * B);
    }
}

struct fftw_plan_s {
    int kind; /* 0 = r2c, 1 = c2r */
    int n0, n1, nh;
    int nthreads;
    shim_cfft col;   /* length n0 */
    shim_cfft row;   /* length n1/2 when n1 is even, else n1 */
    double *pr, *pi; /* exp(-2 pi i k/n1), k < n1/2, for the even/odd split */
};

static fftw_plan shim_plan(int kind, int n0, int n1) {
    fftw_plan p = (fftw_plan)calloc(1, sizeof(*p));
    if (!p) return NULL;
    p->kind = kind;
    p->n0 = n0;
    p->n1 = n1;
    p->nh = n1 / 2 + 1;
    p->nthreads = g_nthreads > 0 ? g_nthreads : 1;
    int rowlen = (n1 % 2 == 0) ? n1 / 2 : n1;
    if (shim_cfft_init(&p->col, n0) || shim_cfft_init(&p->row, rowlen)) {
        fftw_destroy_plan(p);
        return NULL;
    }
    if (n1 % 2 == 0) {
        p->pr = (double *)malloc(sizeof(double) * (size_t)(n1 / 2 + 1));
        p->pi = (double *)malloc(sizeof(double) * (size_t)(n1 / 2 + 1));
        for (int k = 0; k <= n1 / 2; ++k) {
            double c, s;
            shim_cossin(k, n1, &c, &s);
            p->pr[k] = c;
            p->pi[k] = -s;
        }
    }
    return p;
}

fftw_plan fftw_plan_dft_r2c_2d(int n0, int n1, double *in, fftw_complex *out, unsigned flags) {
    (void)in; (void)out; (void)flags;
    return shim_plan(0, n0, n1);
}

fftw_plan fftw_plan_dft_c2r_2d(int n0, int n1, fftw_complex *in, double *out, unsigned flags) {
    (void)in; (void)out; (void)flags;
    return shim_plan(1, n0, n1);
}

void fftw_destroy_plan(fftw_plan p) {
    if (!p) return;
    shim_cfft_free(&p->col);
    shim_cfft_free(&p->row);
    free(p->pr);
    free(p->pi);
    free(p);
}

/* real row of length n1 -> half spectrum [0, n1/2] */
static void shim_row_r2c(const fftw_plan p, const double *x, double *outr, double *outi,
                         double *wr, double *wi, double *scratch) {
    const int n1 = p->n1;
    if (n1 % 2 == 0) {
        const int h = n1 / 2;
        for (int m = 0; m < h; ++m) {
            wr[m] = x[2 * m];
            wi[m] = x[2 * m + 1];
        }
        shim_cfft_batch(&p->row, wr, wi, 1, -1, scratch);
        for (int k = 0; k <= h; ++k) {
            const int a = k % h;
            const int b = (h - k) % h;
            /* E = (Z[k] + conj Z[h-k]) / 2,  O = (Z[k] - conj Z[h-k]) / (2i) */
            const double er = 0.5 * (wr[a] + wr[b]);
            const double ei = 0.5 * (wi[a] - wi[b]);
            const double orr = 0.5 * (wi[a] + wi[b]);
            const double oi = -0.5 * (wr[a] - wr[b]);
            const double tr = p->pr[k], ti = p->pi[k];
            outr[k] = er + (orr * tr - oi * ti);
            outi[k] = ei + (orr * ti + oi * tr);
        }
    } else {
        for (int m = 0; m < n1; ++m) {
            wr[m] = x[m];
            wi[m] = 0.0;
        }
        shim_cfft_batch(&p->row, wr, wi, 1, -1, scratch);
        for (int k = 0; k < p->nh; ++k) {
            outr[k] = wr[k];
            outi[k] = wi[k];
        }
    }
}

/* half spectrum [0, n1/2] -> real row of length n1 (imag of DC and Nyquist ignored) */
static void shim_row_c2r(const fftw_plan p, const double *inr, const double *ini, double *x,
                         double *wr, double *wi, double *scratch) {
    const int n1 = p->n1;
    if (n1 % 2 == 0) {
        const int h = n1 / 2;
        for (int k = 0; k < h; ++k) {
            double ar = inr[k], ai = ini[k];
            double br = inr[h - k], bi = -ini[h - k]; /* conj X[h-k] */
            if (k == 0) {
                ai = 0.0;
                bi = 0.0;
            }
            /* Z[k] = (X[k] + conj X[h-k]) + i * exp(+2 pi i k/n1) * (X[k] - conj X[h-k]) */
            const double sr = ar + br, si = ai + bi;
            const double dr = ar - br, di = ai - bi;
            const double tr = p->pr[k], ti = -p->pi[k];
            const double mr = dr * tr - di * ti;
            const double mi = dr * ti + di * tr;
            wr[k] = sr - mi;
            wi[k] = si + mr;
        }
        shim_cfft_batch(&p->row, wr, wi, 1, +1, scratch);
        for (int m = 0; m < h; ++m) {
            x[2 * m] = wr[m];
            x[2 * m + 1] = wi[m];
        }
    } else {
        const int nh = p->nh;
        for (int k = 0; k < n1; ++k) {
            if (k < nh) {
                wr[k] = inr[k];
                wi[k] = (k == 0) ? 0.0 : ini[k];
            } else {
                wr[k] = inr[n1 - k];
                wi[k] = -ini[n1 - k];
            }
        }
        shim_cfft_batch(&p->row, wr, wi, 1, +1, scratch);
        for (int m = 0; m < n1; ++m) x[m] = wr[m];
    }
}

/* column transforms over a complex [n0][nh] array, in place, sign as given */
static void shim_columns(const fftw_plan p, double *data /* interleaved re,im */, int sign) {
    const int n0 = p->n0, nh = p->nh;
    const int nblocks = (nh + SHIM_COL_BLOCK - 1) / SHIM_COL_BLOCK;
#pragma omp parallel num_threads(p->nthreads)
    {
        double *re = (double *)malloc(sizeof(double) * (size_t)n0 * SHIM_COL_BLOCK);
        double *im = (double *)malloc(sizeof(double) * (size_t)n0 * SHIM_COL_BLOCK);
        double *scratch = (double *)malloc(sizeof(double) * 2 * (size_t)n0 * SHIM_COL_BLOCK);
#pragma omp for schedule(static)
        for (int blk = 0; blk < nblocks; ++blk) {
            const int c0 = blk * SHIM_COL_BLOCK;
            const int B = (c0 + SHIM_COL_BLOCK <= nh) ? SHIM_COL_BLOCK : nh - c0;
            for (int t = 0; t < n0; ++t) {
                const double *src = data + 2 * ((size_t)t * nh + c0);
                for (int b = 0; b < B; ++b) {
                    re[t * B + b] = src[2 * b];
                    im[t * B + b] = src[2 * b + 1];
                }
            }
            shim_cfft_batch(&p->col, re, im, B, sign, scratch);
            for (int t = 0; t < n0; ++t) {
                double *dst = data + 2 * ((size_t)t * nh + c0);
                for (int b = 0; b < B; ++b) {
                    dst[2 * b] = re[t * B + b];
                    dst[2 * b + 1] = im[t * B + b];
                }
            }
        }
        free(re);
        free(im);
        free(scratch);
    }
}

void fftw_execute_dft_r2c(const fftw_plan p, double *in, fftw_complex *out) {
    if (!p || p->kind != 0) return;
    const int n0 = p->n0, n1 = p->n1, nh = p->nh;
    double *o = (double *)out;
#pragma omp parallel num_threads(p->nthreads)
    {
        double *wr = (double *)malloc(sizeof(double) * (size_t)n1);
        double *wi = (double *)malloc(sizeof(double) * (size_t)n1);
        double *outr = (double *)malloc(sizeof(double) * (size_t)nh);
        double *outi = (double *)malloc(sizeof(double) * (size_t)nh);
        double *scratch = (double *)malloc(sizeof(double) * 2 * (size_t)n1);
#pragma omp for schedule(static)
        for (int j = 0; j < n0; ++j) {
            shim_row_r2c(p, in + (size_t)j * n1, outr, outi, wr, wi, scratch);
            double *dst = o + 2 * (size_t)j * nh;
            for (int k = 0; k < nh; ++k) {
                dst[2 * k] = outr[k];
                dst[2 * k + 1] = outi[k];
            }
        }
        free(wr);
        free(wi);
        free(outr);
        free(outi);
        free(scratch);
    }
    shim_columns(p, o, -1);
}

void fftw_execute_dft_c2r(const fftw_plan p, fftw_complex *in, double *out) {
    if (!p || p->kind != 1) return;
    const int n0 = p->n0, n1 = p->n1, nh = p->nh;
    /* FFTW may destroy the input of a c2r; this shim works on a copy instead */
    double *tmp = (double *)malloc(sizeof(double) * 2 * (size_t)n0 * nh);
    if (!tmp) return;
    memcpy(tmp, in, sizeof(double) * 2 * (size_t)n0 * nh);
    shim_columns(p, tmp, +1);
#pragma omp parallel num_threads(p->nthreads)
    {
        double *wr = (double *)malloc(sizeof(double) * (size_t)n1);
        double *wi = (double *)malloc(sizeof(double) * (size_t)n1);
        double *inr = (double *)malloc(sizeof(double) * (size_t)nh);
        double *ini = (double *)malloc(sizeof(double) * (size_t)nh);
        double *scratch = (double *)malloc(sizeof(double) * 2 * (size_t)n1);
#pragma omp for schedule(static)
        for (int j = 0; j < n0; ++j) {
            const double *src = tmp + 2 * (size_t)j * nh;
            for (int k = 0; k < nh; ++k) {
                inr[k] = src[2 * k];
                ini[k] = src[2 * k + 1];
            }
            shim_row_c2r(p, inr, ini, out + (size_t)j * n1, wr, wi, scratch);
        }
        free(wr);
        free(wi);
        free(inr);
        free(ini);
        free(scratch);
    }
    free(tmp);
}

double *fftw_alloc_real(size_t n) {
    void *ptr = NULL;
    if (posix_memalign(&ptr, 64, n * sizeof(double) + 64) != 0) return NULL;
    memset(ptr, 0, n * sizeof(double));
    return (double *)ptr;
}

fftw_complex *fftw_alloc_complex(size_t n) {
    void *ptr = NULL;
    if (posix_memalign(&ptr, 64, n * sizeof(fftw_complex) + 64) != 0) return NULL;
    memset(ptr, 0, n * sizeof(fftw_complex));
    return (fftw_complex *)ptr;
}

void fftw_free(void *p) { free(p); }

void fftw_cleanup(void) {}

int fftw_init_threads(void) { return 1; }

void fftw_plan_with_nthreads(int nthreads) { g_nthreads = nthreads > 0 ? nthreads : 1; }

void fftw_cleanup_threads(void) {}
