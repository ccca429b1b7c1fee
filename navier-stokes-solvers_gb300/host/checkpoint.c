/*
 * Checkpoint / resume of the spectral state (include/checkpoint.h).
 *
 * The reference writes HDF5 (src/common/checkpoint.c:266-360); HDF5 is not a
 * dependency here, so the same attribute and dataset names go into an
 * uncompressed .npz archive: a zip file whose entries are NumPy .npy arrays
 * ("stored" method, CRC-32 per entry, little-endian data).  The writer and the
 * reader below handle exactly that subset of the zip and .npy formats.
 */
#include "checkpoint.h"

#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "ns_gpu.h"
#include "ns_spectral_internal.h"

/* ------------------------------------------------------------- byte helpers */

static void put16(unsigned char *p, uint32_t v) { p[0] = (unsigned char)v; p[1] = (unsigned char)(v >> 8); }
static void put32(unsigned char *p, uint32_t v) {
    p[0] = (unsigned char)v;
    p[1] = (unsigned char)(v >> 8);
    p[2] = (unsigned char)(v >> 16);
    p[3] = (unsigned char)(v >> 24);
}
static uint32_t get16(const unsigned char *p) { return (uint32_t)p[0] | ((uint32_t)p[1] << 8); }
static uint32_t get32(const unsigned char *p) {
    return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
}

static int host_is_little_endian(void) {
    const uint16_t one = 1;
    return *(const unsigned char *)&one == 1;
}

/* CRC-32 (reflected polynomial 0xEDB88320), as the zip format specifies */
static uint32_t crc32_update(uint32_t crc, const unsigned char *p, size_t n) {
    static uint32_t table[256];
    static int ready = 0;
    if (!ready) {
        for (uint32_t i = 0; i < 256; ++i) {
            uint32_t c = i;
            for (int k = 0; k < 8; ++k) c = (c & 1u) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
            table[i] = c;
        }
        ready = 1;
    }
    crc = ~crc;
    for (size_t i = 0; i < n; ++i) crc = table[(crc ^ p[i]) & 0xFFu] ^ (crc >> 8);
    return ~crc;
}

/* ------------------------------------------------------------- .npz writer */

#define NPZ_MAX_ENTRIES 64

typedef struct {
    char name[64];
    uint32_t crc, size, offset;
} npz_entry;

typedef struct {
    FILE *f;
    uint32_t n;
    uint64_t pos;
    int failed;
    npz_entry e[NPZ_MAX_ENTRIES];
} npz_writer;

/* .npy version 1.0 header for descr and shape, padded so the data starts on a
 * 64-byte boundary; returns its length */
static size_t npy_header(char *out, size_t cap, const char *descr, int ndim, const size_t *shape) {
    char dict[256];
    int k = snprintf(dict, sizeof(dict), "{'descr': '%s', 'fortran_order': False, 'shape': (", descr);
    for (int i = 0; i < ndim; ++i) k += snprintf(dict + k, sizeof(dict) - (size_t)k, ndim == 1 ? "%zu," : (i ? ", %zu" : "%zu"), shape[i]);
    k += snprintf(dict + k, sizeof(dict) - (size_t)k, "), }");
    size_t total = 10 + (size_t)k + 1;
    total = (total + 63) & ~(size_t)63;
    if (total > cap) return 0;
    const size_t hlen = total - 10;
    memcpy(out, "\x93NUMPY\x01\x00", 8);
    put16((unsigned char *)out + 8, (uint32_t)hlen);
    memcpy(out + 10, dict, (size_t)k);
    memset(out + 10 + k, ' ', hlen - (size_t)k - 1);
    out[total - 1] = '\n';
    return total;
}

static void npz_write_bytes(npz_writer *z, const void *p, size_t n) {
    if (z->failed) return;
    if (n && fwrite(p, 1, n, z->f) != n) z->failed = 1;
    z->pos += n;
}

static void npz_add(npz_writer *z, const char *name, const char *descr, int ndim, const size_t *shape, const void *data,
                    size_t nbytes) {
    if (z->failed) return;
    if (z->n >= NPZ_MAX_ENTRIES || strlen(name) >= sizeof(z->e[0].name) || (data == NULL && nbytes)) {
        z->failed = 1;
        return;
    }
    char hdr[256];
    const size_t hl = npy_header(hdr, sizeof(hdr), descr, ndim, shape);
    const uint64_t size = (uint64_t)hl + nbytes;
    if (hl == 0 || size > 0xFFFFFFFFull || z->pos > 0xFFFFFFFFull) {
        z->failed = 1;
        return;
    }
    uint32_t crc = crc32_update(0, (const unsigned char *)hdr, hl);
    crc = crc32_update(crc, (const unsigned char *)data, nbytes);
    npz_entry *e = &z->e[z->n++];
    snprintf(e->name, sizeof(e->name), "%s", name);
    e->crc = crc;
    e->size = (uint32_t)size;
    e->offset = (uint32_t)z->pos;
    unsigned char lh[30];
    const size_t nl = strlen(name);
    put32(lh, 0x04034b50u);
    put16(lh + 4, 20);         /* version needed */
    put16(lh + 6, 0);          /* flags */
    put16(lh + 8, 0);          /* stored */
    put16(lh + 10, 0);         /* time */
    put16(lh + 12, 33);        /* date 1980-01-01 */
    put32(lh + 14, crc);
    put32(lh + 18, e->size);   /* compressed */
    put32(lh + 22, e->size);   /* uncompressed */
    put16(lh + 26, (uint32_t)nl);
    put16(lh + 28, 0);
    npz_write_bytes(z, lh, sizeof(lh));
    npz_write_bytes(z, name, nl);
    npz_write_bytes(z, hdr, hl);
    npz_write_bytes(z, data, nbytes);
}

static int npz_finish(npz_writer *z) {
    const uint64_t cd_start = z->pos;
    for (uint32_t i = 0; i < z->n && !z->failed; ++i) {
        const npz_entry *e = &z->e[i];
        const size_t nl = strlen(e->name);
        unsigned char ch[46];
        put32(ch, 0x02014b50u);
        put16(ch + 4, 20);
        put16(ch + 6, 20);
        put16(ch + 8, 0);
        put16(ch + 10, 0);
        put16(ch + 12, 0);
        put16(ch + 14, 33);
        put32(ch + 16, e->crc);
        put32(ch + 20, e->size);
        put32(ch + 24, e->size);
        put16(ch + 28, (uint32_t)nl);
        put16(ch + 30, 0);
        put16(ch + 32, 0);
        put16(ch + 34, 0);
        put16(ch + 36, 0);
        put32(ch + 38, 0);
        put32(ch + 42, e->offset);
        npz_write_bytes(z, ch, sizeof(ch));
        npz_write_bytes(z, e->name, nl);
    }
    unsigned char end[22];
    put32(end, 0x06054b50u);
    put16(end + 4, 0);
    put16(end + 6, 0);
    put16(end + 8, z->n);
    put16(end + 10, z->n);
    put32(end + 12, (uint32_t)(z->pos - cd_start));
    put32(end + 16, (uint32_t)cd_start);
    put16(end + 20, 0);
    npz_write_bytes(z, end, sizeof(end));
    return z->failed ? -1 : 0;
}

/* ------------------------------------------------------------- .npz reader */

typedef struct {
    unsigned char *buf;  /* whole file */
    size_t len;
} npz_reader;

/* locate entry name; returns the .npy payload (header included) or NULL */
static const unsigned char *npz_find(const npz_reader *r, const char *name, size_t *size) {
    if (r->len < 22) return NULL;
    size_t eocd = r->len - 22;
    for (;; --eocd) {
        if (get32(r->buf + eocd) == 0x06054b50u) break;
        if (eocd == 0 || r->len - eocd > 22 + 65535) return NULL;
    }
    const uint32_t n = get16(r->buf + eocd + 10);
    size_t p = get32(r->buf + eocd + 16);
    const size_t nl_want = strlen(name);
    for (uint32_t i = 0; i < n; ++i) {
        if (p + 46 > r->len || get32(r->buf + p) != 0x02014b50u) return NULL;
        const uint32_t method = get16(r->buf + p + 10);
        const uint32_t csize = get32(r->buf + p + 20);
        const uint32_t nl = get16(r->buf + p + 28), xl = get16(r->buf + p + 30), cl = get16(r->buf + p + 32);
        const uint32_t off = get32(r->buf + p + 42);
        if (p + 46 + nl > r->len) return NULL;
        if (nl == nl_want && memcmp(r->buf + p + 46, name, nl) == 0) {
            if (method != 0 || (size_t)off + 30 > r->len) return NULL;
            const size_t data = (size_t)off + 30 + get16(r->buf + off + 26) + get16(r->buf + off + 28);
            if (data + csize > r->len) return NULL;
            *size = csize;
            return r->buf + data;
        }
        p += 46 + nl + xl + cl;
    }
    return NULL;
}

/* copy the data of a .npy payload whose descr and element count match */
static int npy_read(const unsigned char *p, size_t size, const char *descr, size_t count, size_t elem, void *out) {
    if (size < 10 || memcmp(p, "\x93NUMPY", 6) != 0) return -1;
    size_t hl, off;
    if (p[6] == 1) { hl = get16(p + 8); off = 10; }
    else { if (size < 12) return -1; hl = get32(p + 8); off = 12; }
    if (off + hl > size) return -1;
    char dict[512];
    const size_t dl = hl < sizeof(dict) - 1 ? hl : sizeof(dict) - 1;
    memcpy(dict, p + off, dl);
    dict[dl] = 0;
    char want[64];
    snprintf(want, sizeof(want), "'descr': '%s'", descr);
    if (!strstr(dict, want) || strstr(dict, "'fortran_order': True")) return -1;
    if (size - off - hl != count * elem) return -1;
    if (out) memcpy(out, p + off + hl, count * elem); /* out == NULL: check only */
    return 0;
}

static int npz_get(const npz_reader *r, const char *name, const char *descr, size_t count, size_t elem, void *out) {
    size_t size = 0;
    const unsigned char *p = npz_find(r, name, &size);
    if (!p) return -1;
    return npy_read(p, size, descr, count, elem, out);
}

/* ------------------------------------------------------------------ API */

int ns_checkpoint_write_spectral(const char *filename, const NSSpectralData *state) {
    if (!filename || !state || !host_is_little_endian()) return -1;
    NSSpectralData *d = (NSSpectralData *)state;
    /* device-resident steps newer than the host arrays are downloaded first */
    if (d->gpu && ns_spectral_gpu_sync_host(d) != SOLVER_SUCCESS) return -1;
    npz_writer z;
    memset(&z, 0, sizeof(z));
    z.f = fopen(filename, "wb");
    if (!z.f) return -1;
    const size_t none[1] = {0};
    const size_t rs[2] = {(size_t)d->ny, (size_t)d->nx};
    const size_t cs[2] = {(size_t)d->nky, (size_t)d->nkx};
    const size_t nr = rs[0] * rs[1], nc = cs[0] * cs[1];
    /* attributes (checkpoint.c:272-279) */
    npz_add(&z, "solver.npy", "|S8", 0, none, "spectral", 8);
    npz_add(&z, "time.npy", "<f8", 0, none, &d->t, sizeof(double));
    npz_add(&z, "dt.npy", "<f8", 0, none, &d->dt, sizeof(double));
    npz_add(&z, "Re.npy", "<f8", 0, none, &d->Re, sizeof(double));
    npz_add(&z, "nx.npy", "<i4", 0, none, &d->nx, sizeof(int));
    npz_add(&z, "ny.npy", "<i4", 0, none, &d->ny, sizeof(int));
    npz_add(&z, "Lx.npy", "<f8", 0, none, &d->Lx, sizeof(double));
    npz_add(&z, "Ly.npy", "<f8", 0, none, &d->Ly, sizeof(double));
    /* datasets (checkpoint.c:290-297) */
    npz_add(&z, "fields/u.npy", "<f8", 2, rs, d->u, nr * sizeof(double));
    npz_add(&z, "fields/v.npy", "<f8", 2, rs, d->v, nr * sizeof(double));
    npz_add(&z, "fields/omega.npy", "<f8", 2, rs, d->omega, nr * sizeof(double));
    npz_add(&z, "fields/psi.npy", "<f8", 2, rs, d->psi, nr * sizeof(double));
    npz_add(&z, "fields/u_hat.npy", "<c16", 2, cs, d->u_hat, nc * sizeof(fftw_complex));
    npz_add(&z, "fields/v_hat.npy", "<c16", 2, cs, d->v_hat, nc * sizeof(fftw_complex));
    npz_add(&z, "fields/omega_hat.npy", "<c16", 2, cs, d->omega_hat, nc * sizeof(fftw_complex));
    /* what an exact resume needs beyond the reference's datasets */
    npz_add(&z, "fields/psi_hat.npy", "<c16", 2, cs, d->psi_hat, nc * sizeof(fftw_complex));
    npz_add(&z, "fields/sfd_hat.npy", "<c16", 2, cs, d->sfd_hat, nc * sizeof(fftw_complex));
    npz_add(&z, "cfl_factor.npy", "<f8", 0, none, &d->cfl_factor, sizeof(double));
    const NSSpectralHyperviscosityConfig *h = &d->hyperviscosity;
    const double hv[10] = {(double)h->enabled, h->coefficient, (double)h->order, h->cutoff_ratio, h->sfd_strength,
                           h->sfd_timescale, (double)h->sfd_enabled, h->kmax, h->cutoff_wavenumber, h->inv_bandwidth};
    const size_t s10[1] = {10};
    npz_add(&z, "hyperviscosity.npy", "<f8", 1, s10, hv, sizeof(hv));
    if (d->gpu) {
        const double fc[4] = {(double)d->gpu->forcing_enabled, d->gpu->forcing_kmin, d->gpu->forcing_kmax,
                              d->gpu->forcing_epsilon};
        const size_t s4[1] = {4};
        const uint64_t seed = d->gpu->forcing_seed, step = d->gpu->step;
        npz_add(&z, "gpu/forcing.npy", "<f8", 1, s4, fc, sizeof(fc));
        npz_add(&z, "gpu/forcing_seed.npy", "<u8", 0, none, &seed, sizeof(seed));
        npz_add(&z, "gpu/step.npy", "<u8", 0, none, &step, sizeof(step));
        npz_add(&z, "gpu/scheme.npy", "<i4", 0, none, &d->gpu->scheme, sizeof(int));
        npz_add(&z, "gpu/precision.npy", "<i4", 0, none, &d->gpu->precision, sizeof(int));
    }
    int st = npz_finish(&z);
    if (fclose(z.f) != 0) st = -1;
    return st;
}

int ns_checkpoint_read_spectral(const char *filename, NSSpectralData *state) {
    if (!filename || !state || !host_is_little_endian()) return -1;
    FILE *f = fopen(filename, "rb");
    if (!f) return -1;
    npz_reader r = {NULL, 0};
    if (fseek(f, 0, SEEK_END) == 0) {
        const long len = ftell(f);
        if (len > 0 && fseek(f, 0, SEEK_SET) == 0) {
            r.buf = (unsigned char *)malloc((size_t)len);
            if (r.buf && fread(r.buf, 1, (size_t)len, f) == (size_t)len) r.len = (size_t)len;
        }
    }
    fclose(f);
    if (!r.len) {
        free(r.buf);
        return -1;
    }
    NSSpectralData *d = state;
    int nx = 0, ny = 0;
    double Lx = 0.0, Ly = 0.0, Re = 0.0, t = 0.0, dt = 0.0;
    int st = 0;
    st |= npz_get(&r, "nx.npy", "<i4", 1, sizeof(int), &nx);
    st |= npz_get(&r, "ny.npy", "<i4", 1, sizeof(int), &ny);
    st |= npz_get(&r, "Lx.npy", "<f8", 1, sizeof(double), &Lx);
    st |= npz_get(&r, "Ly.npy", "<f8", 1, sizeof(double), &Ly);
    st |= npz_get(&r, "Re.npy", "<f8", 1, sizeof(double), &Re);
    st |= npz_get(&r, "time.npy", "<f8", 1, sizeof(double), &t);
    st |= npz_get(&r, "dt.npy", "<f8", 1, sizeof(double), &dt);
    if (st || nx != d->nx || ny != d->ny) {
        free(r.buf);
        return -1;
    }
    const size_t nr = (size_t)d->nx * d->ny, nc = (size_t)d->nkx * d->nky;
    /* every required dataset is checked (name, type, element count) before the
     * first one is copied, so a bad file leaves the state untouched */
    static const char *const req_real[] = {"fields/u.npy", "fields/v.npy", "fields/omega.npy", "fields/psi.npy"};
    static const char *const req_cplx[] = {"fields/u_hat.npy", "fields/v_hat.npy", "fields/omega_hat.npy"};
    for (size_t i = 0; i < sizeof(req_real) / sizeof(req_real[0]); ++i)
        st |= npz_get(&r, req_real[i], "<f8", nr, sizeof(double), NULL);
    for (size_t i = 0; i < sizeof(req_cplx) / sizeof(req_cplx[0]); ++i)
        st |= npz_get(&r, req_cplx[i], "<c16", nc, sizeof(fftw_complex), NULL);
    if (st) {
        free(r.buf);
        return -1;
    }
    /* newer device-resident steps must not overwrite what is read below */
    if (d->gpu && ns_spectral_gpu_sync_host(d) != SOLVER_SUCCESS) {
        free(r.buf);
        return -1;
    }
    st |= npz_get(&r, "fields/u.npy", "<f8", nr, sizeof(double), d->u);
    st |= npz_get(&r, "fields/v.npy", "<f8", nr, sizeof(double), d->v);
    st |= npz_get(&r, "fields/omega.npy", "<f8", nr, sizeof(double), d->omega);
    st |= npz_get(&r, "fields/psi.npy", "<f8", nr, sizeof(double), d->psi);
    st |= npz_get(&r, "fields/u_hat.npy", "<c16", nc, sizeof(fftw_complex), d->u_hat);
    st |= npz_get(&r, "fields/v_hat.npy", "<c16", nc, sizeof(fftw_complex), d->v_hat);
    st |= npz_get(&r, "fields/omega_hat.npy", "<c16", nc, sizeof(fftw_complex), d->omega_hat);
    if (st == 0) {
        d->Lx = Lx;
        d->Ly = Ly;
        d->Re = Re;
        d->t = t;
        d->dt = dt;
        /* optional entries: absent in files from other writers */
        npz_get(&r, "fields/psi_hat.npy", "<c16", nc, sizeof(fftw_complex), d->psi_hat);
        npz_get(&r, "cfl_factor.npy", "<f8", 1, sizeof(double), &d->cfl_factor);
        double hv[10];
        if (npz_get(&r, "hyperviscosity.npy", "<f8", 10, sizeof(double), hv) == 0) {
            NSSpectralHyperviscosityConfig c = d->hyperviscosity;
            c.enabled = (int)hv[0];
            c.coefficient = hv[1];
            c.order = (int)hv[2];
            c.cutoff_ratio = hv[3];
            c.sfd_strength = hv[4];
            c.sfd_timescale = hv[5];
            c.sfd_enabled = (int)hv[6];
            if (d->gpu) {
                /* not ns_spectral_hyperviscosity_set: it re-seeds the SFD filter
                 * with omega_hat (hyperviscosity.c:38-57), and the filter state is
                 * part of the checkpoint */
                d->hyperviscosity = c;
                if (!c.enabled) memset(d->hyperviscosity_weights, 0, nc * sizeof(double));
                ns_spectral_hyperviscosity_update_weights(d);  /* kmax, cutoff and the weights */
            } else {
                c.kmax = hv[7];
                c.cutoff_wavenumber = hv[8];
                c.inv_bandwidth = hv[9];
                d->hyperviscosity = c;
            }
        }
        if (!d->gpu) npz_get(&r, "fields/sfd_hat.npy", "<c16", nc, sizeof(fftw_complex), d->sfd_hat);
        if (d->gpu) {
            double fc[4];
            uint64_t seed = 0, step = 0;
            int scheme = 0;
            if (npz_get(&r, "gpu/forcing.npy", "<f8", 4, sizeof(double), fc) == 0 &&
                npz_get(&r, "gpu/forcing_seed.npy", "<u8", 1, sizeof(uint64_t), &seed) == 0)
                ns_spectral_gpu_set_forcing(d, (int)fc[0], fc[1], fc[2], fc[3], (unsigned long long)seed);
            if (npz_get(&r, "gpu/step.npy", "<u8", 1, sizeof(uint64_t), &step) == 0) d->gpu->step = step;
            if (npz_get(&r, "gpu/scheme.npy", "<i4", 1, sizeof(int), &scheme) == 0) ns_spectral_gpu_set_scheme(d, scheme);
            npz_get(&r, "fields/sfd_hat.npy", "<c16", nc, sizeof(fftw_complex), d->sfd_hat);
            /* the host arrays are the state: the next call uploads them */
            d->gpu->host_stale = 0;
            d->gpu->device_current = 0;
        }
    }
    free(r.buf);
    return st ? -1 : 0;
}
