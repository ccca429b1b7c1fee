// Device kernels of the GB300 pseudospectral step.
//
// Data layout in HBM (per instance, T = float or double, C = complex of T):
//   kept modes     kx columns i in [0, Kx), Kx = floor(2*nkx/3)+1, and ky rows
//                  |band| <= Kyh = floor(ny/3), stored as kept-row index
//                  jj in [0, Ky), Ky = 2*Kyh+1 (jj <= Kyh -> j = jj, else j = ny-Ky+jj)
//   state arrays   W0 (omega_hat at the step start), WS (stage state), ACC (RK
//                  accumulator), PSI0, SFD: C[Kxp][Ky]  (column i contiguous)
//   F[4]           y-transformed fields Psi, Psi_y, Omega, Omega_y: C[ny/B][Kxp][B]
//                  in blocks of B = 2^fLB rows (B = 1: row-contiguous, the
//                  generic kernels; B = ny: kx-column-contiguous)
//   G              x-transformed Jacobian: C[ny][Kxp] or C[Kxp][ny]
// Only the dealiased modes are ever stored or transformed on the hot path;
// the 2/3 rule is the layout (reference mask: spectral_initialization.c:46-49).
//
// One RK stage = one row kernel (x-pass over ny rows: 4 inverse half-length
// c2r, the Jacobian, one forward half-length r2c) + one column kernel (y-pass
// over the Kx kept columns: forward FFT of J, the RK stage algebra of
// spectral_time_integration.c:50-100 with hyperviscosity/SFD, forcing and the
// SFD post-step at stage 4, then the four inverse FFTs of the next stage).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "ns_fft.cuh"

namespace nsg {

struct Geo {
    int nx, ny, nkx, nky;
    int H;          // nx / 2: length of the packed real row transforms
    int Kx, Kxp;    // kept kx columns, padded to a multiple of CW
    int Kyh, Ky;    // kept |ky band| bound and kept row count
    int logny, logH;
    double Lx, Ly;
    int CW;         // columns per column-kernel CTA
    int RPC;        // rows per row-kernel CTA
    int fLB;        // F stored in blocks of 2^fLB rows: [ny >> fLB][Kxp][1 << fLB]
    int fTG;        // G stored kx-column-contiguous
    // mixed-radix transforms (lengths that are not powers of two; the stage
    // bodies instantiated with E = 0): radix lists of the row (length H) and
    // column (length ny) transforms, their pass counts and threads per sequence.
    // oddx: nx is odd, so the row transform is the full complex length nx
    // (H = nx) with Hermitian-extended input instead of the half-length packing.
    unsigned long long rxa, rxb, rya, ryb;
    int nrx, nry, TTr, TTc, oddx;
    // fields in parallel: the row pass gives each row
    // one group of transform threads per field (fpr), the column pass gives each
    // column block four groups, one per inverse-transformed field (fpc), so that
    // a small grid's transforms run side by side instead of one after another
    int fpr, fpc;
};

__host__ __device__ constexpr int clog2(int n) { return n <= 1 ? 0 : 1 + clog2(n / 2); }

// The size fields of a square N x N grid (N a power of two, generic stage bodies)
// as compile-time constants; the tiling fields (CW, RPC, Kxp, fpr, fpc) stay as
// stored.  Inlined into the stage bodies it turns their loop bounds, divisions and
// index arithmetic into constants.  Used only for a geometry whose stored values
// equal these (fold_sizes_match), so the arithmetic is unchanged.
template <int N> __host__ __device__ __forceinline__ void fold_sizes(Geo& g) {
    constexpr int nkx = N / 2 + 1, Kx = (2 * nkx) / 3 + 1, Kyh = (2 * N) / 6;
    g.nx = N;
    g.ny = N;
    g.nkx = nkx;
    g.nky = N;
    g.H = N / 2;
    g.Kx = Kx;
    g.Kyh = Kyh;
    g.Ky = 2 * Kyh + 1;
    g.logny = clog2(N);
    g.logH = clog2(N / 2);
    g.fLB = 0;
    g.fTG = 0;
    g.oddx = 0;
}
template <int N> inline bool fold_sizes_match(const Geo& g) {
    Geo f = g;
    fold_sizes<N>(f);
    return f.nx == g.nx && f.ny == g.ny && f.nkx == g.nkx && f.nky == g.nky && f.H == g.H && f.Kx == g.Kx &&
           f.Kyh == g.Kyh && f.Ky == g.Ky && f.logny == g.logny && f.logH == g.logH && f.fLB == g.fLB &&
           f.fTG == g.fTG && f.oddx == g.oddx;
}

// one transform of a row or column buffer b: the power-of-two engine for E > 0,
// the mixed-radix engine (through the scratch sequence sc) for E == 0; sy is
// the pass barrier (fft_sync)
template <int E, bool INV, typename C>
__device__ __forceinline__ void fft_any(C* b, C* sc, int L, int logL, unsigned long long ra, unsigned long long rb, int np,
                                        int t, int TT, const C* __restrict__ tw, int sy) {
    if constexpr (E == 0) fft_smem_mr<INV>(b, sc, L, ra, rb, np, t, TT, tw, sy);
    else fft_smem<E, INV>(b, L, logL, t, TT, tw, sy);
}

// pass barrier of a transform of TT threads: one warp when TT divides the warp
// size (every transform of the CTA then lies inside a warp), else named barrier
// id over the group's n threads when the CTA runs groups independently (id > 0),
// else the CTA
__device__ __forceinline__ int sync_mode(int TT, int id, int n) {
    if (TT <= 32 && (32 % TT) == 0) return 1;
    return id > 0 ? ((id << 16) | n) : 0;
}

// element (row y, kept column c) of an F buffer / of the G buffer
__device__ __forceinline__ size_t fidx(const Geo& g, int y, int c) {
    return (((size_t)(y >> g.fLB) * g.Kxp + c) << g.fLB) + (y & ((1 << g.fLB) - 1));
}
__device__ __forceinline__ size_t gidx(const Geo& g, int y, int c) {
    return g.fTG ? (size_t)c * g.ny + y : (size_t)y * g.Kxp + c;
}

// kx^2 + ky^2 rounded as the reference's host code does (no fused multiply-add)
__device__ __forceinline__ double k2sum(double kx, double ky) { return __dadd_rn(__dmul_rn(kx, kx), __dmul_rn(ky, ky)); }
__device__ __forceinline__ float k2sum(float kx, float ky) { return kx * kx + ky * ky; }

__device__ __forceinline__ int kept_j(const Geo& g, int jj) { return jj <= g.Kyh ? jj : g.ny - g.Ky + jj; }
__device__ __forceinline__ int kept_jj(const Geo& g, int j) {
    if (j <= g.Kyh) return j;
    if (j >= g.ny - g.Kyh) return j - (g.ny - g.Ky);
    return -1;
}

// Device scalars shared by the kernels of one instance.
struct DevScalars {
    double t;
    double dt;
    double dt_fixed;
    unsigned long long maxvel2;    // bit pattern of max(u^2+v^2) (non-negative double)
    unsigned long long step_next;  // forcing counter of the next step
    unsigned long long step_cur;   // forcing counter of the running step
    unsigned long long kmax_bits;  // bit pattern of max |k| (hyperviscosity setup)
    unsigned long long aux_max;    // bit pattern of a max reduction of the host-array API
    int flag;                      // outside-mode presence / non-finite detection
    int pad;
    unsigned long long fsub;       // forcing draws per step (counter advance per step; 0 means 1)
};

struct StepParams {
    double inv_re, Re, cfl, dxmin, scale;
    int adaptive, hv, sfd, forcing;
    int ifrk;  // 1: integrating-factor RK4 stage algebra
    int fsub;  // forcing draws summed per step (>= 1)
    double sfd_tau;
    double f_kmin, f_kmax, f_sigma;
    unsigned long long f_seed;
};

// ------------------------------------------------------------ Philox4x64-10
// Salmon, Moraes, Dror, Shaw, "Parallel Random Numbers: As Easy as 1, 2, 3" (SC'11)
__device__ __forceinline__ void philox4x64(unsigned long long c[4], unsigned long long k0, unsigned long long k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r > 0) {
            k0 += 0x9E3779B97F4A7C15ULL;
            k1 += 0xBB67AE8584CAA73BULL;
        }
        const unsigned long long m0 = 0xD2E7470EE14C6C93ULL, m1 = 0xCA5A826395121157ULL;
        const unsigned long long hi0 = __umul64hi(m0, c[0]), lo0 = m0 * c[0];
        const unsigned long long hi1 = __umul64hi(m1, c[2]), lo1 = m1 * c[2];
        const unsigned long long n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
        c[0] = n0; c[1] = lo1; c[2] = n2; c[3] = lo0;
    }
}
__device__ __forceinline__ double u53(unsigned long long b) { return (double)(b >> 11) * (1.0 / 9007199254740992.0); }

#define NSG_TAG_IC 0x49430000ULL
#define NSG_TAG_FORCE 0x464f5243ULL

// Forcing noise of the kept mode (kx index i, row j): the sum over s < M of
// xi(base + s), xi = (g1 + i g2) / sqrt 2 from Box-Muller on Philox4x64-10 keyed
// by the seed with counter (mode id, base + s, TAG, 0).  The mode id is
// (signed ky) << 32 | kx, so a physical mode draws the same noise on every grid;
// kx = 0 rows with ky < 0 take the conjugate of the ky > 0 row (Hermitian).
__device__ __forceinline__ double2 forcing_xi_sum(int i, int j, int ny, unsigned long long base, int M,
                                                  unsigned long long seed) {
    int ky = (j <= ny / 2) ? j : j - ny;
    int flip = 0;
    if (i == 0 && ky < 0) { ky = -ky; flip = 1; }
    const unsigned long long id = ((unsigned long long)(unsigned int)ky << 32) | (unsigned int)i;
    double sx = 0.0, sy = 0.0;
    for (int s = 0; s < M; ++s) {
        unsigned long long ctr[4] = {id, base + (unsigned long long)s, NSG_TAG_FORCE, 0ULL};
        philox4x64(ctr, seed, 0ULL);
        const double u1 = fmax(u53(ctr[0]), 2.2250738585072014e-308);
        const double u2 = u53(ctr[1]);
        const double rad = sqrt(-2.0 * log(u1)) * 0.70710678118654752440;
        double sn, cs;
        sincos(2.0 * 3.141592653589793 * u2, &sn, &cs);
        sx = __dadd_rn(sx, __dmul_rn(rad, cs));
        sy = __dadd_rn(sy, __dmul_rn(rad, sn));
    }
    return make_double2(sx, flip ? -sy : sy);
}

// One term of the noise table of a step: draw s of mode (kx index i, ky) with
// counter base + s, as forcing_xi_sum forms it (the conjugate row of kx = 0,
// ky < 0 negated); zero outside the shell kmin <= |k| <= kmax.
__device__ __forceinline__ double2 forcing_noise_term(int i, int ky, int s, unsigned long long base,
                                                      unsigned long long seed, double Lx, double Ly, double kmin,
                                                      double kmax) {
    const double kxd = 2.0 * 3.141592653589793 * i / Lx;
    const double kyd = 2.0 * 3.141592653589793 * ky / Ly;
    const double k2d = kxd * kxd + kyd * kyd;
    const double km = sqrt(k2d);
    if (!(k2d > 1e-12 && km >= kmin && km <= kmax)) return make_double2(0.0, 0.0);
    int flip = 0;
    if (i == 0 && ky < 0) { ky = -ky; flip = 1; }
    const unsigned long long id = ((unsigned long long)(unsigned int)ky << 32) | (unsigned int)i;
    unsigned long long ctr[4] = {id, base + (unsigned long long)s, NSG_TAG_FORCE, 0ULL};
    philox4x64(ctr, seed, 0ULL);
    const double u1 = fmax(u53(ctr[0]), 2.2250738585072014e-308);
    const double u2 = u53(ctr[1]);
    const double rad = sqrt(-2.0 * log(u1)) * 0.70710678118654752440;
    double sn, cs;
    sincos(2.0 * 3.141592653589793 * u2, &sn, &cs);
    return make_double2(__dmul_rn(rad, cs), flip ? -__dmul_rn(rad, sn) : __dmul_rn(rad, sn));
}

// ---------------------------------------------------------------- reductions
struct DD { double s, c; };  // Neumaier pair: value = s + c
__device__ __forceinline__ void dd_add(DD& a, double x) {
    const double t = a.s + x;
    if (fabs(a.s) >= fabs(x)) a.c += (a.s - t) + x;
    else a.c += (x - t) + a.s;
    a.s = t;
}
__device__ __forceinline__ DD dd_merge(DD a, DD b) {
    DD r = a;
    dd_add(r, b.s);
    r.c += b.c;
    return r;
}
// block-wide merge; returns the total in thread 0
static __device__ DD block_dd(DD v) {
    __shared__ double ss[32], sc[32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        DD w;
        w.s = __shfl_xor_sync(0xffffffffu, v.s, o);
        w.c = __shfl_xor_sync(0xffffffffu, v.c, o);
        v = dd_merge(v, w);
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    __syncthreads();
    if (lane == 0) { ss[wid] = v.s; sc[wid] = v.c; }
    __syncthreads();
    if (wid == 0) {
        DD w;
        w.s = lane < nw ? ss[lane] : 0.0;
        w.c = lane < nw ? sc[lane] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            DD u;
            u.s = __shfl_xor_sync(0xffffffffu, w.s, o);
            u.c = __shfl_xor_sync(0xffffffffu, w.c, o);
            w = dd_merge(w, u);
        }
        v = w;
    }
    return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// =============================================================== row kernel
enum { ROW_STAGE = 0, ROW_DUMP = 1, ROW_UVW = 2, ROW_INV1 = 3, ROW_FWD1 = 4 };
// thread groups per row of the row pass (nf = fields inverse-transformed per row)
__host__ __device__ inline int row_groups(int fpr, int E, int nf) { return (fpr && nf > 1) ? nf : 1; }

template <typename T> struct RowArgs {
    typedef typename CT<T>::C C;
    const C* F[4];            // field inputs C[ny][Kxp]
    int dx[4];                // 1: multiply by i kx before the transform
    C* G;                     // C[ny][Kxp] output (ROW_STAGE, ROW_DUMP, ROW_FWD1)
    const double* in_real;    // ROW_FWD1 input double[ny][nx]
    const float* in_f32;      // ROW_FWD1: float[ny][nx] input instead of in_real (when set)
    float* out_f32;           // ROW_INV1: float[ny][nx] output instead of out_real[0] (when set)
    double* out_real[5];      // physical outputs double[ny][nx]
    const T* kxv;             // kx of kept columns
    const C* twr;             // exp(-2 pi i t/H), t < H
    const C* twh;             // exp(-2 pi i k/nx), k < H
    DevScalars* ds;
    int cfl;                  // reduce max(u^2+v^2) into ds->maxvel2
    int marker;               // 1: stage 1 (advance step counters), 2: stage 2 (reset maxvel2)
};

template <int MODE> struct RowNF { static const int v = (MODE == ROW_STAGE || MODE == ROW_DUMP) ? 4 : (MODE == ROW_UVW ? 3 : 1); };

// grid = ny / RPC, block = RPC * P * TT with TT = H / E (E > 0) or g.TTr (E = 0)
// and P = row_groups(g.fpr, E, NF) thread groups per row, dynamic smem = NF * RPC *
// spad_len(H) * sizeof(C), plus P * RPC * spad_len(H) * sizeof(C) of mixed-radix
// scratch (one sequence per group) when E = 0
// body of the row pass for row block bx (rows bx*RPC .. bx*RPC + RPC - 1); the
// block must have exactly RPC * P * TT threads.  With P > 1 (fields in parallel;
// TT a multiple of 32 or a divisor of 32, RPC * P <= 15 when TT > 32) group f of a
// row loads, unpacks and inverse-transforms field f, the row's threads form the
// products together, and group 0 makes the forward transform (every group, on its
// own copy, when TT < 32).
// FG = false compiles the field-group logic out (callers that always run one
// group per row, such as the persistent ensemble kernel)
template <typename T, int E, int MODE, bool FG = true>
__device__ __forceinline__ void row_body(const Geo& g, const RowArgs<T>& a, const int bx) {
    typedef typename CT<T>::C C;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C* sm = reinterpret_cast<C*>(smem_raw);
    constexpr int NF = RowNF<MODE>::v;
    const int H = g.H, TT = (E == 0) ? g.TTr : H / E, LP = spad_len(H);
    const int P = FG ? row_groups(g.fpr, E, NF) : 1, TQ = P * TT;
    const int r = threadIdx.x / TQ, q = threadIdx.x - r * TQ;
    const int fg = q / TT, t = q - fg * TT;
    const int sy = sync_mode(TT, P > 1 ? 1 + r * P + fg : 0, TT);
    // groups narrower than a warp all transform a copy of the product (their warp
    // barriers stay uniform) and share its stores; wider groups leave both to group 0
    const bool allfwd = P > 1 && TT < 32;
    const int y = bx * g.RPC + r;
    const int nx = g.nx, Kx = g.Kx;
    C* scr = sm + (NF * g.RPC + r * P + fg) * LP;  // mixed-radix scratch of this row and group (E = 0 only)
    const bool oddx = (E == 0) && g.oddx;

    if (MODE == ROW_STAGE && bx == 0 && threadIdx.x == 0) {
        if (a.marker == 1) {
            a.ds->step_cur = a.ds->step_next;
            a.ds->step_next = a.ds->step_next + (a.ds->fsub ? a.ds->fsub : 1ULL);
        } else if (a.marker == 2) {
            a.ds->maxvel2 = 0ULL;
        }
    }

    if constexpr (MODE == ROW_FWD1) {
        C* b = sm + r * LP;
        const double* src = a.in_real + (size_t)y * nx;
        const float* srcf = a.in_f32 ? a.in_f32 + (size_t)y * nx : nullptr;
        for (int m = t; m < H; m += TT) {
            C z;
            if (oddx) {
                z.x = srcf ? (T)srcf[m] : (T)src[m];
                z.y = (T)0;
            } else if (srcf) {
                z.x = (T)srcf[2 * m];
                z.y = (T)srcf[2 * m + 1];
            } else {
                z.x = (T)src[2 * m];
                z.y = (T)src[2 * m + 1];
            }
            b[spad(m)] = z;
        }
        __syncthreads();
        fft_any<E, false>(b, scr, H, g.logH, g.rxa, g.rxb, g.nrx, t, TT, a.twr, sy);
    } else {
        // half spectra X_f[k], k < Kx (zero above); odd nx: the full Hermitian
        // spectrum X[k], X[nx - k] = conj X[k], of the length-nx transform
#pragma unroll
        for (int f = 0; f < NF; ++f) {
            if (P > 1 && f != fg) continue;
            C* b = sm + (f * g.RPC + r) * LP;
            const C* src = a.F[f];
            if constexpr (E > 0) {
                // exactly E elements a thread (H = E TT): all loads in flight before
                // the stores (the fields are L2 round trips on small grids)
                C xv[E];
#pragma unroll
                for (int u = 0; u < E; ++u) {
                    const int k = t + u * TT;
                    C x = cmake<C>(0.0, 0.0);
                    if (k < Kx) {
                        x = src[fidx(g, y, k)];
                        if (a.dx[f]) {
                            const T kx = a.kxv[k];
                            C d;
                            d.x = -kx * x.y;
                            d.y = kx * x.x;
                            x = d;
                        }
                    }
                    xv[u] = x;
                }
#pragma unroll
                for (int u = 0; u < E; ++u) b[spad(t + u * TT)] = xv[u];
            } else {
                for (int k = t; k < H; k += TT) {
                    const bool mirror = oddx && k >= g.nkx;
                    const int kk = mirror ? nx - k : k;
                    C x = cmake<C>(0.0, 0.0);
                    if (kk < Kx) {
                        x = src[fidx(g, y, kk)];
                        if (a.dx[f]) {
                            const T kx = a.kxv[kk];
                            C d;
                            d.x = -kx * x.y;
                            d.y = kx * x.x;
                            x = d;
                        }
                        if (mirror) x.y = -x.y;
                    }
                    b[spad(k)] = x;
                }
            }
        }
        __syncthreads();
        // pack for the half-length inverse: z[m] = x[2m] + i x[2m+1] has spectrum
        // Z[k] = (X[k] + conj X[H-k]) + i exp(+2 pi i k/nx) (X[k] - conj X[H-k]);
        // the imaginary parts of X[0] and the Nyquist bin (zero here) are ignored.
#pragma unroll
        for (int f = 0; f < NF && !oddx; ++f) {
            if (P > 1 && f != fg) continue;
            C* b = sm + (f * g.RPC + r) * LP;
            for (int k = t; 2 * k <= H; k += TT) {
                if (k == 0) {
                    const C x0 = b[spad(0)];
                    b[spad(0)] = cmake<C>(x0.x, x0.x);
                    continue;
                }
                const C xa = b[spad(k)], xb = b[spad(H - k)];
                const C e = cconj(__ldg(&a.twh[k]));  // exp(+2 pi i k/nx)
                const C A = cadd(xa, cconj(xb));
                const C D = cmul(csub(xa, cconj(xb)), e);
                b[spad(k)] = cmake<C>(A.x - D.y, A.y + D.x);
                if (2 * k != H) {
                    C e2;  // exp(+2 pi i (H-k)/nx) = -conj(e)
                    e2.x = -e.x;
                    e2.y = e.y;
                    const C A2 = cadd(xb, cconj(xa));
                    const C D2 = cmul(csub(xb, cconj(xa)), e2);
                    b[spad(H - k)] = cmake<C>(A2.x - D2.y, A2.y + D2.x);
                }
            }
        }
        if (!oddx) __syncthreads();
        if (P > 1) {
            // one call site for every group: groups that share a warp (TT < 32) meet
            // the same warp barriers in the same order
            fft_any<E, true>(sm + (fg * g.RPC + r) * LP, scr, H, g.logH, g.rxa, g.rxb, g.nrx, t, TT, a.twr, sy);
            __syncthreads();  // the loops below read every field of the row
        } else {
#pragma unroll
            for (int f = 0; f < NF; ++f)
                fft_any<E, true>(sm + (f * g.RPC + r) * LP, scr, H, g.logH, g.rxa, g.rxb, g.nrx, t, TT, a.twr, sy);
        }

        if constexpr (MODE == ROW_STAGE || MODE == ROW_DUMP) {
            C* b0 = sm + (0 * g.RPC + r) * LP;
            C* b1 = sm + (1 * g.RPC + r) * LP;
            C* b2 = sm + (2 * g.RPC + r) * LP;
            C* b3 = sm + (3 * g.RPC + r) * LP;
            T vmax2 = (T)0;
            if (oddx) {
                // one grid point per element (the real parts of the length-nx inverse)
                for (int m = q; m < H; m += TQ) {
                    const T p0 = b0[spad(m)].x, p1 = b1[spad(m)].x, p2 = b2[spad(m)].x, p3 = b3[spad(m)].x;
                    const T jv = p0 * p3 - p1 * p2;
                    if (a.cfl) vmax2 = fmax(vmax2, p0 * p0 + p1 * p1);
                    if constexpr (MODE == ROW_DUMP) {
                        const size_t o = (size_t)y * nx + m;
                        a.out_real[0][o] = p0;
                        a.out_real[1][o] = p1;
                        a.out_real[2][o] = p2;
                        a.out_real[3][o] = p3;
                        a.out_real[4][o] = jv;
                    }
                    const C pj = cmake<C>(jv, 0.0);
                    b0[spad(m)] = pj;
                    if (allfwd) { b1[spad(m)] = pj; b2[spad(m)] = pj; b3[spad(m)] = pj; }
                }
            }
            for (int m = oddx ? H : q; m < H; m += TQ) {
                const C z0 = b0[spad(m)], z1 = b1[spad(m)], z2 = b2[spad(m)], z3 = b3[spad(m)];
                // z0 = psi_x, z1 = psi_y, z2 = omega_x, z3 = omega_y at points 2m (re) and 2m+1 (im)
                const T je = z0.x * z3.x - z1.x * z2.x;
                const T jo = z0.y * z3.y - z1.y * z2.y;
                if (a.cfl) {
                    const T ve = z0.x * z0.x + z1.x * z1.x, vo = z0.y * z0.y + z1.y * z1.y;
                    vmax2 = fmax(vmax2, fmax(ve, vo));
                }
                if constexpr (MODE == ROW_DUMP) {
                    const size_t o = (size_t)y * nx + 2 * m;
                    a.out_real[0][o] = z0.x; a.out_real[0][o + 1] = z0.y;
                    a.out_real[1][o] = z1.x; a.out_real[1][o + 1] = z1.y;
                    a.out_real[2][o] = z2.x; a.out_real[2][o + 1] = z2.y;
                    a.out_real[3][o] = z3.x; a.out_real[3][o + 1] = z3.y;
                    a.out_real[4][o] = je;   a.out_real[4][o + 1] = jo;
                }
                const C pj = cmake<C>(je, jo);
                b0[spad(m)] = pj;
                if (allfwd) { b1[spad(m)] = pj; b2[spad(m)] = pj; b3[spad(m)] = pj; }
            }
            if (a.cfl) {
                double v = (double)vmax2;
                if ((blockDim.x & 31) == 0) {  // whole warps: reduce before the atomic
                    v = warp_max(v);
                    if ((threadIdx.x & 31) == 0) atomicMax(&a.ds->maxvel2, (unsigned long long)__double_as_longlong(v));
                } else {
                    atomicMax(&a.ds->maxvel2, (unsigned long long)__double_as_longlong(v));
                }
            }
            __syncthreads();
            if (P > 1 && fg != 0 && !allfwd) return;  // group 0 transforms the product and stores it
            fft_any<E, false>(sm + (fg * g.RPC + r) * LP, scr, H, g.logH, g.rxa, g.rxb, g.nrx, t, TT, a.twr, sy);
        } else {
            const C* b0 = sm + (0 * g.RPC + r) * LP;
            if (oddx) {
                for (int m = q; m < H; m += TQ) {
                    const size_t o = (size_t)y * nx + m;
                    const T p0 = b0[spad(m)].x;
                    if constexpr (MODE == ROW_UVW) {
                        a.out_real[0][o] = p0;                                 // u = psi_y
                        a.out_real[1][o] = -sm[(1 * g.RPC + r) * LP + spad(m)].x;  // v = -psi_x
                        a.out_real[2][o] = sm[(2 * g.RPC + r) * LP + spad(m)].x;   // omega
                    } else if (a.out_f32) {
                        a.out_f32[o] = (float)p0;
                    } else {
                        a.out_real[0][o] = p0;
                    }
                }
                return;
            }
            for (int m = q; m < H; m += TQ) {
                const size_t o = (size_t)y * nx + 2 * m;
                const C z0 = b0[spad(m)];
                if constexpr (MODE == ROW_UVW) {
                    const C z1 = sm[(1 * g.RPC + r) * LP + spad(m)];
                    const C z2 = sm[(2 * g.RPC + r) * LP + spad(m)];
                    a.out_real[0][o] = z0.x; a.out_real[0][o + 1] = z0.y;   // u = psi_y
                    a.out_real[1][o] = -z1.x; a.out_real[1][o + 1] = -z1.y; // v = -psi_x
                    a.out_real[2][o] = z2.x; a.out_real[2][o + 1] = z2.y;   // omega
                } else if (a.out_f32) {
                    a.out_f32[o] = (float)z0.x;
                    a.out_f32[o + 1] = (float)z0.y;
                } else {
                    a.out_real[0][o] = z0.x;
                    a.out_real[0][o + 1] = z0.y;
                }
            }
            return;
        }
    }
    // forward post-processing: X[k] = E[k] + exp(-2 pi i k/nx) O[k],
    // E = (W[k] + conj W[H-k])/2, O = (W[k] - conj W[H-k])/(2i), for the kept k < Kx
    {
        // this group's transformed row; with allfwd every group holds the same
        // transform and stores its share k = q, q + P TT, ...
        const C* b0 = sm + (fg * g.RPC + r) * LP;
        const int k0 = allfwd ? q : t, ks = allfwd ? TQ : TT;
        C* dst = a.G;
        if (oddx) {  // the length-nx transform of the real row: X[k] directly
            for (int k = k0; k < Kx; k += ks) dst[gidx(g, y, k)] = b0[spad(k)];
            return;
        }
        const T half = (T)0.5;
        for (int k = k0; k < Kx; k += ks) {
            const C wa = b0[spad(k)];
            const C wb = b0[spad(k == 0 ? 0 : H - k)];
            C ev, od;
            ev.x = half * (wa.x + wb.x);
            ev.y = half * (wa.y - wb.y);
            od.x = half * (wa.y + wb.y);
            od.y = -half * (wa.x - wb.x);
            dst[gidx(g, y, k)] = cadd(ev, cmul(od, __ldg(&a.twh[k])));
        }
    }
}

// N > 0: the grid's size fields folded to constants (fold_sizes<N>)
template <typename T, int E, int MODE, int N = 0>
__global__ void __launch_bounds__(256) k_row(Geo g, RowArgs<T> a) {
    if constexpr (N > 0) {
        Geo f = g;
        fold_sizes<N>(f);
        row_body<T, E, MODE>(f, a, blockIdx.x);
    } else {
        row_body<T, E, MODE>(g, a, blockIdx.x);
    }
}

// ============================================================ column kernel
// COL_ADD: forward y-transforms of the G rows (a real field's x-transform),
// W0 += (scaled) spectrum on the kept modes, then the stage-1 fields of the new
// W0 (as COL_PROLOGUE with psi from W0): a correction added and the fields ready
// in one pass
enum { COL_STAGE = 0, COL_PROLOGUE = 1, COL_INV1 = 2, COL_FWD_EXPORT = 3, COL_NL_EXPORT = 4, COL_ADD = 5 };
// thread groups per column block of the column pass (the modes with several
// inverse-transformed fields)
__host__ __device__ inline int col_groups(int fpc, int E, int mode) {
    return (fpc && (mode == COL_STAGE || mode == COL_PROLOGUE || mode == COL_ADD)) ? 4 : 1;
}

template <typename T> struct ColArgs {
    typedef typename CT<T>::C C;
    const C* G;                 // C[ny][Kxp]
    C* F[4];                    // C[ny][Kxp]
    C* W0;                      // kept state at the step start (or the prologue input)
    C* WS;                      // stage state
    C* ACC;                     // RK accumulator
    const C* PSI0;              // stored psi_hat (prologue)
    C* SFD;                     // SFD filtered state
    const T* hvw;               // hyperviscosity weight per kept mode
    const T* sfdw;              // sfd_strength * ramp per kept mode
    const T* kxv;
    const T* kyv;
    const C* twc;               // exp(-2 pi i t/ny), t < ny
    DevScalars* ds;
    StepParams sp;
    double2* out_spec;          // FP64 export [nky][nkx]
    double out_scale;           // export scale (1/(nx ny) forward, -1/(nx ny) nonlinear)
    int psi_from_w;             // prologue: Psi = -W0/k^2 instead of PSI0
    int nfields;                // prologue: number of fields (4 for a stage, 3 = Psi,Psi_y,Omega)
    // this step's forcing noise summed per mode (k_forcing_noise, k_forcing_sum), zero
    // outside the forcing shell, or null: entry e = i (2 fkyr + 1) + ky + fkyr for kx
    // index i <= fkxr and |ky| <= fkyr
    const double2* fsum;
    int fkxr, fkyr;
};

// x / k2 for the Poisson solve: IEEE division in FP64 (as the reference), the
// fast reciprocal-based divide in the FP32 bulk path
__device__ __forceinline__ double kdiv(double x, double k2) { return x / k2; }
__device__ __forceinline__ float kdiv(float x, float k2) { return __fdividef(x, k2); }

template <typename T, typename C>
__device__ __forceinline__ C field_value(int f, C w, T kx, T ky) {
    // f: 0 Psi = -w/k^2, 1 Psi_y = i ky Psi, 2 Omega = w, 3 Omega_y = i ky w (spectral_core.c:17-31)
    C v = w;
    if (f < 2) {
        const T k2 = k2sum(kx, ky);
        if (k2 > (T)1e-12) { v.x = -kdiv(w.x, k2); v.y = -kdiv(w.y, k2); }
        else { v.x = (T)0; v.y = (T)0; }
    }
    if (f == 1 || f == 3) {
        C d;
        d.x = -ky * v.y;
        d.y = ky * v.x;
        v = d;
    }
    return v;
}

// FP64 shell test of mode (i, j): kmin <= |k| <= kmax, |k| > 0 (as the reference's k2)
__device__ __forceinline__ bool forcing_in_shell(double Lx, double Ly, int ny, int i, int j, double kmin, double kmax) {
    const double kxd = 2.0 * 3.141592653589793 * i / Lx;
    const double kyd = (j <= ny / 2) ? 2.0 * 3.141592653589793 * j / Ly : 2.0 * 3.141592653589793 * (j - ny) / Ly;
    const double k2d = kxd * kxd + kyd * kyd;
    const double km = sqrt(k2d);
    return k2d > 1e-12 && km >= kmin && km <= kmax;
}

// white-in-time forcing increment of one kept mode: amp times the mode's noise
// (the sum over this step's draws) when kmin <= |k| <= kmax.  With a table the
// draws and their per-mode sums were made for the step by k_forcing_noise and
// k_forcing_sum (beside the step's first three stages), zero outside the shell;
// otherwise they are drawn here (forcing_xi_sum).  The geometry comes by value
// (Lx, Ly, ny): a caller's Geo never escapes into this out-of-line call, so its
// fields stay foldable constants where they are.
static __device__ __noinline__ double2 forcing_increment(double Lx, double Ly, int ny, int i, int j,
                                                         unsigned long long step, int M, unsigned long long seed,
                                                         double kmin, double kmax, double amp, const double2* fsum,
                                                         int fkxr, int fkyr) {
    double2 xi;
    const int ky = (j <= ny / 2) ? j : j - ny;
    if (fsum && i <= fkxr && ky >= -fkyr && ky <= fkyr) {
        xi = fsum[(size_t)i * (2 * fkyr + 1) + (ky + fkyr)];
        if (xi.x == 0.0 && xi.y == 0.0) return make_double2(0.0, 0.0);  // outside the shell
    } else {
        if (!forcing_in_shell(Lx, Ly, ny, i, j, kmin, kmax)) return make_double2(0.0, 0.0);
        xi = forcing_xi_sum(i, j, ny, step, M, seed);
    }
    return make_double2(amp * xi.x, amp * xi.y);
}

// constants of one RK4 stage (spectral_time_integration.c:50-100)
template <typename T> struct StageCoef {
    T inv_re, sc, ch, cf, c6;  // 1/Re, N scale, dt/2, dt, dt/6
    int hv, sfd;
};
template <typename T> __device__ __forceinline__ StageCoef<T> stage_coef(const StepParams& sp, double dt) {
    StageCoef<T> q;
    q.inv_re = (T)sp.inv_re;
    q.sc = (T)sp.scale;
    q.ch = (T)(0.5 * dt);
    q.cf = (T)dt;
    q.c6 = (T)(dt / 6.0);
    q.hv = sp.hv;
    q.sfd = sp.sfd;
    return q;
}

// RK stage STAGE on one kept mode (spectral_time_integration.c:50-100 with
// hyperviscosity.c:104-150): jh = r2c(J) of the mode (N = -sc jh), w0 = omega_hat
// at the step start, ws = stage state, acc0 = accumulator (stages 2-4), hw the
// hyperviscosity weight (0 when off), sw / fb the SFD ramp and filtered state
// (read only when SFD is on), k2 = |k|^2.  Stores ACC and WS at s for stages 1-3
// and returns the next stage state (stage 4: omega_hat^{n+1} before forcing).
// IFRK: integrating-factor RK4, explicit part N - SFD relaxation, exact decay by
// E1 = exp(-(k^2/Re + w) dt/2), E2 = E1^2.
template <typename T, int STAGE, bool IFRK, typename C>
__device__ __forceinline__ C rk_stage_mode(const StageCoef<T>& q, C jh, C w0, C ws, C acc0, T hw, T sw, C fb, T k2,
                                           C* __restrict__ ACC, C* __restrict__ WS, size_t s) {
    C wn;
    if (IFRK) {
        C k;
        k.x = -(jh.x * q.sc);
        k.y = -(jh.y * q.sc);
        if (q.sfd && sw > (T)0) {
            k.x -= sw * (ws.x - fb.x);
            k.y -= sw * (ws.y - fb.y);
        }
        const T lam = k2 * q.inv_re + hw;
        const T e1 = exp(-lam * q.ch), e2 = e1 * e1;
        if (STAGE == 1) {
            ACC[s] = cmake<C>(e2 * k.x, e2 * k.y);
            wn.x = e1 * (w0.x + q.ch * k.x); wn.y = e1 * (w0.y + q.ch * k.y);
            WS[s] = wn;
        } else if (STAGE == 2 || STAGE == 3) {
            C acc = acc0;
            acc.x = acc.x + (T)2 * (e1 * k.x);
            acc.y = acc.y + (T)2 * (e1 * k.y);
            ACC[s] = acc;
            if (STAGE == 2) { wn.x = e1 * w0.x + q.ch * k.x; wn.y = e1 * w0.y + q.ch * k.y; }
            else { wn.x = e2 * w0.x + q.cf * (e1 * k.x); wn.y = e2 * w0.y + q.cf * (e1 * k.y); }
            WS[s] = wn;
        } else {
            wn.x = e2 * w0.x + q.c6 * (acc0.x + k.x);
            wn.y = e2 * w0.y + q.c6 * (acc0.y + k.y);
        }
    } else {
        C k;  // k = N - k^2 omega / Re - damping (spectral_time_integration.c:50-54)
        k.x = -(jh.x * q.sc) - k2 * ws.x * q.inv_re;
        k.y = -(jh.y * q.sc) - k2 * ws.y * q.inv_re;
        if (q.hv || q.sfd) {
            C damp = cmake<C>(0.0, 0.0);
            if (q.hv) { damp.x += hw * ws.x; damp.y += hw * ws.y; }
            if (q.sfd && sw > (T)0) {
                damp.x += sw * (ws.x - fb.x);
                damp.y += sw * (ws.y - fb.y);
            }
            k.x -= damp.x;
            k.y -= damp.y;
        }
        if (STAGE == 1) {
            ACC[s] = k;
            wn.x = w0.x + q.ch * k.x; wn.y = w0.y + q.ch * k.y;
            WS[s] = wn;
        } else if (STAGE == 2 || STAGE == 3) {
            C acc = acc0;
            acc.x = acc.x + (T)2 * k.x;
            acc.y = acc.y + (T)2 * k.y;
            ACC[s] = acc;
            const T cc = (STAGE == 2) ? q.ch : q.cf;
            wn.x = w0.x + cc * k.x; wn.y = w0.y + cc * k.y;
            WS[s] = wn;
        } else {
            wn.x = w0.x + q.c6 * (acc0.x + k.x);
            wn.y = w0.y + q.c6 * (acc0.y + k.y);
        }
    }
    return wn;
}

// stage-4 forcing increment and SFD post-step (hyperviscosity.c:152-178) of kept
// mode (i, j) at s: adds the forcing to wn when its |k| lies in the shell (an
// FP32/FP64 |k|^2 screen, margin far beyond rounding, before the exact FP64
// test), then relaxes the SFD filter toward it; sets forced when wn changed
template <typename T, typename C>
__device__ __forceinline__ C post_step_mode(const Geo& g, const ColArgs<T>& a, int i, int j, size_t s, C wn, T kx, T ky,
                                            double f_amp, double sfd_a, bool& forced) {
    forced = false;
    const T k2f = kx * kx + ky * ky;
    if (a.sp.forcing && (double)kx <= a.sp.f_kmax + 1e-9 && k2f >= (T)(a.sp.f_kmin * a.sp.f_kmin * (1.0 - 1e-3)) &&
        k2f <= (T)(a.sp.f_kmax * a.sp.f_kmax * (1.0 + 1e-3))) {
        // modes of the step's table read their summed noise inline (no out-of-line
        // call in the register-heavy stage kernels); the others go through
        // forcing_increment, which makes the same test and product
        const int kyi = (j <= g.ny / 2) ? j : j - g.ny;
        double2 df;
        if (a.fsum && i <= a.fkxr && kyi >= -a.fkyr && kyi <= a.fkyr) {
            const double2 xi = a.fsum[(size_t)i * (2 * a.fkyr + 1) + (kyi + a.fkyr)];
            df = (xi.x == 0.0 && xi.y == 0.0) ? make_double2(0.0, 0.0) : make_double2(f_amp * xi.x, f_amp * xi.y);
        } else {
            df = forcing_increment(g.Lx, g.Ly, g.ny, i, j, a.ds->step_cur, a.sp.fsub, a.sp.f_seed, a.sp.f_kmin,
                                   a.sp.f_kmax, f_amp, a.fsum, a.fkxr, a.fkyr);
        }
        if (df.x != 0.0 || df.y != 0.0) {
            wn.x = (T)((double)wn.x + df.x);
            wn.y = (T)((double)wn.y + df.y);
            forced = true;
        }
    }
    if (a.sp.sfd) {
        C fb = a.SFD[s];
        const T al = (T)sfd_a, om = (T)(1.0 - sfd_a);
        fb.x = om * fb.x + al * wn.x;
        fb.y = om * fb.y + al * wn.y;
        a.SFD[s] = fb;
    }
    return wn;
}

// grid = Kxp / CW, block = P * CW * TC with TC = ny / E (E > 0) or g.TTc (E = 0)
// and P = col_groups(g.fpc, E, MODE) thread groups, dynamic smem = P * CW *
// spad_len(ny) * sizeof(C), twice that when E = 0 (the mixed-radix scratch)
// body of the column pass for column block bx (kept columns bx*CW .. bx*CW + CW - 1);
// the block must have exactly P * CW * TC threads.  With P > 1 (fields in
// parallel; CW * TC a multiple of 32) group 0 makes the forward transforms, the
// block applies the stage together, and group f inverse-transforms and stores
// the fields f, f + P, ... in its own buffers, synchronised by named barrier 1 + f.
template <typename T, int E, int MODE, int STAGE, bool FG = true>
__device__ __forceinline__ void col_body(const Geo& g, const ColArgs<T>& a, const int bx) {
    typedef typename CT<T>::C C;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C* sm = reinterpret_cast<C*>(smem_raw);
    const int ny = g.ny, TC = (E == 0) ? g.TTc : ny / E, LP = spad_len(ny), CW = g.CW;
    const int P = FG ? col_groups(g.fpc, E, MODE) : 1, GT = CW * TC;
    const int fg = threadIdx.x / GT, u = threadIdx.x - fg * GT;
    const int b = u / TC, t = u - b * TC;
    const int sy = sync_mode(TC, P > 1 ? 1 + fg : 0, GT);
    const int c0 = bx * CW;
    const int Kx = g.Kx, Ky = g.Ky;
    const int nthr = P * GT;  // the block size
    C* gbuf = sm + fg * CW * LP;  // this group's CW column buffers
    C* mybuf = gbuf + b * LP;
    C* myscr = sm + (P * CW + fg * CW + b) * LP;  // mixed-radix scratch of this group (E = 0 only)
    // next-stage state of the block's kept modes, CW * Ky values (COL_STAGE, COL_ADD):
    // the stage loop leaves it here for the inverse transforms of the fields
    C* wsm = sm + (E == 0 ? 2 : 1) * P * CW * LP;
    __shared__ double s_dt;

    if (MODE == COL_STAGE) {
        if (threadIdx.x == 0) {
            double dt;
            if (STAGE == 1) {
                if (a.sp.adaptive) {
                    // spectral_time_integration.c:9-31 on max|u| of the stage-1 fields
                    const double vmax = sqrt(__longlong_as_double((long long)a.ds->maxvel2));
                    const double dt_cfl = a.sp.cfl * a.sp.dxmin / (vmax + 1e-12);
                    const double dt_visc = 0.5 * a.sp.Re * a.sp.dxmin * a.sp.dxmin;
                    dt = fmin(dt_cfl, dt_visc);
                    dt = fmax(dt, 1e-8);
                    dt = fmin(dt, 0.1);
                } else {
                    dt = a.ds->dt_fixed;
                }
                if (bx == 0) a.ds->dt = dt;
            } else {
                dt = a.ds->dt;
            }
            s_dt = dt;
        }
    }

    if (MODE == COL_STAGE || MODE == COL_FWD_EXPORT || MODE == COL_NL_EXPORT || MODE == COL_ADD) {
        // four loads of G in flight per thread before their stores (L2 round trips)
        for (int i0 = threadIdx.x; i0 < ny * CW; i0 += 4 * nthr) {
            C v[4];
            int o[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int idx = i0 + q * nthr;
                v[q] = cmake<C>(0.0, 0.0);
                o[q] = -1;
                if (idx < ny * CW) {
                    int y, c;
                    if (g.fTG) { c = idx / ny; y = idx - c * ny; } else { y = idx / CW; c = idx - y * CW; }
                    o[q] = c * LP + spad(y);
                    if (c0 + c < Kx) v[q] = a.G[gidx(g, y, c0 + c)];
                }
            }
#pragma unroll
            for (int q = 0; q < 4; ++q)
                if (o[q] >= 0) sm[o[q]] = v[q];
        }
        __syncthreads();
        if (fg == 0) fft_any<E, false>(mybuf, myscr, ny, g.logny, g.rya, g.ryb, g.nry, t, TC, a.twc, sy);
        __syncthreads();  // the loops below read every column of the block

        if constexpr (MODE == COL_FWD_EXPORT || MODE == COL_NL_EXPORT) {
            const T sc = (T)a.out_scale;
            for (int idx = threadIdx.x; idx < CW * Ky; idx += nthr) {
                const int c = idx / Ky, jj = idx - c * Ky, i = c0 + c;
                if (i >= Kx) continue;
                const int j = kept_j(g, jj);
                const C v = sm[c * LP + spad(j)];
                a.out_spec[(size_t)j * g.nkx + i] = make_double2((double)(v.x * sc), (double)(v.y * sc));
            }
            return;
        } else if constexpr (MODE == COL_ADD) {
            // the scaled value rounded in T, the sum formed in double and rounded once to
            // T (the roundings of an FP64 export added to the state)
            const T sc = (T)a.out_scale;
            for (int idx = threadIdx.x; idx < CW * Ky; idx += nthr) {
                const int c = idx / Ky, jj = idx - c * Ky, i = c0 + c;
                if (i >= Kx) continue;
                const int j = kept_j(g, jj);
                const C v = sm[c * LP + spad(j)];
                const size_t s = (size_t)i * Ky + jj;
                C w = a.W0[s];
                w.x = (T)((double)w.x + (double)(v.x * sc));
                w.y = (T)((double)w.y + (double)(v.y * sc));
                a.W0[s] = w;
                wsm[idx] = w;
            }
            __syncthreads();  // the inverse phase reads W0 of every column of the block
        } else {
            const double dt = s_dt;
            const StageCoef<T> q = stage_coef<T>(a.sp, dt);
            double f_amp = 0.0;
            double sfd_a = 0.0;
            if (STAGE == 4) {
                if (a.sp.forcing) f_amp = a.sp.f_sigma * sqrt(dt / a.sp.fsub);
                if (a.sp.sfd) {
                    sfd_a = dt / a.sp.sfd_tau;
                    sfd_a = sfd_a > 1.0 ? 1.0 : (sfd_a < 0.0 ? 0.0 : sfd_a);
                }
            }
            // two modes a thread per round: both modes' loads in flight before either
            // mode's arithmetic and stores
            for (int i0 = threadIdx.x; i0 < CW * Ky; i0 += 2 * nthr) {
                C w0v[2], wsv[2], accv[2], fbv[2];
                T hwv[2], swv[2];
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int idx = i0 + h * nthr;
                    const int c = idx / Ky, jj = idx - c * Ky, i = c0 + c;
                    w0v[h] = wsv[h] = accv[h] = fbv[h] = cmake<C>(0.0, 0.0);
                    hwv[h] = swv[h] = (T)0;
                    if (idx >= CW * Ky || i >= Kx) continue;
                    const size_t s = (size_t)i * Ky + jj;
                    w0v[h] = a.W0[s];
                    wsv[h] = (STAGE == 1) ? w0v[h] : a.WS[s];
                    if (STAGE != 1) accv[h] = a.ACC[s];
                    if (a.sp.hv) hwv[h] = a.hvw[s];
                    if (a.sp.sfd) {
                        swv[h] = a.sfdw[s];
                        fbv[h] = a.SFD[s];
                    }
                }
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int idx = i0 + h * nthr;
                    const int c = idx / Ky, jj = idx - c * Ky, i = c0 + c;
                    if (idx >= CW * Ky || i >= Kx) continue;
                    const int j = kept_j(g, jj);
                    const C gh = sm[c * LP + spad(j)];
                    const size_t s = (size_t)i * Ky + jj;
                    const T kx = a.kxv[i], ky = a.kyv[jj];
                    const T k2 = k2sum(kx, ky);
                    C wn = a.sp.ifrk
                               ? rk_stage_mode<T, STAGE, true>(q, gh, w0v[h], wsv[h], accv[h], hwv[h], swv[h], fbv[h], k2,
                                                               a.ACC, a.WS, s)
                               : rk_stage_mode<T, STAGE, false>(q, gh, w0v[h], wsv[h], accv[h], hwv[h], swv[h], fbv[h],
                                                                k2, a.ACC, a.WS, s);
                    if (STAGE == 4) {
                        bool forced;
                        wn = post_step_mode(g, a, i, j, s, wn, kx, ky, f_amp, sfd_a, forced);
                        a.W0[s] = wn;
                    }
                    wsm[idx] = wn;
                }
            }
            if (STAGE == 4 && bx == 0 && threadIdx.x == 0) a.ds->t = a.ds->t + dt;
            __syncthreads();
        }
    }

    if constexpr (MODE == COL_FWD_EXPORT || MODE == COL_NL_EXPORT) return;

    // inverse y-transforms of the next-stage fields
    const int nf = (MODE == COL_INV1) ? 1 : (MODE == COL_PROLOGUE ? a.nfields : 4);  // COL_ADD: 4
    const C* src = (MODE == COL_STAGE) ? ((STAGE == 4) ? a.W0 : a.WS) : a.W0;
    for (int f = fg; f < nf; f += P) {
        for (int idx = u; idx < CW * ny; idx += GT) {
            const int c = idx / ny, j = idx - c * ny, i = c0 + c;
            const int jk = kept_jj(g, j);
            C v = cmake<C>(0.0, 0.0);
            if (i < Kx && jk >= 0) {
                const size_t s = (size_t)i * Ky + jk;
                if (MODE == COL_INV1) {
                    v = src[s];
                } else if (MODE == COL_STAGE || MODE == COL_ADD) {
                    v = field_value<T, C>(f, wsm[c * Ky + jk], a.kxv[i], a.kyv[jk]);
                } else if (MODE == COL_PROLOGUE && !a.psi_from_w && f < 2) {
                    const C p = a.PSI0[s];
                    v = p;
                    if (f == 1) { const T ky = a.kyv[jk]; v.x = -ky * p.y; v.y = ky * p.x; }
                } else {
                    v = field_value<T, C>(f, src[s], a.kxv[i], a.kyv[jk]);
                }
            }
            gbuf[c * LP + spad(j)] = v;
        }
        fft_sync(P > 1 ? ((1 + fg) << 16) | GT : 0);
        fft_any<E, true>(mybuf, myscr, ny, g.logny, g.rya, g.ryb, g.nry, t, TC, a.twc, sy);
        fft_sync(P > 1 ? ((1 + fg) << 16) | GT : 0);  // the store loop reads every column of the group
        C* dstF = a.F[f];
        for (int idx = u; idx < ny * CW; idx += GT) {
            int y, c;
            if (g.fLB) { c = idx / ny; y = idx - c * ny; } else { y = idx / CW; c = idx - y * CW; }
            dstF[fidx(g, y, c0 + c)] = gbuf[c * LP + spad(y)];
        }
        fft_sync(P > 1 ? ((1 + fg) << 16) | GT : 0);
    }
}

template <typename T, int E, int MODE, int STAGE, int N = 0>
__global__ void __launch_bounds__(512) k_col(Geo g, ColArgs<T> a) {
    if constexpr (N > 0) {
        Geo f = g;
        fold_sizes<N>(f);
        col_body<T, E, MODE, STAGE>(f, a, blockIdx.x);
    } else {
        col_body<T, E, MODE, STAGE>(g, a, blockIdx.x);
    }
}

// ======================================================= auxiliary kernels
// (left out of translation units that define NSG_NO_AUX_KERNELS: their host
// stubs are defined once, by the instance engine)
#ifndef NSG_NO_AUX_KERNELS

// grid, wavenumbers, k^2, mask exactly as spectral_initialization.c:15-49
__global__ void k_geometry(Geo g, double* x, double* y, double* kx, double* ky, double* k2, int* mask) {
    const int nx = g.nx, ny = g.ny, nkx = g.nkx;
    const long long n = (long long)nkx * g.nky;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n; idx += (long long)gridDim.x * blockDim.x) {
        const int j = (int)(idx / nkx), i = (int)(idx - (long long)j * nkx);
        const double kxv = 2.0 * 3.14159265358979323846 * i / g.Lx;
        const double kyv = (j <= ny / 2) ? 2.0 * 3.14159265358979323846 * j / g.Ly : 2.0 * 3.14159265358979323846 * (j - ny) / g.Ly;
        if (k2) k2[idx] = k2sum(kxv, kyv);
        if (mask) {
            const int band = (j <= ny / 2) ? j : j - ny;
            mask[idx] = (i <= (2 * nkx) / 3) && (abs(band) <= (2 * ny) / 6);
        }
        if (j == 0 && kx) kx[i] = kxv;
        if (i == 0 && ky) ky[j] = kyv;
        if (j == 0 && i < nx && x) x[i] = i * g.Lx / nx;
        if (i == 0 && y) y[j] = j * g.Ly / ny;
    }
    // x covers i < nx which exceeds nkx: finish the tail
    for (long long i = nkx + blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nx; i += (long long)gridDim.x * blockDim.x)
        if (x) x[i] = i * g.Lx / nx;
}

__device__ __forceinline__ double geo_k2(const Geo& g, int j, int i) {
    const double kxv = 2.0 * 3.14159265358979323846 * i / g.Lx;
    const double kyv = (j <= g.ny / 2) ? 2.0 * 3.14159265358979323846 * j / g.Ly : 2.0 * 3.14159265358979323846 * (j - g.ny) / g.Ly;
    return k2sum(kxv, kyv);
}
__device__ __forceinline__ int geo_kept(const Geo& g, int j, int i) {
    const int band = (j <= g.ny / 2) ? j : j - g.ny;
    return (i <= (2 * g.nkx) / 3) && (abs(band) <= (2 * g.ny) / 6);
}

// max |k| over all modes (hyperviscosity.c:68-72)
__global__ void k_kmax(Geo g, DevScalars* ds) {
    const long long n = (long long)g.nkx * g.nky;
    double m = 0.0;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n; idx += (long long)gridDim.x * blockDim.x) {
        const int j = (int)(idx / g.nkx), i = (int)(idx - (long long)j * g.nkx);
        m = fmax(m, sqrt(geo_k2(g, j, i)));
    }
    m = warp_max(m);
    if ((threadIdx.x & 31) == 0) atomicMax(&ds->kmax_bits, (unsigned long long)__double_as_longlong(m));
}

// weight = c ((|k| - kc) inv_bw)^order above kc (hyperviscosity.c:88-101), FP64 full table
__global__ void k_hv_weights(Geo g, int enabled, double coefficient, int order, double cutoff, double inv_bw,
                             double* w_full) {
    const long long n = (long long)g.nkx * g.nky;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n; idx += (long long)gridDim.x * blockDim.x) {
        const int j = (int)(idx / g.nkx), i = (int)(idx - (long long)j * g.nkx);
        double w = 0.0;
        if (enabled) {
            const double km = sqrt(geo_k2(g, j, i));
            if (km > cutoff) w = coefficient * pow((km - cutoff) * inv_bw, (double)order);
        }
        w_full[idx] = w;
    }
}

// kept-mode tables in the working precision (FP64 generated, rounded once)
template <typename T>
__global__ void k_tables(Geo g, const double* w_full, int sfd, double sfd_strength, int order, double cutoff,
                         double inv_bw, T* kxv, T* kyv, T* hvw, T* sfdw) {
    const long long n = (long long)g.Kxp * g.Ky;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n; idx += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(idx / g.Ky), jj = (int)(idx - (long long)i * g.Ky);
        const int j = kept_j(g, jj);
        double w = 0.0, s = 0.0;
        if (i < g.Kx) {
            w = w_full ? w_full[(size_t)j * g.nkx + i] : 0.0;
            if (sfd && inv_bw > 0.0) {
                const double km = sqrt(geo_k2(g, j, i));
                double ratio = 0.0;
                if (km > cutoff) {
                    double sc = (km - cutoff) * inv_bw;
                    sc = sc < 0.0 ? 0.0 : (sc > 1.0 ? 1.0 : sc);
                    ratio = pow(sc, (double)order);
                }
                s = sfd_strength * ratio;
            }
        }
        hvw[idx] = (T)w;
        sfdw[idx] = (T)s;
        if (jj == 0) kxv[i] = (T)(2.0 * 3.14159265358979323846 * i / g.Lx);
        if (i == 0) {
            kyv[jj] = (T)((j <= g.ny / 2) ? 2.0 * 3.14159265358979323846 * j / g.Ly : 2.0 * 3.14159265358979323846 * (j - g.ny) / g.Ly);
        }
    }
}

// twiddle table tw[t] = exp(-2 pi i t / L), t < n (FP64 sincospi, rounded once)
template <typename C>
__global__ void k_twiddles(C* tw, int n, int L) {
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        double s, c;
        sincospi(-2.0 * (double)t / (double)L, &s, &c);
        tw[t].x = c;
        tw[t].y = s;
    }
}

// host-layout spectrum -> kept state (and masked-out modes into OUT); flag if any masked-out mode is non-zero
template <typename T>
__global__ void k_import(Geo g, const double2* wh, const double2* ph, const double2* sh, typename CT<T>::C* W,
                         typename CT<T>::C* P, typename CT<T>::C* S, double2* out, double2* outsfd, int* flag) {
    typedef typename CT<T>::C C;
    const long long n = (long long)g.nkx * g.nky;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n; idx += (long long)gridDim.x * blockDim.x) {
        const int j = (int)(idx / g.nkx), i = (int)(idx - (long long)j * g.nkx);
        const int jk = kept_jj(g, j);
        const double2 w = wh[idx];
        if (i < g.Kx && jk >= 0) {
            const size_t s = (size_t)i * g.Ky + jk;
            W[s] = cmake<C>(w.x, w.y);
            if (P) { const double2 p = ph[idx]; P[s] = cmake<C>(p.x, p.y); }
            if (S) { const double2 q = sh[idx]; S[s] = cmake<C>(q.x, q.y); }
        } else {
            if (out) out[idx] = w;
            if (outsfd) outsfd[idx] = sh ? sh[idx] : make_double2(0.0, 0.0);
            if (flag && (w.x != 0.0 || w.y != 0.0)) atomicOr(flag, 1);
            if (flag && ph) {  // bit 2: the stream function has a non-zero mode outside the mask
                const double2 p = ph[idx];
                if (p.x != 0.0 || p.y != 0.0) atomicOr(flag, 2);
            }
        }
    }
}

// reference-layout exports of the device state (compute_derivatives' spectral part, spectral_core.c:8-34)
template <typename T>
__global__ void k_export(Geo g, const typename CT<T>::C* W, const typename CT<T>::C* S, const double2* out,
                         const double2* outsfd, double2* wh, double2* ph, double2* uh, double2* vh, double2* sh) {
    const long long n = (long long)g.nkx * g.nky;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n; idx += (long long)gridDim.x * blockDim.x) {
        const int j = (int)(idx / g.nkx), i = (int)(idx - (long long)j * g.nkx);
        const int jk = kept_jj(g, j);
        double2 w = make_double2(0.0, 0.0), q = make_double2(0.0, 0.0);
        if (i < g.Kx && jk >= 0) {
            const size_t s = (size_t)i * g.Ky + jk;
            w = make_double2((double)W[s].x, (double)W[s].y);
            if (S) q = make_double2((double)S[s].x, (double)S[s].y);
        } else {
            if (out) w = out[idx];
            if (outsfd) q = outsfd[idx];
        }
        if (wh) wh[idx] = w;
        if (sh) sh[idx] = q;
        const double kxv = 2.0 * 3.14159265358979323846 * i / g.Lx;
        const double kyv = (j <= g.ny / 2) ? 2.0 * 3.14159265358979323846 * j / g.Ly : 2.0 * 3.14159265358979323846 * (j - g.ny) / g.Ly;
        const double k2 = k2sum(kxv, kyv);
        double2 p = make_double2(0.0, 0.0);
        if (k2 > 1e-12) p = make_double2(-w.x / k2, -w.y / k2);
        if (ph) ph[idx] = p;
        if (uh) uh[idx] = make_double2(-kyv * p.y, kyv * p.x);
        if (vh) vh[idx] = make_double2(kxv * p.y, -kxv * p.x);
    }
}

// FP64 pointwise compat ops over host-layout spectra
__global__ void k_velocity(Geo g, const double2* wh, double2* ph, double2* uh, double2* vh) {
    const long long n = (long long)g.nkx * g.nky;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n; idx += (long long)gridDim.x * blockDim.x) {
        const int j = (int)(idx / g.nkx), i = (int)(idx - (long long)j * g.nkx);
        const double kxv = 2.0 * 3.14159265358979323846 * i / g.Lx;
        const double kyv = (j <= g.ny / 2) ? 2.0 * 3.14159265358979323846 * j / g.Ly : 2.0 * 3.14159265358979323846 * (j - g.ny) / g.Ly;
        const double k2 = k2sum(kxv, kyv);
        const double2 w = wh[idx];
        double2 p = make_double2(0.0, 0.0);
        if (k2 > 1e-12) p = make_double2(-w.x / k2, -w.y / k2);
        ph[idx] = p;
        uh[idx] = make_double2(-kyv * p.y, kyv * p.x);
        vh[idx] = make_double2(kxv * p.y, -kxv * p.x);
    }
}

__global__ void k_dealias(Geo g, double2* fh, double2* masked_copy) {
    const long long n = (long long)g.nkx * g.nky;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n; idx += (long long)gridDim.x * blockDim.x) {
        const int j = (int)(idx / g.nkx), i = (int)(idx - (long long)j * g.nkx);
        double2 v = fh[idx];
        if (!geo_kept(g, j, i)) v = make_double2(0.0, 0.0);
        if (masked_copy) masked_copy[idx] = v;
        else fh[idx] = v;
    }
}

// rhs -= w state + s ramp (state - sfd)   (hyperviscosity.c:104-150)
__global__ void k_hv_apply(Geo g, const double* w_full, int visc, int sfd, double sfd_strength, int order,
                           double cutoff, double inv_bw, double2* rhs, const double2* st, const double2* sf) {
    const long long n = (long long)g.nkx * g.nky;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n; idx += (long long)gridDim.x * blockDim.x) {
        const int j = (int)(idx / g.nkx), i = (int)(idx - (long long)j * g.nkx);
        const double2 s = st[idx];
        double dr = 0.0, di = 0.0;
        if (visc) { const double w = w_full[idx]; dr += w * s.x; di += w * s.y; }
        if (sfd) {
            double ratio = 0.0;
            if (inv_bw > 0.0) {
                const double km = sqrt(geo_k2(g, j, i));
                if (km > cutoff) {
                    double sc = (km - cutoff) * inv_bw;
                    sc = sc < 0.0 ? 0.0 : (sc > 1.0 ? 1.0 : sc);
                    ratio = pow(sc, (double)order);
                }
            }
            const double sw = sfd_strength * ratio;
            if (sw > 0.0) { const double2 f = sf[idx]; dr += sw * (s.x - f.x); di += sw * (s.y - f.y); }
        }
        double2 r = rhs[idx];
        r.x -= dr;
        r.y -= di;
        rhs[idx] = r;
    }
}

// This step's forcing draws, one thread per (mode entry, draw s): entry e is
// kx index i = e / (2 kyr + 1), ky = e % (2 kyr + 1) - kyr; the draw uses the
// counter the stage-4 kernel uses, *counter + s with counter = the running step's
// step_cur (set by the step's stage-1 row pass; the kernel runs after it, beside
// stages 1-3, and is joined before stage 4).  Terms are stored as forcing_xi_sum forms
// them (the conjugate row of kx = 0, ky < 0 negated), modes outside the shell
// as zeros.
__global__ void k_forcing_noise(int ny, double Lx, double Ly, const unsigned long long* counter, int M,
                                unsigned long long seed, double kmin, double kmax, int kxr, int kyr, double2* out) {
    const int n = (kxr + 1) * (2 * kyr + 1) * M;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const int e = t / M, s = t - e * M;
        const int i = e / (2 * kyr + 1);
        const int ky = e - i * (2 * kyr + 1) - kyr;
        out[t] = forcing_noise_term(i, ky, s, *counter, seed, Lx, Ly, kmin, kmax);
    }
}

// per-mode sums of the step's noise table (k_forcing_noise): the M draws of mode
// e = i (2 kyr + 1) + ky + kyr summed in order from zero, as forcing_xi_sum sums
// them, and zero outside the forcing shell (the shell test of forcing_increment)
__global__ void k_forcing_sum(int ny, double Lx, double Ly, int M, double kmin, double kmax, int kxr, int kyr,
                              const double2* __restrict__ terms, double2* __restrict__ out) {
    const int n = (kxr + 1) * (2 * kyr + 1);
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
        const int i = e / (2 * kyr + 1);
        const int ky = e - i * (2 * kyr + 1) - kyr;
        const int j = ky >= 0 ? ky : ny + ky;
        double2 r = make_double2(0.0, 0.0);
        if (forcing_in_shell(Lx, Ly, ny, i, j, kmin, kmax)) {
            const double2* t = terms + (size_t)e * M;
            double sx = 0.0, sy = 0.0;
            for (int s = 0; s < M; ++s) {
                sx = __dadd_rn(sx, t[s].x);
                sy = __dadd_rn(sy, t[s].y);
            }
            r = make_double2(sx, sy);
        }
        out[e] = r;
    }
}

// device scalars from kernel parameters: ordered on the stream, no host copy or sync
__global__ void k_set_scalars(DevScalars* ds, DevScalars h) { *ds = h; }
__global__ void k_set_dt_fixed(DevScalars* ds, double dt) { ds->dt_fixed = dt; }

__global__ void k_hv_post(Geo g, double alpha, const double2* st, double2* sf) {
    const long long n = (long long)g.nkx * g.nky;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n; idx += (long long)gridDim.x * blockDim.x) {
        const double2 p = sf[idx], s = st[idx];
        sf[idx] = make_double2((1.0 - alpha) * p.x + alpha * s.x, (1.0 - alpha) * p.y + alpha * s.y);
    }
}

// masked-out modes evolve by the linear part only (the reference's RK4 on modes
// whose nonlinear term is zeroed by the mask); FP64, reference arithmetic
__global__ void k_outside(Geo g, StepParams sp, const double* w_full, double cutoff, double inv_bw, int order,
                          double sfd_strength, DevScalars* ds, double2* out, double2* outsfd) {
    const long long n = (long long)g.nkx * g.nky;
    const double dt = ds->dt;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n; idx += (long long)gridDim.x * blockDim.x) {
        const int j = (int)(idx / g.nkx), i = (int)(idx - (long long)j * g.nkx);
        if (geo_kept(g, j, i)) continue;
        const double k2 = geo_k2(g, j, i);
        const double w = (sp.hv && w_full) ? w_full[idx] : 0.0;
        double sw = 0.0;
        if (sp.sfd && inv_bw > 0.0) {
            const double km = sqrt(k2);
            if (km > cutoff) {
                double sc = (km - cutoff) * inv_bw;
                sc = sc < 0.0 ? 0.0 : (sc > 1.0 ? 1.0 : sc);
                sw = sfd_strength * pow(sc, (double)order);
            }
        }
        const double2 w0 = out[idx];
        const double2 fb = outsfd ? outsfd[idx] : make_double2(0.0, 0.0);
        double2 wn;
        if (sp.ifrk) {
            // integrating-factor RK4 with a zero (masked) nonlinear term: explicit part is the SFD relaxation
            const double lam = k2 * sp.inv_re + w;
            const double e1 = exp(-lam * (0.5 * dt)), e2 = e1 * e1;
            double2 ws = w0, acc = make_double2(0.0, 0.0);
            for (int s = 0; s < 4; ++s) {
                double2 k = make_double2(0.0, 0.0);
                if (sp.sfd && sw > 0.0) { k.x -= sw * (ws.x - fb.x); k.y -= sw * (ws.y - fb.y); }
                if (s == 0) {
                    acc = make_double2(e2 * k.x, e2 * k.y);
                    ws = make_double2(e1 * (w0.x + (0.5 * dt) * k.x), e1 * (w0.y + (0.5 * dt) * k.y));
                } else if (s == 1) {
                    acc = make_double2(acc.x + 2.0 * (e1 * k.x), acc.y + 2.0 * (e1 * k.y));
                    ws = make_double2(e1 * w0.x + (0.5 * dt) * k.x, e1 * w0.y + (0.5 * dt) * k.y);
                } else if (s == 2) {
                    acc = make_double2(acc.x + 2.0 * (e1 * k.x), acc.y + 2.0 * (e1 * k.y));
                    ws = make_double2(e2 * w0.x + dt * (e1 * k.x), e2 * w0.y + dt * (e1 * k.y));
                } else {
                    wn = make_double2(e2 * w0.x + dt / 6.0 * (acc.x + k.x), e2 * w0.y + dt / 6.0 * (acc.y + k.y));
                }
            }
        } else {
            double2 kk[4];
            double2 ws = w0;
            const double cst[3] = {0.5 * dt, 0.5 * dt, dt};
            for (int s = 0; s < 4; ++s) {
                double2 k;
                k.x = 0.0 - k2 * ws.x * sp.inv_re;
                k.y = 0.0 - k2 * ws.y * sp.inv_re;
                double dr = 0.0, di = 0.0;
                if (sp.hv) { dr += w * ws.x; di += w * ws.y; }
                if (sp.sfd && sw > 0.0) { dr += sw * (ws.x - fb.x); di += sw * (ws.y - fb.y); }
                k.x -= dr;
                k.y -= di;
                kk[s] = k;
                if (s < 3) ws = make_double2(w0.x + cst[s] * k.x, w0.y + cst[s] * k.y);
            }
            wn.x = w0.x + dt / 6.0 * (kk[0].x + 2.0 * kk[1].x + 2.0 * kk[2].x + kk[3].x);
            wn.y = w0.y + dt / 6.0 * (kk[0].y + 2.0 * kk[1].y + 2.0 * kk[2].y + kk[3].y);
        }
        out[idx] = wn;
        if (sp.sfd && outsfd) {
            double a = dt / sp.sfd_tau;
            a = a > 1.0 ? 1.0 : (a < 0.0 ? 0.0 : a);
            outsfd[idx] = make_double2((1.0 - a) * fb.x + a * wn.x, (1.0 - a) * fb.y + a * wn.y);
        }
    }
}

// per-block compensated partial sums of two quantities (s0, s1) -> part[2*block]
// kind 0: energy 0.5(a^2+b^2); 1: enstrophy 0.5 a^2; 2: max sqrt(a^2+b^2) (into ds->maxvel2)
__global__ void k_reduce_real(int kind, const double* a, const double* b, long long n, double2* part, DevScalars* ds) {
    DD acc = {0.0, 0.0};
    double m = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const double x = a[i];
        if (kind == 0) { const double yv = b[i]; dd_add(acc, 0.5 * (x * x + yv * yv)); }
        else if (kind == 1) dd_add(acc, 0.5 * x * x);
        else { const double yv = b[i]; m = fmax(m, sqrt(x * x + yv * yv)); }
    }
    if (kind == 2) {
        m = warp_max(m);
        if ((threadIdx.x & 31) == 0) atomicMax(&ds->aux_max, (unsigned long long)__double_as_longlong(m));
        return;
    }
    DD tot = block_dd(acc);
    if (threadIdx.x == 0) part[blockIdx.x] = make_double2(tot.s, tot.c);
}

// merge n partial pairs into out[0] (value) with one block
__global__ void k_merge_partials(const double2* part, int n, double* out) {
    DD acc = {0.0, 0.0};
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        DD v = {part[i].x, part[i].y};
        acc = dd_merge(acc, v);
    }
    DD tot = block_dd(acc);
    if (threadIdx.x == 0) out[0] = tot.s + tot.c;
}

// Parseval energy and enstrophy of the kept state: E = 1/2 sum_full |w|^2/k^2,
// Z = 1/2 sum_full |w|^2 (Hermitian weight 2 for kx > 0); flags non-finite values
template <typename T>
__global__ void k_diag(Geo g, const typename CT<T>::C* W, const T* kxv, const T* kyv, double2* part, DevScalars* ds) {
    DD e = {0.0, 0.0}, z = {0.0, 0.0};
    int bad = 0;
    const long long n = (long long)g.Kx * g.Ky;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n; idx += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(idx / g.Ky), jj = (int)(idx - (long long)i * g.Ky);
        const double wx = (double)W[idx].x, wy = (double)W[idx].y;
        if (!isfinite(wx) || !isfinite(wy)) bad = 1;
        const int j = kept_j(g, jj);
        const double k2 = geo_k2(g, j, i);
        const double wt = (i == 0) ? 1.0 : 2.0;
        const double m2 = wt * (wx * wx + wy * wy);
        dd_add(z, 0.5 * m2);
        if (k2 > 1e-12) dd_add(e, 0.5 * m2 / k2);
    }
    if (bad) atomicOr(&ds->flag, 2);
    DD te = block_dd(e);
    __syncthreads();
    DD tz = block_dd(z);
    if (threadIdx.x == 0) {
        part[2 * blockIdx.x] = make_double2(te.s, te.c);
        part[2 * blockIdx.x + 1] = make_double2(tz.s, tz.c);
    }
}
__global__ void k_merge_pairs2(const double2* part, int nblocks, double* out) {
    DD a = {0.0, 0.0}, b = {0.0, 0.0};
    for (int i = threadIdx.x; i < nblocks; i += blockDim.x) {
        DD u = {part[2 * i].x, part[2 * i].y}, v = {part[2 * i + 1].x, part[2 * i + 1].y};
        a = dd_merge(a, u);
        b = dd_merge(b, v);
    }
    DD ta = block_dd(a);
    __syncthreads();
    DD tb = block_dd(b);
    if (threadIdx.x == 0) { out[0] = ta.s + ta.c; out[1] = tb.s + tb.c; }
}

// spectral statistics of host-layout spectra (spectral_analysis.c:36-142)
__global__ void k_spec_stats(Geo g, const double2* wh, const double2* uh, const double2* vh, double2* part,
                             DevScalars* ds, double* bins, int* counts, int nbins) {
    const long long n = (long long)g.nkx * g.nky;
    const double k2last = geo_k2(g, g.nky - 1, g.nkx - 1);
    const double max_k = sqrt(k2last);
    DD tot = {0.0, 0.0}, hi = {0.0, 0.0}, acc = {0.0, 0.0};
    double cnt = 0.0, mx = 0.0;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n; idx += (long long)gridDim.x * blockDim.x) {
        const int j = (int)(idx / g.nkx), i = (int)(idx - (long long)j * g.nkx);
        const double k2 = geo_k2(g, j, i);
        if (wh) {
            const double2 w = wh[idx];
            const double m = hypot(w.x, w.y);
            const double m2 = m * m;
            dd_add(tot, m2);
            const double kn = max_k > 0.0 ? sqrt(k2) / max_k : 0.0;
            if (kn > 0.8) dd_add(hi, m2);
            mx = fmax(mx, m);
            if (k2 > 0.25 * k2last) { dd_add(acc, m2); cnt += 1.0; }
        }
        if (uh && bins) {
            const int bin = (int)(sqrt(k2) + 0.5);
            if (bin < nbins) {
                const double2 u = uh[idx], v = vh[idx];
                const double um = hypot(u.x, u.y), vm = hypot(v.x, v.y);
                atomicAdd(&bins[bin], 0.5 * (um * um + vm * vm));
                atomicAdd(&counts[bin], 1);
            }
        }
    }
    mx = warp_max(mx);
    if ((threadIdx.x & 31) == 0) atomicMax(&ds->aux_max, (unsigned long long)__double_as_longlong(mx));
    DD a = block_dd(tot);
    __syncthreads();
    DD b = block_dd(hi);
    __syncthreads();
    DD c = block_dd(acc);
    __syncthreads();
    DD d = {cnt, 0.0};
    d = block_dd(d);
    if (threadIdx.x == 0) {
        part[4 * blockIdx.x + 0] = make_double2(a.s, a.c);
        part[4 * blockIdx.x + 1] = make_double2(b.s, b.c);
        part[4 * blockIdx.x + 2] = make_double2(c.s, c.c);
        part[4 * blockIdx.x + 3] = make_double2(d.s, d.c);
    }
}
__global__ void k_merge_pairs4(const double2* part, int nblocks, double* out) {
    for (int q = 0; q < 4; ++q) {
        DD a = {0.0, 0.0};
        for (int i = threadIdx.x; i < nblocks; i += blockDim.x) {
            DD u = {part[4 * i + q].x, part[4 * i + q].y};
            a = dd_merge(a, u);
        }
        DD t = block_dd(a);
        if (threadIdx.x == 0) out[q] = t.s + t.c;
        __syncthreads();
    }
}

// Taylor-Green fields of spectral_initialization.c:72-88
__global__ void k_taylor_green(Geo g, double* u, double* v, double* w, double* p) {
    const long long n = (long long)g.nx * g.ny;
    const double tp = 2 * 3.14159265358979323846;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n; idx += (long long)gridDim.x * blockDim.x) {
        const int j = (int)(idx / g.nx), i = (int)(idx - (long long)j * g.nx);
        const double x = i * g.Lx / g.nx, y = j * g.Ly / g.ny;
        u[idx] = sin(tp * x / g.Lx) * cos(tp * y / g.Ly);
        v[idx] = -cos(tp * x / g.Lx) * sin(tp * y / g.Ly);
        w[idx] = 2.0 * (tp / g.Lx) * cos(tp * x / g.Lx) * cos(tp * y / g.Ly);
        p[idx] = 0.0;
    }
}

// random-phase spectrum, unnormalised; energy partials (weight 2 for 0 < kx < Nyquist)
__global__ void k_random_spectrum(Geo g, unsigned long long seed, double k0, double2* wh, double2* part) {
    const long long n = (long long)g.nkx * g.nky;
    DD e = {0.0, 0.0};
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n; idx += (long long)gridDim.x * blockDim.x) {
        const int j = (int)(idx / g.nkx), i = (int)(idx - (long long)j * g.nkx);
        const double k2 = geo_k2(g, j, i);
        double2 v = make_double2(0.0, 0.0);
        if (geo_kept(g, j, i) && k2 > 1e-12) {
            int jsrc = j, flip = 0;
            if (i == 0 && j > g.ny / 2) { jsrc = g.ny - j; flip = 1; }
            unsigned long long ctr[4] = {(unsigned long long)jsrc * g.nkx + i, 0ULL, NSG_TAG_IC, 0ULL};
            philox4x64(ctr, seed, 0ULL);
            const double km = sqrt(k2);
            const double ek = km * km * km * km * exp(-(km / k0) * (km / k0));
            const double amp = sqrt(km * ek / 3.14159265358979323846);
            double sn, cs;
            sincos(2.0 * 3.14159265358979323846 * u53(ctr[0]), &sn, &cs);
            v = make_double2(amp * cs, amp * sn);
            if (flip) v.y = -v.y;
            const double wt = (i == 0 || 2 * i == g.nx) ? 1.0 : 2.0;
            const double m2 = v.x * v.x + v.y * v.y;
            dd_add(e, wt * 0.5 * m2 / k2);
        }
        wh[idx] = v;
    }
    DD te = block_dd(e);
    if (threadIdx.x == 0) part[blockIdx.x] = make_double2(te.s, te.c);
}
__global__ void k_scale_spec(long long n, double2* wh, const double* num_den) {
    const double e = num_den[0];
    const double target = num_den[1];
    const double s = e > 0.0 ? sqrt(target / e) : 0.0;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n; idx += (long long)gridDim.x * blockDim.x) {
        double2 v = wh[idx];
        wh[idx] = make_double2(v.x * s, v.y * s);
    }
}

// forcing shell selection (forcing.c:78-96)
__global__ void k_forcing_weights(const double* k2, int n, double kmin, double kmax, double* w, int* active) {
    int cnt = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double km = sqrt(k2[i]);
        const int on = (km >= kmin && km <= kmax);
        w[i] = on ? 1.0 : 0.0;
        cnt += on;
    }
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(active, cnt);
}

__device__ __forceinline__ unsigned long long splitmix_out(unsigned long long z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

// ns_forcing_generate's stream, counter-addressable; single CTA (ranks by block scan)
__global__ void k_forcing_generate(int n, const double* weights, int colored, double alpha, double beta,
                                   double energy_target, unsigned long long state, double2* cs, double2* out) {
    __shared__ int warp_tot[32];
    __shared__ int base_s;
    __shared__ double scale_s;
    if (threadIdx.x == 0) base_s = 0;
    __syncthreads();
    DD tot = {0.0, 0.0};
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int c0 = 0; c0 < n; c0 += blockDim.x) {
        const int idx = c0 + threadIdx.x;
        const int on = (idx < n && weights[idx] > 0.0) ? 1 : 0;
        // block exclusive scan of 'on'
        int incl = on;
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        if (lane == 31) warp_tot[wid] = incl;
        __syncthreads();
        if (wid == 0) {
            int v = lane < nw ? warp_tot[lane] : 0;
            for (int o = 1; o < 32; o <<= 1) {
                const int u = __shfl_up_sync(0xffffffffu, v, o);
                if (lane >= o) v += u;
            }
            if (lane < nw) warp_tot[lane] = v;  // inclusive warp prefix
        }
        __syncthreads();
        const int rank = base_s + (wid > 0 ? warp_tot[wid - 1] : 0) + incl - on;
        if (idx < n) {
            double2 val = make_double2(0.0, 0.0);
            if (on) {
                const unsigned long long G = 0x9E3779B97F4A7C15ULL;
                const unsigned long long d1 = splitmix_out(state + (2ULL * (unsigned long long)rank + 1ULL) * G);
                const unsigned long long d2 = splitmix_out(state + (2ULL * (unsigned long long)rank + 2ULL) * G);
                double u1 = u53(d1);
                const double u2 = u53(d2);
                u1 = fmax(u1, 2.2250738585072014e-308);
                const double rad = sqrt(-2.0 * log(u1));
                const double th = 2.0 * 3.14159265358979323846 * u2;
                double sn, csv;
                sincos(th, &sn, &csv);
                double2 noise = make_double2(rad * csv, rad * sn);
                if (colored) {
                    double2 c = cs[idx];
                    c = make_double2(alpha * c.x + beta * noise.x, alpha * c.y + beta * noise.y);
                    cs[idx] = c;
                    val = c;
                } else {
                    val = noise;
                }
                const double w = weights[idx];
                out[idx] = make_double2(w * val.x, w * val.y);
                dd_add(tot, w * w * (val.x * val.x + val.y * val.y));
            } else {
                out[idx] = make_double2(0.0, 0.0);
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) base_s += warp_tot[nw - 1];
        __syncthreads();
    }
    DD t = block_dd(tot);
    if (threadIdx.x == 0) {
        const double total = fmax(t.s + t.c, 1e-16);
        scale_s = sqrt(energy_target / total);
    }
    __syncthreads();
    const double sc = scale_s;
    for (int idx = threadIdx.x; idx < n; idx += blockDim.x) {
        double2 v = out[idx];
        out[idx] = make_double2(v.x * sc, v.y * sc);
        if (colored) { double2 c = cs[idx]; cs[idx] = make_double2(c.x * sc, c.y * sc); }
    }
}

// Shell-binned energy spectrum of the kept-mode state with the reference's
// binning (spectral_analysis.c:103-123): bin (int)(|k| + 0.5) for bins < nbins,
// per-mode energy 0.5 (|u_hat|^2 + |v_hat|^2) with psi = -omega/k^2,
// u_hat = i ky psi, v_hat = -i kx psi (spectral_core.c:17-31).  Wavenumbers in
// FP64 as the reference's tables; per-block shared-memory bins, then one
// atomic per bin and block.  dynamic smem = nbins doubles.
template <typename T>
__global__ void k_energy_spectrum(Geo g, const typename CT<T>::C* W, int nbins, double* bins) {
    extern __shared__ double sbin[];
    for (int b = threadIdx.x; b < nbins; b += blockDim.x) sbin[b] = 0.0;
    __syncthreads();
    const long long n = (long long)g.Kx * g.Ky;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n; idx += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(idx / g.Ky), jj = (int)(idx - (long long)i * g.Ky);
        const int j = kept_j(g, jj);
        const double kx = 2.0 * 3.14159265358979323846 * i / g.Lx;
        const double ky = (j <= g.ny / 2) ? 2.0 * 3.14159265358979323846 * j / g.Ly
                                          : 2.0 * 3.14159265358979323846 * (j - g.ny) / g.Ly;
        const double k2 = k2sum(kx, ky);
        const int bin = (int)(sqrt(k2) + 0.5);
        if (bin >= nbins || k2 <= 1e-12) continue;
        const typename CT<T>::C w = W[(size_t)i * g.Ky + jj];
        const double px = -(double)w.x / k2, py = -(double)w.y / k2;
        const double p2 = px * px + py * py;
        atomicAdd(&sbin[bin], 0.5 * (ky * ky * p2 + kx * kx * p2));
    }
    __syncthreads();
    for (int b = threadIdx.x; b < nbins; b += blockDim.x)
        if (sbin[b] != 0.0) atomicAdd(&bins[b], sbin[b]);
}

// modes per bin over the whole half spectrum [nky][nkx] (the reference counts
// every mode, dealiased or not, spectral_analysis.c:116-121)
__global__ void k_spectrum_counts(Geo g, int nbins, int* counts) {
    const long long n = (long long)g.nkx * g.nky;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n; idx += (long long)gridDim.x * blockDim.x) {
        const int j = (int)(idx / g.nkx), i = (int)(idx - (long long)j * g.nkx);
        const double kx = 2.0 * 3.14159265358979323846 * i / g.Lx;
        const double ky = (j <= g.ny / 2) ? 2.0 * 3.14159265358979323846 * j / g.Ly
                                          : 2.0 * 3.14159265358979323846 * (j - g.ny) / g.Ly;
        const int bin = (int)(sqrt(k2sum(kx, ky)) + 0.5);
        if (bin < nbins) atomicAdd(&counts[bin], 1);
    }
}

// spectral truncation of a fine state onto a coarse grid of the same box: the
// coarse kept modes are a subset of the fine kept modes (same physical kx, ky)
template <typename T>
__global__ void k_filter(Geo gf, const typename CT<T>::C* Wf, Geo gc, typename CT<T>::C* Wc) {
    const long long n = (long long)gc.Kx * gc.Ky;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n; idx += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(idx / gc.Ky), jj = (int)(idx - (long long)i * gc.Ky);
        const int j = kept_j(gc, jj);
        const int ky = (j <= gc.ny / 2) ? j : j - gc.ny;
        const int jf = ky >= 0 ? ky : ky + gf.ny;
        const int jjf = kept_jj(gf, jf);
        Wc[idx] = (i < gf.Kx && jjf >= 0) ? Wf[(size_t)i * gf.Ky + jjf] : cmake<typename CT<T>::C>(0.0, 0.0);
    }
}

// W[kept] += spec[j][i] (an FP64 half spectrum in the reference layout)


#endif  // NSG_NO_AUX_KERNELS

}  // namespace nsg
