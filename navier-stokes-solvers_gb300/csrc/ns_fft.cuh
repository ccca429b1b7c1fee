// Shared-memory Stockham FFT engine for sm_103a (FP32 and FP64).
//
// One CTA transforms B independent sequences of length L (a power of two)
// held in shared memory.  Each transform is owned by TT = L / E threads; every
// thread keeps E complex values in registers per pass and exchanges them
// through shared memory between passes (load -> sync -> butterflies -> store ->
// sync).  Passes use radix min(E, remaining) in {16, 8, 4, 2}, so a length-2048
// transform with E = 16 takes three passes (16, 16, 8).
//
// Pass p with radix R over Ns = product of earlier radices (Stockham autosort,
// output in natural order):
//   butterfly j in [0, L/R):  a_r = X[j + r L/R]  (r < R)
//                             a_r *= W_{Ns R}^{+-(j mod Ns) r}
//                             a   = DFT_R(a)
//                             Y[(j - j mod Ns) R + j mod Ns + r Ns] = a_r
// Forward uses W = exp(-2 pi i / n), backward its conjugate; both unnormalised.
// Twiddles come from a per-length table tw[t] = exp(-2 pi i t / L) generated in
// FP64 on the device and rounded once to the working precision.
//
// Shared-memory addresses are padded by one element every 16 (spad) so the
// strided butterfly stores of the early passes spread over the banks.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace nsg {

template <typename T> struct CT;
template <> struct CT<float> { typedef float2 C; };
template <> struct CT<double> { typedef double2 C; };

template <typename C> __device__ __forceinline__ C cadd(C a, C b) { C r; r.x = a.x + b.x; r.y = a.y + b.y; return r; }
template <typename C> __device__ __forceinline__ C csub(C a, C b) { C r; r.x = a.x - b.x; r.y = a.y - b.y; return r; }
template <typename C> __device__ __forceinline__ C cmul(C a, C b) {
    C r;
    r.x = a.x * b.x - a.y * b.y;
    r.y = a.x * b.y + a.y * b.x;
    return r;
}
template <typename C, typename T> __device__ __forceinline__ C cscale(C a, T s) { C r; r.x = a.x * s; r.y = a.y * s; return r; }
template <typename C> __device__ __forceinline__ C cconj(C a) { C r; r.x = a.x; r.y = -a.y; return r; }
template <typename C> __device__ __forceinline__ C cmake(double x, double y) { C r; r.x = x; r.y = y; return r; }
// multiply by -i (forward) or +i (backward)
template <bool INV, typename C> __device__ __forceinline__ C cmul_mi(C a) {
    C r;
    if (INV) { r.x = -a.y; r.y = a.x; } else { r.x = a.y; r.y = -a.x; }
    return r;
}

__device__ __forceinline__ int spad(int i) { return i + (i >> 4); }
// padded shared-memory length of one transform of length L
__host__ __device__ inline int spad_len(int L) { return L + (L >> 4) + 4; }

// barrier between the passes of one transform, by sync mode sy:
//   0  the CTA barrier (every thread of the CTA runs the same passes);
//   1  a warp barrier (every transform of the CTA is owned by threads of a single warp);
//   (id << 16) | n  named barrier id (1..15) over n threads (a multiple of 32): the
//      threads of one group of transforms, which run their passes independently of
//      the CTA's other groups
__device__ __forceinline__ void fft_sync(int sy) {
    if (sy == 1) {
        __syncwarp();
    } else if (sy == 0) {
        __syncthreads();
    } else {
        asm volatile("bar.sync %0, %1;" ::"r"(sy >> 16), "r"(sy & 0xffff) : "memory");
    }
}

// ---------------------------------------------------------------- DFTs
template <bool INV, typename C> __device__ __forceinline__ void dft2(C* a) {
    C t = a[0];
    a[0] = cadd(t, a[1]);
    a[1] = csub(t, a[1]);
}

template <bool INV, typename C> __device__ __forceinline__ void dft4(C* a) {
    C t0 = cadd(a[0], a[2]);
    C t1 = csub(a[0], a[2]);
    C t2 = cadd(a[1], a[3]);
    C t3 = cmul_mi<INV>(csub(a[1], a[3]));
    a[0] = cadd(t0, t2);
    a[2] = csub(t0, t2);
    a[1] = cadd(t1, t3);
    a[3] = csub(t1, t3);
}

// y_k = E_k + W8^k O_k, y_{k+4} = E_k - W8^k O_k with E, O the DFT4 of even/odd inputs
template <bool INV, typename C> __device__ __forceinline__ void dft8(C* a) {
    typedef decltype(a[0].x) T;
    const T r = (T)0.70710678118654752440;
    C e[4] = {a[0], a[2], a[4], a[6]};
    C o[4] = {a[1], a[3], a[5], a[7]};
    dft4<INV>(e);
    dft4<INV>(o);
    C w1, w2, w3;
    if (!INV) {
        w1.x = r * (o[1].x + o[1].y); w1.y = r * (o[1].y - o[1].x);
        w3.x = r * (o[3].y - o[3].x); w3.y = -r * (o[3].x + o[3].y);
    } else {
        w1.x = r * (o[1].x - o[1].y); w1.y = r * (o[1].x + o[1].y);
        w3.x = -r * (o[3].x + o[3].y); w3.y = r * (o[3].x - o[3].y);
    }
    w2 = cmul_mi<INV>(o[2]);
    a[0] = cadd(e[0], o[0]); a[4] = csub(e[0], o[0]);
    a[1] = cadd(e[1], w1);   a[5] = csub(e[1], w1);
    a[2] = cadd(e[2], w2);   a[6] = csub(e[2], w2);
    a[3] = cadd(e[3], w3);   a[7] = csub(e[3], w3);
}

// y_k = E_k + W16^k O_k, y_{k+8} = E_k - W16^k O_k
template <bool INV, typename C> __device__ __forceinline__ void dft16(C* a) {
    typedef decltype(a[0].x) T;
    const T c1 = (T)0.92387953251128675613;  // cos(pi/8)
    const T s1 = (T)0.38268343236508977173;  // sin(pi/8)
    const T r = (T)0.70710678118654752440;
    C e[8], o[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) { e[k] = a[2 * k]; o[k] = a[2 * k + 1]; }
    dft8<INV>(e);
    dft8<INV>(o);
    const T sg = INV ? (T)1 : (T)-1;  // sign of the imaginary part of W16^k for k in (0,8)
    C w[8];
    w[0] = cmake<C>(1.0, 0.0);
    w[1] = cmake<C>(c1, sg * s1);
    w[2] = cmake<C>(r, sg * r);
    w[3] = cmake<C>(s1, sg * c1);
    w[4] = cmake<C>(0.0, sg);
    w[5] = cmake<C>(-s1, sg * c1);
    w[6] = cmake<C>(-r, sg * r);
    w[7] = cmake<C>(-c1, sg * s1);
    C ow[8];
    ow[0] = o[0];
    ow[4] = cmul_mi<INV>(o[4]);
#pragma unroll
    for (int k = 1; k < 8; ++k)
        if (k != 4) ow[k] = cmul(o[k], w[k]);
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        a[k] = cadd(e[k], ow[k]);
        a[k + 8] = csub(e[k], ow[k]);
    }
}

template <int R, bool INV, typename C> __device__ __forceinline__ void dftR(C* a) {
    if (R == 2) dft2<INV>(a);
    else if (R == 4) dft4<INV>(a);
    else if (R == 8) dft8<INV>(a);
    else dft16<INV>(a);
}

// ---------------------------------------------------------------- passes
// Load this thread's butterflies of a radix-R pass: v[q R + r] = X[j_q + r L/R], j_q = t + q TT
template <int E, int R, typename C>
__device__ __forceinline__ void pass_load(C (&v)[E], const C* sb, int L, int t, int TT) {
    const int LR = L / R;
#pragma unroll
    for (int q = 0; q < E / R; ++q) {
        const int j = t + q * TT;
#pragma unroll
        for (int r = 0; r < R; ++r) v[q * R + r] = sb[spad(j + r * LR)];
    }
}

template <int E, int R, bool INV, typename C>
__device__ __forceinline__ void pass_compute_store(C (&v)[E], C* sb, int L, int Ns, int t, int TT,
                                                   const C* __restrict__ tw) {
#pragma unroll
    for (int q = 0; q < E / R; ++q) {
        const int j = t + q * TT;
        const int k = j & (Ns - 1);
        C* a = &v[q * R];
        if (Ns > 1) {
            const int step = (L / (Ns * R)) * k;
#pragma unroll
            for (int r = 1; r < R; ++r) {
                C w = __ldg(&tw[step * r]);
                if (INV) w.y = -w.y;
                a[r] = cmul(a[r], w);
            }
        }
        dftR<R, INV>(a);
        const int base = (j - k) * R + k;
#pragma unroll
        for (int r = 0; r < R; ++r) sb[spad(base + r * Ns)] = a[r];
    }
}

template <int LOGE> struct ConstLog;

// In-place FFT of the sequence at sb (padded, natural order in and out).
// Every thread that the sync mode sy (fft_sync) names must call this; thread
// t < TT of this transform, TT = L / E.  With sy != 0 the passes synchronise
// only the warp or the group, and the caller synchronises the CTA before other
// threads read the result.
template <int E, bool INV, typename C>
__device__ void fft_smem(C* sb, int L, int logL, int t, int TT, const C* __restrict__ tw, int ws = 0) {
    C v[E];
    const int logE = (E == 16) ? 4 : (E == 8) ? 3 : (E == 4) ? 2 : 1;
    int Ns = 1;
    int rem = logL;
    while (rem > 0) {
        const int lr = rem < logE ? rem : logE;
        if (lr == 4) {
            if constexpr (E >= 16) {
                pass_load<E, 16>(v, sb, L, t, TT);
                fft_sync(ws);
                pass_compute_store<E, 16, INV>(v, sb, L, Ns, t, TT, tw);
            }
        } else if (lr == 3) {
            if constexpr (E >= 8) {
                pass_load<E, 8>(v, sb, L, t, TT);
                fft_sync(ws);
                pass_compute_store<E, 8, INV>(v, sb, L, Ns, t, TT, tw);
            }
        } else if (lr == 2) {
            if constexpr (E >= 4) {
                pass_load<E, 4>(v, sb, L, t, TT);
                fft_sync(ws);
                pass_compute_store<E, 4, INV>(v, sb, L, Ns, t, TT, tw);
            }
        } else {
            pass_load<E, 2>(v, sb, L, t, TT);
            fft_sync(ws);
            pass_compute_store<E, 2, INV>(v, sb, L, Ns, t, TT, tw);
        }
        fft_sync(ws);
        Ns <<= lr;
        rem -= lr;
    }
}

// ------------------------------------------------ mixed-radix lengths
// Lengths that are not powers of two (any L whose prime factors are all small:
// the reference's FFTW accepts every length) use the same Stockham recurrence
// with a per-length list of radices, packed one per byte (pass p in byte p of
// ra for p < 8, of rb for p >= 8; at most 16 passes).  Radices 2, 3, 4, 5, 7 and
// 8 run from registers; any other (prime) radix R runs as a direct R-point sum.
// Each pass reads one buffer and writes the other (sb and a scratch sequence sc
// of the same padded length), so a thread's butterflies need not fit a fixed
// register budget: thread t of TT takes butterflies t, t + TT, ...  The result
// ends in sb.  The roots of unity of the odd radices are entries of the same
// FP64-generated twiddle table, W_R^m = tw[m L / R].

__device__ __forceinline__ int mr_radix(unsigned long long ra, unsigned long long rb, int p) {
    return (int)(((p < 8) ? (ra >> (8 * p)) : (rb >> (8 * (p - 8)))) & 0xffULL);
}

template <int R, bool INV, typename C>
__device__ __forceinline__ void dft_odd(C* a, const C* __restrict__ tw, int L) {
    const int s = L / R;
    C y[R];
#pragma unroll
    for (int q = 0; q < R; ++q) {
        C acc = a[0];
#pragma unroll
        for (int r = 1; r < R; ++r) {
            C w = __ldg(&tw[((q * r) % R) * s]);
            if (INV) w.y = -w.y;
            acc = cadd(acc, cmul(a[r], w));
        }
        y[q] = acc;
    }
#pragma unroll
    for (int q = 0; q < R; ++q) a[q] = y[q];
}

template <int R, bool INV, typename C>
__device__ __forceinline__ void mr_pass(const C* src, C* dst, int L, int Ns, int t, int TT, const C* __restrict__ tw) {
    const int LR = L / R;
    const int tstep = L / (Ns * R);
    for (int j = t; j < LR; j += TT) {
        const int k = j % Ns;
        C a[R];
#pragma unroll
        for (int r = 0; r < R; ++r) a[r] = src[spad(j + r * LR)];
        if (Ns > 1) {
#pragma unroll
            for (int r = 1; r < R; ++r) {
                C w = __ldg(&tw[tstep * k * r]);
                if (INV) w.y = -w.y;
                a[r] = cmul(a[r], w);
            }
        }
        if constexpr (R == 3 || R == 5 || R == 7) dft_odd<R, INV>(a, tw, L);
        else dftR<R, INV>(a);
        const int base = (j - k) * R + k;
#pragma unroll
        for (int r = 0; r < R; ++r) dst[spad(base + r * Ns)] = a[r];
    }
}

// any radix R as the direct sum y_q = sum_r W_R^{qr} W_{Ns R}^{kr} x_r
template <bool INV, typename C>
__device__ void mr_pass_direct(const C* src, C* dst, int L, int R, int Ns, int t, int TT, const C* __restrict__ tw) {
    const int LR = L / R;
    const int tstep = L / (Ns * R);
    for (int j = t; j < LR; j += TT) {
        const int k = j % Ns;
        const int base = (j - k) * R + k;
        for (int q = 0; q < R; ++q) {
            C acc = src[spad(j)];
            for (int r = 1; r < R; ++r) {
                C x = src[spad(j + r * LR)];
                C w = __ldg(&tw[(tstep * k * r) % L]);
                C v = __ldg(&tw[((q * r) % R) * LR]);
                if (INV) { w.y = -w.y; v.y = -v.y; }
                acc = cadd(acc, cmul(cmul(x, w), v));
            }
            dst[spad(base + q * Ns)] = acc;
        }
    }
}

// In-place (through sc) FFT of the sequence at sb; every thread that the sync
// mode ws names calls it (it synchronises), thread t < TT of this sequence.
template <bool INV, typename C>
__device__ void fft_smem_mr(C* sb, C* sc, int L, unsigned long long ra, unsigned long long rb, int np, int t, int TT,
                            const C* __restrict__ tw, int ws = 0) {
    C* src = sb;
    C* dst = sc;
    int Ns = 1;
    for (int p = 0; p < np; ++p) {
        const int R = mr_radix(ra, rb, p);
        switch (R) {
            case 2: mr_pass<2, INV>(src, dst, L, Ns, t, TT, tw); break;
            case 3: mr_pass<3, INV>(src, dst, L, Ns, t, TT, tw); break;
            case 4: mr_pass<4, INV>(src, dst, L, Ns, t, TT, tw); break;
            case 5: mr_pass<5, INV>(src, dst, L, Ns, t, TT, tw); break;
            case 7: mr_pass<7, INV>(src, dst, L, Ns, t, TT, tw); break;
            case 8: mr_pass<8, INV>(src, dst, L, Ns, t, TT, tw); break;
            default: mr_pass_direct<INV>(src, dst, L, R, Ns, t, TT, tw); break;
        }
        fft_sync(ws);
        C* x = src;
        src = dst;
        dst = x;
        Ns *= R;
    }
    if (src != sb) {
        for (int i = t; i < L; i += TT) sb[spad(i)] = src[spad(i)];
        fft_sync(ws);
    }
}

// Radix list of a length for fft_smem_mr: 8s, then 4, 2, 3, 5, 7, then the
// remaining prime factors in increasing order.  Returns the number of passes,
// or -1 when a prime factor exceeds max_prime or more than 16 passes are needed.
static inline int mr_plan(int L, int max_prime, unsigned long long* ra, unsigned long long* rb) {
    int rad[64];
    int n = 0, m = L;
    while (m % 8 == 0 && n < 64) { rad[n++] = 8; m /= 8; }
    while (m % 4 == 0 && n < 64) { rad[n++] = 4; m /= 4; }
    while (m % 2 == 0 && n < 64) { rad[n++] = 2; m /= 2; }
    for (int p = 3; p <= m && n < 64; p += 2) {
        while (m % p == 0 && n < 64) {
            if (p > max_prime) return -1;
            rad[n++] = p;
            m /= p;
        }
    }
    if (m != 1 || n > 16) return -1;
    *ra = 0;
    *rb = 0;
    for (int p = 0; p < n; ++p) {
        if (p < 8) *ra |= (unsigned long long)rad[p] << (8 * p);
        else *rb |= (unsigned long long)rad[p] << (8 * (p - 8));
    }
    return n;
}

}  // namespace nsg
