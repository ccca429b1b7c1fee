// Register-resident stage kernels (the hot path at nx = 2048 / ny = 2048).
//
// Each RK stage is one row pass (x direction) and one column pass (y
// direction).  Both keep each transform's points in registers and exchange
// them through padded shared-memory buffers (conflict-free pitches).  Every
// transform runs through one forward body: an inverse is conj(DFT(conj x)).
//
//   k_row_t  FP32 row pass: one warp per row, 1024-point half-length transform
//            as a 32 x 32 four-step FFT (32 points per thread).  Inboxes filled
//            by cp.async; Jacobian operands and per-lane twiddles in tensor memory.
//   k_row_w  FP64 row pass: the same transform with the Jacobian operands in
//            shared memory and the next field staged in registers.
//   k_col_q  FP32 column pass: four warps per kept kx column, 2048-point transform
//            as 16 x 16 x 8 (16 points per thread), all columns in flight at once.
//   k_col_w  FP64 column pass: two warps per column, 32 x 64 four-step FFT.
// The forward's output layout equals its input layout for the 32 x 32 row
// transform, so the row pass forms the Jacobian in registers between the
// inverse and forward transforms; the column pass runs its RK stage algebra on
// the forward's output and builds the inverse inputs per mode.
#pragma once
#include "ns_kernels.cuh"

#ifndef NSG_RT_SPREAD
#define NSG_RT_SPREAD 1   // FP32 row pass: equal contiguous row ranges per CTA (measured neutral at 2048^2)
#endif

namespace nsg {

// ------------------------------------------------------------ streamed loads
// Global loads that do not allocate in L1: the column pass streams ~50 KB per
// column through the SM, which would otherwise evict the twiddle and
// wavenumber tables that every FFT pass re-reads from L1.
#ifndef NSG_STREAM
#define NSG_STREAM 1
#endif
#if NSG_STREAM
__device__ __forceinline__ float2 ld_stream(const float2* p) {
    float2 v;
    asm("ld.global.L1::no_allocate.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "l"(p));
    return v;
}
__device__ __forceinline__ double2 ld_stream(const double2* p) {
    double2 v;
    asm("ld.global.L1::no_allocate.v2.f64 {%0, %1}, [%2];" : "=d"(v.x), "=d"(v.y) : "l"(p));
    return v;
}
__device__ __forceinline__ float ld_stream(const float* p) {
    float v;
    asm("ld.global.L1::no_allocate.f32 %0, [%1];" : "=f"(v) : "l"(p));
    return v;
}
__device__ __forceinline__ double ld_stream(const double* p) {
    double v;
    asm("ld.global.L1::no_allocate.f64 %0, [%1];" : "=d"(v) : "l"(p));
    return v;
}
#else
template <typename X> __device__ __forceinline__ X ld_stream(const X* p) { return *p; }
#endif

// wait until the kernel this one was launched after (programmatic stream
// serialization) has completed and its writes are visible
__device__ __forceinline__ void wait_previous_kernel() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// ------------------------------------------------------------------ DFT32
// cos(pi k/16), k = 0..8
__device__ __forceinline__ double cpi16(int k) {
    switch (k) {
        case 0: return 1.0;
        case 1: return 0.98078528040323044913;
        case 2: return 0.92387953251128675613;
        case 3: return 0.83146961230254523708;
        case 4: return 0.70710678118654752440;
        case 5: return 0.55557023301960222474;
        case 6: return 0.38268343236508977173;
        case 7: return 0.19509032201612826785;
        default: return 0.0;
    }
}

// y_k = E_k + W32^k O_k, y_{k+16} = E_k - W32^k O_k (E, O: DFT16 of even/odd inputs)
template <bool INV, typename C> __device__ __forceinline__ void dft32(C* a) {
    typedef decltype(a[0].x) T;
    C e[16], o[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) {
        e[k] = a[2 * k];
        o[k] = a[2 * k + 1];
    }
    dft16<INV>(e);
    dft16<INV>(o);
#pragma unroll
    for (int k = 0; k < 16; ++k) {
        C w;
        if (k == 0) {
            w = o[0];
        } else if (k == 8) {
            w = cmul_mi<INV>(o[8]);
        } else {
            // W32^k = cos(pi k/16) -+ i sin(pi k/16)
            const T cr = (k < 8) ? (T)cpi16(k) : (T)-cpi16(16 - k);
            const T si = (k < 8) ? (T)cpi16(8 - k) : (T)cpi16(k - 8);
            C tw;
            tw.x = cr;
            tw.y = INV ? si : -si;
            w = cmul(o[k], tw);
        }
        a[k] = cadd(e[k], w);
        a[k + 16] = csub(e[k], w);
    }
}

// ============================================================ k_row_w
// NW warps per CTA, one row each (rows y0 .. y0 + NW - 1 of a round), persistent
// over rounds.  F and G are kx-column-contiguous ([Kx][ny]), so the CTA moves
// them together: thread (kb, w) = (tid / NW, tid % NW) handles columns
// k = kb + 32 i of row y0 + w, and for each column the NW consecutive rows are
// one run of NW elements (64 bytes in FP32).  The next field is fetched into
// registers while the current one transforms, then deposited into the warps'
// exchange buffers; every other step of a row stays inside its warp.
// dynamic smem: tw [32][33] (W_1024^{t k1}), twh [1024]; per warp S [32][33]
//               exchange, R [1024] (psi_x, then psi_x * omega_y), Q [1024] (psi_y);
//               kx [704]
#ifndef NSG_RW_WARPS_F32
#define NSG_RW_WARPS_F32 8
#endif
#define NSG_RW_WARPS_F64 3
#define NSG_RW_KXMAX 704   // kept kx columns at nx = 2048 (684) rounded up to 32

// warps that share rows (and barriers): groups of NSG_RW_GROUP warps in FP32
// (4 rows x 8 bytes: one 32-byte sector per column), the whole CTA in FP64
#ifndef NSG_RW_GROUP
#define NSG_RW_GROUP 4
#endif
template <typename T> __host__ __device__ constexpr int rw_warps() { return sizeof(T) == 4 ? NSG_RW_WARPS_F32 : NSG_RW_WARPS_F64; }
template <typename T> __host__ __device__ constexpr int rw_group() { return sizeof(T) == 4 ? NSG_RW_GROUP : NSG_RW_WARPS_F64; }
// per-warp block S | R | Q, padded so that group-wide accesses (GW lanes at one
// offset in the GW warps' S, 32 / GW columns) hit distinct banks
template <typename T> __host__ __device__ constexpr int rw_wstride() { return 32 * 33 + 2048 + 16 / rw_group<T>(); }
template <typename T> __host__ __device__ constexpr size_t rw_smem_bytes() {
    return (size_t)(32 * 33 + 1024 + rw_warps<T>() * rw_wstride<T>()) * (sizeof(T) == 4 ? sizeof(float2) : sizeof(double2)) +
           (size_t)NSG_RW_KXMAX * sizeof(T);
}
// barrier over one group of GW warps (named barrier 1 + group; the CTA barrier when GW is the whole CTA)
template <int GW, int NW> __device__ __forceinline__ void group_sync(int grp) {
    if (GW == NW) {
        __syncthreads();
    } else {
        asm volatile("bar.sync %0, %1;" ::"r"(grp + 1), "r"(32 * GW) : "memory");
    }
}

// flat index k < 1024 inside a [32][33] exchange buffer
__device__ __forceinline__ int sx(int k) { return (k >> 5) * 33 + (k & 31); }

// one 1024-point transform inside a warp: a[] holds x[lane + 32 n1] on entry and
// X[lane + 32 k2] on exit
template <bool INV, typename C>
__device__ __forceinline__ void warp_fft1024(C (&a)[32], C* S, const C* tw, int lane) {
    dft32<INV>(a);
#pragma unroll
    for (int k1 = 1; k1 < 32; ++k1) {
        C w = tw[k1 * 33 + lane];
        if (INV) w.y = -w.y;
        a[k1] = cmul(a[k1], w);
    }
#pragma unroll
    for (int k1 = 0; k1 < 32; ++k1) S[k1 * 33 + lane] = a[k1];
    __syncwarp();
#pragma unroll
    for (int n2 = 0; n2 < 32; ++n2) a[n2] = S[lane * 33 + n2];
    __syncwarp();
    dft32<INV>(a);
}

// kept kx columns at nx = 2048: floor(2 * 1025 / 3) + 1 (spectral_initialization.c:46-49)
#define NSG_RW_KX 684

// fetch X_f[k] of row y, k = kb + 32 i < NSG_RW_KX, into registers (F kx-column-contiguous)
template <typename C>
__device__ __forceinline__ void rows_fetch(C (&pf)[NSG_RW_KXMAX / 32], const C* __restrict__ src, size_t ny, int y,
                                           bool ok, int kb) {
#pragma unroll
    for (int i = 0; i < NSG_RW_KXMAX / 32; ++i) {
        const int k = kb + 32 * i;
        pf[i] = (ok && k < NSG_RW_KX) ? __ldg(&src[(size_t)k * ny + y]) : cmake<C>(0.0, 0.0);
    }
}

// deposit the fetched values (times i kx when dx) into row w's exchange buffer Sw
template <typename T, typename C>
__device__ __forceinline__ void rows_deposit(const C (&pf)[NSG_RW_KXMAX / 32], C* Sw, int dx, const T* kxv, int kb) {
#pragma unroll
    for (int i = 0; i < NSG_RW_KXMAX / 32; ++i) {
        const int k = kb + 32 * i;
        if (k < NSG_RW_KX) {
            C x = pf[i];
            if (dx) {
                const T kx = kxv[k];
                C d;
                d.x = -kx * x.y;
                d.y = kx * x.x;
                x = d;
            }
            Sw[i * 33 + kb] = x;
        }
    }
}

// pack the half-length inverse input Z[lane + 32 n1] = (X[k] + conj X[H-k]) + i e^{+2 pi i k/nx} (X[k] - conj X[H-k])
// from the half spectrum X[k], k < NSG_RW_KX, held in S, and return conj Z (the
// inverse transform runs as conj(DFT(conj Z))).  k = lane + 32 n1 sits at
// S[33 n1 + lane]; H - k at S[33 (31 - n1) + ob] with ob = 32 - lane (lane > 0)
// or 33 (lane = 0), so every address is a per-thread base plus a constant.
template <typename T, typename C>
__device__ __forceinline__ void row_pack(C (&a)[32], const C* S, const C* twh, int lane) {
    const int ob = lane ? 32 - lane : 33;
    const C zero = cmake<C>(0.0, 0.0);
#pragma unroll
    for (int n1 = 0; n1 < 32; ++n1) {
        const int k = lane + 32 * n1;
        const C xa = (k < NSG_RW_KX) ? S[33 * n1 + lane] : zero;
        const C xb = (k > 0 && 1024 - k < NSG_RW_KX) ? S[33 * (31 - n1) + ob] : zero;
        if (n1 == 0 && lane == 0) {
            a[n1] = cmake<C>(xa.x, -xa.x);  // conj of Re X[0] (1 + i); the Nyquist bin is masked
        } else {
            const C e = twh[k];  // exp(-2 pi i k/nx) = conj of the pack twiddle
            const C A = cadd(xa, cconj(xb));
            const C dd = csub(xa, cconj(xb));
            // D = dd * conj(e); Z = (A.x - D.y, A.y + D.x); a = conj Z
            const T Dx = dd.x * e.x + dd.y * e.y;
            const T Dy = dd.y * e.x - dd.x * e.y;
            a[n1] = cmake<C>(A.x - Dy, -(A.y + Dx));
        }
    }
    __syncwarp();
}

template <typename T>
__global__ void __launch_bounds__(32 * rw_warps<T>(), 1) k_row_w(Geo g, RowArgs<T> a) {
    typedef typename CT<T>::C C;
    constexpr int NW = rw_warps<T>();
    constexpr int GW = rw_group<T>();
    constexpr int WS = rw_wstride<T>();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C* tw = reinterpret_cast<C*>(smem_raw);
    C* twh_s = tw + 32 * 33;                          // exp(-2 pi i k/nx), k < 1024
    C* S0 = twh_s + 1024;                             // warp w's block at S0 + w * WS
    T* kx_s = reinterpret_cast<T*>(twh_s + 1024 + NW * WS);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    C* S = S0 + warp * WS;
    C* R = S + 32 * 33;
    C* Q = R + 1024;
    const int ny = g.ny;
    // group grp owns rows y0 + GW grp + w (w < GW); thread (kb, wme) of the group
    // moves columns kb + 32 i of row wme
    const int grp = warp / GW;
    const int tg = threadIdx.x - grp * 32 * GW;
    const int kb = tg / GW, wme = tg - kb * GW;
    C* Sg = S0 + grp * GW * WS;                       // the group's first warp block
    C* Sme = Sg + wme * WS;

    // constant tables first (they do not depend on the previous kernel)
    for (int i = threadIdx.x; i < 1024; i += blockDim.x) {
        const int k1 = i >> 5, t = i & 31;
        tw[k1 * 33 + t] = a.twr[t * k1];
        twh_s[i] = a.twh[i];
    }
    for (int i = threadIdx.x; i < NSG_RW_KXMAX; i += blockDim.x) kx_s[i] = (i < NSG_RW_KX) ? a.kxv[i] : (T)0;
    wait_previous_kernel();
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        if (a.marker == 1) {
            a.ds->step_cur = a.ds->step_next;
            a.ds->step_next = a.ds->step_next + (a.ds->fsub ? a.ds->fsub : 1ULL);
        } else if (a.marker == 2) {
            a.ds->maxvel2 = 0ULL;
        }
    }

    // field order q = 0..3: psi_x (F[0], d/dx), psi_y (F[1]), omega_y (F[3]), omega_x (F[2], d/dx)
    T vmax2 = (T)0;
    C v[32];
    C pf[NSG_RW_KXMAX / 32];
    const int ystep = gridDim.x * NW;
    __syncthreads();  // tables in place
    int y0 = blockIdx.x * NW + grp * GW;  // this group's first row of the round
    rows_fetch(pf, a.F[0], (size_t)ny, y0 + wme, y0 + wme < ny, kb);
    for (; y0 < ny; y0 += ystep) {
        const int y = y0 + (warp - grp * GW);
        // q = 0..3: inverse transforms (conj(DFT(conj Z))) of psi_x, psi_y,
        // omega_y, omega_x; q = 4: forward transform of the packed Jacobian.
        // One transform body serves all five.
#pragma unroll 1
        for (int q = 0; q < 5; ++q) {
            if (q < 4) {
                const int f = (q < 2) ? q : 5 - q;
                const int dx = (f == 0 || f == 2);
                group_sync<GW, NW>(grp);  // every warp of the group is done with its exchange buffer
                rows_deposit<T>(pf, Sme, dx, kx_s, kb);
                group_sync<GW, NW>(grp);
                // fetch the next field (or the next round's psi_x) while this one transforms
                if (q < 3) {
                    rows_fetch(pf, a.F[(q + 1 < 2) ? q + 1 : 4 - q], (size_t)ny, y0 + wme, y0 + wme < ny, kb);
                } else {
                    const int yn = y0 + ystep + wme;
                    rows_fetch(pf, a.F[0], (size_t)ny, yn, yn < ny, kb);
                }
                if (y < ny) row_pack<T>(v, S, twh_s, lane);
            }
            if (y >= ny) continue;
            warp_fft1024<false>(v, S, tw, lane);
            if (q == 4) break;
#pragma unroll
            for (int k = 0; k < 32; ++k) v[k].y = -v[k].y;
            if (q == 0) {
#pragma unroll
                for (int k = 0; k < 32; ++k) R[lane + 32 * k] = v[k];
            } else if (q == 1) {
#pragma unroll
                for (int k = 0; k < 32; ++k) {
                    if (a.cfl) {
                        const C px = R[lane + 32 * k];
                        vmax2 = fmax(vmax2, fmax(px.x * px.x + v[k].x * v[k].x, px.y * px.y + v[k].y * v[k].y));
                    }
                    Q[lane + 32 * k] = v[k];
                }
            } else if (q == 2) {
#pragma unroll
                for (int k = 0; k < 32; ++k) {
                    const C px = R[lane + 32 * k];
                    R[lane + 32 * k] = cmake<C>(px.x * v[k].x, px.y * v[k].y);
                }
            } else {
                // J = psi_x omega_y - psi_y omega_x, packed as w[m] = J[2m] + i J[2m+1]
#pragma unroll
                for (int k = 0; k < 32; ++k) {
                    const C p = R[lane + 32 * k];
                    const C py = Q[lane + 32 * k];
                    v[k] = cmake<C>(p.x - py.x * v[k].x, p.y - py.y * v[k].y);
                }
            }
        }
        if (y < ny) {
#pragma unroll
            for (int k = 0; k < 32; ++k) S[k * 33 + lane] = v[k];
        }
        group_sync<GW, NW>(grp);
        // unpack the kept kx < Kx of the group's GW rows together: element e is
        // (k = e / GW, row y0 + e % GW), so consecutive threads write the GW
        // consecutive rows of one G column
        const T half = (T)0.5;
        const int nrows = (ny - y0 < GW) ? ny - y0 : GW;
        for (int e = tg; e < NSG_RW_KX * GW; e += 32 * GW) {
            const int k = e / GW, w = e - k * GW;
            if (w >= nrows) continue;
            const C* Sw = Sg + w * WS;
            const C wa = Sw[sx(k)];
            const C wb = Sw[sx((1024 - k) & 1023)];
            C ev, od;
            ev.x = half * (wa.x + wb.x);
            ev.y = half * (wa.y - wb.y);
            od.x = half * (wa.y + wb.y);
            od.y = -half * (wa.x - wb.x);
            a.G[(size_t)k * ny + y0 + w] = cadd(ev, cmul(od, twh_s[k]));
        }
    }
    if (a.cfl) {
        const double vm = warp_max((double)vmax2);
        if (lane == 0) atomicMax(&a.ds->maxvel2, (unsigned long long)__double_as_longlong(vm));
    }
}

// ============================================================ k_col_w
// ny = 2048: a team of 64 threads (two warps) per kept kx column.  The 2048-
// point transforms below synchronise the team with a named barrier, so several
// teams share one CTA (and its shared twiddle table) without waiting on each other.

// barrier over one 64-thread team (named barrier bid, 1 <= bid <= 15)
__device__ __forceinline__ void team_sync(int bid) { asm volatile("bar.sync %0, 64;" ::"r"(bid) : "memory"); }

// forward 2048-point transform: a[] = x[64 n1 + t] on entry (t = 32 h + lane),
// X[lane + 32 k2 + 1024 h] on exit; col is this team's exchange buffer, tw the
// shared table tw[k1 * 65 + t] = W_2048^{t k1} (k1 < 32, t < 64): consecutive
// threads read consecutive entries, and column t = 32 holds W_64^{k1}
template <typename C>
__device__ __forceinline__ void col_fwd2048(C (&a)[32], C* col, const C* tw, int t, int lane, int h, int bid) {
    dft32<false>(a);
#pragma unroll
    for (int k1 = 1; k1 < 32; ++k1) a[k1] = cmul(a[k1], tw[k1 * 65 + t]);
#pragma unroll
    for (int k1 = 0; k1 < 32; ++k1) col[k1 * 65 + t] = a[k1];
    team_sync(bid);
#pragma unroll
    for (int m = 0; m < 32; ++m) a[m] = col[lane * 65 + 2 * m + h];
    team_sync(bid);
    dft32<false>(a);
    if (h) {
#pragma unroll
        for (int k2 = 1; k2 < 32; ++k2) a[k2] = cmul(a[k2], tw[k2 * 65 + 32]);  // W_64^{k2} = W_2048^{32 k2}
    }
#pragma unroll
    for (int k2 = 0; k2 < 32; ++k2) col[h * 1056 + k2 * 33 + lane] = a[k2];
    team_sync(bid);
#pragma unroll
    for (int k2 = 0; k2 < 32; ++k2) {
        const C b = col[(1 - h) * 1056 + k2 * 33 + lane];
        a[k2] = h ? csub(b, a[k2]) : cadd(a[k2], b);  // E + W O  |  E - W O
    }
    team_sync(bid);
}

// ------------------------------------------------------------ cp.async staging
// Asynchronous global -> shared copies (no register staging); each thread
// waits for its own copies with cp_async_wait_all, a barrier publishes them.
__device__ __forceinline__ void cp_async(void* s, const float2* gp) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"((unsigned)__cvta_generic_to_shared(s)), "l"(gp)
                 : "memory");
}
__device__ __forceinline__ void cp_async(void* s, const double2* gp) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((unsigned)__cvta_generic_to_shared(s)), "l"(gp)
                 : "memory");
}
__device__ __forceinline__ void cp_async(void* s, const float* gp) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"((unsigned)__cvta_generic_to_shared(s)), "l"(gp)
                 : "memory");
}
__device__ __forceinline__ void cp_async(void* s, const double* gp) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"((unsigned)__cvta_generic_to_shared(s)), "l"(gp)
                 : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// ------------------------------------------------------------ tensor memory
// Per-thread storage in the 32x32b shape: a warp reaches the 32 lanes of its
// quarter (warp index mod 4), thread = lane, one 32-bit value per column.
__device__ __forceinline__ void tm_st16(unsigned ta, const float2 (&v)[32], int c) {
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, %16};" ::"r"(ta),
        "f"(v[8 * c + 0].x), "f"(v[8 * c + 0].y), "f"(v[8 * c + 1].x), "f"(v[8 * c + 1].y), "f"(v[8 * c + 2].x), "f"(v[8 * c + 2].y),
        "f"(v[8 * c + 3].x), "f"(v[8 * c + 3].y), "f"(v[8 * c + 4].x), "f"(v[8 * c + 4].y), "f"(v[8 * c + 5].x), "f"(v[8 * c + 5].y),
        "f"(v[8 * c + 6].x), "f"(v[8 * c + 6].y), "f"(v[8 * c + 7].x), "f"(v[8 * c + 7].y)
        : "memory");
}
__device__ __forceinline__ void tm_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

// issue a 16-column load (8 complex) into r without waiting
__device__ __forceinline__ void tm_ld16_issue(unsigned ta, float (&r)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
        : "=f"(r[0]), "=f"(r[1]), "=f"(r[2]), "=f"(r[3]), "=f"(r[4]), "=f"(r[5]), "=f"(r[6]), "=f"(r[7]), "=f"(r[8]), "=f"(r[9]),
          "=f"(r[10]), "=f"(r[11]), "=f"(r[12]), "=f"(r[13]), "=f"(r[14]), "=f"(r[15])
        : "r"(ta)
        : "memory");
}
// wait for the outstanding loads; the registers pass through the wait so that
// no use of them can be scheduled before it
__device__ __forceinline__ void tm_wait_ld(float (&r)[16]) {
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+f"(r[0]), "+f"(r[1]), "+f"(r[2]), "+f"(r[3]), "+f"(r[4]), "+f"(r[5]), "+f"(r[6]), "+f"(r[7]), "+f"(r[8]),
                   "+f"(r[9]), "+f"(r[10]), "+f"(r[11]), "+f"(r[12]), "+f"(r[13]), "+f"(r[14]), "+f"(r[15])
                 :
                 : "memory");
}
__device__ __forceinline__ void tm_wait_ld2(float (&r)[16], float (&s)[16]) {
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+f"(r[0]), "+f"(r[1]), "+f"(r[2]), "+f"(r[3]), "+f"(r[4]), "+f"(r[5]), "+f"(r[6]), "+f"(r[7]), "+f"(r[8]),
                   "+f"(r[9]), "+f"(r[10]), "+f"(r[11]), "+f"(r[12]), "+f"(r[13]), "+f"(r[14]), "+f"(r[15]), "+f"(s[0]),
                   "+f"(s[1]), "+f"(s[2]), "+f"(s[3]), "+f"(s[4]), "+f"(s[5]), "+f"(s[6]), "+f"(s[7]), "+f"(s[8]), "+f"(s[9]),
                   "+f"(s[10]), "+f"(s[11]), "+f"(s[12]), "+f"(s[13]), "+f"(s[14]), "+f"(s[15])
                 :
                 : "memory");
}


// Persistent column pass: one CTA per SM, NT teams of 64 threads, team q of
// CTA b takes the kept columns i = b + gridDim.x (q + NT r).  The CTA keeps the
// twiddle table W_2048^m and the kept ky values in shared memory (every
// transform reads 31-62 twiddles per thread, so they must not depend on L1
// hits).  Each team stages its column's omega_hat and hyperviscosity weights
// with cp.async before the kernel waits for the row pass, and the stage state
// WS and accumulator ACC into its exchange buffer once the forward transform
// has released it.  All five transforms of a column run through one forward
// transform body (an inverse is conj(DFT(conj x))), which keeps the kernel
// small enough for the instruction caches of five teams at different phases.
//
// dynamic smem: TW [32][65] C | per team: X [XL] C (FFT exchange, then WS | ACC),
// NS [Kyp] C (omega_hat at the step start, then the next stage's state) |
// per team SHV [Kyp] T | KYS [Kyp] T   (Kyp = Ky rounded up to a multiple of 4)
#define NSG_CW_EX 2112
#define NSG_CW_TW (32 * 65)
__host__ __device__ constexpr int cw_kyp(int Ky) { return (Ky + 3) & ~3; }
__host__ __device__ constexpr int cw_xl(int Ky) { return 2 * cw_kyp(Ky) > NSG_CW_EX ? 2 * cw_kyp(Ky) : NSG_CW_EX; }
template <typename T> __host__ __device__ constexpr int cw_teams() { return sizeof(T) == 4 ? 5 : 2; }
template <typename T> __host__ __device__ constexpr size_t cw_smem_bytes(int Ky) {
    return (size_t)(NSG_CW_TW + cw_teams<T>() * (cw_xl(Ky) + cw_kyp(Ky))) * (sizeof(T) == 4 ? sizeof(float2) : sizeof(double2)) +
           (size_t)(cw_teams<T>() + 1) * cw_kyp(Ky) * sizeof(T);
}

template <typename T, int STAGE, bool IFRK>
__global__ void __launch_bounds__(64 * cw_teams<T>(), 1) k_col_w(Geo g, ColArgs<T> a) {
    typedef typename CT<T>::C C;
    constexpr int NT = cw_teams<T>();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int Ky = g.Ky, Kyp = cw_kyp(Ky), XL = cw_xl(Ky), Kx = g.Kx;
    const int team = threadIdx.x >> 6, t = threadIdx.x & 63, lane = t & 31, h = t >> 5;
    const int bid = 1 + team;
    C* TW = reinterpret_cast<C*>(smem_raw);
    C* X = TW + NSG_CW_TW + team * (XL + Kyp);
    C* NS = X + XL;
    T* SHV = reinterpret_cast<T*>(TW + NSG_CW_TW + NT * (XL + Kyp)) + team * Kyp;
    T* KYS = reinterpret_cast<T*>(TW + NSG_CW_TW + NT * (XL + Kyp)) + NT * Kyp;
    const int hv = a.sp.hv, sfd = a.sp.sfd;
    __shared__ double s_dt;

    // constant tables, and the first column's omega_hat / weights: these were
    // written before the previous kernel (the row pass, which waited for them)
    for (int m = threadIdx.x; m < NSG_CW_TW; m += blockDim.x) {
        const int k1 = m / 65, tt = m - 65 * k1;
        TW[m] = a.twc[(tt * k1) & 2047];
    }
    for (int jj = threadIdx.x; jj < Ky; jj += blockDim.x) KYS[jj] = a.kyv[jj];
    const int cstride = gridDim.x * NT;
    int i = blockIdx.x + gridDim.x * team;
    if (i < Kx) {
        const size_t base = (size_t)i * Ky;
        for (int jj = t; jj < Ky; jj += 64) {
            cp_async(&NS[jj], &a.W0[base + jj]);
            if (hv) cp_async(&SHV[jj], &a.hvw[base + jj]);
        }
    }
    wait_previous_kernel();
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
            if (blockIdx.x == 0) a.ds->dt = dt;
        } else {
            dt = a.ds->dt;
        }
        s_dt = dt;
    }
    __syncthreads();  // tables and dt

    const double dt = s_dt;
    const StageCoef<T> sq = stage_coef<T>(a.sp, dt);
    C* __restrict__ W0 = a.W0;
    C* __restrict__ WS = a.WS;
    C* __restrict__ ACC = a.ACC;
    const C zero = cmake<C>(0.0, 0.0);

    for (bool first = true; i < Kx; i += cstride, first = false) {
        if (!first) {
            const size_t base = (size_t)i * Ky;
            for (int jj = t; jj < Ky; jj += 64) {
                cp_async(&NS[jj], &a.W0[base + jj]);
                if (hv) cp_async(&SHV[jj], &a.hvw[base + jj]);
            }
        }
        const T kx = __ldg(&a.kxv[i]);
        const size_t cbase = (size_t)i * Ky;
        C v[32];
        // q = -1: forward transform of the Jacobian column and the RK stage;
        // q = 0..3: inverse transforms of Omega, Omega_y, Psi, Psi_y
#pragma unroll 1
        for (int q = -1; q < 4; ++q) {
            const int f = (q + 2) & 3;
            if (q < 0) {
                const C* __restrict__ Gc = a.G + (size_t)i * 2048;
#pragma unroll
                for (int n1 = 0; n1 < 32; ++n1) v[n1] = ld_stream(&Gc[64 * n1 + t]);
            } else {
                // thread t builds modes j = 64 n1 + t; Psi = -w/k^2 is formed once
                // (written back to NS) and reused for Psi_y by the same thread
#pragma unroll
                for (int n1 = 0; n1 < 32; ++n1) {
                    const int j = 64 * n1 + t;
                    const int jj = kept_jj(g, j);
                    C x = zero;
                    if (jj >= 0) {
                        const T ky = KYS[jj];
                        C w = NS[jj];
                        if (f == 0) {
                            w = field_value<T, C>(0, w, kx, ky);
                            NS[jj] = w;
                        }
                        if (f == 1 || f == 3) {
                            x.x = -ky * w.y;
                            x.y = ky * w.x;
                        } else {
                            x = w;
                        }
                    }
                    v[n1] = cconj(x);
                }
            }
            col_fwd2048(v, X, TW, t, lane, h, bid);  // ends with a team barrier: X is free
            if (q >= 0) {
                C* __restrict__ Fc = a.F[f] + (size_t)i * 2048;
#pragma unroll
                for (int k2 = 0; k2 < 32; ++k2) Fc[lane + 32 * k2 + 1024 * h] = cconj(v[k2]);
                continue;
            }
            if (STAGE != 1) {
                for (int jj = t; jj < Ky; jj += 64) {
                    cp_async(&X[jj], &WS[cbase + jj]);
                    cp_async(&X[Kyp + jj], &ACC[cbase + jj]);
                }
            }
            cp_async_wait_all();
            team_sync(bid);  // the team's staged omega_hat, weights, WS and ACC

            // RK stage algebra (spectral_time_integration.c:50-100) on this
            // thread's forward outputs, modes j = lane + 32 k2 + 1024 h
#pragma unroll
            for (int k2 = 0; k2 < 32; ++k2) {
                const int j = lane + 32 * k2 + 1024 * h;
                const int jj = kept_jj(g, j);
                if (jj < 0) continue;
                const size_t s = cbase + jj;
                const C jh = v[k2];
                const C w0 = NS[jj];
                const C ws = (STAGE == 1) ? w0 : X[jj];
                const C acc0 = (STAGE == 1) ? zero : X[Kyp + jj];
                const T hw = hv ? SHV[jj] : (T)0;
                T sw = (T)0;
                C fb = zero;
                if (sfd) {
                    sw = a.sfdw[s];
                    fb = a.SFD[s];
                }
                const C wn = rk_stage_mode<T, STAGE, IFRK>(sq, jh, w0, ws, acc0, hw, sw, fb, k2sum(kx, KYS[jj]), ACC, WS, s);
                if (STAGE == 4) W0[s] = wn;
                NS[jj] = wn;
            }
            if (STAGE == 4 && (a.sp.forcing || sfd)) {
                // forcing increment (few low-|k| modes), then the SFD post-step, on omega_hat^{n+1}
                // columns beyond the shell only relax the SFD filter (and skip the
                // FP64 amplitude)
                const bool force_col = a.sp.forcing && (double)kx <= a.sp.f_kmax + 1e-9;
                const double f_amp = force_col ? a.sp.f_sigma * sqrt(dt / a.sp.fsub) : 0.0;
                double sa = 0.0;
                if (sfd) {
                    sa = dt / a.sp.sfd_tau;
                    sa = sa > 1.0 ? 1.0 : (sa < 0.0 ? 0.0 : sa);
                }
#pragma unroll 1
                for (int k2 = 0; k2 < 32 && (force_col || sfd); ++k2) {
                    const int j = lane + 32 * k2 + 1024 * h;
                    const int jj = kept_jj(g, j);
                    if (jj < 0) continue;
                    const size_t s = cbase + jj;
                    bool forced;
                    const C wn = post_step_mode(g, a, i, j, s, NS[jj], kx, KYS[jj], f_amp, sa, forced);
                    if (forced) {
                        W0[s] = wn;
                        NS[jj] = wn;
                    }
                }
            }
            team_sync(bid);  // NS complete for the inverse transforms; X is free again
        }
    }
    if (STAGE == 4 && blockIdx.x == 0 && threadIdx.x == 0) a.ds->t = a.ds->t + dt;
}

// ============================================================ k_col_q
// FP32 column pass at ny = 2048 or 4096 with N/128 warps (N/16 threads, 16
// points each) per kept kx column.  At 2048 every SM holds all of its columns at
// once (684 columns, 5 per SM), so the pass takes as long as one column's chain
// of five transforms and the RK algebra; four warps per column run that chain
// with half the serial work per thread of the two-warp teams (k_col_w), in the
// same shared memory per column.  At 4096 two columns of eight warps share an SM.
//
// N-point transform, N = 16 x 16 x M2 with TT = N/16 threads, M2 = TT/16
// (2048: 16 x 16 x 8; 4096: 16 x 16 x 16), thread t < TT, k1 = t & 15, hi = t >> 4:
//   pass A   t holds x[TT n1 + t] (n1 < 16): DFT16 over n1, times W_N^{t k1}
//   pass B1  thread (k1, m2 = hi) takes z[M2 m1 + m2] of column k1 (m1 < 16):
//            DFT16 over m1, times W_TT^{m2 q1}
//   pass B2  thread (k1, hi) takes the M2 values m2 of q1 = R hi + r (r < R = 16/M2):
//            DFT_M2 -> X[k1 + 16 q1 + 256 q2] in a[M2 r + q2]
// The exchange buffer holds [16][TT + 1] values; a pitch of TT + 1 makes every
// exchange store and load conflict-free (16 bank pairs, two wavefronts).
#ifndef NSG_COL_Q
#define NSG_COL_Q 1   // 0: the FP32 column pass at 2048 runs k_col_w
#endif
template <int NL> struct CQ {
    static constexpr int N = 1 << NL, TT = N / 16, M2 = TT / 16, R = 16 / M2, P = TT + 1;
    static constexpr int NT = NL == 11 ? 5 : 2;  // teams per CTA (shared memory: ~38 / 77 KB per column)
    static constexpr int EX = 16 * P;            // exchange buffer extent
};
template <int NL> __host__ __device__ constexpr int cq_xl(int Ky) {
    return 2 * cw_kyp(Ky) > CQ<NL>::EX ? 2 * cw_kyp(Ky) : CQ<NL>::EX;
}
template <int NL> __host__ __device__ constexpr size_t cq_smem_bytes(int Ky) {
    return (size_t)(CQ<NL>::N + CQ<NL>::NT * (cq_xl<NL>(Ky) + cw_kyp(Ky))) * sizeof(float2) +
           (size_t)(CQ<NL>::NT + 1) * cw_kyp(Ky) * sizeof(float);
}
// barrier over one team of TT threads (named barrier bid, 1 <= bid <= 15)
template <int TT> __device__ __forceinline__ void team_bar(int bid) {
    asm volatile("bar.sync %0, %1;" ::"r"(bid), "n"(TT) : "memory");
}

// forward N-point transform of a team: a[n1] = x[TT n1 + t] on entry,
// a[M2 r + q2] = X[k1 + 16 (R hi + r) + 256 q2] on exit; E is the team's exchange
// buffer (free again on return), TW1[k1 * TT + t] = W_N^{t k1}
template <int NL>
__device__ __forceinline__ void col_fwd_q(float2 (&a)[16], float2* E, const float2* TW1, int t, int bid) {
    typedef CQ<NL> Q;
    const int k1 = t & 15, hi = t >> 4;
    dft16<false>(a);
#pragma unroll
    for (int c = 1; c < 16; ++c) a[c] = cmul(a[c], TW1[c * Q::TT + t]);
#pragma unroll
    for (int c = 0; c < 16; ++c) E[c * Q::P + t] = a[c];
    team_bar<Q::TT>(bid);
#pragma unroll
    for (int m1 = 0; m1 < 16; ++m1) a[m1] = E[k1 * Q::P + Q::M2 * m1 + hi];
    team_bar<Q::TT>(bid);
    dft16<false>(a);
#pragma unroll
    for (int q1 = 1; q1 < 16; ++q1) a[q1] = cmul(a[q1], TW1[q1 * Q::TT + 16 * hi]);  // W_TT^{m2 q1}
#pragma unroll
    for (int q1 = 0; q1 < 16; ++q1) E[k1 * Q::P + q1 * Q::M2 + hi] = a[q1];
    team_bar<Q::TT>(bid);
#pragma unroll
    for (int r = 0; r < Q::R; ++r) {
#pragma unroll
        for (int m2 = 0; m2 < Q::M2; ++m2) a[Q::M2 * r + m2] = E[k1 * Q::P + (Q::R * hi + r) * Q::M2 + m2];
    }
    team_bar<Q::TT>(bid);
    if constexpr (Q::M2 == 8) {
        dft8<false>(a);
        dft8<false>(a + 8);
    } else {
        dft16<false>(a);
    }
}

// output mode of a[e] (e = M2 r + q2) in thread t
template <int NL> __device__ __forceinline__ int cq_mode(int t, int e) {
    typedef CQ<NL> Q;
    return (t & 15) + 16 * (Q::R * (t >> 4) + e / Q::M2) + 256 * (e % Q::M2);
}

// Persistent column pass (FP32): one CTA per SM, NT teams of TT threads,
// team q of CTA b takes the kept columns b + gridDim.x (q + NT r).  Staging,
// tables and stage algebra follow k_col_w; only the thread <-> mode maps differ
// (build: j = TT n1 + t; stage algebra: j = cq_mode<NL>(t, e)).
// dynamic smem: TW1 [16][TT] | per team: X [XL] (exchange, then WS | ACC), NS [Kyp]
//               | per team SHV [Kyp] float | KYS [Kyp] float
template <int NL, int STAGE, bool IFRK>
__global__ void __launch_bounds__(CQ<NL>::TT * CQ<NL>::NT, 1) k_col_q(Geo g, ColArgs<float> a) {
    typedef float T;
    typedef float2 C;
    typedef CQ<NL> Q;
    constexpr int NT = Q::NT, TT = Q::TT;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int Ky = g.Ky, Kyp = cw_kyp(Ky), XL = cq_xl<NL>(Ky), Kx = g.Kx;
    const int team = threadIdx.x / TT, t = threadIdx.x % TT;
    const int bid = 1 + team;
    C* TW1 = reinterpret_cast<C*>(smem_raw);
    C* X = TW1 + Q::N + team * (XL + Kyp);
    C* NS = X + XL;
    T* SHV = reinterpret_cast<T*>(TW1 + Q::N + NT * (XL + Kyp)) + team * Kyp;
    T* KYS = reinterpret_cast<T*>(TW1 + Q::N + NT * (XL + Kyp)) + NT * Kyp;
    const int hv = a.sp.hv, sfd = a.sp.sfd;
    __shared__ double s_dt;

    for (int m = threadIdx.x; m < Q::N; m += blockDim.x) TW1[m] = a.twc[((m % TT) * (m / TT)) & (Q::N - 1)];
    for (int jj = threadIdx.x; jj < Ky; jj += blockDim.x) KYS[jj] = a.kyv[jj];
    const int cstride = gridDim.x * NT;
    int i = blockIdx.x + gridDim.x * team;
    if (i < Kx) {
        const size_t base = (size_t)i * Ky;
        for (int jj = t; jj < Ky; jj += TT) {
            cp_async(&NS[jj], &a.W0[base + jj]);
            if (hv) cp_async(&SHV[jj], &a.hvw[base + jj]);
        }
    }
    wait_previous_kernel();
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
            if (blockIdx.x == 0) a.ds->dt = dt;
        } else {
            dt = a.ds->dt;
        }
        s_dt = dt;
    }
    __syncthreads();  // tables and dt

    const double dt = s_dt;
    const StageCoef<T> sq = stage_coef<T>(a.sp, dt);
    C* __restrict__ W0 = a.W0;
    C* __restrict__ WS = a.WS;
    C* __restrict__ ACC = a.ACC;
    const C zero = make_float2(0.f, 0.f);

    for (bool first = true; i < Kx; i += cstride, first = false) {
        if (!first) {
            const size_t base = (size_t)i * Ky;
            for (int jj = t; jj < Ky; jj += TT) {
                cp_async(&NS[jj], &a.W0[base + jj]);
                if (hv) cp_async(&SHV[jj], &a.hvw[base + jj]);
            }
        }
        const T kx = __ldg(&a.kxv[i]);
        const size_t cbase = (size_t)i * Ky;
        C v[16];
        // q = -1: forward transform of the Jacobian column and the RK stage;
        // q = 0..3: inverse transforms of Omega, Omega_y, Psi, Psi_y
#pragma unroll 1
        for (int q = -1; q < 4; ++q) {
            const int f = (q + 2) & 3;
            if (q < 0) {
                const C* __restrict__ Gc = a.G + (size_t)i * Q::N;
#pragma unroll
                for (int n1 = 0; n1 < 16; ++n1) v[n1] = ld_stream(&Gc[TT * n1 + t]);
            } else {
                // thread t builds modes j = TT n1 + t; Psi = -w/k^2 is formed once
                // (written back to NS) and reused for Psi_y by the same thread
#pragma unroll
                for (int n1 = 0; n1 < 16; ++n1) {
                    const int j = TT * n1 + t;
                    const int jj = kept_jj(g, j);
                    C x = zero;
                    if (jj >= 0) {
                        const T ky = KYS[jj];
                        C w = NS[jj];
                        if (f == 0) {
                            w = field_value<T, C>(0, w, kx, ky);
                            NS[jj] = w;
                        }
                        if (f == 1 || f == 3) {
                            x.x = -ky * w.y;
                            x.y = ky * w.x;
                        } else {
                            x = w;
                        }
                    }
                    v[n1] = cconj(x);
                }
            }
            col_fwd_q<NL>(v, X, TW1, t, bid);  // ends with a team barrier: X is free
            if (q >= 0) {
                C* __restrict__ Fc = a.F[f] + (size_t)i * Q::N;
#pragma unroll
                for (int e = 0; e < 16; ++e) Fc[cq_mode<NL>(t, e)] = cconj(v[e]);
                continue;
            }
            if (STAGE != 1) {
                for (int jj = t; jj < Ky; jj += TT) {
                    cp_async(&X[jj], &WS[cbase + jj]);
                    cp_async(&X[Kyp + jj], &ACC[cbase + jj]);
                }
            }
            cp_async_wait_all();
            team_bar<TT>(bid);  // the team's staged omega_hat, weights, WS and ACC

            // RK stage algebra (spectral_time_integration.c:50-100) on this
            // thread's forward outputs, modes j = cq_mode<NL>(t, e)
#pragma unroll
            for (int e = 0; e < 16; ++e) {
                const int j = cq_mode<NL>(t, e);
                const int jj = kept_jj(g, j);
                if (jj < 0) continue;
                const size_t s = cbase + jj;
                const C jh = v[e];
                const C w0 = NS[jj];
                const C ws = (STAGE == 1) ? w0 : X[jj];
                const C acc0 = (STAGE == 1) ? zero : X[Kyp + jj];
                const T hw = hv ? SHV[jj] : (T)0;
                T sw = (T)0;
                C fb = zero;
                if (sfd) {
                    sw = a.sfdw[s];
                    fb = a.SFD[s];
                }
                const C wn = rk_stage_mode<T, STAGE, IFRK>(sq, jh, w0, ws, acc0, hw, sw, fb, k2sum(kx, KYS[jj]), ACC, WS, s);
                if (STAGE == 4) W0[s] = wn;
                NS[jj] = wn;
            }
            if (STAGE == 4 && (a.sp.forcing || sfd)) {
                // forcing increment (few low-|k| modes), then the SFD post-step, on omega_hat^{n+1}
                // columns beyond the shell only relax the SFD filter (and skip the
                // FP64 amplitude)
                const bool force_col = a.sp.forcing && (double)kx <= a.sp.f_kmax + 1e-9;
                const double f_amp = force_col ? a.sp.f_sigma * sqrt(dt / a.sp.fsub) : 0.0;
                double sa = 0.0;
                if (sfd) {
                    sa = dt / a.sp.sfd_tau;
                    sa = sa > 1.0 ? 1.0 : (sa < 0.0 ? 0.0 : sa);
                }
#pragma unroll 1
                for (int e = 0; e < 16 && (force_col || sfd); ++e) {
                    const int j = cq_mode<NL>(t, e);
                    const int jj = kept_jj(g, j);
                    if (jj < 0) continue;
                    const size_t s = cbase + jj;
                    bool forced;
                    const C wn = post_step_mode(g, a, i, j, s, NS[jj], kx, KYS[jj], f_amp, sa, forced);
                    if (forced) {
                        W0[s] = wn;
                        NS[jj] = wn;
                    }
                }
            }
            team_bar<TT>(bid);  // NS complete for the inverse transforms; X is free again
        }
    }
    if (STAGE == 4 && blockIdx.x == 0 && threadIdx.x == 0) a.ds->t = a.ds->t + dt;
}

// ============================================================ k_row_t
// FP32 row pass at nx = 2048 with the Jacobian operands in tensor memory.
// Same transforms and row ownership as k_row_w (groups of GW warps own GW
// consecutive rows; every transform of a row stays inside its warp), with two
// changes to where data waits:
//  * the next field of the group's rows streams into per-warp inboxes with
//    cp.async (no register staging), so its global latency overlaps the
//    current field's transform whatever the register allocator does;
//  * psi_x (then psi_x omega_y) and psi_y live in the warp's 128 columns of
//    tensor memory (tcgen05.st / tcgen05.ld, 32x32b shape: lane = thread),
//    which frees the 16 KB per row that they took in shared memory and moves
//    their traffic off the shared-memory pipe.
// NB inboxes per warp: 2 lets the copy of field q + 1 start as soon as field q
// has landed (one group barrier per field); 1 waits until every warp of the
// group has packed field q (two barriers per field).
// dynamic smem (float2): tw [32][33] | twh [1024] | per warp: S [32][33], IN [NB][712]
//                        | kx [704] float | tensor-memory address
#define NSG_RT_IN 712
#ifndef NSG_ROW_TMEM
#define NSG_ROW_TMEM 1   // 0: the FP32 row pass runs k_row_w
#endif
#ifndef NSG_RT_NW
#define NSG_RT_NW 8
#endif
#ifndef NSG_RT_GW
#define NSG_RT_GW 8     // the whole CTA reads 8 consecutive rows: 64-byte runs per kx column
#endif
#ifndef NSG_RT_NB
#define NSG_RT_NB 1
#endif
#ifndef NSG_RT_TWTM
#define NSG_RT_TWTM 1   // per-lane twiddles of the transforms and the inverse pack in tensor memory
#endif
template <int NB> __host__ __device__ constexpr int rt_wstride() {
    // 16-byte aligned blocks whose bases differ by 4 float2 modulo 16 between
    // neighbouring warps (group-wide deposits and unpack reads hit distinct banks)
    return ((1056 + NB * NSG_RT_IN + 15) / 16) * 16 + 4;
}
template <int NW, int NB> __host__ __device__ constexpr size_t rt_smem_bytes() {
    return (size_t)(32 * 33 + 1024 + NW * rt_wstride<NB>()) * sizeof(float2) + (size_t)NSG_RW_KXMAX * sizeof(float) + 16;
}
template <int NW> __host__ __device__ constexpr int rt_tmem_need() {
    // 128 columns per warp (warps w and w + 4 share lanes) + 128 twiddle columns
    return 128 * ((NW + 3) / 4) + (NSG_RT_TWTM ? 128 : 0);
}
template <int NW> __host__ __device__ constexpr unsigned rt_tmem_cols() { return rt_tmem_need<NW>() <= 256 ? 256u : 512u; }

// the 1024-point transform of warp_fft1024 with the per-lane twiddles
// W_1024^{lane k1} (k1 < 32) read from tensor memory columns ttw .. ttw + 63
__device__ __forceinline__ void warp_fft1024_tm(float2 (&a)[32], float2* S, unsigned ttw, int lane) {
    dft32<false>(a);
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        float r[16];
        tm_ld16_issue(ttw + 16u * c, r);
        tm_wait_ld(r);
#pragma unroll
        for (int m = 0; m < 8; ++m) {
            const int k1 = 8 * c + m;
            if (k1 > 0) a[k1] = cmul(a[k1], make_float2(r[2 * m], r[2 * m + 1]));
        }
    }
#pragma unroll
    for (int k1 = 0; k1 < 32; ++k1) S[k1 * 33 + lane] = a[k1];
    __syncwarp();
#pragma unroll
    for (int n2 = 0; n2 < 32; ++n2) a[n2] = S[lane * 33 + n2];
    __syncwarp();
    dft32<false>(a);
}

// copy X_f[k] of row y, k = kb + 32 i < NSG_RW_KX, into the inbox IN (at sx(k)); always commits a group
__device__ __forceinline__ void rt_issue(float2* IN, const float2* __restrict__ src, int ny, int y, bool ok, int kb) {
    if (ok) {
#pragma unroll
        for (int i = 0; i < NSG_RW_KXMAX / 32; ++i) {
            const int k = kb + 32 * i;
            if (k < NSG_RW_KX) cp_async(&IN[33 * i + kb], &src[(size_t)k * ny + y]);
        }
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
}

// row_pack from an inbox, with the i kx factor of the x-derivative fields applied on the way
// (twh: the shared table exp(-2 pi i k/nx); with TW the pack twiddles of this
// lane, k = lane + 32 n1, come from tensor memory columns ttwh + 2 n1, + 1)
template <bool DX, bool TW>
__device__ __forceinline__ void rt_pack(float2 (&a)[32], const float2* IN, const float* kxs, const float2* twh, unsigned ttwh,
                                        int lane) {
    const int ob = lane ? 32 - lane : 33;
    const float2 zero = make_float2(0.f, 0.f);
    float r[16];
#pragma unroll
    for (int n1 = 0; n1 < 32; ++n1) {
        if (TW && (n1 & 7) == 0) {
            tm_ld16_issue(ttwh + 2u * n1, r);
            tm_wait_ld(r);
        }
        const int k = lane + 32 * n1;
        float2 xa = (k < NSG_RW_KX) ? IN[33 * n1 + lane] : zero;
        float2 xb = (k > 0 && 1024 - k < NSG_RW_KX) ? IN[33 * (31 - n1) + ob] : zero;
        if (DX) {
            const float ka = (k < NSG_RW_KX) ? kxs[k] : 0.f;
            const float kb = (k > 0 && 1024 - k < NSG_RW_KX) ? kxs[1024 - k] : 0.f;
            xa = make_float2(-ka * xa.y, ka * xa.x);
            xb = make_float2(-kb * xb.y, kb * xb.x);
        }
        if (n1 == 0 && lane == 0) {
            a[n1] = make_float2(xa.x, -xa.x);
        } else {
            const float2 e = TW ? make_float2(r[2 * (n1 & 7)], r[2 * (n1 & 7) + 1]) : twh[k];
            const float2 A = cadd(xa, cconj(xb));
            const float2 dd = csub(xa, cconj(xb));
            const float Dx = dd.x * e.x + dd.y * e.y;
            const float Dy = dd.y * e.x - dd.x * e.y;
            a[n1] = make_float2(A.x - Dy, -(A.y + Dx));
        }
    }
}

template <int NW, int GW, int NB>
__global__ void __launch_bounds__(32 * NW, 1) k_row_t(Geo g, RowArgs<float> a) {
    static_assert(NW % GW == 0 && NB >= 1 && NB <= 2, "row tiling");
    static_assert(rt_tmem_need<NW>() <= 512, "tensor-memory columns");
    constexpr int WS = rt_wstride<NB>();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2* tw = reinterpret_cast<float2*>(smem_raw);
    float2* twh_s = tw + 32 * 33;
    float2* S0 = twh_s + 1024;
    float* kx_s = reinterpret_cast<float*>(S0 + NW * WS);
    unsigned* tslot = reinterpret_cast<unsigned*>(kx_s + NSG_RW_KXMAX);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float2* S = S0 + warp * WS;
    const int ny = g.ny;
    const int grp = warp / GW;
    const int tg = threadIdx.x - grp * 32 * GW;
    const int kb = tg / GW, wme = tg - kb * GW;
    float2* Sg = S0 + grp * GW * WS;
    float2* INme = Sg + wme * WS + 1056;   // inbox 0 of the warp whose row this thread copies
    const float2* INw = S + 1056;          // this warp's inbox 0

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         (unsigned)__cvta_generic_to_shared(tslot)),
                     "r"(rt_tmem_cols<NW>()));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    for (int i = threadIdx.x; i < 1024; i += blockDim.x) {
        const int k1 = i >> 5, t = i & 31;
        tw[k1 * 33 + t] = a.twr[t * k1];
        twh_s[i] = a.twh[i];
    }
    for (int i = threadIdx.x; i < NSG_RW_KXMAX; i += blockDim.x) kx_s[i] = (i < NSG_RW_KX) ? a.kxv[i] : 0.f;
    wait_previous_kernel();
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        if (a.marker == 1) {
            a.ds->step_cur = a.ds->step_next;
            a.ds->step_next = a.ds->step_next + (a.ds->fsub ? a.ds->fsub : 1ULL);
        } else if (a.marker == 2) {
            a.ds->maxvel2 = 0ULL;
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();  // tables and the tensor-memory address
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    // this warp's 128 columns: R (psi_x, then psi_x omega_y) at +0, Q (psi_y) at +64
    const unsigned tR = *tslot + ((unsigned)(32 * (warp & 3)) << 16) + 128u * (unsigned)(warp >> 2);
    const unsigned tQ = tR + 64u;
    // per-lane twiddles after the warps' R and Q columns, one copy per lane
    // quarter (written by warps 0-3, read by every warp of the quarter):
    // tTW + 2 k1 (+1) = W_1024^{lane k1}, tTWH + 2 n1 (+1) = exp(-2 pi i (lane + 32 n1)/nx)
    const unsigned tTW = *tslot + ((unsigned)(32 * (warp & 3)) << 16) + 128u * (unsigned)((NW + 3) / 4);
    const unsigned tTWH = tTW + 64u;
    if (NSG_RT_TWTM) {
        if (warp < 4) {
            float2 t[32];
#pragma unroll
            for (int k1 = 0; k1 < 32; ++k1) t[k1] = tw[k1 * 33 + lane];
#pragma unroll
            for (int c = 0; c < 4; ++c) tm_st16(tTW + 16u * c, t, c);
#pragma unroll
            for (int n1 = 0; n1 < 32; ++n1) t[n1] = twh_s[lane + 32 * n1];
#pragma unroll
            for (int c = 0; c < 4; ++c) tm_st16(tTWH + 16u * c, t, c);
            tm_wait_st();
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    }

    float vmax2 = 0.f;
    float2 v[32];
    // rows of this CTA: [r0, yend), in rounds of NW.  NSG_RT_SPREAD gives every
    // CTA an equal contiguous share (13-14 rows at 2048 over 152 CTAs), so the
    // last round is short on every SM instead of full on some and absent on others
    // (the rounds are latency-bound, so at 2048^2 this measured the same as round-robin).
    const int r0 = NSG_RT_SPREAD ? (int)(((long long)ny * blockIdx.x) / gridDim.x) : blockIdx.x * NW;
    const int yend = NSG_RT_SPREAD ? (int)(((long long)ny * (blockIdx.x + 1)) / gridDim.x) : ny;
    const int ystep = NSG_RT_SPREAD ? NW : gridDim.x * NW;
    int y0 = r0 + grp * GW;
    int buf = 0;
    rt_issue(INme, a.F[0], ny, y0 + wme, y0 + wme < yend, kb);
    for (; y0 < yend; y0 += ystep) {
        const int y = y0 + (warp - grp * GW);
        // q = 0..3: inverse transforms of psi_x (F0, d/dx), psi_y (F1), omega_y (F3),
        // omega_x (F2, d/dx); q = 4: forward transform of the packed Jacobian
#pragma unroll 1
        for (int q = 0; q < 5; ++q) {
            if (q < 4) {
                asm volatile("cp.async.wait_all;" ::: "memory");  // field q (the only copies in flight)
                group_sync<GW, NW>(grp);                           // ... from every thread; the other inbox is free
                const int yn = (q < 3) ? y0 + wme : y0 + ystep + wme;
                const float2* src = a.F[(q < 3) ? ((q + 1 < 2) ? q + 1 : 4 - q) : 0];
                if (NB == 2) rt_issue(INme + (buf ^ 1) * NSG_RT_IN, src, ny, yn, yn < yend, kb);
                if (y < yend) {
                    const float2* IN = INw + buf * NSG_RT_IN;
                    if (q == 0 || q == 3) rt_pack<true, NSG_RT_TWTM>(v, IN, kx_s, twh_s, tTWH, lane);
                    else rt_pack<false, NSG_RT_TWTM>(v, IN, kx_s, twh_s, tTWH, lane);
                }
                if (NB == 1) {
                    group_sync<GW, NW>(grp);  // every warp has packed field q
                    rt_issue(INme, src, ny, yn, yn < yend, kb);
                }
                buf ^= (NB - 1);
            }
            if (y >= yend) continue;
            if (NSG_RT_TWTM) warp_fft1024_tm(v, S, tTW, lane);
            else warp_fft1024<false>(v, S, tw, lane);
            if (q == 4) break;
#pragma unroll
            for (int k = 0; k < 32; ++k) v[k].y = -v[k].y;
            if (q == 0) {
#pragma unroll
                for (int c = 0; c < 4; ++c) tm_st16(tR + 16u * c, v, c);
            } else if (q == 1) {
                if (a.cfl) {
                    tm_wait_st();
#pragma unroll
                    for (int c = 0; c < 4; ++c) {
                        float r[16];
                        tm_ld16_issue(tR + 16u * c, r);
                        tm_wait_ld(r);
#pragma unroll
                        for (int m = 0; m < 8; ++m) {
                            const float2 p = v[8 * c + m];
                            vmax2 = fmaxf(vmax2, fmaxf(r[2 * m] * r[2 * m] + p.x * p.x, r[2 * m + 1] * r[2 * m + 1] + p.y * p.y));
                        }
                    }
                }
#pragma unroll
                for (int c = 0; c < 4; ++c) tm_st16(tQ + 16u * c, v, c);
            } else if (q == 2) {
                tm_wait_st();
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    float r[16];
                    tm_ld16_issue(tR + 16u * c, r);
                    tm_wait_ld(r);
                    float2 pr[32];
#pragma unroll
                    for (int m = 0; m < 8; ++m) pr[8 * c + m] = make_float2(r[2 * m] * v[8 * c + m].x, r[2 * m + 1] * v[8 * c + m].y);
                    tm_st16(tR + 16u * c, pr, c);
                }
            } else {
                // J = psi_x omega_y - psi_y omega_x, packed as w[m] = J[2m] + i J[2m+1]
                tm_wait_st();
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    float r[16], s[16];
                    tm_ld16_issue(tR + 16u * c, r);
                    tm_ld16_issue(tQ + 16u * c, s);
                    tm_wait_ld2(r, s);
#pragma unroll
                    for (int m = 0; m < 8; ++m) {
                        const float2 w = v[8 * c + m];
                        v[8 * c + m] = make_float2(r[2 * m] - s[2 * m] * w.x, r[2 * m + 1] - s[2 * m + 1] * w.y);
                    }
                }
            }
        }
        if (y < yend) {
#pragma unroll
            for (int k = 0; k < 32; ++k) S[k * 33 + lane] = v[k];
        }
        group_sync<GW, NW>(grp);
        const float half = 0.5f;
        const int nrows = (yend - y0 < GW) ? yend - y0 : GW;
        for (int e = tg; e < NSG_RW_KX * GW; e += 32 * GW) {
            const int k = e / GW, w = e - k * GW;
            if (w >= nrows) continue;
            const float2* Sw = Sg + w * WS;
            const float2 wa = Sw[sx(k)];
            const float2 wb = Sw[sx((1024 - k) & 1023)];
            float2 ev, od;
            ev.x = half * (wa.x + wb.x);
            ev.y = half * (wa.y - wb.y);
            od.x = half * (wa.y + wb.y);
            od.y = -half * (wa.x - wb.x);
            a.G[(size_t)k * ny + y0 + w] = cadd(ev, cmul(od, twh_s[k]));
        }
    }
    asm volatile("cp.async.wait_all;" ::: "memory");
    tm_wait_st();
    if (a.cfl) {
        const double vm = warp_max((double)vmax2);
        if (lane == 0) atomicMax(&a.ds->maxvel2, (unsigned long long)__double_as_longlong(vm));
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(*tslot), "r"(rt_tmem_cols<NW>()));
    }
}

// ============================================================ k_row_4k
// FP32 row pass at nx = 4096 (H = 2048, 1367 kept kx): two warps (64 threads,
// 32 points each) per row, four rows per CTA, rows assigned to the CTAs
// round-robin in groups of four.  The half-length transforms are the two-warp
// 2048-point transform of the column pass (col_fwd2048: input x[64 n1 + t],
// output X[lane + 32 k2 + 1024 h]); inverses run as conj(DFT(conj z)).  The
// inverse outputs are spatial samples z[m] in the output layout, where the
// Jacobian is formed (psi_x and psi_y in tensor memory, 128 columns per warp);
// J then passes once through the row's exchange buffer (dense, conflict-free
// both ways) into the input layout of its forward transform.
// dynamic smem (float2): tw [32][65] (W_2048^{t k1}) | twh [2048] | per row: IN [1368],
//                        X [2112] (block pitch 3480 = 8 mod 16) | kx [1368] float | tensor-memory address
#define NSG_R4_ROWS 4
#define NSG_R4_KX 1367
#define NSG_R4_IN 1368
#define NSG_R4_BLK (NSG_R4_IN + NSG_CW_EX)
__host__ __device__ constexpr size_t r4_smem_bytes() {
    return (size_t)(32 * 65 + 2048 + NSG_R4_ROWS * NSG_R4_BLK) * sizeof(float2) + (size_t)NSG_R4_IN * sizeof(float) + 16;
}

// the CTA's rows y0 + w (w = tid & 3, valid while < yend) of field src into the
// inboxes: thread tid copies k = (tid >> 2) + 64 i, so the four rows of one kx
// column are one 32-byte run
__device__ __forceinline__ void r4_issue(float2* IN0, const float2* __restrict__ src, int ny, int y0, int yend, int tid) {
    const int w = tid & 3, kb = tid >> 2;
    if (y0 + w < yend) {
#pragma unroll
        for (int i = 0; i < 22; ++i) {
            const int k = kb + 64 * i;
            if (k < NSG_R4_KX) cp_async(&IN0[w * NSG_R4_BLK + k], &src[(size_t)k * ny + y0 + w]);
        }
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
}

// conj of the half-length inverse input Z[k] (k = 64 n1 + t) from the inbox IN
// (half spectrum X[k], k < 1367), with the i kx factor of the x-derivative fields:
// Z[k] = (X[k] + conj X[H-k]) + i e^{+2 pi i k/nx} (X[k] - conj X[H-k])
template <bool DX>
__device__ __forceinline__ void r4_pack(float2 (&a)[32], const float2* IN, const float* kxs, const float2* twh, int t) {
    const float2 zero = make_float2(0.f, 0.f);
#pragma unroll
    for (int n1 = 0; n1 < 32; ++n1) {
        const int k = 64 * n1 + t;
        const bool ka_ok = k < NSG_R4_KX, kb_ok = k > 0 && 2048 - k < NSG_R4_KX;
        float2 xa = ka_ok ? IN[k] : zero;
        float2 xb = kb_ok ? IN[2048 - k] : zero;
        if (DX) {
            const float ka = ka_ok ? kxs[k] : 0.f;
            const float kb = kb_ok ? kxs[2048 - k] : 0.f;
            xa = make_float2(-ka * xa.y, ka * xa.x);
            xb = make_float2(-kb * xb.y, kb * xb.x);
        }
        if (k == 0) {
            a[n1] = make_float2(xa.x, -xa.x);  // conj of Re X[0] (1 + i); the Nyquist bin is masked
        } else {
            const float2 e = twh[k];  // exp(-2 pi i k/nx)
            const float2 A = cadd(xa, cconj(xb));
            const float2 dd = csub(xa, cconj(xb));
            const float Dx = dd.x * e.x + dd.y * e.y;
            const float Dy = dd.y * e.x - dd.x * e.y;
            a[n1] = make_float2(A.x - Dy, -(A.y + Dx));
        }
    }
}

__global__ void __launch_bounds__(64 * NSG_R4_ROWS, 1) k_row_4k(Geo g, RowArgs<float> a) {
    constexpr int NR = NSG_R4_ROWS;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2* tw = reinterpret_cast<float2*>(smem_raw);
    float2* twh_s = tw + 32 * 65;
    float2* B0 = twh_s + 2048;  // row r's block: IN at B0 + r * BLK, X at + NSG_R4_IN
    float* kx_s = reinterpret_cast<float*>(B0 + NR * NSG_R4_BLK);
    unsigned* tslot = reinterpret_cast<unsigned*>(kx_s + NSG_R4_IN);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int rr = warp >> 1, t = tid & 63, h = t >> 5, bid = 1 + rr;
    const float2* INr = B0 + rr * NSG_R4_BLK;
    float2* Xr = B0 + rr * NSG_R4_BLK + NSG_R4_IN;
    const int ny = g.ny;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 256;" ::"r"(
            (unsigned)__cvta_generic_to_shared(tslot)));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    for (int i = tid; i < 32 * 65; i += blockDim.x) {
        const int k1 = i / 65, tt = i - 65 * k1;
        tw[i] = (tt < 64) ? a.twr[(tt * k1) & 2047] : make_float2(0.f, 0.f);
    }
    for (int i = tid; i < 2048; i += blockDim.x) twh_s[i] = a.twh[i];
    for (int i = tid; i < NSG_R4_IN; i += blockDim.x) kx_s[i] = (i < NSG_R4_KX) ? a.kxv[i] : 0.f;
    wait_previous_kernel();
    if (blockIdx.x == 0 && tid == 0) {
        if (a.marker == 1) {
            a.ds->step_cur = a.ds->step_next;
            a.ds->step_next = a.ds->step_next + (a.ds->fsub ? a.ds->fsub : 1ULL);
        } else if (a.marker == 2) {
            a.ds->maxvel2 = 0ULL;
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    // this warp's 128 columns: R (psi_x, then psi_x omega_y) at +0, Q (psi_y) at +64
    const unsigned tR = *tslot + ((unsigned)(32 * (warp & 3)) << 16) + 128u * (unsigned)(warp >> 2);
    const unsigned tQ = tR + 64u;

    // rows round-robin: in one round CTAs b .. b + 3 read rows 16 c .. 16 c + 15, so
    // the four 32-byte sectors of each 128-byte line of F are read together (the
    // fields exceed L2 at 4096^2, so a line split over rounds is fetched again)
    const int yend = ny, ystep = gridDim.x * NR;
    float vmax2 = 0.f;
    float2 v[32];
    r4_issue(B0, a.F[0], ny, blockIdx.x * NR, yend, tid);
    for (int y0 = blockIdx.x * NR; y0 < yend; y0 += ystep) {
        const int y = y0 + rr;
        // q = 0..3: inverse transforms of psi_x (F0, d/dx), psi_y (F1), omega_y (F3),
        // omega_x (F2, d/dx); q = 4: forward transform of the packed Jacobian
#pragma unroll 1
        for (int q = 0; q < 5; ++q) {
            if (q < 4) {
                asm volatile("cp.async.wait_all;" ::: "memory");
                __syncthreads();  // field q of every row has landed
                if (y < yend) {
                    if (q == 0 || q == 3) r4_pack<true>(v, INr, kx_s, twh_s, t);
                    else r4_pack<false>(v, INr, kx_s, twh_s, t);
                }
                __syncthreads();  // every row has packed field q: the inboxes take the next field
                const int yn = (q < 3) ? y0 : y0 + ystep;
                r4_issue(B0, a.F[(q < 3) ? ((q + 1 < 2) ? q + 1 : 4 - q) : 0], ny, yn, yend, tid);
            }
            if (y >= yend) continue;
            if (q == 4) {
                // J from the output layout (m = lane + 32 k2 + 1024 h) to the input layout (64 n1 + t)
#pragma unroll
                for (int k2 = 0; k2 < 32; ++k2) Xr[lane + 32 * k2 + 1024 * h] = v[k2];
                team_sync(bid);
#pragma unroll
                for (int n1 = 0; n1 < 32; ++n1) v[n1] = Xr[64 * n1 + t];
                team_sync(bid);
                col_fwd2048(v, Xr, tw, t, lane, h, bid);
                break;
            }
            col_fwd2048(v, Xr, tw, t, lane, h, bid);
#pragma unroll
            for (int k = 0; k < 32; ++k) v[k].y = -v[k].y;
            if (q == 0) {
#pragma unroll
                for (int c = 0; c < 4; ++c) tm_st16(tR + 16u * c, v, c);
            } else if (q == 1) {
                if (a.cfl) {
                    tm_wait_st();
#pragma unroll
                    for (int c = 0; c < 4; ++c) {
                        float r[16];
                        tm_ld16_issue(tR + 16u * c, r);
                        tm_wait_ld(r);
#pragma unroll
                        for (int m = 0; m < 8; ++m) {
                            const float2 p = v[8 * c + m];
                            vmax2 = fmaxf(vmax2, fmaxf(r[2 * m] * r[2 * m] + p.x * p.x, r[2 * m + 1] * r[2 * m + 1] + p.y * p.y));
                        }
                    }
                }
#pragma unroll
                for (int c = 0; c < 4; ++c) tm_st16(tQ + 16u * c, v, c);
            } else if (q == 2) {
                tm_wait_st();
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    float r[16];
                    tm_ld16_issue(tR + 16u * c, r);
                    tm_wait_ld(r);
                    float2 pr[32];
#pragma unroll
                    for (int m = 0; m < 8; ++m) pr[m] = make_float2(r[2 * m] * v[8 * c + m].x, r[2 * m + 1] * v[8 * c + m].y);
                    tm_st16(tR + 16u * c, pr, 0);
                }
            } else {
                // J = psi_x omega_y - psi_y omega_x, packed as w[m] = J[2m] + i J[2m+1]
                tm_wait_st();
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    float r[16], s2[16];
                    tm_ld16_issue(tR + 16u * c, r);
                    tm_ld16_issue(tQ + 16u * c, s2);
                    tm_wait_ld2(r, s2);
#pragma unroll
                    for (int m = 0; m < 8; ++m) {
                        const float2 w = v[8 * c + m];
                        v[8 * c + m] = make_float2(r[2 * m] - s2[2 * m] * w.x, r[2 * m + 1] - s2[2 * m + 1] * w.y);
                    }
                }
            }
        }
        // the row's half-length spectrum W into its exchange buffer, by frequency
        if (y < yend) {
#pragma unroll
            for (int k2 = 0; k2 < 32; ++k2) Xr[lane + 32 * k2 + 1024 * h] = v[k2];
        }
        __syncthreads();
        // unpack the kept kx < Kx of the CTA's rows together: element e is
        // (k = e / 4, row y0 + e % 4), so four consecutive threads write one
        // 32-byte run of a G column
        const float half = 0.5f;
        const int nrows = (yend - y0 < NR) ? yend - y0 : NR;
        for (int e = tid; e < NSG_R4_KX * NR; e += blockDim.x) {
            const int k = e >> 2, w = e & 3;
            if (w >= nrows) continue;
            const float2* Sw = B0 + w * NSG_R4_BLK + NSG_R4_IN;
            const float2 wa = Sw[k];
            const float2 wb = Sw[(2048 - k) & 2047];
            float2 ev, od;
            ev.x = half * (wa.x + wb.x);
            ev.y = half * (wa.y - wb.y);
            od.x = half * (wa.y + wb.y);
            od.y = -half * (wa.x - wb.x);
            a.G[(size_t)k * ny + y0 + w] = cadd(ev, cmul(od, twh_s[k]));
        }
    }
    asm volatile("cp.async.wait_all;" ::: "memory");
    tm_wait_st();
    if (a.cfl) {
        const double vm = warp_max((double)vmax2);
        if (lane == 0) atomicMax(&a.ds->maxvel2, (unsigned long long)__double_as_longlong(vm));
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 256;" ::"r"(*tslot));
    }
}

}  // namespace nsg
