// Host engine and C-ABI (include/ns_gpu.h) for the sm_103a pseudospectral step.
//
// One ns_gpu instance owns one CUDA stream and every device buffer of one
// solver (no global state, so many instances can live side by side; the
// reference's global fftw_cleanup in spectral_memory.c:100-103 has no
// counterpart).  All work is issued on the instance stream; the host-array
// entry points synchronise that stream before returning.
#include <type_traits>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

#include "ns_gpu.h"
#include "ns_kernels.cuh"

using namespace nsg;

#include "ns_gpu_impl.h"

static int ilog2(int n) {
    int l = 0;
    while ((1 << l) < n) ++l;
    return l;
}
static int is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

// largest prime factor a transform length may have (one direct p-point pass)
#define NSG_MAX_PRIME 31

static int grid_for(long long n, int threads = 256, int cap = 2048) {
    long long b = (n + threads - 1) / threads;
    if (b < 1) b = 1;
    if (b > cap) b = cap;
    return (int)b;
}

template <typename T> using Cx = typename CT<T>::C;


template <typename T, int E, int MODE> static int row_launch_e(ns_gpu* g, const RowArgs<T>& a) {
    const int NF = RowNF<MODE>::v;
    const int TT = E ? g->g.H / E : g->g.TTr;
    const int P = row_groups(g->g.fpr, E, NF);
    // E = 0 (mixed radix): one scratch sequence per row after the NF field buffers
    const size_t smem = (size_t)(NF + (E ? 0 : P)) * g->g.RPC * spad_len(g->g.H) * sizeof(Cx<T>);
    void (*kern)(Geo, RowArgs<T>) = k_row<T, E, MODE>;
    // the step's radix-4 row pass with the grid's size fields as constants
    // (256^2 in FP32, 128^2 in FP64)
    if constexpr (E == 4 && MODE == ROW_STAGE) {
        if constexpr (std::is_same<T, float>::value) {
            if (g->fold == 256) kern = k_row<T, E, MODE, 256>;
        } else {
            if (g->fold == 128) kern = k_row<T, E, MODE, 128>;
        }
    }
    NSG_TRY(set_smem(g, kern, smem));
    kern<<<g->g.ny / g->g.RPC, g->g.RPC * P * TT, smem, g->st>>>(g->g, a);
    NSG_LAUNCHED(g);
    return NS_GPU_OK;
}
template <typename T, int MODE> static int row_launch(ns_gpu* g, const RowArgs<T>& a) {
    if (g->ER == 0) return row_launch_e<T, 0, MODE>(g, a);
    return g->ER == 16 ? row_launch_e<T, 16, MODE>(g, a) : row_launch_e<T, 4, MODE>(g, a);
}

template <typename T, int E, int MODE, int STAGE> static int col_launch_e(ns_gpu* g, const ColArgs<T>& a) {
    const int TC = E ? g->g.ny / E : g->g.TTc;
    const int P = col_groups(g->g.fpc, E, MODE);
    // the column buffers (and mixed-radix scratch), then the next-stage state of the
    // block's kept modes for the stage and correction passes
    const size_t wsm = (MODE == COL_STAGE || MODE == COL_ADD) ? (size_t)g->g.CW * g->g.Ky : 0;
    const size_t smem = ((size_t)(E ? P : 2 * P) * g->g.CW * spad_len(g->g.ny) + wsm) * sizeof(Cx<T>);
    void (*kern)(Geo, ColArgs<T>) = k_col<T, E, MODE, STAGE>;
    if constexpr (E == 4 && MODE == COL_STAGE) {
        if constexpr (std::is_same<T, float>::value) {
            if (g->fold == 256) kern = k_col<T, E, MODE, STAGE, 256>;
        } else {
            if (g->fold == 128) kern = k_col<T, E, MODE, STAGE, 128>;
        }
    }
    NSG_TRY(set_smem(g, kern, smem));
    kern<<<g->g.Kxp / g->g.CW, P * g->g.CW * TC, smem, g->st>>>(g->g, a);
    NSG_LAUNCHED(g);
    return NS_GPU_OK;
}
template <typename T, int MODE, int STAGE> static int col_launch(ns_gpu* g, const ColArgs<T>& a) {
    if (g->EC == 0) return col_launch_e<T, 0, MODE, STAGE>(g, a);
    return g->EC == 16 ? col_launch_e<T, 16, MODE, STAGE>(g, a) : col_launch_e<T, 4, MODE, STAGE>(g, a);
}

template <typename T> static StepParams step_params(const ns_gpu* g) {
    StepParams sp;
    memset(&sp, 0, sizeof(sp));
    sp.Re = g->p.Re;
    sp.inv_re = 1.0 / g->p.Re;
    sp.cfl = g->p.cfl_factor;
    sp.dxmin = fmin(g->g.Lx / g->g.nx, g->g.Ly / g->g.ny);
    sp.scale = 1.0 / ((double)g->g.nx * (double)g->g.ny);
    sp.adaptive = g->p.adaptive_dt;
    sp.hv = (g->p.hv_enabled && g->p.hv_coefficient > 0.0) ? 1 : 0;
    sp.sfd = (g->p.sfd_enabled && g->p.sfd_strength > 0.0 && g->p.sfd_timescale > 0.0) ? 1 : 0;
    sp.sfd_tau = g->p.sfd_timescale;
    sp.forcing = (g->p.forcing_enabled && g->f_sigma > 0.0) ? 1 : 0;
    sp.f_kmin = g->p.forcing_kmin;
    sp.f_kmax = g->p.forcing_kmax;
    sp.f_sigma = g->f_sigma;
    sp.f_seed = g->p.forcing_seed;
    sp.ifrk = g->p.scheme == NS_GPU_IFRK4 ? 1 : 0;
    sp.fsub = g->p.forcing_substeps > 1 ? g->p.forcing_substeps : 1;
    return sp;
}

template <typename T> static RowArgs<T> row_args(ns_gpu* g) {
    RowArgs<T> a;
    memset(&a, 0, sizeof(a));
    a.kxv = (const T*)g->kxv;
    a.twr = (const Cx<T>*)g->twr;
    a.twh = (const Cx<T>*)g->twh;
    a.ds = g->ds;
    a.G = (Cx<T>*)g->G;
    return a;
}

template <typename T> static ColArgs<T> col_args(ns_gpu* g) {
    ColArgs<T> a;
    memset(&a, 0, sizeof(a));
    a.G = (const Cx<T>*)g->G;
    for (int f = 0; f < 4; ++f) a.F[f] = (Cx<T>*)g->F[f];
    a.W0 = (Cx<T>*)g->W0;
    a.WS = (Cx<T>*)g->WS;
    a.ACC = (Cx<T>*)g->ACC;
    a.PSI0 = (const Cx<T>*)g->PSI0;
    a.SFD = (Cx<T>*)g->SFD;
    a.hvw = (const T*)g->hvw;
    a.sfdw = (const T*)g->sfdw;
    a.kxv = (const T*)g->kxv;
    a.kyv = (const T*)g->kyv;
    a.twc = (const Cx<T>*)g->twc;
    a.ds = g->ds;
    a.sp = step_params<T>(g);
    if (a.sp.forcing && g->fM > 0) {
        a.fsum = g->fsum;
        a.fkxr = g->fkxr;
        a.fkyr = g->fkyr;
    }
    a.nfields = 4;
    return a;
}

// F <- fields of (W, psi) : Psi, Psi_y, Omega[, Omega_y]
template <typename T> static int prologue(ns_gpu* g, void* W, void* P, int psi_from_w, int nfields) {
    ColArgs<T> a = col_args<T>(g);
    a.W0 = (Cx<T>*)W;
    a.PSI0 = (const Cx<T>*)P;
    a.psi_from_w = psi_from_w;
    a.nfields = nfields;
    return col_launch<T, COL_PROLOGUE, 0>(g, a);
}

template <typename T> static int stage_row(ns_gpu* g, int stage) {
    ProfScope ps(g, 0);
    RowArgs<T> a = row_args<T>(g);
    for (int f = 0; f < 4; ++f) a.F[f] = (const Cx<T>*)g->F[f];
    a.dx[0] = 1; a.dx[1] = 0; a.dx[2] = 1; a.dx[3] = 0;  // psi_x, psi_y, omega_x, omega_y
    a.cfl = (stage == 1 && g->p.adaptive_dt) ? 1 : 0;
    a.marker = (stage == 1) ? 1 : (stage == 2 ? 2 : 0);
    if (g->fast_row) {
        if constexpr (sizeof(T) == 4) return nsg_fast_row_f32(g, a);
        else return nsg_fast_row_f64(g, a);
    }
    return row_launch<T, ROW_STAGE>(g, a);
}

template <typename T, int STAGE> static int stage_col(ns_gpu* g, const ColArgs<T>& a) {
    ProfScope ps(g, 1);
    if (g->fast_col) {
        if constexpr (sizeof(T) == 4) return nsg_fast_col_f32(g, a, STAGE);
        else return nsg_fast_col_f64(g, a, STAGE);
    }
    return col_launch<T, COL_STAGE, STAGE>(g, a);
}

static int dalloc(ns_gpu* g, void** p, size_t bytes);

// The per-step forcing-noise table of steps that take several draws: every (kept
// mode with |kx|, |ky| <= kmax, draw) pair gets one thread of k_forcing_noise
// before the step's first stage, instead of one thread per mode drawing them in
// sequence at stage 4.
static int ensure_noise(ns_gpu* g) {
    g->fM = 0;
    const StepParams sp = step_params<double>(g);
    // the draws (FP64 Philox, logarithm, sine and cosine) and their per-mode sums
    // run beside stages 1-3 on a second stream; in the stage-4 column pass, where
    // the forced columns' draws used to run, they cost 7.7 us of a 0.274 ms 2048^2
    // step with one draw per step
    if (!sp.forcing || sp.fsub < 1) return NS_GPU_OK;
    const double two_pi = 2.0 * 3.14159265358979323846;
    const int kxr = std::min((int)floor(sp.f_kmax * g->g.Lx / two_pi + 1e-9), g->g.Kx - 1);
    const int kyr = std::min((int)floor(sp.f_kmax * g->g.Ly / two_pi + 1e-9), g->g.Kyh);
    if (kxr < 0 || kyr < 0) return NS_GPU_OK;
    const size_t need = (size_t)(kxr + 1) * (2 * kyr + 1) * sp.fsub;
    if (need > g->fnoise_cap) {
        if (g->fnoise) cudaFree(g->fnoise);
    if (g->fsum) cudaFree(g->fsum);
        g->fnoise = nullptr;
        g->fnoise_cap = 0;
        NSG_TRY(dalloc(g, (void**)&g->fnoise, need * sizeof(double2)));
        g->fnoise_cap = need;
    }
    const size_t modes = (size_t)(kxr + 1) * (2 * kyr + 1);
    if (modes > g->fsum_cap) {
        if (g->fsum) cudaFree(g->fsum);
        g->fsum = nullptr;
        g->fsum_cap = 0;
        NSG_TRY(dalloc(g, (void**)&g->fsum, modes * sizeof(double2)));
        g->fsum_cap = modes;
    }
    if (!g->stn) {
        NSG_CUDA(g, cudaStreamCreateWithFlags(&g->stn, cudaStreamNonBlocking));
        NSG_CUDA(g, cudaEventCreateWithFlags(&g->evn0, cudaEventDisableTiming));
        NSG_CUDA(g, cudaEventCreateWithFlags(&g->evn1, cudaEventDisableTiming));
    }
    g->fkxr = kxr;
    g->fkyr = kyr;
    g->fM = sp.fsub;
    return NS_GPU_OK;
}

// the step's noise table on its own stream, after the stage-1 row pass (which
// sets step_cur) and joined before the stage-4 column pass: its FP64 draws run
// beside stages 1-3 instead of ahead of them
static int launch_noise(ns_gpu* g) {
    const StepParams sp = step_params<double>(g);
    const int n = (g->fkxr + 1) * (2 * g->fkyr + 1) * g->fM;
    NSG_CUDA(g, cudaEventRecord(g->evn0, g->st));
    NSG_CUDA(g, cudaStreamWaitEvent(g->stn, g->evn0, 0));
    k_forcing_noise<<<(n + 127) / 128, 128, 0, g->stn>>>(g->g.ny, g->g.Lx, g->g.Ly, &g->ds->step_cur, g->fM, sp.f_seed,
                                                         sp.f_kmin, sp.f_kmax, g->fkxr, g->fkyr, g->fnoise);
    NSG_LAUNCHED(g);
    const int modes = (g->fkxr + 1) * (2 * g->fkyr + 1);
    k_forcing_sum<<<(modes + 127) / 128, 128, 0, g->stn>>>(g->g.ny, g->g.Lx, g->g.Ly, g->fM, sp.f_kmin, sp.f_kmax,
                                                             g->fkxr, g->fkyr, g->fnoise, g->fsum);
    NSG_LAUNCHED(g);
    NSG_CUDA(g, cudaEventRecord(g->evn1, g->stn));
    return NS_GPU_OK;
}

// the kernels of one RK4 step on the instance stream
template <typename T> static int one_step(ns_gpu* g, const ColArgs<T>& a) {
    NSG_TRY(stage_row<T>(g, 1));
    if (g->fM > 0) NSG_TRY(launch_noise(g));
    NSG_TRY((stage_col<T, 1>(g, a)));
    NSG_TRY(stage_row<T>(g, 2));
    NSG_TRY((stage_col<T, 2>(g, a)));
    NSG_TRY(stage_row<T>(g, 3));
    NSG_TRY((stage_col<T, 3>(g, a)));
    NSG_TRY(stage_row<T>(g, 4));
    if (g->fM > 0) NSG_CUDA(g, cudaStreamWaitEvent(g->st, g->evn1, 0));
    NSG_TRY((stage_col<T, 4>(g, a)));
    if (g->outside_active) {
        const long long nn = (long long)g->g.nkx * g->g.nky;
        k_outside<<<grid_for(nn), 256, 0, g->st>>>(g->g, a.sp, g->hvw_full, g->hv_cutoff, g->hv_inv_bw,
                                                   g->p.hv_order > 0 ? g->p.hv_order : 1, g->p.sfd_strength, g->ds,
                                                   g->out, g->outsfd);
        NSG_LAUNCHED(g);
    }
    return NS_GPU_OK;
}

// every value a step's launches take by value: a captured step stays valid while
// these bytes are unchanged (the state itself lives in device memory)
template <typename T> static std::vector<unsigned char> step_key(ns_gpu* g, const ColArgs<T>& a) {
    const RowArgs<T> r = row_args<T>(g);
    std::vector<unsigned char> k;
    auto put = [&k](const void* p, size_t n) {
        const unsigned char* c = static_cast<const unsigned char*>(p);
        k.insert(k.end(), c, c + n);
    };
    put(&a, sizeof(a));
    put(&r, sizeof(r));
    put(&g->g, sizeof(g->g));
    const int ints[] = {g->prec, g->ER, g->EC, g->fast_row, g->fast_col, g->outside_active, g->fM, g->fkxr, g->fkyr};
    put(ints, sizeof(ints));
    const double dbl[] = {g->hv_cutoff, g->hv_inv_bw, g->p.sfd_strength, (double)g->p.hv_order};
    put(dbl, sizeof(dbl));
    const void* ptrs[] = {g->fnoise, g->fsum, g->hvw_full, g->out, g->outsfd};
    put(ptrs, sizeof(ptrs));
    return k;
}

static void drop_step_graph(ns_gpu* g) {
    if (g->step_exec) cudaGraphExecDestroy(g->step_exec);
    g->step_exec = nullptr;
    g->step_key.clear();
}

// Capture one step into g->step_exec (relaxed mode: the launch helpers set
// kernel attributes); on any failure the instance keeps launching directly.
template <typename T> static void capture_step(ns_gpu* g, const ColArgs<T>& a, std::vector<unsigned char>&& key) {
    drop_step_graph(g);
    if (cudaStreamBeginCapture(g->st, cudaStreamCaptureModeRelaxed) != cudaSuccess) {
        cudaGetLastError();
        g->step_graph_off = 1;
        return;
    }
    const unsigned long long l0 = g->launches;
    const int s = one_step<T>(g, a);
    cudaGraph_t graph = nullptr;
    const cudaError_t e = cudaStreamEndCapture(g->st, &graph);
    g->step_launches = g->launches - l0;
    g->launches = l0;
    cudaGraphExec_t exec = nullptr;
    if (s != NS_GPU_OK || e != cudaSuccess || !graph || cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) {
        cudaGetLastError();
        g->step_graph_off = 1;
        g->err.clear();
    } else {
        g->step_exec = exec;
        g->step_key = std::move(key);
    }
    if (graph) cudaGraphDestroy(graph);
}

// nsteps RK4 steps.  A step's launches are captured once as a CUDA graph and
// replayed (small grids are launch-bound: a 128^2 step is nine kernels of a few
// microseconds); the first step with new arguments runs directly, which also
// sets the kernels' attributes before a capture.  Profiling runs (per-launch
// events) launch directly.
template <typename T> static int advance_t(ns_gpu* g, int nsteps) {
    NSG_TRY(ensure_noise(g));
    if (!g->fields_valid) {
        NSG_TRY(prologue<T>(g, g->W0, g->PSI0, g->psi0_valid ? 0 : 1, 4));
        g->fields_valid = 1;
        g->psi0_valid = 0;
    }
    ColArgs<T> a = col_args<T>(g);
    if (nsteps > 0 && !g->prof && !g->step_graph_off) {
        std::vector<unsigned char> key = step_key<T>(g, a);
        if (!g->step_exec || key != g->step_key) {
            if (key != g->step_key_seen) {  // new arguments: one direct step first
                NSG_TRY(one_step<T>(g, a));
                g->step_key_seen = key;
                --nsteps;
                if (nsteps == 0) return NS_GPU_OK;
            }
            capture_step<T>(g, a, std::move(key));
        }
        if (g->step_exec) {
            for (int n = 0; n < nsteps; ++n) {
                NSG_CUDA(g, cudaGraphLaunch(g->step_exec, g->st));
                g->launches += g->step_launches;
            }
            return NS_GPU_OK;
        }
    }
    for (int n = 0; n < nsteps; ++n) NSG_TRY(one_step<T>(g, a));
    return NS_GPU_OK;
}

int nsg_prepare_fields(ns_gpu* g) {
    if (g->prec != NS_GPU_FP32) return NS_GPU_ERR_INVALID;
    if (!g->fields_valid) {
        NSG_TRY(prologue<float>(g, g->W0, g->PSI0, g->psi0_valid ? 0 : 1, 4));
        g->fields_valid = 1;
        g->psi0_valid = 0;
    }
    return NS_GPU_OK;
}

void nsg_stage_args(ns_gpu* g, RowArgs<float>* ra, ColArgs<float>* ca) {
    *ra = row_args<float>(g);
    for (int f = 0; f < 4; ++f) ra->F[f] = (const float2*)g->F[f];
    ra->dx[0] = 1; ra->dx[1] = 0; ra->dx[2] = 1; ra->dx[3] = 0;  // psi_x, psi_y, omega_x, omega_y
    *ca = col_args<float>(g);
    ca->fsum = nullptr;  // the ensemble kernel draws its members' forcing itself
}

// ------------------------------------------------------------ allocation
static int dalloc(ns_gpu* g, void** p, size_t bytes) {
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        *p = nullptr;
        NSG_FAIL(g, NS_GPU_ERR_ALLOC, "cudaMalloc(%zu bytes): %s", bytes, cudaGetErrorString(e));
    }
    e = cudaMemsetAsync(*p, 0, bytes, g->st);
    if (e != cudaSuccess) NSG_FAIL(g, NS_GPU_ERR_CUDA, "cudaMemset: %s", cudaGetErrorString(e));
    return NS_GPU_OK;
}

static int ensure_staging(ns_gpu* g) {
    if (g->spec[0]) return NS_GPU_OK;
    const size_t ns = (size_t)g->g.nkx * g->g.nky * sizeof(double2);
    const size_t nr = (size_t)g->g.nx * g->g.ny * sizeof(double);
    for (int i = 0; i < 5; ++i) NSG_TRY(dalloc(g, (void**)&g->spec[i], ns));
    for (int i = 0; i < 5; ++i) NSG_TRY(dalloc(g, (void**)&g->real[i], nr));
    return NS_GPU_OK;
}

static int ensure_outside(ns_gpu* g) {
    if (g->out) return NS_GPU_OK;
    const size_t ns = (size_t)g->g.nkx * g->g.nky * sizeof(double2);
    NSG_TRY(dalloc(g, (void**)&g->out, ns));
    NSG_TRY(dalloc(g, (void**)&g->outsfd, ns));
    return NS_GPU_OK;
}

static int ensure_scratch(ns_gpu* g, size_t bytes) {
    if (g->scratch_bytes >= bytes) return NS_GPU_OK;
    if (g->scratch) cudaFree(g->scratch);
    g->scratch = nullptr;
    g->scratch_bytes = 0;
    NSG_TRY(dalloc(g, &g->scratch, bytes));
    g->scratch_bytes = bytes;
    return NS_GPU_OK;
}

static int h2d(ns_gpu* g, void* dst, const void* src, size_t bytes) {
    NSG_CUDA(g, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, g->st));
    return NS_GPU_OK;
}
static int d2h(ns_gpu* g, void* dst, const void* src, size_t bytes) {
    NSG_CUDA(g, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, g->st));
    return NS_GPU_OK;
}
static int sync(ns_gpu* g) {
    NSG_CUDA(g, cudaStreamSynchronize(g->st));
    return NS_GPU_OK;
}
static size_t spec_bytes(const ns_gpu* g) { return (size_t)g->g.nkx * g->g.nky * sizeof(double2); }
static size_t real_bytes(const ns_gpu* g) { return (size_t)g->g.nx * g->g.ny * sizeof(double); }

// tables in the working precision
template <typename T> static int build_tables(ns_gpu* g) {
    const long long n = (long long)g->g.Kxp * g->g.Ky;
    const int sfd = (g->p.sfd_enabled && g->p.sfd_strength > 0.0) ? 1 : 0;
    const int order = g->p.hv_order > 0 ? g->p.hv_order : 1;
    k_tables<T><<<grid_for(n), 256, 0, g->st>>>(g->g, g->hvw_full, sfd, g->p.sfd_strength, order, g->hv_cutoff,
                                                g->hv_inv_bw, (T*)g->kxv, (T*)g->kyv, (T*)g->hvw, (T*)g->sfdw);
    NSG_LAUNCHED(g);
    return NS_GPU_OK;
}

// hyperviscosity.c:60-102 — kmax on the device, cutoff/inverse bandwidth as the reference, FP64 weight table
static int compute_hv(ns_gpu* g) {
    NSG_CUDA(g, cudaMemsetAsync(&g->ds->kmax_bits, 0, sizeof(unsigned long long), g->st));
    const long long n = (long long)g->g.nkx * g->g.nky;
    k_kmax<<<grid_for(n), 256, 0, g->st>>>(g->g, g->ds);
    NSG_LAUNCHED(g);
    unsigned long long bits = 0;
    NSG_TRY(d2h(g, &bits, &g->ds->kmax_bits, sizeof(bits)));
    NSG_TRY(sync(g));
    double kmax;
    memcpy(&kmax, &bits, sizeof(kmax));
    double ratio = g->p.hv_cutoff_ratio;
    ratio = ratio < 0.0 ? 0.0 : (ratio > 1.0 ? 1.0 : ratio);
    g->hv_kmax = kmax;
    g->hv_cutoff = ratio * kmax;
    const double bw = fmax(kmax - g->hv_cutoff, 1e-12);
    g->hv_inv_bw = (bw > 0.0) ? 1.0 / bw : 0.0;
    const int enabled = (g->p.hv_enabled && g->p.hv_coefficient > 0.0 && kmax > 0.0) ? 1 : 0;
    const int order = g->p.hv_order > 0 ? g->p.hv_order : 1;
    k_hv_weights<<<grid_for(n), 256, 0, g->st>>>(g->g, enabled, g->p.hv_coefficient, order, g->hv_cutoff, g->hv_inv_bw,
                                                 g->hvw_full);
    NSG_LAUNCHED(g);
    return g->prec == NS_GPU_FP64 ? build_tables<double>(g) : build_tables<float>(g);
}

// forcing amplitude sigma = sqrt(2 eps / sum_full 1/k^2) over the kept modes of the shell
__global__ void k_forcing_sigma(Geo g, double kmin, double kmax, double2* part) {
    DD acc = {0.0, 0.0};
    const long long n = (long long)g.nkx * g.nky;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n; idx += (long long)gridDim.x * blockDim.x) {
        const int j = (int)(idx / g.nkx), i = (int)(idx - (long long)j * g.nkx);
        const double k2 = geo_k2(g, j, i);
        const double km = sqrt(k2);
        if (geo_kept(g, j, i) && k2 > 1e-12 && km >= kmin && km <= kmax) dd_add(acc, (i == 0 ? 1.0 : 2.0) / k2);
    }
    DD t = block_dd(acc);
    if (threadIdx.x == 0) part[blockIdx.x] = make_double2(t.s, t.c);
}

static int compute_sigma(ns_gpu* g) {
    g->f_sigma = 0.0;
    if (!g->p.forcing_enabled || g->p.forcing_epsilon <= 0.0) return NS_GPU_OK;
    const long long n = (long long)g->g.nkx * g->g.nky;
    const int nb = grid_for(n, 256, g->part_n);
    k_forcing_sigma<<<nb, 256, 0, g->st>>>(g->g, g->p.forcing_kmin, g->p.forcing_kmax, g->part);
    NSG_LAUNCHED(g);
    k_merge_partials<<<1, 256, 0, g->st>>>(g->part, nb, g->dres);
    NSG_LAUNCHED(g);
    double acc = 0.0;
    NSG_TRY(d2h(g, &acc, g->dres, sizeof(double)));
    NSG_TRY(sync(g));
    g->f_sigma = acc > 0.0 ? sqrt(2.0 * g->p.forcing_epsilon / acc) : 0.0;
    return NS_GPU_OK;
}

// ================================================================== C-ABI
// (C linkage comes from the declarations in ns_gpu.h)

const char* ns_gpu_status_string(int s) {
    switch (s) {
        case NS_GPU_OK: return "ok";
        case NS_GPU_ERR_INVALID: return "invalid argument";
        case NS_GPU_ERR_NO_DEVICE: return "no CUDA device";
        case NS_GPU_ERR_CUDA: return "CUDA error";
        case NS_GPU_ERR_ALLOC: return "device allocation failed";
        case NS_GPU_ERR_DIVERGED: return "non-finite values in the state";
        default: return "unknown status";
    }
}

const char* ns_gpu_last_error(const ns_gpu* g) { return g ? g->err.c_str() : "null instance"; }

void ns_gpu_destroy(ns_gpu* g) {
    if (!g) return;
    if (g->st) cudaStreamSynchronize(g->st);
    drop_step_graph(g);
    void* bufs[] = {g->F[0], g->F[1], g->F[2], g->F[3], g->G, g->W0, g->WS, g->ACC, g->PSI0, g->SFD, g->KS,
                    g->KP, g->hvw, g->sfdw, g->kxv, g->kyv, g->twc, g->twr, g->twh, g->hvw_full, g->ds, g->part,
                    g->dres, g->dflag, g->out, g->outsfd, g->scratch, g->flushbuf};
    for (void* b : bufs)
        if (b) cudaFree(b);
    for (int i = 0; i < 5; ++i) {
        if (g->spec[i]) cudaFree(g->spec[i]);
        if (g->real[i]) cudaFree(g->real[i]);
    }
    if (g->fnoise) cudaFree(g->fnoise);
    if (g->fsum) cudaFree(g->fsum);
    if (g->st2) cudaStreamDestroy(g->st2);
    if (g->ev_a) cudaEventDestroy(g->ev_a);
    if (g->ev_b) cudaEventDestroy(g->ev_b);
    if (g->stn) cudaStreamDestroy(g->stn);
    if (g->evn0) cudaEventDestroy(g->evn0);
    if (g->evn1) cudaEventDestroy(g->evn1);
    if (g->st) cudaStreamDestroy(g->st);
    delete g;
}

// Create an instance.  kc (may be NULL) fixes the generic stage kernels' tiling:
// values per thread of the row / column transforms (er, ec), rows per row block
// (rpc), kept columns per column block (cw), and the alignment of the padded
// kept-column count Kxp; zero fields are chosen automatically.
int nsg_create(int nx, int ny, double Lx, double Ly, int precision, const NsgTiling* kc, ns_gpu** out) {
    if (!out) return NS_GPU_ERR_INVALID;
    *out = nullptr;
    // Any side in [8, 4096] whose transform lengths (nx/2 for even nx, nx for odd
    // nx; ny) factor into primes up to NSG_MAX_PRIME: a prime factor p is one
    // direct p-point pass, p operations per output, so large primes are refused
    // rather than run at quadratic cost.
    unsigned long long rxa = 0, rxb = 0, rya = 0, ryb = 0;
    const int oddx = (nx & 1);
    const int Hlen = oddx ? nx : nx / 2;
    const int nrx = (nx >= 8 && nx <= 4096) ? mr_plan(Hlen, NSG_MAX_PRIME, &rxa, &rxb) : -1;
    const int nry = (ny >= 8 && ny <= 4096) ? mr_plan(ny, NSG_MAX_PRIME, &rya, &ryb) : -1;
    if (nrx < 0 || nry < 0) {
        fprintf(stderr,
                "ns_gpu_create: nx=%d ny=%d: each side must lie in [8, 4096] and its transform length (nx/2 for even "
                "nx, nx for odd nx; ny) have no prime factor above %d\n",
                nx, ny, NSG_MAX_PRIME);
        return NS_GPU_ERR_INVALID;
    }
    const int pow2_grid = is_pow2(nx) && is_pow2(ny);
    if (!(Lx > 0.0) || !(Ly > 0.0) || (precision != NS_GPU_FP64 && precision != NS_GPU_FP32)) return NS_GPU_ERR_INVALID;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev < 1) {
        fprintf(stderr, "ns_gpu_create: no CUDA device (%s)\n", cudaGetErrorString(e));
        return NS_GPU_ERR_NO_DEVICE;
    }
    ns_gpu* g = new ns_gpu();
    memset(g->F, 0, sizeof(g->F));
    g->G = g->W0 = g->WS = g->ACC = g->PSI0 = g->SFD = g->KS = g->KP = nullptr;
    g->hvw = g->sfdw = g->kxv = g->kyv = g->twc = g->twr = g->twh = nullptr;
    g->hvw_full = nullptr;
    g->ds = nullptr;
    g->part = nullptr;
    g->dres = nullptr;
    g->dflag = nullptr;
    for (int i = 0; i < 5; ++i) { g->spec[i] = nullptr; g->real[i] = nullptr; }
    g->out = g->outsfd = nullptr;
    g->scratch = nullptr;
    g->scratch_bytes = 0;
    g->flushbuf = nullptr;
    g->flush_bytes = 0;
    g->prof = nullptr;
    g->step_exec = nullptr;
    g->stn = nullptr;
    g->evn0 = g->evn1 = nullptr;
    g->step_launches = 0;
    g->step_graph_off = 0;
    g->launches = 0;
    g->outside_active = 0;
    g->fields_valid = 0;
    g->psi0_valid = 0;
    g->params_set = 0;
    g->f_sigma = 0.0;
    g->prec = precision;
    cudaGetDevice(&g->device);
    g->num_sms = 1;
    cudaDeviceGetAttribute(&g->num_sms, cudaDevAttrMultiProcessorCount, g->device);
    {
        // NS_GB300_GENERIC_KERNELS=1 selects the generic Stockham stage kernels at every size
        const char* gen = getenv("NS_GB300_GENERIC_KERNELS");
        const int generic = (gen && gen[0] == '1') || (kc && (kc->er || kc->ec));
        // FP32 also has register-resident row and column passes at 4096
        // (their F/G layouts assume a power-of-two ny)
        g->fast_row = (!generic && pow2_grid && (nx == 2048 || (nx == 4096 && precision == NS_GPU_FP32))) ? 1 : 0;
        g->fast_col = (!generic && pow2_grid && (ny == 2048 || (ny == 4096 && precision == NS_GPU_FP32 && nsg_fast_col_q())))
                          ? 1
                          : 0;
    }
    if (cudaStreamCreateWithFlags(&g->st, cudaStreamNonBlocking) != cudaSuccess) {
        delete g;
        return NS_GPU_ERR_CUDA;
    }
    Geo& G = g->g;
    G.nx = nx;
    G.ny = ny;
    G.nkx = nx / 2 + 1;
    G.nky = ny;
    G.H = Hlen;
    G.Kx = (2 * G.nkx) / 3 + 1;
    G.Kyh = (2 * ny) / 6;
    G.Ky = 2 * G.Kyh + 1;
    G.logny = ilog2(ny);
    G.logH = ilog2(G.H);
    G.rxa = rxa;
    G.rxb = rxb;
    G.rya = rya;
    G.ryb = ryb;
    G.nrx = nrx;
    G.nry = nry;
    G.oddx = oddx;
    // mixed-radix threads per sequence: about one per eight points, whole warps, at most 256
    G.TTr = std::min(256, std::max(32, ((G.H + 7) / 8 + 31) / 32 * 32));
    G.TTc = std::min(256, std::max(32, ((ny + 7) / 8 + 31) / 32 * 32));
    G.Lx = Lx;
    G.Ly = Ly;
    // With the register-resident stage kernels F and G are both kx-column-contiguous
    // (F in blocks of ny rows): the column pass reads G and writes F as whole
    // columns, and the row pass reads F and writes G group-wide, as runs of one
    // column over the group's consecutive rows.
    G.fLB = (g->fast_row || g->fast_col) ? G.logny : 0;
    G.fTG = G.fLB ? 1 : 0;
    // automatic tiling (timed on GB300 at 128^2 .. 1024^2, FP32 and FP64): rows
    // with 4 values per thread up to 512-point row transforms (1024^2) and 16 from
    // 1024 points; columns with 16 values per thread from 512 points, 4 below
    // (E = 0: the mixed-radix bodies, for lengths that are not powers of two)
    const int mr_row = oddx || !is_pow2(G.H), mr_col = !is_pow2(ny);
    g->ER = mr_row ? 0 : (kc && kc->er) ? kc->er : (G.H >= 1024 ? 16 : 4);
    g->EC = mr_col ? 0 : (kc && kc->ec) ? kc->ec : (ny >= 512 ? 16 : 4);
    const size_t cs = (precision == NS_GPU_FP64) ? sizeof(double2) : sizeof(float2);
    // fields in parallel (a thread group per field): automatic when the
    // transforms are short (row groups of at most two warps, column groups of at
    // most four) and too few to give the SMs more than a few warps each one after
    // another: 64 warps per SM in FP32, 8 in FP64 (timed on GB300 from 32^2 to
    // 1024^2: FP64 768^2 rows, 49152 threads of 64-thread transforms, ran 2 %
    // slower with groups, 384^2 columns 23 % faster).  Row groups narrower than a
    // warp share warps (TT divides 32); column groups narrower than a warp take
    // 32 / TC columns each, so that they are whole warps.
    const int TTp = g->ER ? G.H / g->ER : G.TTr, TCp = g->EC ? ny / g->EC : G.TTc;
    const long long busy = (precision == NS_GPU_FP32 ? 64LL : 8LL) * 32 * g->num_sms;
    const bool row_fits = TTp % 32 == 0 || 32 % TTp == 0;
    const bool col_fits = TCp % 32 == 0 || (32 % TCp == 0 && G.Kx >= 32 / TCp);
    G.fpr = (kc && kc->fpr) ? (kc->fpr > 0) : (row_fits && TTp <= 64 && (long long)ny * TTp < busy);
    G.fpc = (kc && kc->fpc) ? (kc->fpc > 0) : (col_fits && TCp <= 128 && (long long)G.Kx * TCp < busy);
    // column tile width: up to 16 columns, <= 512 threads, <= ~100 KB shared memory
    {
        const int TC = g->EC ? ny / g->EC : G.TTc;
        const int P = G.fpc ? 4 : 1;
        const int nbuf = g->EC ? P : 2 * P;
        int CW = (G.fpc && TC < 32) ? 32 / TC : 1;
        // with a group per field a column block is already four groups: widen it
        // only while that still leaves two blocks per SM
        while (CW < 16 && 2 * CW * TC * P <= 512 && (size_t)nbuf * 2 * CW * spad_len(ny) * cs <= 100 * 1024 && CW < G.Kx &&
               G.Kx / (2 * CW) >= (G.fpc ? 2 : 1) * g->num_sms)
            CW *= 2;
        if (kc && kc->cw) CW = kc->cw;
        G.CW = CW;
        int al = CW;
        if (kc && kc->kxp_align > al) al = kc->kxp_align;
        G.Kxp = ((G.Kx + al - 1) / al) * al;
    }
    // rows per CTA: up to 256 threads (128 for FP64 rows of one group), <= ~100 KB
    // shared memory for four fields
    {
        const int TT = g->ER ? G.H / g->ER : G.TTr;
        const int P = G.fpr ? 4 : 1;
        const int nbuf = g->ER ? 4 : 4 + P;  // four field buffers (+ the mixed-radix scratch per group)
        const int budget = (G.fpr || precision == NS_GPU_FP32) ? 256 : 128;
        int RPC = 1;
        while (2 * RPC * TT * P <= budget && 2 * RPC <= ny && ny % (2 * RPC) == 0 &&
               (size_t)nbuf * 2 * RPC * spad_len(G.H) * cs <= 100 * 1024 && ny / (2 * RPC) >= g->num_sms &&
               (TT <= 32 || !G.fpr || 2 * RPC * P <= 15))
            RPC *= 2;
        if (kc && kc->rpc) RPC = kc->rpc;
        G.RPC = RPC;
    }
    // a group per field needs row groups of whole warps or of a divisor of a warp,
    // column groups of whole warps, at most 256 (row) / 512 (column) threads per
    // CTA, and at most 15 named barriers per CTA (groups wider than a warp)
    if (G.fpr && !((TTp % 32 == 0 || 32 % TTp == 0) && G.RPC * 4 * TTp <= 256 && (TTp <= 32 || G.RPC * 4 <= 15))) {
        fprintf(stderr, "ns_gpu_create: nx=%d ny=%d: the row pass cannot run a thread group per field with this tiling\n",
                nx, ny);
        cudaStreamDestroy(g->st);
        delete g;
        return NS_GPU_ERR_INVALID;
    }
    if (G.fpc && !((G.CW * TCp) % 32 == 0 && 4 * G.CW * TCp <= 512)) {
        fprintf(stderr, "ns_gpu_create: nx=%d ny=%d: the column pass cannot run a thread group per field with this tiling\n",
                nx, ny);
        cudaStreamDestroy(g->st);
        delete g;
        return NS_GPU_ERR_INVALID;
    }
    {
        // the resolved tiling: radix 4 or 16 (or the mixed-radix bodies), row blocks
        // that cover ny exactly, CTAs within the stage kernels' launch bounds
        const int TT = g->ER ? G.H / g->ER : G.TTr, TC = g->EC ? ny / g->EC : G.TTc;
        const int rthr = G.RPC * (G.fpr ? 4 : 1) * TT, cthr = G.CW * (G.fpc ? 4 : 1) * TC;
        const bool ok = (g->ER == 0 || g->ER == 4 || g->ER == 16) && (g->EC == 0 || g->EC == 4 || g->EC == 16) &&
                        TT >= 1 && TC >= 1 && G.RPC >= 1 && ny % G.RPC == 0 && G.CW >= 1 && rthr <= 256 && cthr <= 512;
        if (!ok) {
            fprintf(stderr,
                    "ns_gpu_create: nx=%d ny=%d: invalid stage tiling (row radix %d, column radix %d, %d rows and %d "
                    "columns per CTA)\n",
                    nx, ny, g->ER, g->EC, G.RPC, G.CW);
            cudaStreamDestroy(g->st);
            delete g;
            return NS_GPU_ERR_INVALID;
        }
    }
    // grids whose step kernels have a copy with the size fields as constants
    g->fold = (precision == NS_GPU_FP32 && fold_sizes_match<256>(G))   ? 256
              : (precision == NS_GPU_FP64 && fold_sizes_match<128>(G)) ? 128
                                                                       : 0;
    // the stage kernels' shared memory must fit one CTA (odd nx near the upper
    // bound needs the full length-nx row in five buffers)
    {
        int optin = 0;
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, g->device);
        const size_t row_sm = (size_t)(g->ER ? 4 : 4 + (G.fpr ? 4 : 1)) * G.RPC * spad_len(G.H) * cs;
        const size_t col_sm = ((size_t)(g->EC ? 1 : 2) * (G.fpc ? 4 : 1) * G.CW * spad_len(ny) + (size_t)G.CW * G.Ky) * cs;
        if (optin > 0 && (row_sm > (size_t)optin || col_sm > (size_t)optin)) {
            fprintf(stderr,
                    "ns_gpu_create: nx=%d ny=%d: the stage kernels need %zu / %zu bytes of shared memory per CTA, above "
                    "the device's %d\n",
                    nx, ny, row_sm, col_sm, optin);
            cudaStreamDestroy(g->st);
            delete g;
            return NS_GPU_ERR_INVALID;
        }
    }
    const size_t A = (size_t)ny * G.Kxp * cs;
    const size_t Cb = (size_t)G.Kxp * G.Ky * cs;
    const size_t Rb = (size_t)G.Kxp * G.Ky * (cs / 2);
    int s = NS_GPU_OK;
    for (int f = 0; f < 4 && s == NS_GPU_OK; ++f) s = dalloc(g, &g->F[f], A);
    if (s == NS_GPU_OK) s = dalloc(g, &g->G, A);
    void** states[] = {&g->W0, &g->WS, &g->ACC, &g->PSI0, &g->SFD, &g->KS, &g->KP};
    for (void** p : states)
        if (s == NS_GPU_OK) s = dalloc(g, p, Cb);
    if (s == NS_GPU_OK) s = dalloc(g, &g->hvw, Rb);
    if (s == NS_GPU_OK) s = dalloc(g, &g->sfdw, Rb);
    if (s == NS_GPU_OK) s = dalloc(g, &g->kxv, (size_t)G.Kxp * (cs / 2));
    if (s == NS_GPU_OK) s = dalloc(g, &g->kyv, (size_t)G.Ky * (cs / 2));
    if (s == NS_GPU_OK) s = dalloc(g, &g->twc, (size_t)ny * cs);
    if (s == NS_GPU_OK) s = dalloc(g, &g->twr, (size_t)G.H * cs);
    if (s == NS_GPU_OK) s = dalloc(g, &g->twh, (size_t)G.H * cs);
    if (s == NS_GPU_OK) s = dalloc(g, (void**)&g->hvw_full, (size_t)G.nkx * G.nky * sizeof(double));
    if (s == NS_GPU_OK) s = dalloc(g, (void**)&g->ds, sizeof(DevScalars));
    g->part_n = 2048;
    if (s == NS_GPU_OK) s = dalloc(g, (void**)&g->part, (size_t)4 * g->part_n * sizeof(double2));
    if (s == NS_GPU_OK) s = dalloc(g, (void**)&g->dres, 16 * sizeof(double));
    if (s == NS_GPU_OK) s = dalloc(g, (void**)&g->dflag, sizeof(int));
    if (s != NS_GPU_OK) {
        fprintf(stderr, "ns_gpu_create: %s\n", g->err.c_str());
        ns_gpu_destroy(g);
        return s;
    }
    if (precision == NS_GPU_FP64) {
        k_twiddles<<<grid_for(ny), 256, 0, g->st>>>((double2*)g->twc, ny, ny);
        k_twiddles<<<grid_for(G.H), 256, 0, g->st>>>((double2*)g->twr, G.H, G.H);
        k_twiddles<<<grid_for(G.H), 256, 0, g->st>>>((double2*)g->twh, G.H, nx);
    } else {
        k_twiddles<<<grid_for(ny), 256, 0, g->st>>>((float2*)g->twc, ny, ny);
        k_twiddles<<<grid_for(G.H), 256, 0, g->st>>>((float2*)g->twr, G.H, G.H);
        k_twiddles<<<grid_for(G.H), 256, 0, g->st>>>((float2*)g->twh, G.H, nx);
    }
    g->launches += 3;
    // default parameters: the reference allocate defaults (spectral_memory.c:17-19, hyperviscosity.c:15-30)
    ns_gpu_params p;
    memset(&p, 0, sizeof(p));
    p.Re = 1.0;
    p.cfl_factor = 0.3;
    p.dt = 0.01;
    p.hv_order = 8;
    p.hv_cutoff_ratio = 0.65;
    p.sfd_timescale = 1.0;
    s = ns_gpu_set_params(g, &p);
    if (s != NS_GPU_OK) {
        fprintf(stderr, "ns_gpu_create: %s\n", g->err.c_str());
        ns_gpu_destroy(g);
        return s;
    }
    *out = g;
    return NS_GPU_OK;
}

int ns_gpu_create(int nx, int ny, double Lx, double Ly, int precision, ns_gpu** out) {
    return nsg_create(nx, ny, Lx, Ly, precision, nullptr, out);
}

int ns_gpu_create_tiled(int nx, int ny, double Lx, double Ly, int precision, const ns_gpu_tiling* t, ns_gpu** out) {
    if (!t) return nsg_create(nx, ny, Lx, Ly, precision, nullptr, out);
    if (out) *out = nullptr;
    auto pow2_or_zero = [](int v) { return v == 0 || is_pow2(v); };
    if (!(t->row_radix == 0 || t->row_radix == 4 || t->row_radix == 16) ||
        !(t->col_radix == 0 || t->col_radix == 4 || t->col_radix == 16) || !pow2_or_zero(t->rows_per_cta) ||
        !pow2_or_zero(t->cols_per_cta) || t->rows_per_cta < 0 || t->cols_per_cta < 0 || t->cols_per_cta > 64 ||
        t->row_field_groups < -1 || t->row_field_groups > 1 || t->col_field_groups < -1 || t->col_field_groups > 1)
        return NS_GPU_ERR_INVALID;
    NsgTiling k;
    memset(&k, 0, sizeof(k));
    k.er = t->row_radix;
    k.ec = t->col_radix;
    k.rpc = t->rows_per_cta;
    k.cw = t->cols_per_cta;
    k.fpr = t->row_field_groups;
    k.fpc = t->col_field_groups;
    return nsg_create(nx, ny, Lx, Ly, precision, &k, out);
}

int ns_gpu_get_tiling(const ns_gpu* g, ns_gpu_tiling* t) {
    if (!g || !t) return NS_GPU_ERR_INVALID;
    t->row_radix = g->ER;
    t->col_radix = g->EC;
    t->rows_per_cta = g->g.RPC;
    t->cols_per_cta = g->g.CW;
    t->row_field_groups = g->g.fpr ? 1 : -1;
    t->col_field_groups = g->g.fpc ? 1 : -1;
    t->register_resident = (g->fast_row ? 1 : 0) | (g->fast_col ? 2 : 0);
    return NS_GPU_OK;
}

int ns_gpu_dims(const ns_gpu* g, int* kx_kept, int* ky_kept) {
    if (!g) return NS_GPU_ERR_INVALID;
    if (kx_kept) *kx_kept = g->g.Kx;
    if (ky_kept) *ky_kept = g->g.Ky;
    return NS_GPU_OK;
}

uint64_t ns_gpu_launch_count(const ns_gpu* g) { return g ? g->launches : 0; }

int ns_gpu_synchronize(ns_gpu* g) {
    if (!g) return NS_GPU_ERR_INVALID;
    return sync(g);
}

int ns_gpu_set_params(ns_gpu* g, const ns_gpu_params* p) {
    if (!g || !p) return NS_GPU_ERR_INVALID;
    if (!(p->Re > 0.0)) NSG_FAIL(g, NS_GPU_ERR_INVALID, "Re must be positive (got %g)", p->Re);
    if (p->scheme != NS_GPU_RK4 && p->scheme != NS_GPU_IFRK4)
        NSG_FAIL(g, NS_GPU_ERR_INVALID, "unknown time scheme %d", p->scheme);
    const int hv_changed = !g->params_set || p->hv_enabled != g->p.hv_enabled || p->hv_coefficient != g->p.hv_coefficient ||
                           p->hv_order != g->p.hv_order || p->hv_cutoff_ratio != g->p.hv_cutoff_ratio ||
                           p->sfd_enabled != g->p.sfd_enabled || p->sfd_strength != g->p.sfd_strength;
    const int f_changed = !g->params_set || p->forcing_enabled != g->p.forcing_enabled ||
                          p->forcing_kmin != g->p.forcing_kmin || p->forcing_kmax != g->p.forcing_kmax ||
                          p->forcing_epsilon != g->p.forcing_epsilon;
    const int dt_changed = !g->params_set || p->dt != g->p.dt;
    const int fsub_changed = !g->params_set || p->forcing_substeps != g->p.forcing_substeps;
    if (p->forcing_substeps < 0 || p->forcing_substeps > 1024)
        NSG_FAIL(g, NS_GPU_ERR_INVALID, "forcing_substeps %d not in [0, 1024]", p->forcing_substeps);
    g->p = *p;
    g->params_set = 1;
    if (hv_changed) NSG_TRY(compute_hv(g));
    if (f_changed) NSG_TRY(compute_sigma(g));
    if (dt_changed) {  // a kernel parameter, ordered on the stream: no host copy, no sync
        k_set_dt_fixed<<<1, 1, 0, g->st>>>(g->ds, p->dt);
        NSG_LAUNCHED(g);
    }
    if (fsub_changed) {
        unsigned long long m = p->forcing_substeps > 1 ? (unsigned long long)p->forcing_substeps : 1ULL;
        NSG_TRY(h2d(g, &g->ds->fsub, &m, sizeof(m)));
        NSG_TRY(sync(g));
    }
    return NS_GPU_OK;
}

int ns_gpu_geometry(ns_gpu* g, double* x, double* y, double* kx, double* ky, double* k2, int* mask) {
    if (!g) return NS_GPU_ERR_INVALID;
    NSG_TRY(ensure_staging(g));
    const Geo& G = g->g;
    double* dx = g->real[0];
    double* dy = g->real[0] + G.nx;
    double* dkx = g->real[0] + G.nx + G.ny;
    double* dky = g->real[0] + G.nx + G.ny + G.nkx;
    double* dk2 = (double*)g->spec[0];
    int* dmask = (int*)g->spec[1];
    const long long n = (long long)G.nkx * G.nky;
    k_geometry<<<grid_for(n), 256, 0, g->st>>>(G, dx, dy, dkx, dky, dk2, dmask);
    NSG_LAUNCHED(g);
    if (x) NSG_TRY(d2h(g, x, dx, G.nx * sizeof(double)));
    if (y) NSG_TRY(d2h(g, y, dy, G.ny * sizeof(double)));
    if (kx) NSG_TRY(d2h(g, kx, dkx, G.nkx * sizeof(double)));
    if (ky) NSG_TRY(d2h(g, ky, dky, G.nky * sizeof(double)));
    if (k2) NSG_TRY(d2h(g, k2, dk2, n * sizeof(double)));
    if (mask) NSG_TRY(d2h(g, mask, dmask, n * sizeof(int)));
    return sync(g);
}

int ns_gpu_hv_weights(ns_gpu* g, double* kmax, double* cutoff, double* inv_bw, double* weights_out) {
    if (!g) return NS_GPU_ERR_INVALID;
    NSG_TRY(compute_hv(g));
    if (kmax) *kmax = g->hv_kmax;
    if (cutoff) *cutoff = g->hv_cutoff;
    if (inv_bw) *inv_bw = g->hv_inv_bw;
    if (weights_out) NSG_TRY(d2h(g, weights_out, g->hvw_full, (size_t)g->g.nkx * g->g.nky * sizeof(double)));
    return sync(g);
}

// ------------------------------------------------- host-array transforms
template <typename T> static int forward_t(ns_gpu* g, const double* field, double* field_hat) {
    NSG_TRY(h2d(g, g->real[0], field, real_bytes(g)));
    RowArgs<T> a = row_args<T>(g);
    a.in_real = g->real[0];
    NSG_TRY(row_launch<T, ROW_FWD1>(g, a));
    NSG_CUDA(g, cudaMemsetAsync(g->spec[0], 0, spec_bytes(g), g->st));
    ColArgs<T> c = col_args<T>(g);
    c.out_spec = g->spec[0];
    c.out_scale = 1.0 / ((double)g->g.nx * (double)g->g.ny);
    NSG_TRY((col_launch<T, COL_FWD_EXPORT, 0>(g, c)));
    g->fields_valid = 0;
    NSG_TRY(d2h(g, field_hat, g->spec[0], spec_bytes(g)));
    return sync(g);
}

int ns_gpu_forward(ns_gpu* g, const double* field, double* field_hat) {
    if (!g || !field || !field_hat) return NS_GPU_ERR_INVALID;
    NSG_TRY(ensure_staging(g));
    return g->prec == NS_GPU_FP64 ? forward_t<double>(g, field, field_hat) : forward_t<float>(g, field, field_hat);
}

template <typename T> static int import_kept(ns_gpu* g, const double2* spec, void* W, void* P, const double2* pspec) {
    const long long n = (long long)g->g.nkx * g->g.nky;
    k_import<T><<<grid_for(n), 256, 0, g->st>>>(g->g, spec, pspec, nullptr, (Cx<T>*)W, (Cx<T>*)P, nullptr, nullptr,
                                                nullptr, nullptr);
    NSG_LAUNCHED(g);
    return NS_GPU_OK;
}

template <typename T> static int inverse_t(ns_gpu* g, const double* field_hat, double* field, double* masked) {
    NSG_TRY(h2d(g, g->spec[0], field_hat, spec_bytes(g)));
    NSG_TRY(import_kept<T>(g, g->spec[0], g->KS, nullptr, nullptr));
    ColArgs<T> c = col_args<T>(g);
    c.W0 = (Cx<T>*)g->KS;
    NSG_TRY((col_launch<T, COL_INV1, 0>(g, c)));
    RowArgs<T> a = row_args<T>(g);
    a.F[0] = (const Cx<T>*)g->F[0];
    a.out_real[0] = g->real[0];
    NSG_TRY(row_launch<T, ROW_INV1>(g, a));
    g->fields_valid = 0;
    if (masked) {
        const long long n = (long long)g->g.nkx * g->g.nky;
        k_dealias<<<grid_for(n), 256, 0, g->st>>>(g->g, g->spec[0], g->spec[1]);
        NSG_LAUNCHED(g);
        NSG_TRY(d2h(g, masked, g->spec[1], spec_bytes(g)));
    }
    NSG_TRY(d2h(g, field, g->real[0], real_bytes(g)));
    return sync(g);
}

int ns_gpu_inverse(ns_gpu* g, const double* field_hat, double* field, double* masked_copy) {
    if (!g || !field_hat || !field) return NS_GPU_ERR_INVALID;
    NSG_TRY(ensure_staging(g));
    return g->prec == NS_GPU_FP64 ? inverse_t<double>(g, field_hat, field, masked_copy)
                                  : inverse_t<float>(g, field_hat, field, masked_copy);
}

int ns_gpu_dealias(ns_gpu* g, double* field_hat) {
    if (!g || !field_hat) return NS_GPU_ERR_INVALID;
    NSG_TRY(ensure_staging(g));
    NSG_TRY(h2d(g, g->spec[0], field_hat, spec_bytes(g)));
    const long long n = (long long)g->g.nkx * g->g.nky;
    k_dealias<<<grid_for(n), 256, 0, g->st>>>(g->g, g->spec[0], nullptr);
    NSG_LAUNCHED(g);
    NSG_TRY(d2h(g, field_hat, g->spec[0], spec_bytes(g)));
    return sync(g);
}

int ns_gpu_velocity(ns_gpu* g, const double* omega_hat, double* psi_hat, double* u_hat, double* v_hat) {
    if (!g || !omega_hat) return NS_GPU_ERR_INVALID;
    NSG_TRY(ensure_staging(g));
    NSG_TRY(h2d(g, g->spec[0], omega_hat, spec_bytes(g)));
    const long long n = (long long)g->g.nkx * g->g.nky;
    k_velocity<<<grid_for(n), 256, 0, g->st>>>(g->g, g->spec[0], g->spec[1], g->spec[2], g->spec[3]);
    NSG_LAUNCHED(g);
    if (psi_hat) NSG_TRY(d2h(g, psi_hat, g->spec[1], spec_bytes(g)));
    if (u_hat) NSG_TRY(d2h(g, u_hat, g->spec[2], spec_bytes(g)));
    if (v_hat) NSG_TRY(d2h(g, v_hat, g->spec[3], spec_bytes(g)));
    return sync(g);
}

template <typename T> static int uvw_from_spec(ns_gpu* g, const double2* wspec, double* u, double* v, double* w) {
    NSG_TRY(import_kept<T>(g, wspec, g->KS, nullptr, nullptr));
    NSG_TRY(prologue<T>(g, g->KS, nullptr, 1, 3));
    RowArgs<T> a = row_args<T>(g);
    a.F[0] = (const Cx<T>*)g->F[1];  // Psi_y -> u
    a.F[1] = (const Cx<T>*)g->F[0];  // Psi (x-derivative) -> v = -psi_x
    a.F[2] = (const Cx<T>*)g->F[2];  // Omega -> omega
    a.dx[0] = 0; a.dx[1] = 1; a.dx[2] = 0;
    a.out_real[0] = g->real[0];
    a.out_real[1] = g->real[1];
    a.out_real[2] = g->real[2];
    NSG_TRY(row_launch<T, ROW_UVW>(g, a));
    g->fields_valid = 0;
    if (u) NSG_TRY(d2h(g, u, g->real[0], real_bytes(g)));
    if (v) NSG_TRY(d2h(g, v, g->real[1], real_bytes(g)));
    if (w) NSG_TRY(d2h(g, w, g->real[2], real_bytes(g)));
    return NS_GPU_OK;
}

int ns_gpu_derivatives(ns_gpu* g, const double* omega_hat, double* psi_hat, double* u_hat, double* v_hat, double* u,
                       double* v, double* omega, double* masked_copy) {
    if (!g || !omega_hat) return NS_GPU_ERR_INVALID;
    NSG_TRY(ensure_staging(g));
    NSG_TRY(h2d(g, g->spec[0], omega_hat, spec_bytes(g)));
    const long long n = (long long)g->g.nkx * g->g.nky;
    k_velocity<<<grid_for(n), 256, 0, g->st>>>(g->g, g->spec[0], g->spec[1], g->spec[2], g->spec[3]);
    NSG_LAUNCHED(g);
    if (psi_hat) NSG_TRY(d2h(g, psi_hat, g->spec[1], spec_bytes(g)));
    if (u_hat) NSG_TRY(d2h(g, u_hat, g->spec[2], spec_bytes(g)));
    if (v_hat) NSG_TRY(d2h(g, v_hat, g->spec[3], spec_bytes(g)));
    if (g->prec == NS_GPU_FP64) NSG_TRY(uvw_from_spec<double>(g, g->spec[0], u, v, omega));
    else NSG_TRY(uvw_from_spec<float>(g, g->spec[0], u, v, omega));
    if (masked_copy) {
        k_dealias<<<grid_for(n), 256, 0, g->st>>>(g->g, g->spec[0], g->spec[4]);
        NSG_LAUNCHED(g);
        NSG_TRY(d2h(g, masked_copy, g->spec[4], spec_bytes(g)));
    }
    return sync(g);
}

template <typename T>
static int nonlinear_t(ns_gpu* g, const double* wh, const double* ph, double* nl, double* const* phys) {
    NSG_TRY(h2d(g, g->spec[0], wh, spec_bytes(g)));
    NSG_TRY(h2d(g, g->spec[1], ph, spec_bytes(g)));
    NSG_TRY(import_kept<T>(g, g->spec[0], g->KS, g->KP, g->spec[1]));
    NSG_TRY(prologue<T>(g, g->KS, g->KP, 0, 4));
    RowArgs<T> a = row_args<T>(g);
    for (int f = 0; f < 4; ++f) a.F[f] = (const Cx<T>*)g->F[f];
    a.dx[0] = 1; a.dx[1] = 0; a.dx[2] = 1; a.dx[3] = 0;
    int dump = 0;
    for (int i = 0; i < 5; ++i) {
        a.out_real[i] = g->real[i];
        if (phys[i]) dump = 1;
    }
    if (dump) NSG_TRY(row_launch<T, ROW_DUMP>(g, a));
    else NSG_TRY(row_launch<T, ROW_STAGE>(g, a));
    NSG_CUDA(g, cudaMemsetAsync(g->spec[2], 0, spec_bytes(g), g->st));
    ColArgs<T> c = col_args<T>(g);
    c.out_spec = g->spec[2];
    c.out_scale = -1.0 / ((double)g->g.nx * (double)g->g.ny);
    NSG_TRY((col_launch<T, COL_NL_EXPORT, 0>(g, c)));
    g->fields_valid = 0;
    if (nl) NSG_TRY(d2h(g, nl, g->spec[2], spec_bytes(g)));
    for (int i = 0; i < 5; ++i)
        if (phys[i]) NSG_TRY(d2h(g, phys[i], g->real[i], real_bytes(g)));
    return sync(g);
}

int ns_gpu_nonlinear(ns_gpu* g, const double* omega_hat, const double* psi_hat, double* nonlinear_hat, double* psi_x,
                     double* psi_y, double* omega_x, double* omega_y, double* jacobian) {
    if (!g || !omega_hat || !psi_hat) return NS_GPU_ERR_INVALID;
    NSG_TRY(ensure_staging(g));
    double* phys[5] = {psi_x, psi_y, omega_x, omega_y, jacobian};
    return g->prec == NS_GPU_FP64 ? nonlinear_t<double>(g, omega_hat, psi_hat, nonlinear_hat, phys)
                                  : nonlinear_t<float>(g, omega_hat, psi_hat, nonlinear_hat, phys);
}

int ns_gpu_hv_apply(ns_gpu* g, double* rhs_hat, const double* state_hat, const double* sfd_hat) {
    if (!g || !rhs_hat || !state_hat) return NS_GPU_ERR_INVALID;
    const int visc = (g->p.hv_enabled && g->p.hv_coefficient > 0.0) ? 1 : 0;
    const int sfd = (g->p.sfd_enabled && g->p.sfd_strength > 0.0) ? 1 : 0;
    if (!visc && !sfd) return NS_GPU_OK;
    if (sfd && !sfd_hat) return NS_GPU_ERR_INVALID;
    NSG_TRY(ensure_staging(g));
    NSG_TRY(h2d(g, g->spec[0], rhs_hat, spec_bytes(g)));
    NSG_TRY(h2d(g, g->spec[1], state_hat, spec_bytes(g)));
    if (sfd) NSG_TRY(h2d(g, g->spec[2], sfd_hat, spec_bytes(g)));
    const long long n = (long long)g->g.nkx * g->g.nky;
    k_hv_apply<<<grid_for(n), 256, 0, g->st>>>(g->g, g->hvw_full, visc, sfd, g->p.sfd_strength,
                                               g->p.hv_order > 0 ? g->p.hv_order : 1, g->hv_cutoff, g->hv_inv_bw,
                                               g->spec[0], g->spec[1], g->spec[2]);
    NSG_LAUNCHED(g);
    NSG_TRY(d2h(g, rhs_hat, g->spec[0], spec_bytes(g)));
    return sync(g);
}

int ns_gpu_hv_post_step(ns_gpu* g, const double* state_hat, double* sfd_hat, double dt) {
    if (!g || !state_hat || !sfd_hat) return NS_GPU_ERR_INVALID;
    if (dt <= 0.0 || !g->p.sfd_enabled || g->p.sfd_strength <= 0.0 || g->p.sfd_timescale <= 0.0) return NS_GPU_OK;
    double a = dt / g->p.sfd_timescale;
    a = a > 1.0 ? 1.0 : (a < 0.0 ? 0.0 : a);
    NSG_TRY(ensure_staging(g));
    NSG_TRY(h2d(g, g->spec[1], state_hat, spec_bytes(g)));
    NSG_TRY(h2d(g, g->spec[2], sfd_hat, spec_bytes(g)));
    const long long n = (long long)g->g.nkx * g->g.nky;
    k_hv_post<<<grid_for(n), 256, 0, g->st>>>(g->g, a, g->spec[1], g->spec[2]);
    NSG_LAUNCHED(g);
    NSG_TRY(d2h(g, sfd_hat, g->spec[2], spec_bytes(g)));
    return sync(g);
}

int ns_gpu_reduce(ns_gpu* g, int kind, const double* a, const double* b, double* out) {
    if (!g || !a || !out || kind < 0 || kind > 2) return NS_GPU_ERR_INVALID;
    if (kind != NS_GPU_REDUCE_ENSTROPHY && !b) return NS_GPU_ERR_INVALID;
    NSG_TRY(ensure_staging(g));
    const long long n = (long long)g->g.nx * g->g.ny;
    NSG_TRY(h2d(g, g->real[0], a, real_bytes(g)));
    if (b) NSG_TRY(h2d(g, g->real[1], b, real_bytes(g)));
    const int nb = grid_for(n, 256, g->part_n);
    if (kind == NS_GPU_REDUCE_CFL) {
        NSG_CUDA(g, cudaMemsetAsync(&g->ds->aux_max, 0, sizeof(unsigned long long), g->st));
        k_reduce_real<<<nb, 256, 0, g->st>>>(2, g->real[0], g->real[1], n, g->part, g->ds);
        NSG_LAUNCHED(g);
        unsigned long long bits = 0;
        NSG_TRY(d2h(g, &bits, &g->ds->aux_max, sizeof(bits)));
        NSG_TRY(sync(g));
        double vmax;
        memcpy(&vmax, &bits, sizeof(vmax));
        // spectral_time_integration.c:22-30
        const double dxmin = fmin(g->g.Lx / g->g.nx, g->g.Ly / g->g.ny);
        const double dt_cfl = g->p.cfl_factor * dxmin / (vmax + 1e-12);
        const double dt_visc = 0.5 * g->p.Re * dxmin * dxmin;
        double dt = fmin(dt_cfl, dt_visc);
        dt = fmax(dt, 1e-8);
        dt = fmin(dt, 0.1);
        *out = dt;
        return NS_GPU_OK;
    }
    k_reduce_real<<<nb, 256, 0, g->st>>>(kind == NS_GPU_REDUCE_ENERGY ? 0 : 1, g->real[0], g->real[1], n, g->part, g->ds);
    NSG_LAUNCHED(g);
    k_merge_partials<<<1, 256, 0, g->st>>>(g->part, nb, g->dres);
    NSG_LAUNCHED(g);
    double s = 0.0;
    NSG_TRY(d2h(g, &s, g->dres, sizeof(double)));
    NSG_TRY(sync(g));
    *out = s / ((double)g->g.nx * g->g.ny);
    return NS_GPU_OK;
}

int ns_gpu_spectral_stats(ns_gpu* g, const double* omega_hat, const double* u_hat, const double* v_hat,
                          double* resolution_fraction, double* max_abs, double* spectral_error, double* bin_energy,
                          int* bin_count) {
    if (!g) return NS_GPU_ERR_INVALID;
    if ((bin_energy || bin_count) && (!u_hat || !v_hat)) return NS_GPU_ERR_INVALID;
    NSG_TRY(ensure_staging(g));
    const int nbins = (int)fmin((double)g->g.nkx, (double)(g->g.nky / 2));
    if (omega_hat) NSG_TRY(h2d(g, g->spec[0], omega_hat, spec_bytes(g)));
    if (u_hat) NSG_TRY(h2d(g, g->spec[1], u_hat, spec_bytes(g)));
    if (v_hat) NSG_TRY(h2d(g, g->spec[2], v_hat, spec_bytes(g)));
    double* dbins = g->real[0];
    int* dcount = (int*)g->real[1];
    const int want_bins = (bin_energy || bin_count) ? 1 : 0;
    if (want_bins) {
        NSG_CUDA(g, cudaMemsetAsync(dbins, 0, nbins * sizeof(double), g->st));
        NSG_CUDA(g, cudaMemsetAsync(dcount, 0, nbins * sizeof(int), g->st));
    }
    NSG_CUDA(g, cudaMemsetAsync(&g->ds->aux_max, 0, sizeof(unsigned long long), g->st));
    const long long n = (long long)g->g.nkx * g->g.nky;
    const int nb = grid_for(n, 256, g->part_n);
    k_spec_stats<<<nb, 256, 0, g->st>>>(g->g, omega_hat ? g->spec[0] : nullptr, want_bins ? g->spec[1] : nullptr,
                                        want_bins ? g->spec[2] : nullptr, g->part, g->ds, dbins, dcount, nbins);
    NSG_LAUNCHED(g);
    k_merge_pairs4<<<1, 256, 0, g->st>>>(g->part, nb, g->dres);
    NSG_LAUNCHED(g);
    double r[4];
    unsigned long long bits = 0;
    NSG_TRY(d2h(g, r, g->dres, 4 * sizeof(double)));
    NSG_TRY(d2h(g, &bits, &g->ds->aux_max, sizeof(bits)));
    if (bin_energy) NSG_TRY(d2h(g, bin_energy, dbins, nbins * sizeof(double)));
    if (bin_count) NSG_TRY(d2h(g, bin_count, dcount, nbins * sizeof(int)));
    NSG_TRY(sync(g));
    double mx;
    memcpy(&mx, &bits, sizeof(mx));
    if (resolution_fraction) *resolution_fraction = (r[0] > 1e-16) ? r[1] / r[0] : 0.0;
    if (max_abs) *max_abs = mx;
    if (spectral_error) *spectral_error = (r[3] > 0.0) ? sqrt(r[2] / r[3]) : 0.0;
    return NS_GPU_OK;
}

int ns_gpu_taylor_green(ns_gpu* g, double* u, double* v, double* omega, double* p) {
    if (!g) return NS_GPU_ERR_INVALID;
    NSG_TRY(ensure_staging(g));
    const long long n = (long long)g->g.nx * g->g.ny;
    k_taylor_green<<<grid_for(n), 256, 0, g->st>>>(g->g, g->real[0], g->real[1], g->real[2], g->real[3]);
    NSG_LAUNCHED(g);
    if (u) NSG_TRY(d2h(g, u, g->real[0], real_bytes(g)));
    if (v) NSG_TRY(d2h(g, v, g->real[1], real_bytes(g)));
    if (omega) NSG_TRY(d2h(g, omega, g->real[2], real_bytes(g)));
    if (p) NSG_TRY(d2h(g, p, g->real[3], real_bytes(g)));
    return sync(g);
}

// ---------------------------------------------------------------- stepping
template <typename T>
static int upload_t(ns_gpu* g, const double2* wspec, const double2* pspec, const double2* sspec) {
    NSG_TRY(ensure_outside(g));
    NSG_CUDA(g, cudaMemsetAsync(g->dflag, 0, sizeof(int), g->st));
    const long long n = (long long)g->g.nkx * g->g.nky;
    k_import<T><<<grid_for(n), 256, 0, g->st>>>(g->g, wspec, pspec, sspec, (Cx<T>*)g->W0,
                                                pspec ? (Cx<T>*)g->PSI0 : nullptr, sspec ? (Cx<T>*)g->SFD : nullptr,
                                                g->out, g->outsfd, g->dflag);
    NSG_LAUNCHED(g);
    return NS_GPU_OK;
}

int ns_gpu_upload_state(ns_gpu* g, const double* omega_hat, const double* psi_hat, const double* sfd_hat, double t,
                        double dt, uint64_t step0) {
    if (!g || !omega_hat) return NS_GPU_ERR_INVALID;
    NSG_TRY(ensure_staging(g));
    NSG_TRY(h2d(g, g->spec[0], omega_hat, spec_bytes(g)));
    if (psi_hat) NSG_TRY(h2d(g, g->spec[1], psi_hat, spec_bytes(g)));
    if (sfd_hat) NSG_TRY(h2d(g, g->spec[2], sfd_hat, spec_bytes(g)));
    const double2* pp = psi_hat ? g->spec[1] : nullptr;
    const double2* sp = sfd_hat ? g->spec[2] : nullptr;
    if (g->prec == NS_GPU_FP64) NSG_TRY(upload_t<double>(g, g->spec[0], pp, sp));
    else NSG_TRY(upload_t<float>(g, g->spec[0], pp, sp));
    DevScalars h;
    memset(&h, 0, sizeof(h));
    h.t = t;
    h.dt = dt;
    h.dt_fixed = dt;
    h.step_next = step0;
    h.step_cur = step0;
    h.fsub = g->p.forcing_substeps > 1 ? (unsigned long long)g->p.forcing_substeps : 1ULL;
    NSG_TRY(h2d(g, g->ds, &h, sizeof(h)));
    int flag = 0;
    NSG_TRY(d2h(g, &flag, g->dflag, sizeof(int)));
    NSG_TRY(sync(g));
    g->p.dt = dt;
    g->outside_active = (flag & 1) ? 1 : 0;
    g->fields_valid = 0;
    g->psi0_valid = psi_hat ? 1 : 0;
    return NS_GPU_OK;
}

int ns_gpu_advance(ns_gpu* g, int nsteps) {
    if (!g || nsteps < 0) return NS_GPU_ERR_INVALID;
    return g->prec == NS_GPU_FP64 ? advance_t<double>(g, nsteps) : advance_t<float>(g, nsteps);
}

template <typename T>
static int download_t(ns_gpu* g, double* wh, double* ph, double* uh, double* vh, double* sh, double* u, double* v,
                      double* w) {
    if ((u || v || w) && !g->fields_valid) {
        NSG_TRY(prologue<T>(g, g->W0, g->PSI0, g->psi0_valid ? 0 : 1, 4));
        g->fields_valid = 1;
    }
    const long long n = (long long)g->g.nkx * g->g.nky;
    const int sfd_on = (g->p.sfd_enabled && g->p.sfd_strength > 0.0);
    k_export<T><<<grid_for(n), 256, 0, g->st>>>(g->g, (const Cx<T>*)g->W0, sfd_on ? (const Cx<T>*)g->SFD : nullptr,
                                                g->outside_active ? g->out : nullptr,
                                                (g->outside_active && sfd_on) ? g->outsfd : nullptr, g->spec[0],
                                                g->spec[1], g->spec[2], g->spec[3], g->spec[4]);
    NSG_LAUNCHED(g);
    if (u || v || w) {
        RowArgs<T> a = row_args<T>(g);
        a.F[0] = (const Cx<T>*)g->F[1];
        a.F[1] = (const Cx<T>*)g->F[0];
        a.F[2] = (const Cx<T>*)g->F[2];
        a.dx[0] = 0; a.dx[1] = 1; a.dx[2] = 0;
        a.out_real[0] = g->real[0];
        a.out_real[1] = g->real[1];
        a.out_real[2] = g->real[2];
        NSG_TRY(row_launch<T, ROW_UVW>(g, a));
    }
    if (wh) NSG_TRY(d2h(g, wh, g->spec[0], spec_bytes(g)));
    if (ph) NSG_TRY(d2h(g, ph, g->spec[1], spec_bytes(g)));
    if (uh) NSG_TRY(d2h(g, uh, g->spec[2], spec_bytes(g)));
    if (vh) NSG_TRY(d2h(g, vh, g->spec[3], spec_bytes(g)));
    if (sh) NSG_TRY(d2h(g, sh, g->spec[4], spec_bytes(g)));
    if (u) NSG_TRY(d2h(g, u, g->real[0], real_bytes(g)));
    if (v) NSG_TRY(d2h(g, v, g->real[1], real_bytes(g)));
    if (w) NSG_TRY(d2h(g, w, g->real[2], real_bytes(g)));
    return NS_GPU_OK;
}

int ns_gpu_download_state(ns_gpu* g, double* omega_hat, double* psi_hat, double* u_hat, double* v_hat, double* sfd_hat,
                          double* u, double* v, double* omega, double* t, double* dt) {
    if (!g) return NS_GPU_ERR_INVALID;
    NSG_TRY(ensure_staging(g));
    if (g->prec == NS_GPU_FP64) NSG_TRY(download_t<double>(g, omega_hat, psi_hat, u_hat, v_hat, sfd_hat, u, v, omega));
    else NSG_TRY(download_t<float>(g, omega_hat, psi_hat, u_hat, v_hat, sfd_hat, u, v, omega));
    DevScalars h;
    NSG_TRY(d2h(g, &h, g->ds, sizeof(h)));
    NSG_TRY(sync(g));
    if (t) *t = h.t;
    if (dt) *dt = h.dt;
    return NS_GPU_OK;
}

// --------------------------------------------- one step over host arrays
static int ensure_aux_stream(ns_gpu* g) {
    if (g->st2) return NS_GPU_OK;
    NSG_CUDA(g, cudaStreamCreateWithFlags(&g->st2, cudaStreamNonBlocking));
    NSG_CUDA(g, cudaEventCreateWithFlags(&g->ev_a, cudaEventDisableTiming));
    NSG_CUDA(g, cudaEventCreateWithFlags(&g->ev_b, cudaEventDisableTiming));
    return NS_GPU_OK;
}

// kept modes of a host-layout spectrum [nky][nkx]: the kx < Kx columns of the
// rows |band| <= Kyh, two row ranges
static int d2h_kept(ns_gpu* g, double* dst, const double2* src, cudaStream_t st) {
    const Geo& G = g->g;
    const size_t pitch = (size_t)G.nkx * sizeof(double2), width = (size_t)G.Kx * sizeof(double2);
    NSG_CUDA(g, cudaMemcpy2DAsync(dst, pitch, src, pitch, width, (size_t)G.Kyh + 1, cudaMemcpyDeviceToHost, st));
    const size_t r0 = (size_t)(G.ny - G.Kyh);
    NSG_CUDA(g, cudaMemcpy2DAsync(dst + 2 * r0 * G.nkx, pitch, src + r0 * G.nkx, pitch, width, (size_t)G.Kyh,
                                  cudaMemcpyDeviceToHost, st));
    return NS_GPU_OK;
}

template <typename T>
static int step_host_t(ns_gpu* g, double* wh, double* ph, double* uh, double* vh, double* sh, double* u, double* v,
                       double* w, double t, double dt, uint64_t step0, double* t_out, double* dt_out) {
    const size_t sb = spec_bytes(g), rb = real_bytes(g);
    // inputs: omega_hat on the instance stream, psi_hat (and the SFD state) on the
    // second stream, after everything already queued on the instance stream
    NSG_CUDA(g, cudaEventRecord(g->ev_a, g->st));
    NSG_CUDA(g, cudaStreamWaitEvent(g->st2, g->ev_a, 0));
    NSG_TRY(h2d(g, g->spec[0], wh, sb));
    NSG_CUDA(g, cudaMemcpyAsync(g->spec[1], ph, sb, cudaMemcpyHostToDevice, g->st2));
    if (sh) NSG_CUDA(g, cudaMemcpyAsync(g->spec[2], sh, sb, cudaMemcpyHostToDevice, g->st2));
    NSG_CUDA(g, cudaEventRecord(g->ev_b, g->st2));
    NSG_CUDA(g, cudaStreamWaitEvent(g->st, g->ev_b, 0));
    NSG_TRY(ensure_outside(g));
    NSG_CUDA(g, cudaMemsetAsync(g->dflag, 0, sizeof(int), g->st));
    const long long n = (long long)g->g.nkx * g->g.nky;
    k_import<T><<<grid_for(n), 256, 0, g->st>>>(g->g, g->spec[0], g->spec[1], sh ? g->spec[2] : nullptr, (Cx<T>*)g->W0,
                                                (Cx<T>*)g->PSI0, sh ? (Cx<T>*)g->SFD : nullptr, g->out, g->outsfd,
                                                g->dflag);
    NSG_LAUNCHED(g);
    DevScalars h;
    memset(&h, 0, sizeof(h));
    h.t = t;
    h.dt = dt;
    h.dt_fixed = dt;
    h.step_next = step0;
    h.step_cur = step0;
    h.fsub = g->p.forcing_substeps > 1 ? (unsigned long long)g->p.forcing_substeps : 1ULL;
    k_set_scalars<<<1, 1, 0, g->st>>>(g->ds, h);
    NSG_LAUNCHED(g);
    int flag = 0;
    NSG_TRY(d2h(g, &flag, g->dflag, sizeof(int)));
    NSG_TRY(sync(g));
    g->p.dt = dt;
    g->outside_active = (flag & 1) ? 1 : 0;
    g->fields_valid = 0;
    g->psi0_valid = 1;
    NSG_TRY(advance_t<T>(g, 1));
    // outputs: the spectra leave on the second stream while the instance stream
    // computes u, v, omega and copies them out
    const int sfd_on = (g->p.sfd_enabled && g->p.sfd_strength > 0.0);
    k_export<T><<<grid_for(n), 256, 0, g->st>>>(g->g, (const Cx<T>*)g->W0, sfd_on ? (const Cx<T>*)g->SFD : nullptr,
                                                g->outside_active ? g->out : nullptr,
                                                (g->outside_active && sfd_on) ? g->outsfd : nullptr, g->spec[0],
                                                g->spec[1], g->spec[2], g->spec[3], g->spec[4]);
    NSG_LAUNCHED(g);
    NSG_CUDA(g, cudaEventRecord(g->ev_a, g->st));
    NSG_CUDA(g, cudaStreamWaitEvent(g->st2, g->ev_a, 0));
    // modes outside the mask that were zero in the caller's omega_hat (bit 0) and
    // psi_hat (bit 1) stay zero after the step: those arrays only take their
    // kept modes back
    if (flag & 1) NSG_CUDA(g, cudaMemcpyAsync(wh, g->spec[0], sb, cudaMemcpyDeviceToHost, g->st2));
    else NSG_TRY(d2h_kept(g, wh, g->spec[0], g->st2));
    if (flag & 3) NSG_CUDA(g, cudaMemcpyAsync(ph, g->spec[1], sb, cudaMemcpyDeviceToHost, g->st2));
    else NSG_TRY(d2h_kept(g, ph, g->spec[1], g->st2));
    if (uh) NSG_CUDA(g, cudaMemcpyAsync(uh, g->spec[2], sb, cudaMemcpyDeviceToHost, g->st2));
    if (vh) NSG_CUDA(g, cudaMemcpyAsync(vh, g->spec[3], sb, cudaMemcpyDeviceToHost, g->st2));
    if (sh) NSG_CUDA(g, cudaMemcpyAsync(sh, g->spec[4], sb, cudaMemcpyDeviceToHost, g->st2));
    NSG_CUDA(g, cudaEventRecord(g->ev_b, g->st2));
    if (u || v || w) {
        RowArgs<T> a = row_args<T>(g);
        a.F[0] = (const Cx<T>*)g->F[1];
        a.F[1] = (const Cx<T>*)g->F[0];
        a.F[2] = (const Cx<T>*)g->F[2];
        a.dx[0] = 0; a.dx[1] = 1; a.dx[2] = 0;
        a.out_real[0] = g->real[0];
        a.out_real[1] = g->real[1];
        a.out_real[2] = g->real[2];
        NSG_TRY(row_launch<T, ROW_UVW>(g, a));
        if (u) NSG_TRY(d2h(g, u, g->real[0], rb));
        if (v) NSG_TRY(d2h(g, v, g->real[1], rb));
        if (w) NSG_TRY(d2h(g, w, g->real[2], rb));
    }
    NSG_CUDA(g, cudaStreamWaitEvent(g->st, g->ev_b, 0));
    DevScalars hs;
    NSG_TRY(d2h(g, &hs, g->ds, sizeof(hs)));
    NSG_TRY(sync(g));
    if (t_out) *t_out = hs.t;
    if (dt_out) *dt_out = hs.dt;
    return NS_GPU_OK;
}

int ns_gpu_step_host(ns_gpu* g, double* omega_hat, double* psi_hat, double* u_hat, double* v_hat, double* sfd_hat,
                     double* u, double* v, double* omega, double t, double dt, uint64_t step0, double* t_out,
                     double* dt_out) {
    if (!g || !omega_hat || !psi_hat) return NS_GPU_ERR_INVALID;
    NSG_TRY(ensure_staging(g));
    NSG_TRY(ensure_aux_stream(g));
    return g->prec == NS_GPU_FP64
               ? step_host_t<double>(g, omega_hat, psi_hat, u_hat, v_hat, sfd_hat, u, v, omega, t, dt, step0, t_out,
                                     dt_out)
               : step_host_t<float>(g, omega_hat, psi_hat, u_hat, v_hat, sfd_hat, u, v, omega, t, dt, step0, t_out,
                                    dt_out);
}

static int flush_l2(ns_gpu* g, size_t bytes, int salt) {
    if (bytes == 0) return NS_GPU_OK;
    if (g->flush_bytes < bytes) {
        if (g->flushbuf) cudaFree(g->flushbuf);
        g->flushbuf = nullptr;
        g->flush_bytes = 0;
        NSG_TRY(dalloc(g, &g->flushbuf, bytes));
        g->flush_bytes = bytes;
    }
    NSG_CUDA(g, cudaMemsetAsync(g->flushbuf, salt & 0xff, bytes, g->st));
    return NS_GPU_OK;
}

int ns_gpu_advance_timed(ns_gpu* g, int nsteps, size_t flush_bytes, double* total_ms, double* step_ms) {
    if (!g || nsteps < 0) return NS_GPU_ERR_INVALID;
    std::vector<cudaEvent_t> ev(2 * (size_t)nsteps);
    for (auto& e : ev) NSG_CUDA(g, cudaEventCreate(&e));
    int st = NS_GPU_OK;
    for (int n = 0; n < nsteps && st == NS_GPU_OK; ++n) {
        st = flush_l2(g, flush_bytes, n);
        if (st != NS_GPU_OK) break;
        cudaEventRecord(ev[2 * n], g->st);
        st = ns_gpu_advance(g, 1);
        cudaEventRecord(ev[2 * n + 1], g->st);
    }
    if (st == NS_GPU_OK) st = sync(g);
    double tot = 0.0;
    for (int n = 0; n < nsteps && st == NS_GPU_OK; ++n) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ev[2 * n], ev[2 * n + 1]);
        tot += ms;
        if (step_ms) step_ms[n] = ms;
    }
    for (auto& e : ev) cudaEventDestroy(e);
    if (total_ms) *total_ms = tot;
    return st;
}

int ns_gpu_profile_kernels(ns_gpu* g, int nsteps, size_t flush_bytes, double* kernel_ms, int* counts) {
    if (!g || nsteps < 0 || !kernel_ms || !counts) return NS_GPU_ERR_INVALID;
    std::vector<ns_gpu::ProfRec> recs;
    int st = NS_GPU_OK;
    for (int n = 0; n < nsteps && st == NS_GPU_OK; ++n) {
        st = flush_l2(g, flush_bytes, n);
        if (st != NS_GPU_OK) break;
        g->prof = &recs;
        st = ns_gpu_advance(g, 1);
        g->prof = nullptr;
    }
    g->prof = nullptr;
    if (st == NS_GPU_OK) st = sync(g);
    kernel_ms[0] = kernel_ms[1] = 0.0;
    counts[0] = counts[1] = 0;
    for (auto& r : recs) {
        float ms = 0.f;
        if (st == NS_GPU_OK) cudaEventElapsedTime(&ms, r.a, r.b);
        kernel_ms[r.kind] += ms;
        counts[r.kind] += 1;
        cudaEventDestroy(r.a);
        cudaEventDestroy(r.b);
    }
    return st;
}

int ns_gpu_diagnostics(ns_gpu* g, double* energy, double* enstrophy, double* t, double* dt) {
    if (!g) return NS_GPU_ERR_INVALID;
    const long long n = (long long)g->g.Kx * g->g.Ky;
    const int nb = grid_for(n, 256, g->part_n);
    NSG_CUDA(g, cudaMemsetAsync(&g->ds->flag, 0, sizeof(int), g->st));
    if (g->prec == NS_GPU_FP64)
        k_diag<double><<<nb, 256, 0, g->st>>>(g->g, (const double2*)g->W0, (const double*)g->kxv, (const double*)g->kyv,
                                              g->part, g->ds);
    else
        k_diag<float><<<nb, 256, 0, g->st>>>(g->g, (const float2*)g->W0, (const float*)g->kxv, (const float*)g->kyv,
                                             g->part, g->ds);
    NSG_LAUNCHED(g);
    k_merge_pairs2<<<1, 256, 0, g->st>>>(g->part, nb, g->dres);
    NSG_LAUNCHED(g);
    double r[2];
    DevScalars h;
    NSG_TRY(d2h(g, r, g->dres, 2 * sizeof(double)));
    NSG_TRY(d2h(g, &h, g->ds, sizeof(h)));
    NSG_TRY(sync(g));
    if (energy) *energy = r[0];
    if (enstrophy) *enstrophy = r[1];
    if (t) *t = h.t;
    if (dt) *dt = h.dt;
    if (h.flag & 2) NSG_FAIL(g, NS_GPU_ERR_DIVERGED, "non-finite vorticity in the device state at t=%g", h.t);
    return NS_GPU_OK;
}

int ns_gpu_energy_spectrum(ns_gpu* g, int nbins, double* energy_sum, double* energy_mean, int* count) {
    if (!g || nbins < 1 || nbins > 65536) return NS_GPU_ERR_INVALID;
    if (g->outside_active)
        NSG_FAIL(g, NS_GPU_ERR_INVALID, "energy spectrum: the state has modes outside the 2/3 mask (host-array path only)");
    const size_t need = (size_t)nbins * (sizeof(double) + sizeof(int));
    NSG_TRY(ensure_scratch(g, need));
    double* dbins = (double*)g->scratch;
    int* dcnt = (int*)(dbins + nbins);
    NSG_CUDA(g, cudaMemsetAsync(g->scratch, 0, need, g->st));
    const long long n = (long long)g->g.Kx * g->g.Ky;
    const size_t sm = (size_t)nbins * sizeof(double);
    if (sm > 48 * 1024) {
        if (g->prec == NS_GPU_FP64) NSG_CUDA(g, cudaFuncSetAttribute(k_energy_spectrum<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        else NSG_CUDA(g, cudaFuncSetAttribute(k_energy_spectrum<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    }
    if (g->prec == NS_GPU_FP64)
        k_energy_spectrum<double><<<grid_for(n, 256, 4 * g->num_sms), 256, sm, g->st>>>(g->g, (const double2*)g->W0, nbins, dbins);
    else
        k_energy_spectrum<float><<<grid_for(n, 256, 4 * g->num_sms), 256, sm, g->st>>>(g->g, (const float2*)g->W0, nbins, dbins);
    NSG_LAUNCHED(g);
    k_spectrum_counts<<<grid_for((long long)g->g.nkx * g->g.nky), 256, 0, g->st>>>(g->g, nbins, dcnt);
    NSG_LAUNCHED(g);
    std::vector<double> hs(nbins);
    std::vector<int> hc(nbins);
    NSG_TRY(d2h(g, hs.data(), dbins, (size_t)nbins * sizeof(double)));
    NSG_TRY(d2h(g, hc.data(), dcnt, (size_t)nbins * sizeof(int)));
    NSG_TRY(sync(g));
    for (int b = 0; b < nbins; ++b) {
        if (energy_sum) energy_sum[b] = hs[b];
        if (energy_mean) energy_mean[b] = hc[b] > 0 ? hs[b] / hc[b] : 0.0;
        if (count) count[b] = hc[b];
    }
    return NS_GPU_OK;
}

template <typename T> static int vorticity_t(ns_gpu* g, float* out) {
    if (!g->fields_valid) {
        NSG_TRY(prologue<T>(g, g->W0, g->PSI0, g->psi0_valid ? 0 : 1, 4));
        g->fields_valid = 1;
    }
    RowArgs<T> a = row_args<T>(g);
    a.F[0] = (const Cx<T>*)g->F[2];  // Omega, no derivative
    a.dx[0] = 0;
    a.out_f32 = out;  // the physical field leaves as float directly
    NSG_TRY(row_launch<T, ROW_INV1>(g, a));
    return NS_GPU_OK;
}

int ns_gpu_vorticity_device(ns_gpu* g, float* omega_dev) {
    if (!g || !omega_dev) return NS_GPU_ERR_INVALID;
    if (g->outside_active) NSG_FAIL(g, NS_GPU_ERR_INVALID, "vorticity_device: state has modes outside the 2/3 mask");
    NSG_TRY(ensure_staging(g));
    return g->prec == NS_GPU_FP64 ? vorticity_t<double>(g, omega_dev) : vorticity_t<float>(g, omega_dev);
}

// W0 += the forward transform of the float field delta (kept modes), and the
// next step's stage-1 fields from the new W0 in the same column pass (COL_ADD):
// two kernels, where an exported spectrum, an add and a separate prologue took four
template <typename T> static int add_vorticity_t(ns_gpu* g, const float* delta) {
    RowArgs<T> a = row_args<T>(g);
    a.in_f32 = delta;  // the row pass reads the float field directly
    NSG_TRY(row_launch<T, ROW_FWD1>(g, a));
    ColArgs<T> c = col_args<T>(g);
    c.out_scale = 1.0 / ((double)g->g.nx * (double)g->g.ny);
    c.psi_from_w = 1;
    c.nfields = 4;
    NSG_TRY((col_launch<T, COL_ADD, 0>(g, c)));
    g->fields_valid = 1;
    g->psi0_valid = 0;
    return NS_GPU_OK;
}

int ns_gpu_add_vorticity_device(ns_gpu* g, const float* delta_dev) {
    if (!g || !delta_dev) return NS_GPU_ERR_INVALID;
    NSG_TRY(ensure_staging(g));
    return g->prec == NS_GPU_FP64 ? add_vorticity_t<double>(g, delta_dev) : add_vorticity_t<float>(g, delta_dev);
}

int ns_gpu_filter_state(ns_gpu* fine, ns_gpu* coarse) {
    if (!fine || !coarse) return NS_GPU_ERR_INVALID;
    if (fine->prec != coarse->prec || fine->g.nx < coarse->g.nx || fine->g.ny < coarse->g.ny ||
        fine->g.Lx != coarse->g.Lx || fine->g.Ly != coarse->g.Ly)
        NSG_FAIL(coarse, NS_GPU_ERR_INVALID, "filter_state: needs the same precision and box and a finer source grid");
    NSG_CUDA(coarse, cudaStreamSynchronize(fine->st));
    const long long n = (long long)coarse->g.Kx * coarse->g.Ky;
    if (coarse->prec == NS_GPU_FP64)
        k_filter<double><<<grid_for(n), 256, 0, coarse->st>>>(fine->g, (const double2*)fine->W0, coarse->g, (double2*)coarse->W0);
    else
        k_filter<float><<<grid_for(n), 256, 0, coarse->st>>>(fine->g, (const float2*)fine->W0, coarse->g, (float2*)coarse->W0);
    NSG_LAUNCHED(coarse);
    NSG_CUDA(coarse, cudaMemcpyAsync(&coarse->ds->t, &fine->ds->t, sizeof(double), cudaMemcpyDeviceToDevice, coarse->st));
    NSG_CUDA(coarse, cudaMemcpyAsync(&coarse->ds->step_next, &fine->ds->step_next, sizeof(unsigned long long),
                                     cudaMemcpyDeviceToDevice, coarse->st));
    coarse->fields_valid = 0;
    coarse->psi0_valid = 0;
    coarse->outside_active = 0;
    return NS_GPU_OK;
}

int ns_gpu_init_random_spectrum(ns_gpu* g, uint64_t seed, double k0, double energy) {
    if (!g || !(k0 > 0.0) || energy < 0.0) return NS_GPU_ERR_INVALID;
    NSG_TRY(ensure_staging(g));
    const long long n = (long long)g->g.nkx * g->g.nky;
    const int nb = grid_for(n, 256, g->part_n);
    k_random_spectrum<<<nb, 256, 0, g->st>>>(g->g, (unsigned long long)seed, k0, g->spec[0], g->part);
    NSG_LAUNCHED(g);
    k_merge_partials<<<1, 256, 0, g->st>>>(g->part, nb, g->dres);
    NSG_LAUNCHED(g);
    NSG_TRY(h2d(g, g->dres + 1, &energy, sizeof(double)));
    k_scale_spec<<<grid_for(n), 256, 0, g->st>>>(n, g->spec[0], g->dres);
    NSG_LAUNCHED(g);
    if (g->prec == NS_GPU_FP64) NSG_TRY(upload_t<double>(g, g->spec[0], nullptr, nullptr));
    else NSG_TRY(upload_t<float>(g, g->spec[0], nullptr, nullptr));
    DevScalars h;
    memset(&h, 0, sizeof(h));
    h.dt = g->p.dt;
    h.dt_fixed = g->p.dt;
    h.fsub = g->p.forcing_substeps > 1 ? (unsigned long long)g->p.forcing_substeps : 1ULL;
    NSG_TRY(h2d(g, g->ds, &h, sizeof(h)));
    NSG_TRY(sync(g));
    g->outside_active = 0;
    g->fields_valid = 0;
    g->psi0_valid = 0;
    return NS_GPU_OK;
}

// copy the random spectrum of the device state into a host-layout array (used by the drop-in IC)
int ns_gpu_random_spectrum_host(ns_gpu* g, uint64_t seed, double k0, double energy, double* omega_hat) {
    if (!g || !omega_hat) return NS_GPU_ERR_INVALID;
    NSG_TRY(ns_gpu_init_random_spectrum(g, seed, k0, energy));
    NSG_TRY(d2h(g, omega_hat, g->spec[0], spec_bytes(g)));
    return sync(g);
}

int ns_gpu_forcing_weights(ns_gpu* g, const double* k2, int n, double kmin, double kmax, double* weights, int* active) {
    if (!g || !k2 || !weights || !active || n <= 0) return NS_GPU_ERR_INVALID;
    NSG_TRY(ensure_scratch(g, (size_t)n * 2 * sizeof(double) + 64));
    double* dk2 = (double*)g->scratch;
    double* dw = dk2 + n;
    NSG_TRY(h2d(g, dk2, k2, n * sizeof(double)));
    NSG_CUDA(g, cudaMemsetAsync(g->dflag, 0, sizeof(int), g->st));
    k_forcing_weights<<<grid_for(n), 256, 0, g->st>>>(dk2, n, kmin, kmax, dw, g->dflag);
    NSG_LAUNCHED(g);
    NSG_TRY(d2h(g, weights, dw, n * sizeof(double)));
    NSG_TRY(d2h(g, active, g->dflag, sizeof(int)));
    return sync(g);
}

int ns_gpu_forcing_generate(ns_gpu* g, int n, const double* weights, int active, int colored, double dt,
                            double correlation_time, double energy_target, uint64_t* rng_state, double* colored_state,
                            double* forcing_out) {
    if (!g || !weights || !rng_state || !forcing_out || n <= 0) return NS_GPU_ERR_INVALID;
    if (colored && !colored_state) return NS_GPU_ERR_INVALID;
    NSG_TRY(ensure_scratch(g, (size_t)n * (sizeof(double) + 2 * sizeof(double2)) + 64));
    double* dw = (double*)g->scratch;
    double2* dcs = (double2*)(dw + n);
    double2* dout = dcs + n;
    if (active == 0 || energy_target <= 0.0) {
        // forcing.c:121-133: zero output (and colored state when the target is not positive)
        memset(forcing_out, 0, (size_t)n * sizeof(double2));
        if (colored && energy_target <= 0.0 && active != 0) memset(colored_state, 0, (size_t)n * sizeof(double2));
        return NS_GPU_OK;
    }
    const double tau = fmax(correlation_time, 1e-6);
    double alpha = 0.0, beta = 1.0;
    if (colored) {
        alpha = exp(-dt / tau);
        beta = sqrt(fmax(1.0 - alpha * alpha, 0.0));
    }
    NSG_TRY(h2d(g, dw, weights, n * sizeof(double)));
    if (colored) NSG_TRY(h2d(g, dcs, colored_state, n * sizeof(double2)));
    k_forcing_generate<<<1, 1024, 0, g->st>>>(n, dw, colored, alpha, beta, energy_target,
                                              (unsigned long long)*rng_state, dcs, dout);
    NSG_LAUNCHED(g);
    NSG_TRY(d2h(g, forcing_out, dout, n * sizeof(double2)));
    if (colored) NSG_TRY(d2h(g, colored_state, dcs, n * sizeof(double2)));
    NSG_TRY(sync(g));
    *rng_state = *rng_state + 2ULL * (unsigned long long)active * 0x9E3779B97F4A7C15ULL;
    return NS_GPU_OK;
}

void* ns_gpu_state_device_ptr(ns_gpu* g) { return g ? g->W0 : nullptr; }

void* ns_gpu_host_alloc(size_t bytes) {
    void* p = nullptr;
    if (bytes == 0) bytes = 1;
    if (cudaMallocHost(&p, bytes) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    memset(p, 0, bytes);
    return p;
}

void ns_gpu_host_free(void* ptr) {
    if (ptr) cudaFreeHost(ptr);
}
