// Batched ensembles: many independent pseudospectral solvers of mixed sizes
// advanced by ONE persistent kernel launch (replayed from a CUDA graph).
//
// Every member is an ordinary FP32 ns_gpu instance (its own state, tables,
// seeds, forcing stream and device-side dt); the ensemble only adds a device
// array of member descriptors and a static work schedule.  Each CTA of the
// persistent kernel walks its list of members and runs, for every step, the
// four RK stages of the reference step (spectral_time_integration.c:34-106)
// with the generic stage bodies of ns_kernels.cuh: the row pass over the
// member's row blocks, a barrier, the column pass over its column blocks, a
// barrier.  A member whose work exceeds one CTA's share is processed by a
// whole thread-block cluster (its CTAs split the row and column blocks and
// meet at hardware cluster barriers); smaller members are processed by one
// CTA each, with CTA barriers only.  Nothing spins: the only waits are
// __syncthreads and barrier.cluster, and every CTA of a cluster executes the
// same sequence of cluster barriers.
//
// The schedule is a longest-processing-time assignment of members to CTAs
// with cost n^2 log2(n^2) per member step.  The tiling (threads per CTA, the
// radix of the row and column transforms, the cluster size) is chosen by
// ns_gpu_ensemble_autotune, which times every valid candidate on a probe
// ensemble of the same member mix and caches the winner in a JSON-lines file.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#define NSG_NO_AUX_KERNELS
#include "ns_gpu.h"
#include "ns_gpu_impl.h"
#include "ns_kernels.cuh"

using namespace nsg;

namespace {

struct EnsMember {
    Geo g;                 // geometry with the ensemble's row / column tiling
    RowArgs<float> ra;
    ColArgs<float> ca;
    int nrb;               // row blocks: ny / RPC
    int ncb;               // column blocks: ceil(Kx / CW)
    int adaptive;          // device-side CFL dt
    int fold;              // N: the geometry equals fold_geo<N> (bodies with constant sizes), 0: as stored
};

// The geometry of a side-N member (N a power of two) under the 256-thread tiling of
// radix ER rows and EC columns, with kept columns padded to 64: every field the
// stage bodies read is a compile-time constant.  Inlined into the generic bodies it
// turns their loop bounds, divisions and index arithmetic into constants.  The host
// enables it for a member only when the member's own geometry has exactly these
// values (fold_matches), so the arithmetic is unchanged.
template <int N, int ER, int EC>
__host__ __device__ __forceinline__ void fold_geo(Geo& g) {
    fold_sizes<N>(g);
    g.Kxp = ((g.Kx + 63) / 64) * 64;
    g.CW = 256 / (N / EC);
    g.RPC = 256 / ((N / 2) / ER);
    g.fpr = 0;
    g.fpc = 0;
}

template <int N, int ER, int EC> bool fold_matches(const Geo& g) {
    Geo f = g;
    fold_geo<N, ER, EC>(f);
    return f.nx == g.nx && f.ny == g.ny && f.nkx == g.nkx && f.nky == g.nky && f.H == g.H && f.Kx == g.Kx &&
           f.Kxp == g.Kxp && f.Kyh == g.Kyh && f.Ky == g.Ky && f.logny == g.logny && f.logH == g.logH &&
           f.CW == g.CW && f.RPC == g.RPC && f.fLB == g.fLB && f.fTG == g.fTG && f.oddx == g.oddx &&
           f.fpr == g.fpr && f.fpc == g.fpc;
}

__device__ __forceinline__ unsigned cluster_ctarank() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}

// all threads of all CTAs of the cluster; global writes before it are visible after it
__device__ __forceinline__ void cluster_barrier() {
    __threadfence();
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

template <int EC, int STAGE>
__device__ __forceinline__ void col_pass(const Geo& g, const EnsMember& M, int r, int team) {
    for (int b = r; b < M.ncb; b += team) {
        col_body<float, EC, COL_STAGE, STAGE, false>(g, M.ca, b);
        __syncthreads();
    }
}

// nsteps RK4 steps of member M by this CTA (rank r of a team of CTAs that split
// its row and column blocks); N > 0: the member's geometry folded to constants
template <int ER, int EC, int N>
__device__ __forceinline__ void member_steps(const EnsMember& M, int shared, int team, int r, int nsteps) {
    Geo g = M.g;
    if constexpr (N > 0) fold_geo<N, ER, EC>(g);
    for (int s = 0; s < nsteps; ++s) {
#pragma unroll 1
        for (int stage = 1; stage <= 4; ++stage) {
            RowArgs<float> ra = M.ra;
            ra.cfl = (stage == 1 && M.adaptive) ? 1 : 0;
            ra.marker = stage == 1 ? 1 : (stage == 2 ? 2 : 0);
            for (int b = r; b < M.nrb; b += team) {
                row_body<float, ER, ROW_STAGE, false>(g, ra, b);
                __syncthreads();
            }
            if (shared) cluster_barrier();
            if (stage == 1) col_pass<EC, 1>(g, M, r, team);
            else if (stage == 2) col_pass<EC, 2>(g, M, r, team);
            else if (stage == 3) col_pass<EC, 3>(g, M, r, team);
            else col_pass<EC, 4>(g, M, r, team);
            if (shared) cluster_barrier();
        }
    }
}

// largest CTA: the radix-16 transforms keep 16 complex values per thread and
// need the registers of a 256-thread CTA, and a member's own stage kernels
// (its prologue and downloads, or a solo run with the same tiling) take at
// most 256 threads per row block
__host__ __device__ constexpr int ens_max_threads(int, int) { return 256; }
// CTAs per SM the compiler budgets registers for: five for the radix-4 bodies (at
// most 51 registers a thread, some spilled to L1; the members' small transforms
// are latency-bound, so more resident warps pay: 3, 4 and 5 CTAs per SM gave 0.658,
// 0.592 and 0.582 ms per config-3 step on GB300), one for the radix-16 ones (16
// values a thread)
__host__ __device__ constexpr int ens_min_ctas(int er, int ec) { return (er == 4 && ec == 4) ? 5 : 1; }

// work[w] = 2 * member + shared (1: the member is split over the CTA's cluster)
template <int ER, int EC>
__global__ void __launch_bounds__(ens_max_threads(ER, EC), ens_min_ctas(ER, EC)) k_ensemble(const EnsMember* __restrict__ mem, const int* __restrict__ work,
                                                  const int* __restrict__ woff, int nsteps, int csize) {
    const int rank = csize > 1 ? (int)cluster_ctarank() : 0;
    for (int w = woff[blockIdx.x]; w < woff[blockIdx.x + 1]; ++w) {
        const int code = work[w];
        const EnsMember& M = mem[code >> 1];
        const int shared = code & 1;
        const int team = shared ? csize : 1;
        const int r = shared ? rank : 0;
        // constant-size bodies for the radix-4 tiling's 64^2, 128^2 and 256^2 members
        if constexpr (ER == 4 && EC == 4) {
            if (M.fold == 64) { member_steps<ER, EC, 64>(M, shared, team, r, nsteps); continue; }
            if (M.fold == 128) { member_steps<ER, EC, 128>(M, shared, team, r, nsteps); continue; }
            if (M.fold == 256) { member_steps<ER, EC, 256>(M, shared, team, r, nsteps); continue; }
        }
        member_steps<ER, EC, 0>(M, shared, team, r, nsteps);
    }
}

typedef void (*EnsKernel)(const EnsMember*, const int*, const int*, int, int);

EnsKernel pick_kernel(int er, int ec) {
    if (er == 16 && ec == 16) return k_ensemble<16, 16>;
    if (er == 16 && ec == 4) return k_ensemble<16, 4>;
    if (er == 4 && ec == 16) return k_ensemble<4, 16>;
    if (er == 4 && ec == 4) return k_ensemble<4, 4>;
    return nullptr;
}

bool is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

// Tiling of one member of side n under a configuration, or false when the
// configuration cannot run it (a block must hold whole transforms and exactly
// cfg.threads threads).
bool member_tiling(int n, const ns_gpu_ensemble_config& c, NsgTiling* t) {
    const int H = n / 2;
    if (c.row_radix != 4 && c.row_radix != 16) return false;
    if (c.col_radix != 4 && c.col_radix != 16) return false;
    if (H < c.row_radix || n < c.col_radix) return false;
    const int TT = H / c.row_radix, TC = n / c.col_radix;
    if (c.threads % TT || c.threads % TC || c.threads > ens_max_threads(c.row_radix, c.col_radix)) return false;
    const int rpc = c.threads / TT, cw = c.threads / TC;
    if (rpc > n || cw > 64) return false;
    t->er = c.row_radix;
    t->ec = c.col_radix;
    t->rpc = rpc;
    t->cw = cw;
    t->kxp_align = 64;
    t->fpr = t->fpc = -1;
    return true;
}

// dynamic shared memory of a member's stage bodies: four row buffers per row of a
// row block; a column block's buffers plus its next-stage state (cw x Ky modes)
size_t member_smem(int n, int Ky, const NsgTiling& t) {
    const size_t row = (size_t)4 * t.rpc * spad_len(n / 2) * sizeof(float2);
    const size_t col = ((size_t)t.cw * spad_len(n) + (size_t)t.cw * Ky) * sizeof(float2);
    return row > col ? row : col;
}

double member_cost(int n) { return (double)n * n * std::log2((double)n * n); }

}  // namespace

struct ns_gpu_ensemble {
    std::vector<ns_gpu*> m;
    std::vector<int> n;
    ns_gpu_ensemble_config cfg;
    int device = 0, num_sms = 1;
    cudaStream_t st = nullptr;
    cudaEvent_t done = nullptr;
    EnsMember* dmem = nullptr;
    int* dwork = nullptr;
    int* dwoff = nullptr;
    std::vector<EnsMember> hmem;   // descriptors last uploaded
    std::vector<int> hwork, hwoff;
    int grid = 0;
    size_t smem = 0;
    EnsKernel kern = nullptr;
    cudaGraphExec_t gexec = nullptr;
    int gsteps = -1;
    unsigned long long launches = 0;
    std::string err;
};

#define ENS_FAIL(e, code, ...)                        \
    do {                                              \
        char _b[512];                                 \
        snprintf(_b, sizeof(_b), __VA_ARGS__);        \
        (e)->err = _b;                                \
        return (code);                                \
    } while (0)
#define ENS_CUDA(e, call)                                                                              \
    do {                                                                                               \
        cudaError_t _c = (call);                                                                       \
        if (_c != cudaSuccess) ENS_FAIL(e, NS_GPU_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(_c)); \
    } while (0)

static void drop_graph(ns_gpu_ensemble* e) {
    if (e->gexec) cudaGraphExecDestroy(e->gexec);
    e->gexec = nullptr;
    e->gsteps = -1;
}

// Build the descriptors and the schedule for e->cfg; upload them.
static int configure(ns_gpu_ensemble* e) {
    const int M = (int)e->m.size();
    const ns_gpu_ensemble_config& c = e->cfg;
    e->kern = pick_kernel(c.row_radix, c.col_radix);
    if (!e->kern) ENS_FAIL(e, NS_GPU_ERR_INVALID, "ensemble: radix (%d, %d) not in {4, 16}", c.row_radix, c.col_radix);
    if (c.threads < 32 || c.threads > ens_max_threads(c.row_radix, c.col_radix) || (c.threads & 31)) ENS_FAIL(e, NS_GPU_ERR_INVALID, "ensemble: threads %d", c.threads);
    if (c.cluster != 1 && c.cluster != 2 && c.cluster != 4 && c.cluster != 8)
        ENS_FAIL(e, NS_GPU_ERR_INVALID, "ensemble: cluster %d not in {1, 2, 4, 8}", c.cluster);
    e->hmem.resize(M);
    size_t smem = 0;
    for (int i = 0; i < M; ++i) {
        NsgTiling t;
        if (!member_tiling(e->n[i], c, &t))
            ENS_FAIL(e, NS_GPU_ERR_INVALID, "ensemble: member %d (%d^2) cannot run with threads=%d radix=(%d,%d)", i,
                     e->n[i], c.threads, c.row_radix, c.col_radix);
        ns_gpu* g = e->m[i];
        if (g->outside_active)
            ENS_FAIL(e, NS_GPU_ERR_INVALID, "ensemble: member %d has state outside the 2/3 mask", i);
        if (((g->g.Kx + t.cw - 1) / t.cw) * t.cw > g->g.Kxp)
            ENS_FAIL(e, NS_GPU_ERR_INVALID, "ensemble: member %d column padding too small for %d columns per block", i, t.cw);
        // the member's own launches (prologue, downloads, a later solo run)
        // use the same tiling, so its arithmetic matches the ensemble's
        g->ER = t.er;
        g->EC = t.ec;
        g->g.RPC = t.rpc;
        g->g.CW = t.cw;
        g->g.fpr = g->g.fpc = 0;  // the persistent kernel runs one thread group per row / column block
        EnsMember& d = e->hmem[i];
        memset(&d, 0, sizeof(d));
        nsg_stage_args(g, &d.ra, &d.ca);
        d.g = g->g;
        d.nrb = d.g.ny / t.rpc;
        d.ncb = (d.g.Kx + t.cw - 1) / t.cw;
        d.adaptive = g->p.adaptive_dt;
        d.fold = 0;
        if (c.threads == 256 && c.row_radix == 4 && c.col_radix == 4) {
            if (e->n[i] == 64 && fold_matches<64, 4, 4>(d.g)) d.fold = 64;
            else if (e->n[i] == 128 && fold_matches<128, 4, 4>(d.g)) d.fold = 128;
            else if (e->n[i] == 256 && fold_matches<256, 4, 4>(d.g)) d.fold = 256;
        }
        smem = std::max(smem, member_smem(e->n[i], g->g.Ky, t));
    }
    e->smem = smem;
    if (smem > 48 * 1024) ENS_CUDA(e, cudaFuncSetAttribute(e->kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    if (c.cluster > 1) ENS_CUDA(e, cudaFuncSetAttribute(e->kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    int per_sm = 0;
    ENS_CUDA(e, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, e->kern, c.threads, smem));
    if (per_sm < 1) ENS_FAIL(e, NS_GPU_ERR_INVALID, "ensemble: %zu B shared memory, %d threads do not fit an SM", smem, c.threads);
    int grid = per_sm * e->num_sms;
    if (c.cluster > 1) {
        cudaLaunchConfig_t lc = {};
        lc.gridDim = dim3(grid - grid % c.cluster);
        lc.blockDim = dim3(c.threads);
        lc.dynamicSmemBytes = smem;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = c.cluster;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        lc.attrs = at;
        lc.numAttrs = 1;
        int nclusters = 0;
        ENS_CUDA(e, cudaOccupancyMaxActiveClusters(&nclusters, e->kern, &lc));
        if (nclusters < 1) ENS_FAIL(e, NS_GPU_ERR_INVALID, "ensemble: cluster of %d CTAs does not fit", c.cluster);
        grid = std::min(grid - grid % c.cluster, nclusters * c.cluster);
    }
    // never more CTAs than there is work to give them
    double total = 0.0;
    for (int i = 0; i < M; ++i) total += member_cost(e->n[i]);
    e->grid = grid;

    // longest-processing-time schedule: members that exceed one CTA's fair
    // share go to the least-loaded cluster (all of its CTAs), the rest to the
    // least-loaded CTA
    const double share = total / grid;
    std::vector<int> order(M);
    for (int i = 0; i < M; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return e->n[a] > e->n[b]; });
    std::vector<double> load(grid, 0.0);
    std::vector<std::vector<int>> shared_items(grid), solo_items(grid);
    for (int i : order) {
        const double cst = member_cost(e->n[i]);
        if (c.cluster > 1 && cst > share) {
            int best = 0;
            double bl = 1e300;
            for (int k = 0; k < grid; k += c.cluster) {
                double l = 0.0;
                for (int q = 0; q < c.cluster; ++q) l = std::max(l, load[k + q]);
                if (l < bl) { bl = l; best = k; }
            }
            for (int q = 0; q < c.cluster; ++q) {
                load[best + q] += cst / c.cluster;
                shared_items[best + q].push_back(2 * i + 1);
            }
        } else {
            int best = (int)(std::min_element(load.begin(), load.end()) - load.begin());
            load[best] += cst;
            solo_items[best].push_back(2 * i);
        }
    }
    e->hwork.clear();
    e->hwoff.assign(grid + 1, 0);
    for (int b = 0; b < grid; ++b) {
        e->hwoff[b] = (int)e->hwork.size();
        // shared members first, in the same order on every CTA of the cluster
        for (int w : shared_items[b]) e->hwork.push_back(w);
        for (int w : solo_items[b]) e->hwork.push_back(w);
    }
    e->hwoff[grid] = (int)e->hwork.size();

    if (e->dmem) cudaFree(e->dmem);
    if (e->dwork) cudaFree(e->dwork);
    if (e->dwoff) cudaFree(e->dwoff);
    e->dmem = nullptr;
    e->dwork = e->dwoff = nullptr;
    ENS_CUDA(e, cudaMalloc((void**)&e->dmem, sizeof(EnsMember) * M));
    ENS_CUDA(e, cudaMalloc((void**)&e->dwork, sizeof(int) * std::max<size_t>(1, e->hwork.size())));
    ENS_CUDA(e, cudaMalloc((void**)&e->dwoff, sizeof(int) * (grid + 1)));
    ENS_CUDA(e, cudaMemcpy(e->dmem, e->hmem.data(), sizeof(EnsMember) * M, cudaMemcpyHostToDevice));
    ENS_CUDA(e, cudaMemcpy(e->dwork, e->hwork.data(), sizeof(int) * e->hwork.size(), cudaMemcpyHostToDevice));
    ENS_CUDA(e, cudaMemcpy(e->dwoff, e->hwoff.data(), sizeof(int) * (grid + 1), cudaMemcpyHostToDevice));
    drop_graph(e);
    return NS_GPU_OK;
}

static int launch(ns_gpu_ensemble* e, int nsteps) {
    cudaLaunchConfig_t lc = {};
    lc.gridDim = dim3(e->grid);
    lc.blockDim = dim3(e->cfg.threads);
    lc.dynamicSmemBytes = e->smem;
    lc.stream = e->st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = e->cfg.cluster;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    lc.attrs = at;
    lc.numAttrs = e->cfg.cluster > 1 ? 1 : 0;
    const EnsMember* dm = e->dmem;
    const int* dw = e->dwork;
    const int* dwo = e->dwoff;
    int cs = e->cfg.cluster;
    ENS_CUDA(e, cudaLaunchKernelEx(&lc, e->kern, dm, dw, dwo, nsteps, cs));
    return NS_GPU_OK;
}

// Members' pending work (initial conditions, parameter tables, prologues)
// finishes before the ensemble kernel reads their state.
static int prepare(ns_gpu_ensemble* e) {
    bool changed = false;
    for (size_t i = 0; i < e->m.size(); ++i) {
        ns_gpu* g = e->m[i];
        const int s = nsg_prepare_fields(g);
        if (s != NS_GPU_OK) ENS_FAIL(e, s, "ensemble: member %zu prologue: %s", i, g->err.c_str());
        ENS_CUDA(e, cudaStreamSynchronize(g->st));
        EnsMember d = e->hmem[i];
        RowArgs<float> ra;
        ColArgs<float> ca;
        nsg_stage_args(g, &ra, &ca);
        if (memcmp(&ca.sp, &d.ca.sp, sizeof(StepParams)) != 0 || d.adaptive != g->p.adaptive_dt) changed = true;
    }
    if (changed) return configure(e);
    return NS_GPU_OK;
}

// the members' streams wait for the ensemble's work before their next call
static int publish(ns_gpu_ensemble* e) {
    ENS_CUDA(e, cudaEventRecord(e->done, e->st));
    for (ns_gpu* g : e->m) ENS_CUDA(e, cudaStreamWaitEvent(g->st, e->done, 0));
    return NS_GPU_OK;
}

static int run_graph(ns_gpu_ensemble* e, int nsteps) {
    if (!e->gexec || e->gsteps != nsteps) {
        drop_graph(e);
        cudaGraph_t graph = nullptr;
        ENS_CUDA(e, cudaStreamBeginCapture(e->st, cudaStreamCaptureModeThreadLocal));
        const int s = launch(e, nsteps);
        const cudaError_t ce = cudaStreamEndCapture(e->st, &graph);
        if (s != NS_GPU_OK) {
            if (graph) cudaGraphDestroy(graph);
            return s;
        }
        if (ce != cudaSuccess) ENS_FAIL(e, NS_GPU_ERR_CUDA, "ensemble graph capture: %s", cudaGetErrorString(ce));
        const cudaError_t ie = cudaGraphInstantiate(&e->gexec, graph, 0);
        cudaGraphDestroy(graph);
        if (ie != cudaSuccess) ENS_FAIL(e, NS_GPU_ERR_CUDA, "ensemble graph instantiate: %s", cudaGetErrorString(ie));
        e->gsteps = nsteps;
    }
    ENS_CUDA(e, cudaGraphLaunch(e->gexec, e->st));
    e->launches++;
    return NS_GPU_OK;
}

extern "C" {

int ns_gpu_create_for_ensemble(int nx, int ny, double Lx, double Ly, int precision, const ns_gpu_ensemble_config* cfg,
                               ns_gpu** out) {
    if (!cfg || !out || nx != ny || !is_pow2(nx)) return NS_GPU_ERR_INVALID;
    NsgTiling t;
    if (!member_tiling(nx, *cfg, &t)) return NS_GPU_ERR_INVALID;
    return nsg_create(nx, ny, Lx, Ly, precision, &t, out);
}

int ns_gpu_ensemble_create(int nmembers, const int* n, double L, const ns_gpu_ensemble_config* cfg, ns_gpu_ensemble** out) {
    if (!out || !n || !cfg || nmembers < 1 || !(L > 0.0)) return NS_GPU_ERR_INVALID;
    *out = nullptr;
    for (int i = 0; i < nmembers; ++i) {
        if (!is_pow2(n[i]) || n[i] < 16 || n[i] > 1024) {
            fprintf(stderr, "ns_gpu_ensemble_create: member %d side %d must be a power of two in [16, 1024]\n", i, n[i]);
            return NS_GPU_ERR_INVALID;
        }
        NsgTiling t;
        if (!member_tiling(n[i], *cfg, &t)) {
            fprintf(stderr, "ns_gpu_ensemble_create: member %d (%d^2) cannot run with threads=%d radix=(%d,%d)\n", i, n[i],
                    cfg->threads, cfg->row_radix, cfg->col_radix);
            return NS_GPU_ERR_INVALID;
        }
    }
    ns_gpu_ensemble* e = new ns_gpu_ensemble();
    e->cfg = *cfg;
    e->n.assign(n, n + nmembers);
    cudaGetDevice(&e->device);
    cudaDeviceGetAttribute(&e->num_sms, cudaDevAttrMultiProcessorCount, e->device);
    int s = NS_GPU_OK;
    if (cudaStreamCreateWithFlags(&e->st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&e->done, cudaEventDisableTiming) != cudaSuccess)
        s = NS_GPU_ERR_CUDA;
    for (int i = 0; i < nmembers && s == NS_GPU_OK; ++i) {
        NsgTiling t;
        member_tiling(n[i], *cfg, &t);
        ns_gpu* g = nullptr;
        s = nsg_create(n[i], n[i], L, L, NS_GPU_FP32, &t, &g);
        if (s == NS_GPU_OK) e->m.push_back(g);
    }
    if (s == NS_GPU_OK) s = configure(e);
    if (s != NS_GPU_OK) {
        fprintf(stderr, "ns_gpu_ensemble_create: %s\n", e->err.empty() ? ns_gpu_status_string(s) : e->err.c_str());
        ns_gpu_ensemble_destroy(e);
        return s;
    }
    *out = e;
    return NS_GPU_OK;
}

void ns_gpu_ensemble_destroy(ns_gpu_ensemble* e) {
    if (!e) return;
    if (e->st) cudaStreamSynchronize(e->st);
    drop_graph(e);
    for (ns_gpu* g : e->m) ns_gpu_destroy(g);
    if (e->dmem) cudaFree(e->dmem);
    if (e->dwork) cudaFree(e->dwork);
    if (e->dwoff) cudaFree(e->dwoff);
    if (e->done) cudaEventDestroy(e->done);
    if (e->st) cudaStreamDestroy(e->st);
    delete e;
}

ns_gpu* ns_gpu_ensemble_member(ns_gpu_ensemble* e, int m) {
    if (!e || m < 0 || m >= (int)e->m.size()) return nullptr;
    return e->m[m];
}

const char* ns_gpu_ensemble_last_error(const ns_gpu_ensemble* e) { return e ? e->err.c_str() : "null ensemble"; }

int ns_gpu_ensemble_info(const ns_gpu_ensemble* e, int* grid, int* threads, size_t* smem, int* cluster,
                         uint64_t* launches) {
    if (!e) return NS_GPU_ERR_INVALID;
    if (grid) *grid = e->grid;
    if (threads) *threads = e->cfg.threads;
    if (smem) *smem = e->smem;
    if (cluster) *cluster = e->cfg.cluster;
    if (launches) *launches = e->launches;
    return NS_GPU_OK;
}

int ns_gpu_ensemble_advance(ns_gpu_ensemble* e, int nsteps) {
    if (!e || nsteps < 0) return NS_GPU_ERR_INVALID;
    if (nsteps == 0) return NS_GPU_OK;
    int s = prepare(e);
    if (s != NS_GPU_OK) return s;
    s = run_graph(e, nsteps);
    if (s != NS_GPU_OK) return s;
    return publish(e);
}

int ns_gpu_ensemble_synchronize(ns_gpu_ensemble* e) {
    if (!e) return NS_GPU_ERR_INVALID;
    ENS_CUDA(e, cudaStreamSynchronize(e->st));
    return NS_GPU_OK;
}

int ns_gpu_ensemble_advance_timed(ns_gpu_ensemble* e, int nsteps, int reps, double* ms_per_rep) {
    if (!e || nsteps < 1 || reps < 1 || !ms_per_rep) return NS_GPU_ERR_INVALID;
    int s = prepare(e);
    if (s != NS_GPU_OK) return s;
    s = run_graph(e, nsteps);  // instantiate and warm
    if (s != NS_GPU_OK) return s;
    cudaEvent_t a, b;
    ENS_CUDA(e, cudaEventCreate(&a));
    ENS_CUDA(e, cudaEventCreate(&b));
    cudaEventRecord(a, e->st);
    for (int r = 0; r < reps && s == NS_GPU_OK; ++r) s = run_graph(e, nsteps);
    cudaEventRecord(b, e->st);
    const cudaError_t se = cudaEventSynchronize(b);
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (s != NS_GPU_OK) return s;
    if (se != cudaSuccess) ENS_FAIL(e, NS_GPU_ERR_CUDA, "ensemble timing: %s", cudaGetErrorString(se));
    *ms_per_rep = ms / reps;
    return publish(e);
}

int ns_gpu_ensemble_reconfigure(ns_gpu_ensemble* e, const ns_gpu_ensemble_config* cfg) {
    if (!e || !cfg) return NS_GPU_ERR_INVALID;
    // member layouts pad the kept columns to a multiple of 64, so every valid
    // tiling runs on them
    for (size_t i = 0; i < e->m.size(); ++i) {
        NsgTiling t;
        if (!member_tiling(e->n[i], *cfg, &t)) ENS_FAIL(e, NS_GPU_ERR_INVALID, "ensemble: member %zu cannot run this tiling", i);
    }
    ENS_CUDA(e, cudaStreamSynchronize(e->st));
    for (ns_gpu* g : e->m) ENS_CUDA(e, cudaStreamSynchronize(g->st));
    const ns_gpu_ensemble_config old = e->cfg;
    e->cfg = *cfg;
    const int s = configure(e);
    if (s != NS_GPU_OK) {
        e->cfg = old;
        configure(e);
    }
    return s;
}

}  // extern "C"

// ---------------------------------------------------------------- autotuner
static std::string tune_key(const ns_gpu_ensemble* e) {
    cudaDeviceProp prop;
    cudaGetDeviceProperties(&prop, e->device);
    std::vector<int> sizes = e->n;
    std::sort(sizes.begin(), sizes.end());
    std::string k = std::string(prop.name) + "|" + std::to_string(e->num_sms) + "|";
    for (size_t i = 0; i < sizes.size();) {
        size_t j = i;
        while (j < sizes.size() && sizes[j] == sizes[i]) ++j;
        k += std::to_string(sizes[i]) + "x" + std::to_string(j - i) + ",";
        i = j;
    }
    return k;
}

static bool cache_lookup(const char* path, const std::string& key, ns_gpu_ensemble_config* c, double* ms) {
    if (!path || !path[0]) return false;
    FILE* f = fopen(path, "r");
    if (!f) return false;
    char line[1024], k[512];
    bool found = false;
    while (fgets(line, sizeof(line), f)) {
        ns_gpu_ensemble_config t;
        double m = 0.0;
        if (sscanf(line, "{\"key\": \"%511[^\"]\", \"threads\": %d, \"row_radix\": %d, \"col_radix\": %d, \"cluster\": %d, "
                         "\"ms_per_step\": %lf}",
                   k, &t.threads, &t.row_radix, &t.col_radix, &t.cluster, &m) == 6 &&
            key == k) {
            *c = t;  // the last entry for a key wins
            *ms = m;
            found = true;
        }
    }
    fclose(f);
    return found;
}

extern "C" int ns_gpu_ensemble_autotune(ns_gpu_ensemble* e, int steps, const char* cache_path, ns_gpu_ensemble_config* best,
                                        double* best_ms_per_step) {
    if (!e || steps < 1) return NS_GPU_ERR_INVALID;
    const std::string key = tune_key(e);
    ns_gpu_ensemble_config bc = e->cfg;
    double bms = 0.0;
    if (cache_lookup(cache_path, key, &bc, &bms)) {
        const int s = ns_gpu_ensemble_reconfigure(e, &bc);
        if (s == NS_GPU_OK) {
            if (best) *best = bc;
            if (best_ms_per_step) *best_ms_per_step = bms;
            return NS_GPU_OK;
        }
    }
    const ns_gpu_ensemble_config start = e->cfg;
    bms = 1e300;
    bool any = false;
    const int threads[] = {64, 128, 256};
    const int radix[] = {4, 16};
    const int clusters[] = {1, 2, 4, 8};
    for (int th : threads)
        for (int er : radix)
            for (int ec : radix)
                for (int cs : clusters) {
                    ns_gpu_ensemble_config c = {th, er, ec, cs};
                    bool ok = true;
                    for (int n : e->n) {
                        NsgTiling t;
                        if (!member_tiling(n, c, &t)) { ok = false; break; }
                    }
                    if (!ok || ns_gpu_ensemble_reconfigure(e, &c) != NS_GPU_OK) continue;
                    double ms = 0.0;
                    if (ns_gpu_ensemble_advance_timed(e, steps, 1, &ms) != NS_GPU_OK) continue;  // graph build + warm
                    if (ns_gpu_ensemble_advance_timed(e, steps, 2, &ms) != NS_GPU_OK) continue;
                    ms /= steps;
                    if (ms < bms) { bms = ms; bc = c; any = true; }
                }
    if (!any) {
        ns_gpu_ensemble_reconfigure(e, &start);
        ENS_FAIL(e, NS_GPU_ERR_INVALID, "ensemble autotune: no candidate tiling ran");
    }
    const int s = ns_gpu_ensemble_reconfigure(e, &bc);
    if (s != NS_GPU_OK) return s;
    if (cache_path && cache_path[0]) {
        FILE* f = fopen(cache_path, "a");
        if (f) {
            fprintf(f,
                    "{\"key\": \"%s\", \"threads\": %d, \"row_radix\": %d, \"col_radix\": %d, \"cluster\": %d, "
                    "\"ms_per_step\": %.6f}\n",
                    key.c_str(), bc.threads, bc.row_radix, bc.col_radix, bc.cluster, bms);
            fclose(f);
        }
    }
    if (best) *best = bc;
    if (best_ms_per_step) *best_ms_per_step = bms;
    return NS_GPU_OK;
}
