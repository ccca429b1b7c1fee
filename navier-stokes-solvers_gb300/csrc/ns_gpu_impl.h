// Private host-side definition of an ns_gpu instance and the error-handling
// macros shared by the translation units of the library (not installed).
#pragma once
#include <cuda_runtime.h>

#include <cstdio>
#include <string>
#include <utility>
#include <vector>

#include "ns_gpu.h"
#include "ns_kernels.cuh"

using nsg::Geo;
using nsg::DevScalars;

struct ns_gpu {
    Geo g;
    int prec;
    int ER, EC;
    int fold;  // N: the step's radix-4 stage kernels run with the N x N size fields as constants (fold_sizes)
    int device;
    int num_sms;
    int fast_row;       // radix-32 warp row kernel (nx = 2048)
    int fast_col;       // radix-32 column kernel (ny = 2048)
    cudaStream_t st;
    cudaStream_t st2;              // copies that overlap the instance stream (ns_gpu_step_host)
    // one RK4 step captured as a CUDA graph (advance): replayed while the kernel
    // arguments it was captured with (key) still hold
    cudaGraphExec_t step_exec;
    std::vector<unsigned char> step_key;      // arguments of the captured step
    std::vector<unsigned char> step_key_seen; // arguments of the last step launched directly
    unsigned long long step_launches;         // kernels per captured step
    int step_graph_off;                       // capture failed once: launch directly
    cudaEvent_t ev_a, ev_b;        // ordering between st and st2
    cudaStream_t stn;              // the forcing-noise table of a step, beside its stages 1-3
    cudaEvent_t evn0, evn1;        // fork after the stage-1 row pass, join before the stage-4 column pass
    std::string err;
    unsigned long long launches;
    ns_gpu_params p;
    int params_set;
    double hv_kmax, hv_cutoff, hv_inv_bw;
    double f_sigma;
    // device buffers (complex of the instance precision unless noted)
    void* F[4];
    void* G;
    void *W0, *WS, *ACC, *PSI0, *SFD, *KS, *KP;
    void *hvw, *sfdw, *kxv, *kyv, *twc, *twr, *twh;
    double* hvw_full;   // FP64 [nky][nkx]
    DevScalars* ds;
    double2* part;      // reduction partials
    int part_n;
    double* dres;       // small FP64 results
    int* dflag;
    // host-layout FP64 staging (allocated on first use)
    double2* spec[5];
    double* real[5];
    double2 *out, *outsfd;  // masked-out modes of the state (FP64)
    double2* fnoise;        // this step's forcing draws (k_forcing_noise), [entries][draws]
    size_t fnoise_cap;      // entries x draws allocated
    double2* fsum;          // their per-entry sums, zero outside the shell (k_forcing_sum)
    size_t fsum_cap;        // entries allocated
    int fkxr, fkyr, fM;     // table extent (kx index, |ky|) and draws per step; fM = 0: no table
    int outside_active;
    int fields_valid;   // F holds the stage-1 fields of the current state
    int psi0_valid;     // PSI0 holds the caller's psi_hat for the next prologue
    void* scratch;
    size_t scratch_bytes;
    void* flushbuf;     // L2 flush target of the timed entry points
    size_t flush_bytes;
    // kernel-level profiling: events around every launch while non-null
    struct ProfRec { cudaEvent_t a, b; int kind; };
    std::vector<ProfRec>* prof;
};

// record an event pair around one launch when kernel profiling is on
struct ProfScope {
    ns_gpu* g;
    int kind;
    cudaEvent_t a, b;
    ProfScope(ns_gpu* g_, int kind_) : g(g_), kind(kind_), a(nullptr), b(nullptr) {
        if (g->prof) {
            cudaEventCreate(&a);
            cudaEventCreate(&b);
            cudaEventRecord(a, g->st);
        }
    }
    ~ProfScope() {
        if (g->prof) {
            cudaEventRecord(b, g->st);
            g->prof->push_back({a, b, kind});
        }
    }
};

#define NSG_FAIL(g, code, ...)                                             \
    do {                                                                   \
        char _b[512];                                                      \
        snprintf(_b, sizeof(_b), __VA_ARGS__);                             \
        if (g) (g)->err = _b;                                              \
        return (code);                                                     \
    } while (0)

#define NSG_CUDA(g, call)                                                                    \
    do {                                                                                     \
        cudaError_t _e = (call);                                                             \
        if (_e != cudaSuccess) NSG_FAIL(g, NS_GPU_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(_e)); \
    } while (0)

#define NSG_LAUNCHED(g)                                                                          \
    do {                                                                                         \
        (g)->launches++;                                                                         \
        cudaError_t _e = cudaGetLastError();                                                     \
        if (_e != cudaSuccess) NSG_FAIL(g, NS_GPU_ERR_CUDA, "kernel launch: %s", cudaGetErrorString(_e)); \
    } while (0)

#define NSG_TRY(...)            \
    do {                        \
        int _s = (__VA_ARGS__); \
        if (_s != NS_GPU_OK) return _s; \
    } while (0)

// ------------------------------------------------------------- launchers
// Launch a stage kernel with programmatic stream serialization: it may be
// scheduled while the previous kernel on the stream drains, runs its
// independent prologue, and waits (griddepcontrol.wait) before it touches
// anything the previous kernel wrote.
#ifndef NSG_PDL
#define NSG_PDL 1
#endif
template <typename... KArgs, typename... Args>
static inline cudaError_t launch_stage(void (*kern)(KArgs...), int grid, int block, size_t smem, cudaStream_t st,
                                Args&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = NSG_PDL;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kern, std::forward<Args>(args)...);
}

template <typename K> static inline int set_smem(ns_gpu* g, K kernel, size_t bytes) {
    if (bytes > 48 * 1024) NSG_CUDA(g, cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    return NS_GPU_OK;
}


// Register-resident stage kernels at nx or ny = 2048 (and 4096 in FP32), in
// their own translation unit (csrc/ns_fast.cu); stage is 1..4.
int nsg_fast_row_f32(ns_gpu* g, const nsg::RowArgs<float>& a);
int nsg_fast_row_f64(ns_gpu* g, const nsg::RowArgs<double>& a);
int nsg_fast_col_f32(ns_gpu* g, const nsg::ColArgs<float>& a, int stage);
int nsg_fast_col_f64(ns_gpu* g, const nsg::ColArgs<double>& a, int stage);
// 1 when the FP32 column pass at 2048 / 4096 is k_col_q (else k_col_w)
int nsg_fast_col_q();

// Tiling of the generic stage kernels (zero: automatic), see nsg_create.
struct NsgTiling {
    int er, ec;       // complex values per thread in the row / column transforms (4, 8 or 16)
    int rpc, cw;      // rows per row block, kept columns per column block
    int kxp_align;    // the padded kept-column count Kxp is a multiple of this
    int fpr, fpc;     // fields in parallel in the row / column pass: 1 on, -1 off, 0 automatic
};
int nsg_create(int nx, int ny, double Lx, double Ly, int precision, const NsgTiling* kc, ns_gpu** out);
// Run the stage-1 field prologue of an instance if its fields are stale (FP32
// generic kernels; instance stream, asynchronous).
int nsg_prepare_fields(ns_gpu* g);
// Kernel arguments of an FP32 instance as its stage kernels see them.
void nsg_stage_args(ns_gpu* g, nsg::RowArgs<float>* ra, nsg::ColArgs<float>* ca);
