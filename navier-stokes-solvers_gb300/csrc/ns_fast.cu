// Launchers of the register-resident stage kernels (csrc/ns_wkernels.cuh): the
// FP32 row pass at nx = 2048 (k_row_t) and 4096 (k_row_4k), the FP32 column pass
// at ny = 2048 / 4096 (k_col_q), and the FP64 pair at 2048 (k_row_w, k_col_w).
// They form their own translation unit so that the library builds in parallel
// without splitting the compilation of these kernels.
#include <cuda_runtime.h>

#define NSG_NO_AUX_KERNELS
#include "ns_gpu.h"
#include "ns_gpu_impl.h"
#include "ns_wkernels.cuh"

using namespace nsg;

int nsg_fast_col_q() { return NSG_COL_Q; }

template <typename T> static int fast_row_w(ns_gpu* g, const RowArgs<T>& a) {
    const size_t smem = rw_smem_bytes<T>();
    NSG_TRY(set_smem(g, k_row_w<T>, smem));
    const int nw = rw_warps<T>();
    int grid = g->g.ny / nw;
    if (grid > g->num_sms) grid = g->num_sms;
    const cudaError_t e = launch_stage(k_row_w<T>, grid, 32 * nw, smem, g->st, g->g, a);
    if (e != cudaSuccess) NSG_FAIL(g, NS_GPU_ERR_CUDA, "k_row_w launch: %s", cudaGetErrorString(e));
    NSG_LAUNCHED(g);
    return NS_GPU_OK;
}

int nsg_fast_row_f32(ns_gpu* g, const RowArgs<float>& a) {
    if (g->g.nx == 4096) {
        // FP32, nx = 4096: two warps per row
        const size_t smem = r4_smem_bytes();
        NSG_TRY(set_smem(g, k_row_4k, smem));
        int grid = g->g.ny / NSG_R4_ROWS;
        if (grid > g->num_sms) grid = g->num_sms;
        const cudaError_t e = launch_stage(k_row_4k, grid, 64 * NSG_R4_ROWS, smem, g->st, g->g, a);
        if (e != cudaSuccess) NSG_FAIL(g, NS_GPU_ERR_CUDA, "k_row_4k launch: %s", cudaGetErrorString(e));
        NSG_LAUNCHED(g);
        return NS_GPU_OK;
    }
    if (NSG_ROW_TMEM) {
        // FP32: Jacobian operands in tensor memory, inboxes filled by cp.async
        auto kern = k_row_t<NSG_RT_NW, NSG_RT_GW, NSG_RT_NB>;
        const size_t smem = rt_smem_bytes<NSG_RT_NW, NSG_RT_NB>();
        NSG_TRY(set_smem(g, kern, smem));
        int grid = g->g.ny / NSG_RT_NW;
        if (grid > g->num_sms) grid = g->num_sms;
        const cudaError_t e = launch_stage(kern, grid, 32 * NSG_RT_NW, smem, g->st, g->g, a);
        if (e != cudaSuccess) NSG_FAIL(g, NS_GPU_ERR_CUDA, "k_row_t launch: %s", cudaGetErrorString(e));
        NSG_LAUNCHED(g);
        return NS_GPU_OK;
    }
    return fast_row_w<float>(g, a);
}

int nsg_fast_row_f64(ns_gpu* g, const RowArgs<double>& a) { return fast_row_w<double>(g, a); }

// FP32 column pass k_col_q for ny = 2^NL (NL = 11, 12)
template <int NL, int STAGE> static int launch_col_q(ns_gpu* g, const ColArgs<float>& a) {
    const size_t smem = cq_smem_bytes<NL>(g->g.Ky);
    auto kern = a.sp.ifrk ? k_col_q<NL, STAGE, true> : k_col_q<NL, STAGE, false>;
    NSG_TRY(set_smem(g, kern, smem));
    int grid = g->num_sms;
    if (grid > g->g.Kx) grid = g->g.Kx;
    const cudaError_t e = launch_stage(kern, grid, CQ<NL>::TT * CQ<NL>::NT, smem, g->st, g->g, a);
    if (e != cudaSuccess) NSG_FAIL(g, NS_GPU_ERR_CUDA, "k_col_q launch: %s", cudaGetErrorString(e));
    NSG_LAUNCHED(g);
    return NS_GPU_OK;
}

template <typename T, int STAGE> static int fast_col_w(ns_gpu* g, const ColArgs<T>& a) {
    const size_t smem = cw_smem_bytes<T>(g->g.Ky);
    auto kern = a.sp.ifrk ? k_col_w<T, STAGE, true> : k_col_w<T, STAGE, false>;
    NSG_TRY(set_smem(g, kern, smem));
    int grid = g->num_sms;
    if (grid > g->g.Kx) grid = g->g.Kx;
    const cudaError_t e = launch_stage(kern, grid, 64 * cw_teams<T>(), smem, g->st, g->g, a);
    if (e != cudaSuccess) NSG_FAIL(g, NS_GPU_ERR_CUDA, "k_col_w launch: %s", cudaGetErrorString(e));
    NSG_LAUNCHED(g);
    return NS_GPU_OK;
}

template <int STAGE> static int fast_col_f32(ns_gpu* g, const ColArgs<float>& a) {
    if (NSG_COL_Q) return g->g.ny == 4096 ? launch_col_q<12, STAGE>(g, a) : launch_col_q<11, STAGE>(g, a);
    return fast_col_w<float, STAGE>(g, a);
}

int nsg_fast_col_f32(ns_gpu* g, const ColArgs<float>& a, int stage) {
    switch (stage) {
        case 1: return fast_col_f32<1>(g, a);
        case 2: return fast_col_f32<2>(g, a);
        case 3: return fast_col_f32<3>(g, a);
        default: return fast_col_f32<4>(g, a);
    }
}

int nsg_fast_col_f64(ns_gpu* g, const ColArgs<double>& a, int stage) {
    switch (stage) {
        case 1: return fast_col_w<double, 1>(g, a);
        case 2: return fast_col_w<double, 2>(g, a);
        case 3: return fast_col_w<double, 3>(g, a);
        default: return fast_col_w<double, 4>(g, a);
    }
}
