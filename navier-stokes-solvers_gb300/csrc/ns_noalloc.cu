// Allocation-free forward transform (physical -> dealiased spectrum) for callers
// that cannot allocate device memory.
//
// Some callers of this library cannot call cudaMalloc at all: code that runs
// inside a host framework owning every device allocation through its own pool
// (a second allocator would break its accounting or its memory cap), real-time
// loops where an allocation's latency or failure mode is not acceptable, and
// plugins loaded into a process whose device memory is already fully reserved.
// They hold the input and output buffers themselves and need the transform to
// bring nothing else.
//
// ns_gpu_forward_noalloc therefore keeps its only scratch -- the twiddle tables
// and the x-transformed intermediate between the row and the column pass -- in
// the file-scope array below, reserved once in every GPU that loads this library
// and held until the process exits.  It allocates nothing on any call (no
// cudaMalloc, cudaFree, or allocating library routine).
//
// Set-up: the first call on a device looks the array's device address up with
// cudaGetSymbolAddress while that device is current and caches it; that first
// call should come before any stream capture.  Later calls reuse the address.
// Calls share one array, which keeps the previous call's contents: every call
// rewrites the tables and the intermediate before reading them, and zeroes the
// masked modes of its own output.  Calls that overlap on the GPU (two streams, or
// two threads issuing at once) race on the array; serialise them.
#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>
#include <cstring>
#include <mutex>

#include "ns_gpu.h"

// the kernels get internal linkage in this translation unit (their host stubs
// would otherwise collide with the instance path's at link time)
namespace {
#include "ns_kernels.cuh"
}

using namespace nsg;

// 8 MiB: the FP64 intermediate of every power-of-two grid up to 1024 x 1024
#define NS_NOALLOC_SCRATCH_BYTES (8u << 20)
static __device__ __align__(256) unsigned char g_noalloc_scratch[NS_NOALLOC_SCRATCH_BYTES];

#define NS_NOALLOC_MAX_DEVICES 64
static std::mutex g_noalloc_mu;
static void* g_noalloc_addr[NS_NOALLOC_MAX_DEVICES];

static size_t round256(size_t b) { return (b + 255) & ~(size_t)255; }

// geometry of the instance path (ns_gpu_create) for a grid, FP64
static void noalloc_geo(int nx, int ny, Geo& G, int& ER, int& EC) {
    memset(&G, 0, sizeof(G));
    G.nx = nx;
    G.ny = ny;
    G.nkx = nx / 2 + 1;
    G.nky = ny;
    G.H = nx / 2;
    G.Kx = (2 * G.nkx) / 3 + 1;
    G.Kyh = (2 * ny) / 6;
    G.Ky = 2 * G.Kyh + 1;
    int l = 0;
    while ((1 << l) < ny) ++l;
    G.logny = l;
    l = 0;
    while ((1 << l) < G.H) ++l;
    G.logH = l;
    G.Lx = 1.0;
    G.Ly = 1.0;
    G.fLB = 0;
    G.fTG = 0;
    ER = G.H >= 16 ? 16 : 4;
    EC = ny >= 16 ? 16 : 4;
    const size_t cs = sizeof(double2);
    const int TC = ny / EC;
    int CW = 1;
    while (CW < 16 && 2 * CW * TC <= 512 && (size_t)2 * CW * spad_len(ny) * cs <= 100 * 1024 && CW < G.Kx) CW *= 2;
    G.CW = CW;
    G.Kxp = ((G.Kx + CW - 1) / CW) * CW;
    const int TT = G.H / ER;
    int RPC = 1;
    while (2 * RPC * TT <= 128 && 2 * RPC <= ny && (size_t)4 * 2 * RPC * spad_len(G.H) * cs <= 100 * 1024) RPC *= 2;
    G.RPC = RPC;
}

static size_t noalloc_bytes(const Geo& G) {
    return round256((size_t)G.ny * sizeof(double2)) + 2 * round256((size_t)G.H * sizeof(double2)) +
           round256((size_t)G.ny * G.Kxp * sizeof(double2));
}

// per-device set-up: the array's device address, and the shared-memory limit of
// the two kernels raised to the largest size a supported grid needs
static int noalloc_setup(void** base) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        fprintf(stderr, "ns_gpu_forward_noalloc: cudaGetDevice: %s\n", cudaGetErrorString(e));
        return NS_GPU_ERR_NO_DEVICE;
    }
    if (dev < 0 || dev >= NS_NOALLOC_MAX_DEVICES) return NS_GPU_ERR_INVALID;
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            fprintf(stderr, "ns_gpu_forward_noalloc: cudaGetSymbolAddress: %s\n", cudaGetErrorString(e));
            return NS_GPU_ERR_CUDA;
        }
        const int smem = 100 * 1024 + 4096;
        const void* kerns[] = {(const void*)k_row<double, 16, ROW_FWD1>, (const void*)k_row<double, 4, ROW_FWD1>,
                               (const void*)k_col<double, 16, COL_FWD_EXPORT, 0>,
                               (const void*)k_col<double, 4, COL_FWD_EXPORT, 0>};
        for (const void* k : kerns) {
            e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
            if (e != cudaSuccess) {
                fprintf(stderr, "ns_gpu_forward_noalloc: cudaFuncSetAttribute: %s\n", cudaGetErrorString(e));
                return NS_GPU_ERR_CUDA;
            }
        }
        g_noalloc_addr[dev] = p;
    }
    *base = g_noalloc_addr[dev];
    return NS_GPU_OK;
}

// one launch; the returned status is this launch's own (a <<<>>> launch is only
// checked through cudaGetLastError, which would also report and clear an
// unrelated earlier error of the caller)
template <typename... KArgs, typename... Args>
static cudaError_t noalloc_launch(void (*kern)(KArgs...), int grid, int block, size_t smem, cudaStream_t st,
                                  Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    return cudaLaunchKernelEx(&cfg, kern, args...);
}

static int noalloc_fail(const char* what, cudaError_t e) {
    fprintf(stderr, "ns_gpu_forward_noalloc: %s: %s\n", what, cudaGetErrorString(e));
    return NS_GPU_ERR_CUDA;
}

template <int ER, int EC>
static int noalloc_run(const Geo& G, unsigned char* base, const double* field, double* field_hat, cudaStream_t st) {
    double2* twc = (double2*)base;
    double2* twr = (double2*)(base + round256((size_t)G.ny * sizeof(double2)));
    double2* twh = (double2*)((unsigned char*)twr + round256((size_t)G.H * sizeof(double2)));
    double2* Gbuf = (double2*)((unsigned char*)twh + round256((size_t)G.H * sizeof(double2)));
    cudaError_t e = noalloc_launch(k_twiddles<double2>, (G.ny + 255) / 256, 256, 0, st, twc, G.ny, G.ny);
    if (e != cudaSuccess) return noalloc_fail("twiddle launch", e);
    e = noalloc_launch(k_twiddles<double2>, (G.H + 255) / 256, 256, 0, st, twr, G.H, G.H);
    if (e != cudaSuccess) return noalloc_fail("twiddle launch", e);
    e = noalloc_launch(k_twiddles<double2>, (G.H + 255) / 256, 256, 0, st, twh, G.H, G.nx);
    if (e != cudaSuccess) return noalloc_fail("twiddle launch", e);
    RowArgs<double> ra;
    memset(&ra, 0, sizeof(ra));
    ra.G = Gbuf;
    ra.in_real = field;
    ra.twr = twr;
    ra.twh = twh;
    const int TT = G.H / ER;
    const size_t rsm = (size_t)G.RPC * spad_len(G.H) * sizeof(double2);
    e = noalloc_launch(k_row<double, ER, ROW_FWD1>, G.ny / G.RPC, G.RPC * TT, rsm, st, G, ra);
    if (e != cudaSuccess) return noalloc_fail("row-pass launch", e);
    e = cudaMemsetAsync(field_hat, 0, (size_t)G.nkx * G.nky * sizeof(double2), st);
    if (e != cudaSuccess) return noalloc_fail("cudaMemsetAsync", e);
    ColArgs<double> ca;
    memset(&ca, 0, sizeof(ca));
    ca.G = Gbuf;
    ca.twc = twc;
    ca.out_spec = (double2*)field_hat;
    ca.out_scale = 1.0 / ((double)G.nx * (double)G.ny);
    const int TC = G.ny / EC;
    const size_t csm = (size_t)G.CW * spad_len(G.ny) * sizeof(double2);
    e = noalloc_launch(k_col<double, EC, COL_FWD_EXPORT, 0>, G.Kxp / G.CW, G.CW * TC, csm, st, G, ca);
    if (e != cudaSuccess) return noalloc_fail("column-pass launch", e);
    return NS_GPU_OK;
}

int ns_gpu_forward_noalloc(int nx, int ny, const double* field, double* field_hat, void* stream) {
    if (!field || !field_hat) return NS_GPU_ERR_INVALID;
    if (nx < 8 || ny < 8 || nx > 4096 || ny > 4096 || (nx & (nx - 1)) || (ny & (ny - 1))) {
        fprintf(stderr, "ns_gpu_forward_noalloc: nx=%d ny=%d must be powers of two in [8, 4096]\n", nx, ny);
        return NS_GPU_ERR_INVALID;
    }
    if (((uintptr_t)field & 15) || ((uintptr_t)field_hat & 15)) {
        fprintf(stderr, "ns_gpu_forward_noalloc: field and field_hat must be 16-byte aligned device pointers\n");
        return NS_GPU_ERR_INVALID;
    }
    Geo G;
    int ER = 16, EC = 16;
    noalloc_geo(nx, ny, G, ER, EC);
    const size_t need = noalloc_bytes(G);
    if (need > NS_NOALLOC_SCRATCH_BYTES) {
        fprintf(stderr,
                "ns_gpu_forward_noalloc: a %d x %d grid needs %zu bytes of scratch, more than the %u-byte static "
                "array (grids up to 1024 x 1024 fit); use ns_gpu_forward on an instance instead\n",
                nx, ny, need, (unsigned)NS_NOALLOC_SCRATCH_BYTES);
        return NS_GPU_ERR_INVALID;
    }
    void* base = nullptr;
    int s = noalloc_setup(&base);
    if (s != NS_GPU_OK) return s;
    cudaStream_t st = (cudaStream_t)stream;
    unsigned char* b = (unsigned char*)base;
    if (ER == 16 && EC == 16) return noalloc_run<16, 16>(G, b, field, field_hat, st);
    if (ER == 4 && EC == 16) return noalloc_run<4, 16>(G, b, field, field_hat, st);
    if (ER == 16 && EC == 4) return noalloc_run<16, 4>(G, b, field, field_hat, st);
    return noalloc_run<4, 4>(G, b, field, field_hat, st);
}
