// dsmc_noalloc.cu -- cell start offsets without any device allocation.
//
// Some callers cannot allocate device memory at the point where they need the
// occupancy offsets: an application that hands every byte of HBM to its own
// pool allocator up front, a plugin that runs inside a host code's time loop
// with no licence to grow that footprint, or a caller that may not create new
// allocations at all.  dsmc_cell_starts_noalloc serves them: the caller passes
// device buffers for the per-cell counts and the starts, and the block sums
// the scan needs live in a fixed array inside this library.
//
// That array is a file-scope __device__ variable of NA_MAX_BLOCKS (4096)
// ints (16 KiB): every GPU that loads the library holds it until the process
// exits.  Host code cannot use its name as an address, so every call made
// outside stream capture looks the address up with cudaGetSymbolAddress (with
// the calling device current) and keeps it for captured calls; make the first
// call on a device, and the first one after a device reset, outside capture.
// All calls share the one array and it keeps what the last call left there;
// each call writes every entry it reads before reading it.  Calls whose
// kernels overlap on the GPU race on the array: serialise them (one stream,
// or events between streams).

#include <cstdio>
#include <mutex>

#include "dsmc_kernels.h"

namespace {

constexpr int NA_THREADS = 1024;
constexpr int NA_ITEMS = 4;
constexpr int NA_TILE = NA_THREADS * NA_ITEMS;                  // cells per block
constexpr long long NA_MAX_CELLS = 1LL << 24;                   // 16,777,216 cells
constexpr int NA_MAX_BLOCKS = (int)(NA_MAX_CELLS / NA_TILE);    // 4096 block sums

static __device__ __align__(256) int g_noalloc_block_sums[NA_MAX_BLOCKS];

constexpr int NA_MAX_DEVICES = 64;
std::mutex g_na_mutex;
int* g_na_ptr[NA_MAX_DEVICES] = {nullptr};

__device__ __forceinline__ int na_block_scan(int v, int* total) {
    __shared__ int warpSums[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xFFFFFFFFu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warpSums[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int ws = (lane < (int)(blockDim.x >> 5)) ? warpSums[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xFFFFFFFFu, ws, o);
            if (lane >= o) ws += y;
        }
        warpSums[lane] = ws;
    }
    __syncthreads();
    const int warpOff = wid ? warpSums[wid - 1] : 0;
    *total = warpSums[(blockDim.x >> 5) - 1];
    __syncthreads();
    return warpOff + x - v;
}

__global__ void __launch_bounds__(NA_THREADS) k_na_reduce(const int* __restrict__ count, long long C, int* sums) {
    const long long base = (long long)blockIdx.x * NA_TILE + (long long)threadIdx.x * NA_ITEMS;
    int s = 0;
#pragma unroll
    for (int k = 0; k < NA_ITEMS; ++k)
        if (base + k < C) s += count[base + k];
    int total;
    na_block_scan(s, &total);
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(NA_THREADS) k_na_top(int* sums, int nb, int* start, long long C) {
    int carry = 0;
    for (int b0 = 0; b0 < nb; b0 += NA_THREADS) {
        const int b = b0 + threadIdx.x;
        const int v = (b < nb) ? sums[b] : 0;
        int total;
        const int ex = na_block_scan(v, &total);
        if (b < nb) sums[b] = carry + ex;
        carry += total;
    }
    if (threadIdx.x == 0) start[C] = carry;
}

__global__ void __launch_bounds__(NA_THREADS) k_na_down(const int* __restrict__ count, long long C,
                                                        const int* __restrict__ sums, int* start) {
    const long long base = (long long)blockIdx.x * NA_TILE + (long long)threadIdx.x * NA_ITEMS;
    int v[NA_ITEMS];
    int s = 0;
#pragma unroll
    for (int k = 0; k < NA_ITEMS; ++k) {
        v[k] = (base + k < C) ? count[base + k] : 0;
        s += v[k];
    }
    int total;
    int ex = na_block_scan(s, &total) + sums[blockIdx.x];
#pragma unroll
    for (int k = 0; k < NA_ITEMS; ++k) {
        if (base + k < C) start[base + k] = ex;
        ex += v[k];
    }
}

thread_local char g_na_msg[256];

int na_fail(int code, const char* msg) {
    snprintf(g_na_msg, sizeof(g_na_msg), "%s", msg);
    return code;
}

}  // namespace

extern "C" {

const char* dsmc_noalloc_last_error(void) { return g_na_msg; }

int dsmc_cell_starts_noalloc(const int* d_counts, long long n_cells, int* d_start, void* stream) {
    if (n_cells <= 0 || n_cells > NA_MAX_CELLS)
        return na_fail(DSMC_ERR_INVALID, "dsmc_cell_starts_noalloc: n_cells must be 1..16777216");
    if (!d_counts || !d_start)
        return na_fail(DSMC_ERR_INVALID, "dsmc_cell_starts_noalloc: null device buffer");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return na_fail(DSMC_ERR_CUDA, cudaGetErrorString(e));
    if (dev < 0 || dev >= NA_MAX_DEVICES)
        return na_fail(DSMC_ERR_INVALID, "dsmc_cell_starts_noalloc: device index beyond 63");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // The array's address is looked up again on every call made outside
    // stream capture, so a device reset (which reloads the module and may
    // move the array) never leaves a stale address behind; a captured call
    // uses the address of the last uncaptured one.
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    e = cudaStreamIsCapturing(st, &cap);
    if (e != cudaSuccess) return na_fail(DSMC_ERR_CUDA, cudaGetErrorString(e));
    int* sums = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_na_mutex);
        if (!g_na_ptr[dev] || cap == cudaStreamCaptureStatusNone) {
            void* p = nullptr;
            e = cudaGetSymbolAddress(&p, g_noalloc_block_sums);
            if (e != cudaSuccess) return na_fail(DSMC_ERR_CUDA, cudaGetErrorString(e));
            g_na_ptr[dev] = static_cast<int*>(p);
        }
        sums = g_na_ptr[dev];
    }
    const int nb = (int)((n_cells + NA_TILE - 1) / NA_TILE);
    k_na_reduce<<<nb, NA_THREADS, 0, st>>>(d_counts, n_cells, sums);
    k_na_top<<<1, NA_THREADS, 0, st>>>(sums, nb, d_start, n_cells);
    k_na_down<<<nb, NA_THREADS, 0, st>>>(d_counts, n_cells, sums, d_start);
    e = cudaGetLastError();
    if (e != cudaSuccess) return na_fail(DSMC_ERR_CUDA, cudaGetErrorString(e));
    return DSMC_OK;
}

}  // extern "C"
