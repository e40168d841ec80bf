// fsim_noalloc.cu — a cell sort that allocates no memory.
//
// fsim_cell_sort_noalloc performs the same counting sort as the cell phase of
// a handle (cell index of every position, exclusive scan of the per-cell
// counts, order inside a cell by input index), but on caller-owned device
// buffers and with its scratch in one file-scope __device__ array instead of
// cudaMalloc'ed memory.  It exists for callers that must not allocate device
// memory once they are running: hosts that reserve all GPU memory up front
// under their own allocator or budget, and real-time loops that cannot afford
// the implicit device synchronisation cudaMalloc/cudaFree bring.
//
// The scratch array below lives in every GPU that loads this library, from
// module load until the process exits: 4 * (3 * kMaxParticles + kMaxCells)
// bytes, i.e. 4 MiB.  Every call shares it, so calls that overlap on the GPU
// (different streams, different host threads) race on it; the caller must
// order them.
#include "fsim_internal.h"

#include <cuda_runtime.h>

namespace {

constexpr int kMaxParticles = FSIM_NOALLOC_MAX_PARTICLES;
constexpr int kMaxCells = FSIM_NOALLOC_MAX_CELLS;
constexpr int kThreads = 256;
constexpr int kScanThreads = 1024;
constexpr size_t kScratchWords = 3 * (size_t)kMaxParticles + (size_t)kMaxCells;

// layout: key[kMaxParticles] | slot[kMaxParticles] | tmp[kMaxParticles] | count[kMaxCells]
static __device__ __align__(256) int g_sort_scratch[kScratchWords];

struct Grid {
    float cmin[3], cinv[3];
    int n[3];
};

// cell index of src/pair.cu:8-24; positions outside the grid are clamped into
// its boundary cells
__global__ void k_na_count(Grid g, const float *__restrict__ pos, int np, int *__restrict__ key,
                           int *__restrict__ slot, int *__restrict__ count)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= np) return;
    int c[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        c[a] = (int)__fmul_rn(__fsub_rn(pos[3 * s + a], g.cmin[a]), g.cinv[a]);
        c[a] = min(max(c[a], 0), g.n[a] - 1);
    }
    const int k = (c[0] * g.n[1] + c[1]) * g.n[2] + c[2];
    key[s] = k;
    slot[s] = atomicAdd(&count[k], 1);
}

// single-block exclusive scan of count[0..nc) into start[0..nc]
__global__ void __launch_bounds__(kScanThreads) k_na_scan(const int *__restrict__ count, int nc,
                                                          int *__restrict__ start)
{
    __shared__ int warp_tot[32];
    const int per = (nc + kScanThreads - 1) / kScanThreads;
    const int b = threadIdx.x * per, e = min(b + per, nc);
    int sum = 0;
    for (int i = b; i < e; ++i) sum += count[i];
    // block exclusive scan of the per-thread sums
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int inc = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += t;
    }
    if (lane == 31) warp_tot[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        int w = warp_tot[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += t;
        }
        warp_tot[lane] = w;
    }
    __syncthreads();
    int run = (warp ? warp_tot[warp - 1] : 0) + inc - sum;
    for (int i = b; i < e; ++i) {
        start[i] = run;
        run += count[i];
    }
    if (threadIdx.x == kScanThreads - 1) start[nc] = warp_tot[31];
}

__global__ void k_na_scatter(const int *__restrict__ key, const int *__restrict__ slot,
                             const int *__restrict__ start, int *__restrict__ tmp, int np)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < np) tmp[start[key[s]] + slot[s]] = s;
}

// final slot = cell start + number of same-cell particles with a smaller input
// index.  The scan costs the cell's count per particle; a cell of more than
// kRankMax particles (positions outside the grid or NaN, clamped into one
// boundary cell, or a smoothing length of several particle spacings) keeps the
// scatter's order instead, so the work stays bounded.
constexpr int kRankMax = FSIM_NOALLOC_RANK_MAX;
__global__ void k_na_rank(const int *__restrict__ key, const int *__restrict__ start, const int *__restrict__ tmp,
                          int *__restrict__ ids, int np)
{
    const int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= np) return;
    const int src = tmp[d];
    const int c = key[src];
    const int b = start[c], e = start[c + 1];
    if (e - b > kRankMax) {
        ids[d] = src;
        return;
    }
    int rank = 0;
    for (int t = b; t < e; ++t) rank += tmp[t] < src;
    ids[b + rank] = src;
}

// Device address of the scratch array on the current device.  In host code
// g_sort_scratch names a host-side stand-in, never the device memory.  The
// address is looked up on every call (a table lookup in the runtime once the
// module is loaded on the device) rather than cached, so that it stays right
// after cudaDeviceReset or a new primary context reloads the module.  The
// first call on a device loads the module there, so make it before any stream
// capture.
fsim_status scratch_for_current_device(int **out)
{
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_sort_scratch);
    if (e != cudaSuccess) {
        fsim_set_error("cudaGetSymbolAddress(scratch) failed: %s", cudaGetErrorString(e));
        return FSIM_ECUDA;
    }
    *out = (int *)p;
    return FSIM_OK;
}

} // namespace

extern "C" fsim_status fsim_cell_sort_noalloc(const fsim_derived *grid, const float *d_pos, int n,
                                              int *d_cell_start, int *d_ids, void *stream)
{
    if (!grid || n < 0 || (n > 0 && (!d_pos || !d_ids)) || !d_cell_start) {
        fsim_set_error("fsim_cell_sort_noalloc: invalid arguments");
        return FSIM_EINVAL;
    }
    const int nc = grid->cell_number_total;
    if (n > kMaxParticles || nc < 1 || nc > kMaxCells ||
        (long long)grid->cell_number[0] * grid->cell_number[1] * grid->cell_number[2] != nc) {
        fsim_set_error("fsim_cell_sort_noalloc: %d particles / %d cells exceed the fixed scratch "
                       "(at most %d particles and %d cells)", n, nc, kMaxParticles, kMaxCells);
        return FSIM_EINVAL;
    }
    int *scratch = nullptr;
    fsim_status st = scratch_for_current_device(&scratch);
    if (st) return st;
    int *key = scratch, *slot = scratch + kMaxParticles, *tmp = scratch + 2 * kMaxParticles;
    int *count = scratch + 3 * kMaxParticles;
    cudaStream_t s = (cudaStream_t)stream;
    Grid g;
    for (int a = 0; a < 3; ++a) {
        g.cmin[a] = grid->cell_min[a];
        g.cinv[a] = grid->interval_inv[a];
        g.n[a] = grid->cell_number[a];
    }
    // the scratch keeps the previous call's contents: the counts must start at zero
    cudaError_t e = cudaMemsetAsync(count, 0, sizeof(int) * (size_t)nc, s);
    if (e != cudaSuccess) {
        fsim_set_error("cudaMemsetAsync failed: %s", cudaGetErrorString(e));
        return FSIM_ECUDA;
    }
    const int blocks = (n + kThreads - 1) / kThreads;
    if (n > 0) k_na_count<<<blocks, kThreads, 0, s>>>(g, d_pos, n, key, slot, count);
    k_na_scan<<<1, kScanThreads, 0, s>>>(count, nc, d_cell_start);
    if (n > 0) {
        k_na_scatter<<<blocks, kThreads, 0, s>>>(key, slot, d_cell_start, tmp, n);
        k_na_rank<<<blocks, kThreads, 0, s>>>(key, d_cell_start, tmp, d_ids, n);
    }
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        fsim_set_error("fsim_cell_sort_noalloc launch failed: %s", cudaGetErrorString(e));
        return FSIM_ECUDA;
    }
    return FSIM_OK;
}
