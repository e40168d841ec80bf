// fsim_sim.cu — device state, sm_103a kernels and the simulation half of the
// C ABI (include/fluidsim.h).
//
// Layout in HBM (one handle = one instance):
//   fluid    float4 posr = (x, y, z, rho), float4 velp = (u, v, w, p), int orig,
//            all double-buffered; particles are kept sorted by cell.  The cell
//            phase sorts buffer `cur` into the other one; the fused fluid
//            sweep + update reads the sorted buffer and writes the updated
//            state into the other, in the same order.
//   solid    float4 pos/vel/ref, int type/orig, double-buffered the same way;
//            per-step products (normal+pressure, F, P, L^-1, du/dt) single.
//   virtual  sorted by cell once at creation (walls never move); float4 posr
//            (rho in .w) and velp (mirrored velocity, pressure) rewritten every
//            step; float4 normal computed once (a static quantity).
//   cells    per species an exclusive-scan start array of cell_number_total+1
//            ints: the particles of cell c are [start[c], start[c+1]).
//            Because cells are linearised x-major (src/pair.cu:20-23), the
//            three cells (x, y, z-1..z+1) are contiguous, so the 27-cell
//            neighbourhood is 9 contiguous index ranges.
//
// The neighbour sweeps gather every particle's neighbours (one owner per
// output, no atomics on physics sums): results are deterministic.
#include "fsim_internal.h"

#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

namespace {

// ---------------------------------------------------------------- params
struct DevParams {
    // kernel (src/kernel.cpp:43-60)
    float R2, h, h_inv2, kdiff, kc1, kc2, eps_h2, exp2_scale;
    // fluid (src/properties.cpp:47-57)
    float c0, c0_inv, rho0, rho0_inv, gamma, rho2p, min_p, min_rho, max_rho, mu10, vmax;
    int viscid;
    // solid (src/properties.cpp:59-66)
    float rho_s_inv, lambda, mu_s, cs_s, alpha, beta;
    // physics, time
    float gx, gy, gz, dt, dt_sub;
    // domain
    float dmin[3], dmax[3], cmin[3], cinv[3];
    int nx, ny, nz, ncell;
    // mixed form: cell size, domain bounds relative to the grid origin,
    // density-deviation clamp, FP16 scales of the gathered deviations
    float cdx[3], dlo_rel[3], dhi_rel[3];
    float dlt_min, dlt_max, p_unit, p_unit_inv;
    int mixed;
};

enum : unsigned { FLAG_OUT_OF_GRID = 1u, FLAG_BARRIER_TIMEOUT = 2u };
constexpr unsigned kFull = 0xffffffffu;

constexpr int kBlock = 256;
constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;
constexpr int kMaxScanTiles = 16384; // cell grids up to 67M cells

__host__ __device__ inline int blocks_for(long long n, int b) { return (int)((n + b - 1) / b); }

// ------------------------------------------------------------- cell math
// findPositionCell (src/pair.cu:8-24): per-axis truncation of the FP32
// (p - min) * inv.  Out-of-grid indices (impossible for clamped positions)
// are clamped and flagged instead of indexing out of bounds.
__device__ __forceinline__ int axis_cell(float p, float mn, float inv, int n, bool &bad)
{
    int c = (int)__fmul_rn(__fsub_rn(p, mn), inv);
    if (c < 0 || c >= n) {
        bad = true;
        c = c < 0 ? 0 : n - 1;
    }
    return c;
}

__device__ __forceinline__ int cell_index(const DevParams &P, float x, float y, float z, unsigned *flags)
{
    bool bad = false;
    const int cx = axis_cell(x, P.cmin[0], P.cinv[0], P.nx, bad);
    const int cy = axis_cell(y, P.cmin[1], P.cinv[1], P.ny, bad);
    const int cz = axis_cell(z, P.cmin[2], P.cinv[2], P.nz, bad);
    if (bad && flags) atomicOr(flags, FLAG_OUT_OF_GRID);
    return cx * P.ny * P.nz + cy * P.nz + cz;
}

// FP32 squared distance; the oracle's neighbour counts use the same formula.
__device__ __forceinline__ float dist2(float dx, float dy, float dz)
{
    return __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
}

// The 9 z-contiguous rows of the 27-cell neighbourhood of cell c.
struct Rows {
    int base[9];
    int z0, z1, count;
};
__device__ __forceinline__ void neighbor_rows(const DevParams &P, int c, Rows &r)
{
    const int cx = c / (P.ny * P.nz);
    const int rem = c - cx * P.ny * P.nz;
    const int cy = rem / P.nz;
    const int cz = rem - cy * P.nz;
    r.z0 = max(cz - 1, 0);
    r.z1 = min(cz + 1, P.nz - 1) + 1;
    r.count = 0;
    for (int ox = -1; ox <= 1; ++ox) {
        const int x = cx + ox;
        if (x < 0 || x >= P.nx) continue;
        for (int oy = -1; oy <= 1; ++oy) {
            const int y = cy + oy;
            if (y < 0 || y >= P.ny) continue;
            r.base[r.count++] = (x * P.ny + y) * P.nz;
        }
    }
}

// ------------------------------------------------------- batched launches
// Every step kernel has a body taking (params, args, local block index) and a
// batched wrapper: one launch serves many instances, each with its own
// parameters and buffers.  The wrapper finds its instance by binary search in
// a per-launch prefix table of block counts (bstart[ninst] = total blocks) and
// reads that instance's {params, args} item from the read-only item array.
template <class Args>
struct Item {
    DevParams P;
    Args A;
};

__device__ __forceinline__ int locate_instance(const int *__restrict__ bstart, int ninst, int b)
{
    int lo = 0, hi = ninst;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (bstart[mid] <= b) lo = mid;
        else hi = mid;
    }
    return lo;
}

#define FSIM_BATCHED_KERNEL(NAME, ARGS, BODY, BOUNDS)                                                      \
    __global__ void __launch_bounds__(BOUNDS) NAME(const Item<ARGS> *__restrict__ items,                 \
                                                   const int *__restrict__ bstart, int ninst)            \
    {                                                                                                     \
        const int inst = locate_instance(bstart, ninst, blockIdx.x);                                     \
        const DevParams P = items[inst].P;                                                                \
        const ARGS &A = items[inst].A;                                                                    \
        BODY(P, A, (int)blockIdx.x - bstart[inst]);                                                       \
    }

// ------------------------------------------------------- counting sort
struct HashArgs {
    const float4 *pos;
    int n;
    int *key, *slot, *cnt;
    unsigned *flags;
};
// A slot in cell c's count: lanes of a warp with the same cell share one
// atomic (particles arrive sorted by their previous cell, so a warp holds few
// distinct cells).  Slots only need to be distinct within a cell: the gather
// orders a cell's particles by their previous position.  All lanes call it.
__device__ __forceinline__ int cell_slot(int *cnt, int c, bool active)
{
    const unsigned act = __ballot_sync(kFull, active);
    if (!active) return 0;
    const unsigned peers = __match_any_sync(act, c);
    const int lane = threadIdx.x & 31, leader = __ffs(peers) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(&cnt[c], __popc(peers));
    base = __shfl_sync(peers, base, leader);
    return base + __popc(peers & ((1u << lane) - 1u));
}

__device__ __forceinline__ void hash_body(const DevParams &P, const HashArgs &A, int blk)
{
    const int s = blk * blockDim.x + threadIdx.x;
    const bool active = s < A.n;
    int c = 0;
    if (active) {
        const float4 p = A.pos[s];
        c = cell_index(P, p.x, p.y, p.z, A.flags);
        A.key[s] = c;
    }
    const int slot = cell_slot(A.cnt, c, active);
    if (active) A.slot[s] = slot;
}
FSIM_BATCHED_KERNEL(kb_hash, HashArgs, hash_body, kBlock)

struct ZeroArgs {
    int *p;
    int n;
};
__device__ __forceinline__ void zero_body(const DevParams &, const ZeroArgs &A, int blk)
{
    const int s = blk * blockDim.x + threadIdx.x;
    if (s < A.n) A.p[s] = 0;
}
FSIM_BATCHED_KERNEL(kb_zero, ZeroArgs, zero_body, kBlock)

struct ScanArgs {
    const int *in;
    int *out;
    int n;
    int *partial;
};

__device__ __forceinline__ int warp_inclusive_scan(int v)
{
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

// exclusive scan of one value per thread over a 1024-thread block; returns the
// block total in *total
__device__ __forceinline__ int block_exclusive_scan(int v, int *total)
{
    __shared__ int warp_sums[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int inc = warp_inclusive_scan(v);
    if (lane == 31) warp_sums[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        const int nw = blockDim.x >> 5;
        int w = lane < nw ? warp_sums[lane] : 0;
        w = warp_inclusive_scan(w);
        warp_sums[lane] = w;
    }
    __syncthreads();
    const int before = warp == 0 ? 0 : warp_sums[warp - 1];
    *total = warp_sums[(blockDim.x >> 5) - 1];
    __syncthreads();
    return before + inc - v;
}

// scan pass 1: per-tile sums (one block per 4096-entry tile)
__device__ __forceinline__ void scan_reduce_body(const DevParams &, const ScanArgs &J, int blk)
{
    const int base = blk * kScanTile + threadIdx.x * kScanItems;
    int s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k)
        if (base + k < J.n) s += J.in[base + k];
    int total;
    block_exclusive_scan(s, &total);
    if (threadIdx.x == 0) J.partial[blk] = total;
}
FSIM_BATCHED_KERNEL(kb_scan_reduce, ScanArgs, scan_reduce_body, kScanThreads)

// scan pass 2: exclusive scan of the tile sums (one block per array)
__device__ __forceinline__ void scan_partials_body(const DevParams &, const ScanArgs &J, int)
{
    const int tiles = blocks_for(J.n, kScanTile);
    int carry = 0;
    for (int b0 = 0; b0 < tiles; b0 += kScanThreads) {
        const int i = b0 + threadIdx.x;
        const int v = i < tiles ? J.partial[i] : 0;
        int total;
        const int ex = block_exclusive_scan(v, &total);
        if (i < tiles) J.partial[i] = carry + ex;
        carry += total;
    }
    if (threadIdx.x == 0) J.out[J.n] = carry;
}
FSIM_BATCHED_KERNEL(kb_scan_partials, ScanArgs, scan_partials_body, kScanThreads)

// scan pass 3: scan inside each tile plus its offset
__device__ __forceinline__ void scan_apply_body(const DevParams &, const ScanArgs &J, int blk)
{
    const int base = blk * kScanTile + threadIdx.x * kScanItems;
    int v[kScanItems];
    int s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        v[k] = base + k < J.n ? J.in[base + k] : 0;
        s += v[k];
    }
    int total;
    int run = block_exclusive_scan(s, &total) + J.partial[blk];
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        if (base + k < J.n) J.out[base + k] = run;
        run += v[k];
    }
}
FSIM_BATCHED_KERNEL(kb_scan_apply, ScanArgs, scan_apply_body, kScanThreads)

struct ScatterArgs {
    const int *key, *slot, *start;
    int *tmp;
    int n;
};
__device__ __forceinline__ void scatter_body(const DevParams &, const ScatterArgs &A, int blk)
{
    const int s = blk * blockDim.x + threadIdx.x;
    if (s >= A.n) return;
    A.tmp[A.start[A.key[s]] + A.slot[s]] = s;
}
FSIM_BATCHED_KERNEL(kb_scatter, ScatterArgs, scatter_body, kBlock)

// Rank inside the cell by previous position: the new order is sorted by
// (cell, previous sorted position), a stable and deterministic order.
__device__ __forceinline__ int stable_dst(const int *__restrict__ tmp, const int *__restrict__ key,
                                          const int *__restrict__ start, int d, int &src, int &cell)
{
    src = tmp[d];
    cell = key[src];
    const int b = start[cell], e = start[cell + 1];
    int rank = 0;
    for (int t = b; t < e; ++t) rank += tmp[t] < src;
    return b + rank;
}

struct GatherFluidArgs {
    const int *tmp, *key, *start;
    int n;
    const float4 *posr_in, *velp_in;
    const int *orig_in;
    float4 *posr_out, *velp_out;
    int *orig_out, *cell_out;
};
__device__ __forceinline__ void gather_fluid_body(const DevParams &, const GatherFluidArgs &A, int blk)
{
    const int d = blk * blockDim.x + threadIdx.x;
    if (d >= A.n) return;
    int src, cell;
    const int dst = stable_dst(A.tmp, A.key, A.start, d, src, cell);
    A.posr_out[dst] = A.posr_in[src];
    A.velp_out[dst] = A.velp_in[src];
    A.orig_out[dst] = A.orig_in[src];
    A.cell_out[dst] = cell;
}
FSIM_BATCHED_KERNEL(kb_gather_fluid, GatherFluidArgs, gather_fluid_body, kBlock)

struct GatherSolidArgs {
    const int *tmp, *key, *start;
    int n;
    const float4 *pos_in, *vel_in, *ref_in;
    const int *type_in, *orig_in;
    float4 *pos_out, *vel_out, *ref_out;
    int *type_out, *orig_out, *cell_out;
    int *inv_out;       // sorted position of every input id
    unsigned *cxyz_out; // cell coordinates packed x | y << 11 | z << 21
};
__device__ __forceinline__ unsigned pack_cell(const DevParams &P, int c)
{
    const int cx = c / (P.ny * P.nz), rem = c - cx * P.ny * P.nz;
    const int cy = rem / P.nz, cz = rem - cy * P.nz;
    return (unsigned)cx | ((unsigned)cy << 11) | ((unsigned)cz << 21);
}
// neighbouring cells (each coordinate within one), from packed coordinates
__device__ __forceinline__ bool cells_adjacent(unsigned a, unsigned b)
{
    const int dx = (int)(a & 0x7ffu) - (int)(b & 0x7ffu);
    const int dy = (int)((a >> 11) & 0x3ffu) - (int)((b >> 11) & 0x3ffu);
    const int dz = (int)(a >> 21) - (int)(b >> 21);
    return abs(dx) <= 1 && abs(dy) <= 1 && abs(dz) <= 1;
}
__device__ __forceinline__ void gather_solid_body(const DevParams &P, const GatherSolidArgs &A, int blk)
{
    const int d = blk * blockDim.x + threadIdx.x;
    if (d >= A.n) return;
    int src, cell;
    const int dst = stable_dst(A.tmp, A.key, A.start, d, src, cell);
    A.pos_out[dst] = A.pos_in[src];
    A.vel_out[dst] = A.vel_in[src];
    A.ref_out[dst] = A.ref_in[src];
    A.type_out[dst] = A.type_in[src];
    const int o = A.orig_in[src];
    A.orig_out[dst] = o;
    A.cell_out[dst] = cell;
    A.inv_out[o] = dst;
    A.cxyz_out[dst] = pack_cell(P, cell);
}
FSIM_BATCHED_KERNEL(kb_gather_solid, GatherSolidArgs, gather_solid_body, kBlock)

// ------------------------------------------------------------ EOS
// densityToPressure (src/fluid.cu:16-24): Tait EOS, floored at min_pressure.
__device__ __forceinline__ float tait_pressure(const DevParams &P, float rho)
{
    const float p = (__powf(rho * P.rho0_inv, P.gamma) - 1.0f) * P.rho2p;
    return fmaxf(p, P.min_p);
}

// ------------------------------------------------------ Riemann pair term
// fluidFluidCalculate / fluidSolidCalculate / fluidVirtCalculate
// (src/fluid.cu:26-167), algebraically regrouped:
//   P*   = (rho_i p_j + rho_j p_i)/(rho_i+rho_j) [+ rho_i rho_j du/(rho_i+rho_j) * lim  if du >= 0]
//   (u_i - v*).dx = (rho_j (u_i-u_j).dx - (p_i-p_j) r / c0) / (rho_i+rho_j)
//   du/dt += w dx (-2 P* + 10 mu vis) / rho_i,  drho/dt += 2 rho_i w (u_i - v*).dx
// with w = exp(-r^2/h^2) * kernel_differential (so that w dx = V grad W).
// The caller multiplies by 1/rho_i and 2 rho_i once per particle.  The
// transcendental parts use the PTX approximations ex2/rsqrt/rcp.approx (the
// reference's release build is compiled with -use_fast_math).
struct PairAcc {
    float drho, ax, ay, az;
    float drho_c; // compensation term of the density-rate sum (KAHAN)
};

__device__ __forceinline__ float ex2_approx(float x)
{
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float rsqrt_approx(float x)
{
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float rcp_approx(float x)
{
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// LIMITER: min(3 du, c0) (fluid, wall) or c0 (solid).  clamp_ps: P* >= 0 (wall).
// KAHAN: the density-rate sum is Kahan-compensated (mixed form).
template <bool LIMITER, int VISCID, bool KAHAN = false>
__device__ __forceinline__ void riemann_pair(const DevParams &P, float dx, float dy, float dz, float r2, float uix,
                                             float uiy, float uiz, float rhoi, float pi, float ujx, float ujy,
                                             float ujz, float rhoj, float pj, bool clamp_ps, PairAcc &A)
{
    if (KAHAN) {
        // The same terms with every rounding spelled out (no contraction
        // freedom left to the compiler), so that every kernel inlining this
        // rounds identically, and a Kahan-compensated density-rate sum.
        const float w = __fmul_rn(ex2_approx(__fmul_rn(r2, P.exp2_scale)), P.kdiff);
        const float inv_r = rsqrt_approx(fmaxf(r2, 1e-30f));
        const float rs_inv = rcp_approx(__fadd_rn(rhoi, rhoj));
        const float a = fmaf(__fsub_rn(uiz, ujz), dz, fmaf(__fsub_rn(uiy, ujy), dy, __fmul_rn(__fsub_rn(uix, ujx), dx)));
        const float du = fmaxf(__fmul_rn(a, inv_r), 0.0f);
        const float lim = LIMITER ? fminf(__fmul_rn(3.0f, du), P.c0) : P.c0;
        float ps = __fmul_rn(fmaf(rhoi, pj, __fmul_rn(rhoj, pi)), rs_inv);
        ps = fmaf(__fmul_rn(__fmul_rn(__fmul_rn(rhoi, rhoj), rs_inv), du), lim, ps);
        if (clamp_ps) ps = fmaxf(ps, 0.0f);
        const float r = __fmul_rn(r2, inv_r);
        const float x = fmaf(rhoj, a, -__fmul_rn(__fmul_rn(__fsub_rn(pi, pj), r), P.c0_inv));
        const float y = __fsub_rn(__fmul_rn(__fmul_rn(x, rs_inv), w), A.drho_c);
        const float t = __fadd_rn(A.drho, y);
        A.drho_c = __fsub_rn(__fsub_rn(t, A.drho), y);
        A.drho = t;
        float f = __fmul_rn(-2.0f, ps);
        if (VISCID == 1 || (VISCID == 2 && P.viscid))
            f = fmaf(__fmul_rn(P.mu10, -a), rcp_approx(__fadd_rn(r2, P.eps_h2)), f);
        f = __fmul_rn(f, w);
        A.ax = fmaf(f, dx, A.ax);
        A.ay = fmaf(f, dy, A.ay);
        A.az = fmaf(f, dz, A.az);
        return;
    }
    const float w = ex2_approx(r2 * P.exp2_scale) * P.kdiff;
    const float inv_r = rsqrt_approx(fmaxf(r2, 1e-30f)); // r2 = 0 (the particle itself) contributes 0
    const float rs_inv = rcp_approx(rhoi + rhoj);
    const float a = (uix - ujx) * dx + (uiy - ujy) * dy + (uiz - ujz) * dz;
    const float du = fmaxf(a * inv_r, 0.0f); // only du >= 0 adds dissipation
    const float lim = LIMITER ? fminf(3.0f * du, P.c0) : P.c0;
    float ps = (rhoi * pj + rhoj * pi) * rs_inv;
    ps = fmaf(rhoi * rhoj * rs_inv * du, lim, ps);
    if (clamp_ps) ps = fmaxf(ps, 0.0f);
    const float r = r2 * inv_r;
    A.drho = fmaf((rhoj * a - (pi - pj) * r * P.c0_inv) * rs_inv, w, A.drho);
    float f = -2.0f * ps;
    if (VISCID == 1 || (VISCID == 2 && P.viscid)) f = fmaf(P.mu10 * -a, rcp_approx(r2 + P.eps_h2), f);
    f *= w;
    A.ax = fmaf(f, dx, A.ax);
    A.ay = fmaf(f, dy, A.ay);
    A.az = fmaf(f, dz, A.az);
}

// ------------------------------------------------------- fluid sweep
struct FluidSweepArgs {
    const float4 *posr, *velp;   // sorted step-start state
    const int *start_f, *cell_f, *orig_in;
    const float4 *s_pos, *s_vel, *s_np; // solid position, velocity, (normal, pressure)
    const int *start_s;
    const float4 *v_posr, *v_velp;
    const int *start_v;
    float4 *posr_out, *velp_out;
    int *orig_out;
    float *drho_out;
    float4 *dudt_out;
    int n;
    int keep; // write drho/dt and du/dt
    const float2 *cm; // mixed form: per-cell (density deviation, pressure) references
};

// fluidUpdate (src/fluid.cu:234-269) applied to the sums of one particle: NaN
// scrub, Euler step with the old velocity, density clamp, EOS, position clamp,
// speed cap; writes the integrated state into the other buffer.
__device__ __forceinline__ void fluid_update_store(const DevParams &P, const FluidSweepArgs &A, int i, float4 pr,
                                                   float4 vp, const PairAcc &acc)
{
    const float rho_inv = __fdividef(1.0f, pr.w);
    float drho = 2.0f * pr.w * acc.drho;
    float ax = acc.ax * rho_inv, ay = acc.ay * rho_inv, az = acc.az * rho_inv;
    if (!(drho == drho)) drho = 0.0f;
    if (!(ax == ax && ay == ay && az == az)) ax = ay = az = 0.0f;
    float x = pr.x + vp.x * P.dt, y = pr.y + vp.y * P.dt, z = pr.z + vp.z * P.dt;
    float ux = vp.x + (ax + P.gx) * P.dt, uy = vp.y + (ay + P.gy) * P.dt, uz = vp.z + (az + P.gz) * P.dt;
    float rho = pr.w + drho * P.dt;
    rho = fminf(fmaxf(rho, P.min_rho), P.max_rho);
    const float p = tait_pressure(P, rho);
    x = fminf(fmaxf(x, P.dmin[0]), P.dmax[0]);
    y = fminf(fmaxf(y, P.dmin[1]), P.dmax[1]);
    z = fminf(fmaxf(z, P.dmin[2]), P.dmax[2]);
    const float speed = sqrtf(ux * ux + uy * uy + uz * uz);
    if (speed > P.vmax) {
        const float s = P.vmax / speed;
        ux *= s;
        uy *= s;
        uz *= s;
    }
    A.posr_out[i] = make_float4(x, y, z, rho);
    A.velp_out[i] = make_float4(ux, uy, uz, p);
    A.orig_out[i] = A.orig_in[i];
    if (A.keep) {
        A.drho_out[i] = drho;
        A.dudt_out[i] = make_float4(ax, ay, az, 0.0f);
    }
}

// findFluidPair + fluidUpdate (src/fluid.cu:169-269), fused: the sweep reads
// the step-start buffer and writes the integrated state to the other buffer.
//
// Warp-cooperative form.  A warp owns 32 consecutive (cell-sorted) particles,
// one per lane; lanes of the same (x, y) cell row form a group, and the group
// walks the union of its members' neighbour rows — 9 z-contiguous index ranges
// — as ONE warp-uniform candidate stream: every candidate is a broadcast load
// tested by all lanes at once.  Hits go to a per-lane neighbour list in shared
// memory; the list is then evaluated lane-parallel, so the ~40-instruction
// Riemann pair runs with nearly all lanes busy instead of the ~15 % of lanes
// that pass a distance test at any moment.  Candidates in the union but
// outside a lane's own 27 cells are farther than the cell size >= the impact
// distance, so the pair set is exactly the reference's; CHECK_Z re-checks the
// z cell when the grid spacing is too close to the impact distance for that
// argument to survive FP32 rounding.
//
// Launch shape: warps per block, per-lane list capacity (shared memory) and
// candidates between capacity checks.  None of them changes what a lane sums or
// in which order (a warp owns the same 32 particles and walks the same stream
// whatever the block size; flushes evaluate a lane's hits in stream order), so
// results are bit-identical across shapes and the autotuner may pick any.
// Smaller lists leave more of the SM's 256 KB L1 as cache for the gathers.
template <int W, int CAP, int CHUNK>
struct SweepShape {
    static constexpr int warps = W, cap = CAP, chunk = CHUNK;
};
using Shape0 = SweepShape<4, 48, 16>; // 24 KB of lists per 128-thread block
using Shape1 = SweepShape<4, 32, 8>;  // 16 KB per 128-thread block
using Shape2 = SweepShape<8, 32, 8>;  // 32 KB per 256-thread block
constexpr int kSweepShapes = 3;
constexpr int kShapeWarps[kSweepShapes] = {Shape0::warps, Shape1::warps, Shape2::warps};

enum Species { kFluid = 0, kVirt = 1, kSolid = 2 };

template <int SP, int VISCID, bool KAHAN = false>
__device__ __forceinline__ void flush_list(const DevParams &P, const FluidSweepArgs &A, int (*lst)[32], int lane,
                                           int &cnt, float4 pr, float4 vp, PairAcc &acc)
{
    const int m = __reduce_max_sync(kFull, cnt);
    for (int k = 0; k < m; ++k) {
        if (k < cnt) {
            const int j = lst[k][lane];
            if (SP == kSolid) {
                const float4 q = A.s_pos[j], np = A.s_np[j], sv = A.s_vel[j];
                const float dx = q.x - pr.x, dy = q.y - pr.y, dz = q.z - pr.z;
                const float r2 = dist2(dx, dy, dz);
                if (KAHAN) {
                    const float k2 = __fmul_rn(2.0f, fmaf(__fsub_rn(vp.z, sv.z), np.z,
                                                          fmaf(__fsub_rn(vp.y, sv.y), np.y,
                                                               __fmul_rn(__fsub_rn(vp.x, sv.x), np.x))));
                    riemann_pair<false, VISCID, true>(P, dx, dy, dz, r2, vp.x, vp.y, vp.z, pr.w, vp.w,
                                                      fmaf(-k2, np.x, vp.x), fmaf(-k2, np.y, vp.y),
                                                      fmaf(-k2, np.z, vp.z), pr.w, np.w, false, acc);
                } else {
                    const float k2 = 2.0f * ((vp.x - sv.x) * np.x + (vp.y - sv.y) * np.y + (vp.z - sv.z) * np.z);
                    riemann_pair<false, VISCID>(P, dx, dy, dz, r2, vp.x, vp.y, vp.z, pr.w, vp.w, vp.x - k2 * np.x,
                                                vp.y - k2 * np.y, vp.z - k2 * np.z, pr.w, np.w, false, acc);
                }
            } else {
                const float4 q = SP == kFluid ? A.posr[j] : A.v_posr[j];
                const float4 u = SP == kFluid ? A.velp[j] : A.v_velp[j];
                const float dx = q.x - pr.x, dy = q.y - pr.y, dz = q.z - pr.z;
                const float r2 = dist2(dx, dy, dz);
                riemann_pair<true, VISCID, KAHAN>(P, dx, dy, dz, r2, vp.x, vp.y, vp.z, pr.w, vp.w, u.x, u.y, u.z, q.w,
                                                u.w, SP == kVirt, acc);
            }
        }
    }
    cnt = 0;
}

template <int SP, bool CHECK_Z, int VISCID, class SH, bool KAHAN = false>
__device__ __forceinline__ void gather_species(const DevParams &P, const FluidSweepArgs &A, int (*lst)[32], int lane,
                                               int &cnt, bool in, int cz, int cx, int cy, int z0, int z1, float4 pr,
                                               float4 vp, PairAcc &acc)
{
    const int *start = SP == kFluid ? A.start_f : SP == kVirt ? A.start_v : A.start_s;
    const float4 *pos = SP == kFluid ? A.posr : SP == kVirt ? A.v_posr : A.s_pos;
    for (int ox = -1; ox <= 1; ++ox) {
        const int x = cx + ox;
        if (x < 0 || x >= P.nx) continue;
        for (int oy = -1; oy <= 1; ++oy) {
            const int y = cy + oy;
            if (y < 0 || y >= P.ny) continue;
            const int base = (x * P.ny + y) * P.nz;
            int j = start[base + z0];
            const int je = start[base + z1];
            while (j < je) {
                if (__reduce_max_sync(kFull, cnt) > SH::cap - SH::chunk)
                    flush_list<SP, VISCID, KAHAN>(P, A, lst, lane, cnt, pr, vp, acc);
                const int jend = min(j + SH::chunk, je);
#pragma unroll 4
                for (; j < jend; ++j) {
                    const float4 q = pos[j]; // same address in every lane: a broadcast
                    const float r2 = dist2(q.x - pr.x, q.y - pr.y, q.z - pr.z);
                    bool hit = in && r2 < P.R2;
                    if (CHECK_Z && hit) {
                        const int czj = (int)__fmul_rn(__fsub_rn(q.z, P.cmin[2]), P.cinv[2]);
                        hit = abs(czj - cz) <= 1;
                    }
                    if (hit) lst[cnt++][lane] = j;
                }
            }
        }
    }
    flush_list<SP, VISCID, KAHAN>(P, A, lst, lane, cnt, pr, vp, acc);
}

template <bool CHECK_Z, int VISCID, class SH>
__device__ __forceinline__ void fluid_sweep_body(const DevParams &P, const FluidSweepArgs &A, int blk)
{
    __shared__ int lists[SH::warps][SH::cap][32];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int i = (blk * SH::warps + warp) * 32 + lane;
    const bool valid = i < A.n;
    int(*lst)[32] = lists[warp];
    const float4 pr = valid ? A.posr[i] : make_float4(0.0f, 0.0f, 0.0f, 1.0f);
    const float4 vp = valid ? A.velp[i] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const int cell = valid ? A.cell_f[i] : 0;
    const int row = cell / P.nz, cz = cell - row * P.nz;
    PairAcc acc = {0.0f, 0.0f, 0.0f, 0.0f};
    int cnt = 0;
    unsigned remaining = __ballot_sync(kFull, valid);
    while (remaining) {
        const int leader = __ffs(remaining) - 1;
        const int grow = __shfl_sync(kFull, row, leader);
        const unsigned grp = __ballot_sync(kFull, valid && row == grow);
        remaining &= ~grp;
        const bool in = (grp >> lane) & 1u;
        const int zlo = __reduce_min_sync(kFull, in ? cz : INT_MAX);
        const int zhi = __reduce_max_sync(kFull, in ? cz : INT_MIN);
        const int z0 = max(zlo - 1, 0), z1 = min(zhi + 1, P.nz - 1) + 1;
        const int cx = grow / P.ny, cy = grow - cx * P.ny;
        gather_species<kFluid, CHECK_Z, VISCID, SH>(P, A, lst, lane, cnt, in, cz, cx, cy, z0, z1, pr, vp, acc);
        gather_species<kVirt, CHECK_Z, VISCID, SH>(P, A, lst, lane, cnt, in, cz, cx, cy, z0, z1, pr, vp, acc);
        gather_species<kSolid, CHECK_Z, VISCID, SH>(P, A, lst, lane, cnt, in, cz, cx, cy, z0, z1, pr, vp, acc);
    }
    if (valid) fluid_update_store(P, A, i, pr, vp, acc);
}

template <bool CHECK_Z, int VISCID, class SH>
__global__ void __launch_bounds__(SH::warps * 32) kb_fluid_sweep(const Item<FluidSweepArgs> *__restrict__ items,
                                                                 const int *__restrict__ bstart, int ninst)
{
    const int inst = locate_instance(bstart, ninst, blockIdx.x);
    const DevParams P = items[inst].P;
    fluid_sweep_body<CHECK_Z, VISCID, SH>(P, items[inst].A, (int)blockIdx.x - bstart[inst]);
}

// The one-instance sweep takes {params, args} by value: kernel parameters live
// in the constant bank, where its hot loops read them without extra loads.
template <bool CHECK_Z, int VISCID, class SH>
__global__ void __launch_bounds__(SH::warps * 32) kb_fluid_sweep_1(const DevParams P, const FluidSweepArgs A)
{
    fluid_sweep_body<CHECK_Z, VISCID, SH>(P, A, (int)blockIdx.x);
}

// ------------------------------------------------------- virtual particles
// getVirtData (src/virt.cu:9-75): nearest fluid particle's rho, hydrostatically
// corrected p and velocity mirrored about the (static) wall normal.  Ties in
// distance go to the smaller input id.
struct VirtArgs {
    const float4 *v_posr_in, *v_normal;
    const int *v_cell;
    const float4 *fposr, *fvelp;
    const int *forig, *start_f;
    float4 *v_posr, *v_velp;
    int n;
};
__device__ __forceinline__ void virt_body(const DevParams &P, const VirtArgs &A, int blk)
{
    const int i = blk * blockDim.x + threadIdx.x;
    if (i >= A.n) return;
    const float4 xi = A.v_posr_in[i];
    Rows rows;
    neighbor_rows(P, A.v_cell[i], rows);
    float best = FSIM_LARGE_FLOAT;
    int best_j = -1, best_orig = INT_MAX;
    for (int r = 0; r < rows.count; ++r) {
        for (int j = A.start_f[rows.base[r] + rows.z0], je = A.start_f[rows.base[r] + rows.z1]; j < je; ++j) {
            const float4 q = A.fposr[j];
            const float d2 = dist2(q.x - xi.x, q.y - xi.y, q.z - xi.z);
            if (d2 < best) {
                best = d2;
                best_j = j;
                best_orig = A.forig[j];
            } else if (d2 == best) {
                const int o = A.forig[j];
                if (o < best_orig) {
                    best_j = j;
                    best_orig = o;
                }
            }
        }
    }
    float rho = P.rho0, p = 0.0f, ux = 0.0f, uy = 0.0f, uz = 0.0f;
    if (best_j >= 0) {
        const float4 q = A.fposr[best_j], u = A.fvelp[best_j];
        rho = q.w;
        p = u.w - rho * (P.gx * (q.x - xi.x) + P.gy * (q.y - xi.y) + P.gz * (q.z - xi.z));
        ux = u.x;
        uy = u.y;
        uz = u.z;
    }
    const float4 nrm = A.v_normal[i];
    const float k2 = 2.0f * (ux * nrm.x + uy * nrm.y + uz * nrm.z);
    A.v_posr[i] = make_float4(xi.x, xi.y, xi.z, rho);
    A.v_velp[i] = make_float4(ux - k2 * nrm.x, uy - k2 * nrm.y, uz - k2 * nrm.z, p);
}
FSIM_BATCHED_KERNEL(kb_virt, VirtArgs, virt_body, kBlock)

// Wall normal of every virtual particle (src/virt.cu:52-70): minus the kernel
// gradient sum over the other virtual particles, normalised, zero when its
// squared length is below EPS_FOR_SUM.  Walls never move: computed once.
__global__ void k_virt_normal(const DevParams P, const float4 *__restrict__ v_posr, const int *__restrict__ v_cell,
                              const int *__restrict__ start_v, float4 *__restrict__ v_normal, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 xi = v_posr[i];
    Rows rows;
    neighbor_rows(P, v_cell[i], rows);
    float nx = 0.0f, ny = 0.0f, nz = 0.0f;
    for (int r = 0; r < rows.count; ++r) {
        for (int j = start_v[rows.base[r] + rows.z0], je = start_v[rows.base[r] + rows.z1]; j < je; ++j) {
            if (j == i) continue;
            const float4 q = v_posr[j];
            const float dx = q.x - xi.x, dy = q.y - xi.y, dz = q.z - xi.z;
            const float r2 = dist2(dx, dy, dz);
            if (r2 < P.R2) {
                const float w = __expf(-r2 * P.h_inv2) * P.kdiff;
                nx -= dx * w;
                ny -= dy * w;
                nz -= dz * w;
            }
        }
    }
    const float l2 = nx * nx + ny * ny + nz * nz;
    if (l2 < FSIM_EPS_FOR_SUM) {
        nx = ny = nz = 0.0f;
    } else {
        const float s = rsqrtf(l2);
        nx *= s;
        ny *= s;
        nz *= s;
    }
    v_normal[i] = make_float4(nx, ny, nz, 0.0f);
}

// --------------------------------------------------- warp-per-particle sweeps
// The solid-side sweeps have few particles (27 k at the 4M case) and long
// neighbour loops; one warp per particle splits each row's candidates over the
// 32 lanes and combines the lane sums with a butterfly shuffle reduction (a
// fixed pairing, so results are deterministic).
__device__ __forceinline__ float warp_sum(float v)
{
#pragma unroll
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
    return v;
}

// kSolidGroup lanes share one solid particle: they split its candidates and
// combine their sums with shuffles (a fixed pairing: deterministic).
constexpr int kSolidGroup = 4;

__device__ __forceinline__ float group_sum(float v)
{
#pragma unroll
    for (int o = 1; o < kSolidGroup; o <<= 1) v += __shfl_xor_sync(kFull, v, o);
    return v;
}

// ------------------------------------------------------- fluid-solid coupling
// solidCoupleUpdate (src/solid.cu:262-344): solid normal from the solid
// neighbours' kernel gradients, solid pressure as the Shepard average of the
// fluid pressure.  kSolidGroup lanes per solid particle.
struct CoupleArgs {
    const float4 *s_pos;
    const int *s_cell, *start_s;
    const float4 *fposr, *fvelp;
    const int *start_f;
    float4 *s_np;
    int n;
};
__device__ __forceinline__ void couple_body(const DevParams &P, const CoupleArgs &A, int blk)
{
    const int t = blk * blockDim.x + threadIdx.x;
    const int i = t / kSolidGroup, g = t % kSolidGroup;
    const bool valid = i < A.n;
    float nx = 0.0f, ny = 0.0f, nz = 0.0f, psum = 0.0f, wsum = 0.0f;
    if (valid) {
        const float4 xi = A.s_pos[i];
        Rows rows;
        neighbor_rows(P, A.s_cell[i], rows);
        for (int r = 0; r < rows.count; ++r) {
            const int c0 = rows.base[r] + rows.z0, c1 = rows.base[r] + rows.z1;
            for (int j = A.start_f[c0] + g, je = A.start_f[c1]; j < je; j += kSolidGroup) {
                const float4 q = A.fposr[j];
                const float dx = q.x - xi.x, dy = q.y - xi.y, dz = q.z - xi.z;
                const float r2 = dist2(dx, dy, dz);
                if (r2 < P.R2) {
                    const float w = (__expf(-r2 * P.h_inv2) - P.kc1) * P.kc2;
                    wsum += w;
                    psum += A.fvelp[j].w * w;
                }
            }
            for (int j = A.start_s[c0] + g, je = A.start_s[c1]; j < je; j += kSolidGroup) {
                const float4 q = A.s_pos[j];
                const float dx = q.x - xi.x, dy = q.y - xi.y, dz = q.z - xi.z;
                const float r2 = dist2(dx, dy, dz);
                if (r2 < P.R2) {
                    const float w = __expf(-r2 * P.h_inv2) * P.kdiff;
                    nx -= dx * w;
                    ny -= dy * w;
                    nz -= dz * w;
                }
            }
        }
    }
    nx = group_sum(nx);
    ny = group_sum(ny);
    nz = group_sum(nz);
    psum = group_sum(psum);
    wsum = group_sum(wsum);
    if (!valid || g) return;
    const float l2 = nx * nx + ny * ny + nz * nz;
    if (l2 < FSIM_EPS_FOR_SUM) {
        nx = ny = nz = 0.0f;
    } else {
        const float s = rsqrtf(l2);
        nx *= s;
        ny *= s;
        nz *= s;
    }
    const float p = wsum > FSIM_EPS_FLOAT ? fmaxf(psum / wsum, P.min_p) : 0.0f;
    A.s_np[i] = make_float4(nx, ny, nz, p);
}
FSIM_BATCHED_KERNEL(kb_couple, CoupleArgs, couple_body, kBlock)

// =================================================================== mixed form
// Fluid state of the mixed form (same 2 x 16 bytes per particle as the plain
// form, different contents):
//   posr = (offset from the particle's cell corner, x y z FP32;
//           FP16 pair: density deviation and pressure, each relative to the
//           per-cell FP32 reference cm[cell], for neighbour gathers)
//   velp = (u, v, w, delta = rho/rho0 - 1 in FP32: the particle's own density)
// The cell of sorted particle i is cell_f[i] (kept valid for the current
// order at all times), so x = cell_min + cell * interval + offset.  Pair
// distances are differences of offsets plus whole cells, exact to the FP32
// resolution of a cell (~1e-9 m) instead of the domain (~2e-7 m at 2.5 m).
// The pressure is the Tait EOS of delta (expm1/log1p, no cancellation).
// Wall particles store offsets from their own (static) cells the same way;
// the solid keeps absolute FP32 positions.
constexpr int kCodeShift = 26;                   // neighbour-list entry = j | cell code << 26
constexpr int kIndexMask = (1 << kCodeShift) - 1;
constexpr float kDeltaScale = 1024.0f;           // FP16 density-deviation scale
constexpr float kDeltaUnit = 1.0f / 1024.0f;

__device__ __forceinline__ float eos_delta(const DevParams &P, float d)
{
    return fmaxf(__fmul_rn(P.rho2p, expm1f(__fmul_rn(P.gamma, log1pf(d)))), P.min_p);
}
__device__ __forceinline__ void cell_xyz(const DevParams &P, int c, int &cx, int &cy, int &cz)
{
    const int row = c / P.nz;
    cz = c - row * P.nz;
    cx = row / P.ny;
    cy = row - cx * P.ny;
}
__device__ __forceinline__ unsigned half2_bits(float a, float b)
{
    const __half2 h = __floats2half2_rn(a, b);
    unsigned u;
    memcpy(&u, &h, sizeof u);
    return u;
}
__device__ __forceinline__ float2 half2_floats(float bits)
{
    const unsigned u = __float_as_uint(bits);
    __half2 h;
    memcpy(&h, &u, sizeof h);
    return __half22float2(h);
}

// Cell phase, fluid hash of the mixed form: move every particle to the cell
// its offset now lies in (offset -= whole cells) and hash it there.
__device__ __forceinline__ int rebin_axis(float &off, int c, float inv, float d, int n, bool &bad)
{
    int t = c + (int)floorf(off * inv);
    if (t < 0 || t >= n) {
        bad = true;
        t = t < 0 ? 0 : n - 1;
    }
    if (t != c) off -= (float)(t - c) * d;
    return t;
}
struct HashMixedArgs {
    float4 *pos;
    const int *cell_old;
    int n;
    int *key, *slot, *cnt;
    unsigned *flags;
};
__device__ __forceinline__ void hash_mixed_body(const DevParams &P, const HashMixedArgs &A, int blk)
{
    const int s = blk * blockDim.x + threadIdx.x;
    const bool active = s < A.n;
    int c = 0;
    if (active) {
        float4 p = A.pos[s];
        int cx, cy, cz;
        cell_xyz(P, A.cell_old[s], cx, cy, cz);
        bool bad = false;
        cx = rebin_axis(p.x, cx, P.cinv[0], P.cdx[0], P.nx, bad);
        cy = rebin_axis(p.y, cy, P.cinv[1], P.cdx[1], P.ny, bad);
        cz = rebin_axis(p.z, cz, P.cinv[2], P.cdx[2], P.nz, bad);
        if (bad) atomicOr(A.flags, FLAG_OUT_OF_GRID);
        c = (cx * P.ny + cy) * P.nz + cz;
        A.pos[s] = p;
        A.key[s] = c;
    }
    const int slot = cell_slot(A.cnt, c, active);
    if (active) A.slot[s] = slot;
}
FSIM_BATCHED_KERNEL(kb_hash_mixed, HashMixedArgs, hash_mixed_body, kBlock)

// Per-cell references and the FP16 gather pair (after the sort): cm[c] =
// mean (delta, p) of the cell's particles; each particle stores its
// deviations from them as FP16 in posr.w.  Deviations inside a 2h cell are
// small, so FP16 keeps them to ~1e-3 relative, i.e. ~0.01 Pa for hydrostatic
// water at dx = 5 mm, where an absolute FP16 pressure would be ~3 Pa.
struct CellRefArgs {
    float4 *posr;
    const float4 *velp;
    const int *start;
    float2 *cm;
    int ncell;
};
__device__ __forceinline__ void cell_ref_body(const DevParams &P, const CellRefArgs &A, int blk)
{
    const int c = blk * blockDim.x + threadIdx.x;
    if (c >= A.ncell) return;
    const int b = A.start[c], e = A.start[c + 1];
    if (b == e) return; // never read: no particle refers to an empty cell
    float sd = 0.0f, sp = 0.0f;
    for (int j = b; j < e; ++j) {
        const float d = A.velp[j].w;
        sd += d;
        sp += eos_delta(P, d);
    }
    const float inv_n = 1.0f / (float)(e - b);
    const float dm = sd * inv_n, pm = sp * inv_n;
    A.cm[c] = make_float2(dm, pm);
    float *w = reinterpret_cast<float *>(A.posr);
    for (int j = b; j < e; ++j) {
        const float d = A.velp[j].w;
        w[4 * (size_t)j + 3] = __uint_as_float(half2_bits((d - dm) * kDeltaScale, (eos_delta(P, d) - pm) * P.p_unit_inv));
    }
}
FSIM_BATCHED_KERNEL(kb_cell_ref, CellRefArgs, cell_ref_body, kBlock)

// Own particle of the mixed sweep.
struct OwnMixed {
    float bx, by, bz; // offset + one cell: the list's cell code b in {0,1,2} gives offset - (b - 1) cell
    int cbase;        // linear cell of code (0, 0, 0)
    float rho, p;
};

template <int SP, int VISCID>
__device__ __forceinline__ void flush_list_m(const DevParams &P, const FluidSweepArgs &A, int (*lst)[32], int lane,
                                             int &cnt, const OwnMixed &o, float4 vp, PairAcc &acc)
{
    const int m = __reduce_max_sync(kFull, cnt);
    const int nynz = P.ny * P.nz;
    for (int k = 0; k < m; ++k) {
        if (k < cnt) {
            const unsigned e = (unsigned)lst[k][lane];
            const int j = (int)(e & kIndexMask);
            const int bx = (e >> kCodeShift) & 3u, by = (e >> (kCodeShift + 2)) & 3u, bz = e >> (kCodeShift + 4);
            const float4 q = SP == kFluid ? A.posr[j] : A.v_posr[j];
            const float4 u = SP == kFluid ? A.velp[j] : A.v_velp[j];
            const float dx = q.x - fmaf(-(float)bx, P.cdx[0], o.bx);
            const float dy = q.y - fmaf(-(float)by, P.cdx[1], o.by);
            const float dz = q.z - fmaf(-(float)bz, P.cdx[2], o.bz);
            const float r2 = dist2(dx, dy, dz);
            float rhoj, pj;
            if (SP == kFluid) {
                const float2 ref = A.cm[o.cbase + bx * nynz + by * P.nz + bz];
                const float2 dev = half2_floats(q.w);
                rhoj = fmaf(P.rho0, fmaf(dev.x, kDeltaUnit, ref.x), P.rho0);
                pj = fmaf(dev.y, P.p_unit, ref.y);
            } else {
                rhoj = q.w;
                pj = u.w;
            }
            riemann_pair<true, VISCID, true>(P, dx, dy, dz, r2, vp.x, vp.y, vp.z, o.rho, o.p, u.x, u.y, u.z, rhoj,
                                             pj, SP == kVirt, acc);
        }
    }
    cnt = 0;
}

// Candidate stream of the mixed sweep: the union rows, cell by cell, so that
// every candidate's cell (relative to the lane's own) is known; it travels
// with the list entry as a 6-bit code.  Each lane only takes candidates from
// its own 27 cells.
template <int SP, int VISCID, class SH>
__device__ __forceinline__ void gather_species_m(const DevParams &P, const FluidSweepArgs &A, int (*lst)[32], int lane,
                                                 int &cnt, bool in, int cz, int cx, int cy, int z0, int z1,
                                                 float4 off, const OwnMixed &o, float4 vp, PairAcc &acc)
{
    const int *start = SP == kFluid ? A.start_f : A.start_v;
    const float4 *pos = SP == kFluid ? A.posr : A.v_posr;
    for (int ox = -1; ox <= 1; ++ox) {
        const int x = cx + ox;
        if (x < 0 || x >= P.nx) continue;
        const float psx = fmaf(-(float)ox, P.cdx[0], off.x);
        for (int oy = -1; oy <= 1; ++oy) {
            const int y = cy + oy;
            if (y < 0 || y >= P.ny) continue;
            const float psy = fmaf(-(float)oy, P.cdx[1], off.y);
            const int rb = (x * P.ny + y) * P.nz;
            const unsigned code_xy = (unsigned)(ox + 1) | ((unsigned)(oy + 1) << 2);
            int j = start[rb + z0];
            for (int z = z0; z < z1; ++z) {
                const int je = start[rb + z + 1];
                const int dzc = z - cz;
                const bool inz = in && dzc >= -1 && dzc <= 1;
                const float psz = fmaf(-(float)dzc, P.cdx[2], off.z);
                const unsigned code = (code_xy | ((unsigned)(dzc + 1) << 4)) << kCodeShift;
                while (j < je) {
                    if (__reduce_max_sync(kFull, cnt) > SH::cap - SH::chunk)
                        flush_list_m<SP, VISCID>(P, A, lst, lane, cnt, o, vp, acc);
                    const int jend = min(j + SH::chunk, je);
#pragma unroll 4
                    for (; j < jend; ++j) {
                        const float4 q = pos[j]; // a broadcast
                        const float r2 = dist2(q.x - psx, q.y - psy, q.z - psz);
                        if (inz && r2 < P.R2) lst[cnt++][lane] = (int)(code | (unsigned)j);
                    }
                }
            }
        }
    }
    flush_list_m<SP, VISCID>(P, A, lst, lane, cnt, o, vp, acc);
}

// fluidUpdate (src/fluid.cu:234-269) in the mixed form: delta and offsets.
__device__ __forceinline__ void fluid_update_store_m(const DevParams &P, const FluidSweepArgs &A, int i, float4 off,
                                                     float4 vp, float rho, const PairAcc &acc, int cx, int cy, int cz)
{
    // explicit roundings throughout (see riemann_pair's KAHAN branch)
    const float rho_inv = __fdividef(1.0f, rho);
    float drho = __fmul_rn(__fmul_rn(2.0f, rho), acc.drho);
    float ax = __fmul_rn(acc.ax, rho_inv), ay = __fmul_rn(acc.ay, rho_inv), az = __fmul_rn(acc.az, rho_inv);
    if (!(drho == drho)) drho = 0.0f;
    if (!(ax == ax && ay == ay && az == az)) ax = ay = az = 0.0f;
    float x = fmaf(vp.x, P.dt, off.x), y = fmaf(vp.y, P.dt, off.y), z = fmaf(vp.z, P.dt, off.z);
    float ux = fmaf(__fadd_rn(ax, P.gx), P.dt, vp.x), uy = fmaf(__fadd_rn(ay, P.gy), P.dt, vp.y),
          uz = fmaf(__fadd_rn(az, P.gz), P.dt, vp.z);
    float d = fmaf(__fmul_rn(drho, P.rho0_inv), P.dt, vp.w);
    d = fminf(fmaxf(d, P.dlt_min), P.dlt_max);
    x = fminf(fmaxf(x, fmaf(-(float)cx, P.cdx[0], P.dlo_rel[0])), fmaf(-(float)cx, P.cdx[0], P.dhi_rel[0]));
    y = fminf(fmaxf(y, fmaf(-(float)cy, P.cdx[1], P.dlo_rel[1])), fmaf(-(float)cy, P.cdx[1], P.dhi_rel[1]));
    z = fminf(fmaxf(z, fmaf(-(float)cz, P.cdx[2], P.dlo_rel[2])), fmaf(-(float)cz, P.cdx[2], P.dhi_rel[2]));
    const float speed = __fsqrt_rn(fmaf(uz, uz, fmaf(uy, uy, __fmul_rn(ux, ux))));
    if (speed > P.vmax) {
        const float s = __fdiv_rn(P.vmax, speed);
        ux = __fmul_rn(ux, s);
        uy = __fmul_rn(uy, s);
        uz = __fmul_rn(uz, s);
    }
    A.posr_out[i] = make_float4(x, y, z, 0.0f);
    A.velp_out[i] = make_float4(ux, uy, uz, d);
    A.orig_out[i] = A.orig_in[i];
    if (A.keep) {
        A.drho_out[i] = drho;
        A.dudt_out[i] = make_float4(ax, ay, az, 0.0f);
    }
}

template <int VISCID, class SH>
__device__ __forceinline__ void fluid_sweep_mixed_body(const DevParams &P, const FluidSweepArgs &A, int blk)
{
    __shared__ int lists[SH::warps][SH::cap][32];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int i = (blk * SH::warps + warp) * 32 + lane;
    const bool valid = i < A.n;
    int(*lst)[32] = lists[warp];
    const float4 off = valid ? A.posr[i] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const float4 vp = valid ? A.velp[i] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const int cell = valid ? A.cell_f[i] : 0;
    int cx, cy, cz;
    cell_xyz(P, cell, cx, cy, cz);
    const int row = cell / P.nz;
    OwnMixed o;
    o.bx = __fadd_rn(off.x, P.cdx[0]);
    o.by = __fadd_rn(off.y, P.cdx[1]);
    o.bz = __fadd_rn(off.z, P.cdx[2]);
    o.cbase = cell - P.ny * P.nz - P.nz - 1;
    o.rho = fmaf(P.rho0, vp.w, P.rho0);
    o.p = eos_delta(P, vp.w);
    // absolute position and (rho, p) for the solid pairs, in the plain layout
    const float4 pa = make_float4(__fadd_rn(fmaf((float)cx, P.cdx[0], P.cmin[0]), off.x),
                                  __fadd_rn(fmaf((float)cy, P.cdx[1], P.cmin[1]), off.y),
                                  __fadd_rn(fmaf((float)cz, P.cdx[2], P.cmin[2]), off.z), o.rho);
    const float4 va = make_float4(vp.x, vp.y, vp.z, o.p);
    PairAcc acc = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    int cnt = 0;
    unsigned remaining = __ballot_sync(kFull, valid);
    while (remaining) {
        const int leader = __ffs(remaining) - 1;
        const int grow = __shfl_sync(kFull, row, leader);
        const unsigned grp = __ballot_sync(kFull, valid && row == grow);
        remaining &= ~grp;
        const bool in = (grp >> lane) & 1u;
        const int zlo = __reduce_min_sync(kFull, in ? cz : INT_MAX);
        const int zhi = __reduce_max_sync(kFull, in ? cz : INT_MIN);
        const int z0 = max(zlo - 1, 0), z1 = min(zhi + 1, P.nz - 1) + 1;
        const int gx = grow / P.ny, gy = grow - gx * P.ny;
        gather_species_m<kFluid, VISCID, SH>(P, A, lst, lane, cnt, in, cz, gx, gy, z0, z1, off, o, vp, acc);
        gather_species_m<kVirt, VISCID, SH>(P, A, lst, lane, cnt, in, cz, gx, gy, z0, z1, off, o, vp, acc);
        gather_species<kSolid, false, VISCID, SH, true>(P, A, lst, lane, cnt, in, cz, gx, gy, z0, z1, pa, va, acc);
    }
    if (valid) fluid_update_store_m(P, A, i, off, vp, o.rho, acc, cx, cy, cz);
}

template <int VISCID, class SH>
__global__ void __launch_bounds__(SH::warps * 32) kb_fluid_sweep_m(const Item<FluidSweepArgs> *__restrict__ items,
                                                                   const int *__restrict__ bstart, int ninst)
{
    const int inst = locate_instance(bstart, ninst, blockIdx.x);
    const DevParams P = items[inst].P;
    fluid_sweep_mixed_body<VISCID, SH>(P, items[inst].A, (int)blockIdx.x - bstart[inst]);
}
template <int VISCID, class SH>
__global__ void __launch_bounds__(SH::warps * 32) kb_fluid_sweep_m1(const DevParams P, const FluidSweepArgs A)
{
    fluid_sweep_mixed_body<VISCID, SH>(P, A, (int)blockIdx.x);
}

// getVirtData (src/virt.cu:9-75) in the mixed form.
__device__ __forceinline__ void virt_mixed_body(const DevParams &P, const VirtArgs &A, int blk)
{
    const int i = blk * blockDim.x + threadIdx.x;
    if (i >= A.n) return;
    const float4 xi = A.v_posr_in[i]; // offset from the wall particle's cell
    int cx, cy, cz;
    cell_xyz(P, A.v_cell[i], cx, cy, cz);
    float best = FSIM_LARGE_FLOAT;
    int best_j = -1, best_orig = INT_MAX;
    float bsx = 0.0f, bsy = 0.0f, bsz = 0.0f;
    const int z0 = max(cz - 1, 0), z1 = min(cz + 1, P.nz - 1) + 1;
    for (int ox = -1; ox <= 1; ++ox) {
        const int x = cx + ox;
        if (x < 0 || x >= P.nx) continue;
        const float psx = fmaf(-(float)ox, P.cdx[0], xi.x);
        for (int oy = -1; oy <= 1; ++oy) {
            const int y = cy + oy;
            if (y < 0 || y >= P.ny) continue;
            const float psy = fmaf(-(float)oy, P.cdx[1], xi.y);
            const int rb = (x * P.ny + y) * P.nz;
            for (int z = z0; z < z1; ++z) {
                const float psz = fmaf(-(float)(z - cz), P.cdx[2], xi.z);
                for (int j = A.start_f[rb + z], je = A.start_f[rb + z + 1]; j < je; ++j) {
                    const float4 q = A.fposr[j];
                    const float d2 = dist2(q.x - psx, q.y - psy, q.z - psz);
                    bool take = d2 < best;
                    if (!take && d2 == best) take = A.forig[j] < best_orig;
                    if (take) {
                        best = d2;
                        best_j = j;
                        best_orig = A.forig[j];
                        bsx = psx;
                        bsy = psy;
                        bsz = psz;
                    }
                }
            }
        }
    }
    float rho = P.rho0, p = 0.0f, ux = 0.0f, uy = 0.0f, uz = 0.0f;
    if (best_j >= 0) {
        const float4 q = A.fposr[best_j], u = A.fvelp[best_j];
        rho = fmaf(P.rho0, u.w, P.rho0);
        p = eos_delta(P, u.w) - rho * (P.gx * (q.x - bsx) + P.gy * (q.y - bsy) + P.gz * (q.z - bsz));
        ux = u.x;
        uy = u.y;
        uz = u.z;
    }
    const float4 nrm = A.v_normal[i];
    const float k2 = 2.0f * (ux * nrm.x + uy * nrm.y + uz * nrm.z);
    A.v_posr[i] = make_float4(xi.x, xi.y, xi.z, rho);
    A.v_velp[i] = make_float4(ux - k2 * nrm.x, uy - k2 * nrm.y, uz - k2 * nrm.z, p);
}
FSIM_BATCHED_KERNEL(kb_virt_mixed, VirtArgs, virt_mixed_body, kBlock)

// A fluid candidate of a warp-per-solid-particle row walk in the mixed form:
// its z cell from the row's cell boundaries, its position relative to the
// solid particle from the offset.
struct RowMixed {
    int b1, b2, z0;  // start of the row's 2nd and 3rd cell, first cell
    float sx, sy;    // solid offset minus the row's x/y cell shift
};
__device__ __forceinline__ void fluid_rel(const DevParams &P, const RowMixed &R, int j, float sz0, float4 q, float &dx,
                                          float &dy, float &dz)
{
    const int k = (j >= R.b1) + (j >= R.b2);
    dx = q.x - R.sx;
    dy = q.y - R.sy;
    dz = q.z - fmaf(-(float)k, P.cdx[2], sz0);
}


// The mixed-form row walk of a solid particle: calls f(j, q, dx, dy, dz) for
// every fluid candidate of the 27 cells of solid cell `cell`, lanes of a group
// of `G` taking every G-th candidate of a row.
template <int G, class F>
__device__ __forceinline__ void solid_fluid_walk_m(const DevParams &P, const int *__restrict__ start_f,
                                                   const float4 *__restrict__ fposr, int cell, float4 xi, int g, F &&f)
{
    int cx, cy, cz;
    cell_xyz(P, cell, cx, cy, cz);
    const float sox = xi.x - fmaf((float)cx, P.cdx[0], P.cmin[0]);
    const float soy = xi.y - fmaf((float)cy, P.cdx[1], P.cmin[1]);
    const float soz = xi.z - fmaf((float)cz, P.cdx[2], P.cmin[2]);
    const int z0 = max(cz - 1, 0), z1 = min(cz + 1, P.nz - 1) + 1;
    const float sz0 = fmaf(-(float)(z0 - cz), P.cdx[2], soz);
    for (int ox = -1; ox <= 1; ++ox) {
        const int x = cx + ox;
        if (x < 0 || x >= P.nx) continue;
        for (int oy = -1; oy <= 1; ++oy) {
            const int y = cy + oy;
            if (y < 0 || y >= P.ny) continue;
            const int rb = (x * P.ny + y) * P.nz;
            RowMixed R;
            R.z0 = z0;
            R.b1 = start_f[rb + min(z0 + 1, z1)];
            R.b2 = start_f[rb + min(z0 + 2, z1)];
            R.sx = fmaf(-(float)ox, P.cdx[0], sox);
            R.sy = fmaf(-(float)oy, P.cdx[1], soy);
            for (int j = start_f[rb + z0] + g, je = start_f[rb + z1]; j < je; j += G) {
                const float4 q = fposr[j];
                float dx, dy, dz;
                fluid_rel(P, R, j, sz0, q, dx, dy, dz);
                f(j, dx, dy, dz);
            }
        }
    }
}

// solidCoupleUpdate (src/solid.cu:262-344) in the mixed form.
__device__ __forceinline__ void couple_mixed_body(const DevParams &P, const CoupleArgs &A, int blk)
{
    const int t = blk * blockDim.x + threadIdx.x;
    const int i = t / kSolidGroup, g = t % kSolidGroup;
    const bool valid = i < A.n;
    float nx = 0.0f, ny = 0.0f, nz = 0.0f, psum = 0.0f, wsum = 0.0f;
    if (valid) {
        const float4 xi = A.s_pos[i];
        solid_fluid_walk_m<kSolidGroup>(P, A.start_f, A.fposr, A.s_cell[i], xi, g,
                                        [&](int j, float dx, float dy, float dz) {
                                            const float r2 = dist2(dx, dy, dz);
                                            if (r2 < P.R2) {
                                                const float w = (__expf(-r2 * P.h_inv2) - P.kc1) * P.kc2;
                                                wsum += w;
                                                psum += eos_delta(P, A.fvelp[j].w) * w;
                                            }
                                        });
        Rows rows;
        neighbor_rows(P, A.s_cell[i], rows);
        for (int r = 0; r < rows.count; ++r) {
            const int c0 = rows.base[r] + rows.z0, c1 = rows.base[r] + rows.z1;
            for (int j = A.start_s[c0] + g, je = A.start_s[c1]; j < je; j += kSolidGroup) {
                const float4 q = A.s_pos[j];
                const float dx = q.x - xi.x, dy = q.y - xi.y, dz = q.z - xi.z;
                const float r2 = dist2(dx, dy, dz);
                if (r2 < P.R2) {
                    const float w = __expf(-r2 * P.h_inv2) * P.kdiff;
                    nx -= dx * w;
                    ny -= dy * w;
                    nz -= dz * w;
                }
            }
        }
    }
    nx = group_sum(nx);
    ny = group_sum(ny);
    nz = group_sum(nz);
    psum = group_sum(psum);
    wsum = group_sum(wsum);
    if (!valid || g) return;
    const float l2 = nx * nx + ny * ny + nz * nz;
    if (l2 < FSIM_EPS_FOR_SUM) {
        nx = ny = nz = 0.0f;
    } else {
        const float s = rsqrtf(l2);
        nx *= s;
        ny *= s;
        nz *= s;
    }
    const float p = wsum > FSIM_EPS_FLOAT ? fmaxf(psum / wsum, P.min_p) : 0.0f;
    A.s_np[i] = make_float4(nx, ny, nz, p);
}
FSIM_BATCHED_KERNEL(kb_couple_mixed, CoupleArgs, couple_mixed_body, kBlock)


// ------------------------------------------------------------ solid
struct SolidArgs {
    float4 *pos, *vel;
    const float4 *ref;
    const int *type, *cell, *start_s;
    const float4 *np;
    float *F, *Pk, *L, *PL, *AV; // 9 floats per particle, row-major
    float4 *dudt, *couple;
    const float4 *fposr, *fvelp;
    const int *start_f;
    int n;
    // static reference-configuration neighbours (CSR over input ids)
    const int *orig, *inv, *nbr_off, *nbr_orig;
    const float4 *nbr_dXw; // (X_j - X_i, kernel weight)
    const unsigned *cxyz;
    int nsub;              // this instance's solid sub-steps per step
    unsigned *flags;       // this instance's error flags
};

struct M3 {
    float m[9];
};
__device__ __forceinline__ M3 mmul(const M3 &a, const M3 &b)
{
    M3 r;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
            r.m[3 * i + j] = a.m[3 * i] * b.m[j] + a.m[3 * i + 1] * b.m[3 + j] + a.m[3 * i + 2] * b.m[6 + j];
    return r;
}
__device__ __forceinline__ M3 cofactor(const M3 &a)
{
    M3 c;
    c.m[0] = a.m[4] * a.m[8] - a.m[5] * a.m[7];
    c.m[1] = a.m[5] * a.m[6] - a.m[3] * a.m[8];
    c.m[2] = a.m[3] * a.m[7] - a.m[4] * a.m[6];
    c.m[3] = a.m[2] * a.m[7] - a.m[1] * a.m[8];
    c.m[4] = a.m[0] * a.m[8] - a.m[2] * a.m[6];
    c.m[5] = a.m[1] * a.m[6] - a.m[0] * a.m[7];
    c.m[6] = a.m[1] * a.m[5] - a.m[2] * a.m[4];
    c.m[7] = a.m[2] * a.m[3] - a.m[0] * a.m[5];
    c.m[8] = a.m[0] * a.m[4] - a.m[1] * a.m[3];
    return c;
}

// Solid sub-step sweeps over the static reference-configuration neighbour
// lists: the reference takes the solid candidates from the 27 cells of the
// current cells and keeps those with |X_j - X_i| < 2h (src/solid.cu:53-69,
// 195-203).  The list holds every j with |X_j - X_i| < 2h (built once); a
// sub-step keeps the entries whose current cell is adjacent to i's, which is
// exactly that set.  kSolidGroup lanes share one particle and combine their
// sums with shuffles (a fixed pairing: deterministic).

// solidDeformationCalculate (src/solid.cu:10-79): F and L over the
// reference-configuration neighbours, L^-1 (identity when singular),
// F <- F L^-1, Green strain, St-Venant-Kirchhoff 2nd Piola, P = F S.
// Also stores P L^-1 and cof(F) L^-1 (= det(F) F^-T L^-1) for the force sweep.
// MIXED: L^-1 is formed in FP64 (cofactors, determinant, division) and rounded.
template <bool MIXED>
__device__ __forceinline__ void solid_deform_body(const DevParams &P, const SolidArgs &S, int blk)
{
    const int t = blk * blockDim.x + threadIdx.x;
    const int i = t / kSolidGroup, g = t % kSolidGroup;
    const bool valid = i < S.n;
    M3 F, L;
#pragma unroll
    for (int k = 0; k < 9; ++k) F.m[k] = L.m[k] = 0.0f;
    if (valid) {
        const float4 xi = S.pos[i];
        const unsigned ci = S.cxyz[i];
        const int o = S.orig[i];
        for (int e = S.nbr_off[o] + g, ee = S.nbr_off[o + 1]; e < ee; e += kSolidGroup) {
            const int j = S.inv[S.nbr_orig[e]];
            if (!cells_adjacent(ci, S.cxyz[j])) continue;
            const float4 dXw = S.nbr_dXw[e];
            const float4 xj = S.pos[j];
            const float dx[3] = {xj.x - xi.x, xj.y - xi.y, xj.z - xi.z};
            const float dX[3] = {dXw.x, dXw.y, dXw.z};
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                const float ra = dx[a] * dXw.w, la = dX[a] * dXw.w;
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    F.m[3 * a + c] += ra * dX[c];
                    L.m[3 * a + c] += la * dX[c];
                }
            }
        }
    }
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        F.m[k] = group_sum(F.m[k]);
        L.m[k] = group_sum(L.m[k]);
    }
    if (!valid || g) return;
    M3 Linv;
    if (MIXED) {
        double l[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) l[k] = (double)L.m[k];
        const double c0 = l[4] * l[8] - l[5] * l[7], c1 = l[5] * l[6] - l[3] * l[8], c2 = l[3] * l[7] - l[4] * l[6];
        const double det = l[0] * c0 + l[1] * c1 + l[2] * c2;
        if (det != 0.0) {
            const double id = 1.0 / det;
            const double inv[9] = {c0 * id, (l[2] * l[7] - l[1] * l[8]) * id, (l[1] * l[5] - l[2] * l[4]) * id,
                                   c1 * id, (l[0] * l[8] - l[2] * l[6]) * id, (l[2] * l[3] - l[0] * l[5]) * id,
                                   c2 * id, (l[1] * l[6] - l[0] * l[7]) * id, (l[0] * l[4] - l[1] * l[3]) * id};
#pragma unroll
            for (int k = 0; k < 9; ++k) Linv.m[k] = (float)inv[k];
        } else {
#pragma unroll
            for (int k = 0; k < 9; ++k) Linv.m[k] = (k % 4 == 0) ? 1.0f : 0.0f;
        }
    } else {
    const M3 cl = cofactor(L);
    const float det = L.m[0] * cl.m[0] + L.m[1] * cl.m[1] + L.m[2] * cl.m[2];
    if (det != 0.0f) {
        const float id = 1.0f / det;
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int c = 0; c < 3; ++c) Linv.m[3 * a + c] = cl.m[3 * c + a] * id;
    } else {
#pragma unroll
        for (int k = 0; k < 9; ++k) Linv.m[k] = (k % 4 == 0) ? 1.0f : 0.0f;
    }
    }
    F = mmul(F, Linv);
    // E = (F^T F - I)/2, S = 2 mu E + lambda tr(E) I, P = F S
    M3 E;
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int c = 0; c < 3; ++c)
            E.m[3 * a + c] =
                0.5f * (F.m[a] * F.m[c] + F.m[3 + a] * F.m[3 + c] + F.m[6 + a] * F.m[6 + c] - (a == c ? 1.0f : 0.0f));
    const float tr = E.m[0] + E.m[4] + E.m[8];
    M3 Sm;
#pragma unroll
    for (int k = 0; k < 9; ++k) Sm.m[k] = 2.0f * P.mu_s * E.m[k] + ((k % 4 == 0) ? P.lambda * tr : 0.0f);
    const M3 Pk = mmul(F, Sm);
    const M3 PL = mmul(Pk, Linv);
    const M3 AV = mmul(cofactor(F), Linv);
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        S.F[9 * i + k] = F.m[k];
        S.Pk[9 * i + k] = Pk.m[k];
        S.L[9 * i + k] = Linv.m[k];
        S.PL[9 * i + k] = PL.m[k];
        S.AV[9 * i + k] = AV.m[k];
    }
}
FSIM_BATCHED_KERNEL(kb_solid_deform, SolidArgs, solid_deform_body<false>, kBlock)
FSIM_BATCHED_KERNEL(kb_solid_deform_mixed, SolidArgs, solid_deform_body<true>, kBlock)

// solidForceCalculate (src/solid.cu:81-207): fluid traction over the fluid
// neighbours (current configuration, fluid already advanced; candidates from
// the 27 cells of the step-start cell) plus stress divergence and artificial
// viscosity over the reference-configuration solid neighbours.
// MIXED: fluid positions are cell offsets, fluid (rho, p) come from delta.
template <bool MIXED>
__device__ __forceinline__ void solid_force_body(const DevParams &P, const SolidArgs &S, int blk)
{
    const int t = blk * blockDim.x + threadIdx.x;
    const int i = t / kSolidGroup, g = t % kSolidGroup;
    const bool valid = i < S.n;
    float cx = 0.0f, cy = 0.0f, cz = 0.0f, ax = 0.0f, ay = 0.0f, az = 0.0f;
    if (valid) {
        const float4 xi = S.pos[i], vi = S.vel[i], ni = S.np[i];
        // solidFluidCouple (src/solid.cu:81-117)
        auto traction = [&](float dx, float dy, float dz, float r2, float4 u, float rhoj, float pj) {
            const float w = __expf(-r2 * P.h_inv2) * P.kdiff;
            const float k2 = 2.0f * ((u.x - vi.x) * ni.x + (u.y - vi.y) * ni.y + (u.z - vi.z) * ni.z);
            const float inv_r = r2 > 0.0f ? rsqrtf(r2) : 0.0f;
            const float du = -k2 * (ni.x * dx + ni.y * dy + ni.z * dz) * inv_r;
            float ps = 0.5f * (ni.w + pj);
            if (du >= 0.0f) ps += 0.5f * rhoj * du * P.c0;
            const float f = -2.0f * ps * P.rho_s_inv * w;
            cx += f * dx;
            cy += f * dy;
            cz += f * dz;
        };
        if (MIXED) {
            solid_fluid_walk_m<kSolidGroup>(P, S.start_f, S.fposr, S.cell[i], xi, g,
                                            [&](int j, float dx, float dy, float dz) {
                                                const float r2 = dist2(dx, dy, dz);
                                                if (r2 < P.R2) {
                                                    const float4 u = S.fvelp[j];
                                                    traction(dx, dy, dz, r2, u, fmaf(P.rho0, u.w, P.rho0),
                                                             eos_delta(P, u.w));
                                                }
                                            });
        }
        Rows rows;
        neighbor_rows(P, S.cell[i], rows);
        if (MIXED) rows.count = 0;
        for (int r = 0; r < rows.count; ++r) {
            const int c0 = rows.base[r] + rows.z0, c1 = rows.base[r] + rows.z1;
            for (int j = S.start_f[c0] + g, je = S.start_f[c1]; j < je; j += kSolidGroup) {
                const float4 q = S.fposr[j];
                const float dx = q.x - xi.x, dy = q.y - xi.y, dz = q.z - xi.z;
                const float r2 = dist2(dx, dy, dz);
                if (r2 < P.R2) {
                    const float4 u = S.fvelp[j];
                    const float w = __expf(-r2 * P.h_inv2) * P.kdiff;
                    const float k2 = 2.0f * ((u.x - vi.x) * ni.x + (u.y - vi.y) * ni.y + (u.z - vi.z) * ni.z);
                    // u_i - u_j = -k2 n ; du = (u_i - u_j).e
                    const float inv_r = r2 > 0.0f ? rsqrtf(r2) : 0.0f;
                    const float du = -k2 * (ni.x * dx + ni.y * dy + ni.z * dz) * inv_r;
                    float ps = 0.5f * (ni.w + u.w);
                    if (du >= 0.0f) ps += 0.5f * q.w * du * P.c0;
                    const float f = -2.0f * ps * P.rho_s_inv * w;
                    cx += f * dx;
                    cy += f * dy;
                    cz += f * dz;
                }
            }
        }
        // solidSolidForce (src/solid.cu:119-157)
        float PLi[9], AVi[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) {
            PLi[k] = S.PL[9 * i + k];
            AVi[k] = S.AV[9 * i + k];
        }
        const unsigned ci = S.cxyz[i];
        const int o = S.orig[i];
        for (int e = S.nbr_off[o] + g, ee = S.nbr_off[o + 1]; e < ee; e += kSolidGroup) {
            const int j = S.inv[S.nbr_orig[e]];
            if (!cells_adjacent(ci, S.cxyz[j])) continue;
            const float4 dXw = S.nbr_dXw[e];
            const float dX = dXw.x, dY = dXw.y, dZ = dXw.z, w = dXw.w;
            const float *PLj = S.PL + 9 * j;
            const float ws = w * P.rho_s_inv;
            ax += ((PLj[0] + PLi[0]) * dX + (PLj[1] + PLi[1]) * dY + (PLj[2] + PLi[2]) * dZ) * ws;
            ay += ((PLj[3] + PLi[3]) * dX + (PLj[4] + PLi[4]) * dY + (PLj[5] + PLi[5]) * dZ) * ws;
            az += ((PLj[6] + PLi[6]) * dX + (PLj[7] + PLi[7]) * dY + (PLj[8] + PLi[8]) * dZ) * ws;
            const float4 xj = S.pos[j], vj = S.vel[j];
            const float ddx = xj.x - xi.x, ddy = xj.y - xi.y, ddz = xj.z - xi.z;
            const float dvdx = (vj.x - vi.x) * ddx + (vj.y - vi.y) * ddy + (vj.z - vi.z) * ddz;
            const float nu = P.h * dvdx / (ddx * ddx + ddy * ddy + ddz * ddz + P.eps_h2);
            const float visc = (P.alpha * nu * P.cs_s - P.beta * nu * nu) * w;
            ax += (AVi[0] * dX + AVi[1] * dY + AVi[2] * dZ) * visc;
            ay += (AVi[3] * dX + AVi[4] * dY + AVi[5] * dZ) * visc;
            az += (AVi[6] * dX + AVi[7] * dY + AVi[8] * dZ) * visc;
        }
    }
    cx = group_sum(cx);
    cy = group_sum(cy);
    cz = group_sum(cz);
    ax = group_sum(ax);
    ay = group_sum(ay);
    az = group_sum(az);
    if (!valid || g) return;
    S.couple[i] = make_float4(cx, cy, cz, 0.0f);
    S.dudt[i] = make_float4(ax + cx, ay + cy, az + cz, 0.0f);
}
FSIM_BATCHED_KERNEL(kb_solid_force, SolidArgs, solid_force_body<false>, kBlock)
FSIM_BATCHED_KERNEL(kb_solid_force_mixed, SolidArgs, solid_force_body<true>, kBlock)

// Kernel weight of every static solid neighbour pair (once, at creation).
__global__ void k_solid_pair_weights(const DevParams P, float4 *__restrict__ dXw, int n)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    float4 v = dXw[e];
    const float r2 = dist2(v.x, v.y, v.z);
    v.w = __expf(-r2 * P.h_inv2) * P.kdiff;
    dXw[e] = v;
}

// solidUpdate (src/solid.cu:209-239)
__device__ __forceinline__ void solid_update_body(const DevParams &P, const SolidArgs &S, int blk)
{
    const int i = blk * blockDim.x + threadIdx.x;
    if (i >= S.n) return;
    const int t = S.type[i];
    if (t == 1) { // FIXED_SOLID
        float4 v = S.vel[i];
        S.vel[i] = make_float4(0.0f, 0.0f, 0.0f, v.w);
        S.dudt[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    } else if (t == 0) { // UNCONSTRAINED_SOLID
        const float4 x = S.pos[i], v = S.vel[i], a = S.dudt[i];
        float nx = x.x + v.x * P.dt_sub, ny = x.y + v.y * P.dt_sub, nz = x.z + v.z * P.dt_sub;
        S.vel[i] = make_float4(v.x + (a.x + P.gx) * P.dt_sub, v.y + (a.y + P.gy) * P.dt_sub,
                               v.z + (a.z + P.gz) * P.dt_sub, v.w);
        nx = fminf(fmaxf(nx, P.dmin[0]), P.dmax[0]);
        ny = fminf(fmaxf(ny, P.dmin[1]), P.dmax[1]);
        nz = fminf(fmaxf(nz, P.dmin[2]), P.dmax[2]);
        S.pos[i] = make_float4(nx, ny, nz, x.w);
    }
}
FSIM_BATCHED_KERNEL(kb_solid_update, SolidArgs, solid_update_body, kBlock)




// ------------------------------------------------------- case generator
// The lattice case of fsim_case_generate (fsim_host.cpp), generated on the
// device with the same particles in the same order, bit for bit.  Sites are
// visited there in (i, j, k) order, k fastest; along one (i, j) row the site
// types are intervals in k, so a site's index among the particles of its
// type, and its index among the sites that draw jitter (3 splitmix64 draws
// each, a counter-based stream), follow from per-row bases (prefix sums over
// rows, on the host) plus a closed-form count inside the row.
struct CaseGeom {
    int T[3], FN[3], SL[3], SN[3];
    int fixed_layers, L;
    int has_solid, jitter;
    double dx, jit;
    uint64_t seed;
};
struct RowIv {
    int s0, s1;   // solid sites [s0, s1)
    int f0, f1;   // fluid block sites [f0, f1) (before removing solid)
    int inside;   // the row lies inside the tank in i and j
    int fixed;    // solid sites of this row are FIXED (below the floor)
};
__host__ __device__ inline void case_row(const CaseGeom &g, int i, int j, RowIv &r)
{
    r.inside = !(i < 0 || i >= g.T[0] || j < 0 || j >= g.T[1]);
    r.fixed = j < 0;
    const bool solid_ij = g.has_solid && i >= g.SL[0] && i < g.SL[0] + g.SN[0] && j >= g.SL[1] - g.fixed_layers &&
                          j < g.SL[1] + g.SN[1];
    r.s0 = r.s1 = 0;
    if (solid_ij) {
        int lo = g.SL[2], hi = g.SL[2] + g.SN[2];
        if (j >= 0) { // above the floor a solid site must be inside the tank
            if (!r.inside) hi = lo;
            lo = lo > 0 ? lo : 0;
            hi = hi < g.T[2] ? hi : g.T[2];
        }
        lo = lo > -g.L ? lo : -g.L;
        hi = hi < g.T[2] + g.L ? hi : g.T[2] + g.L;
        if (hi > lo) {
            r.s0 = lo;
            r.s1 = hi;
        }
    }
    r.f0 = r.f1 = 0;
    if (r.inside && i < g.FN[0] && j < g.FN[1]) {
        r.f0 = 0;
        r.f1 = g.FN[2] < g.T[2] ? g.FN[2] : g.T[2];
        if (r.f1 < 0) r.f1 = 0;
    }
}
__host__ __device__ inline int iv_before(int a, int b, int k) // |[a, b) n (-inf, k)|
{
    const int e = b < k ? b : k;
    return e > a ? e - a : 0;
}
__host__ __device__ inline int iv_overlap_before(int a, int b, int c, int d, int k)
{
    return iv_before(a > c ? a : c, b < d ? b : d, k);
}
// per-row particle counts: fluid, solid, virtual, jitter-drawing sites
__host__ __device__ inline void case_row_counts(const CaseGeom &g, const RowIv &r, int c[4])
{
    const int kend = g.T[2] + g.L;
    const int ns = r.s1 - r.s0;
    const int nf = (r.f1 - r.f0) - iv_overlap_before(r.f0, r.f1, r.s0, r.s1, kend);
    const int nv = r.inside ? 2 * g.L : (g.T[2] + 2 * g.L) - ns;
    c[0] = nf;
    c[1] = ns;
    c[2] = nv;
    c[3] = g.jitter ? nf + (r.fixed ? 0 : ns) : 0;
}

struct RowBase {
    int f, s, v, pad;
    long long d; // jitter-drawing sites before the row
};
struct CaseGenArgs {
    CaseGeom g;
    const RowBase *base;
    const float2 *hydro; // (rho, p) per lattice row j of the fluid block
    float rho0;
    float4 *fposr, *fvelp;
    int *forig;
    float4 *spos, *svel, *sref;
    int *stype, *sorig;
    float4 *vpos;
    long long nsite;
};
__device__ __forceinline__ double case_uniform(uint64_t seed, long long n) // draw n of splitmix64(seed)
{
    uint64_t z = seed + (uint64_t)(n + 1) * 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return __dmul_rn((double)(z >> 11), 1.0 / 9007199254740992.0);
}
__global__ void k_case_generate(const CaseGenArgs A)
{
    const long long sidx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (sidx >= A.nsite) return;
    const CaseGeom &g = A.g;
    const int nk = g.T[2] + 2 * g.L, nj = g.T[1] + 2 * g.L;
    const long long row = sidx / nk;
    const int k = (int)(sidx - row * nk) - g.L;
    const int i = (int)(row / nj) - g.L, j = (int)(row % nj) - g.L;
    RowIv r;
    case_row(g, i, j, r);
    const RowBase b = A.base[row];
    const bool in_solid = k >= r.s0 && k < r.s1;
    const bool outside = !r.inside || k < 0 || k >= g.T[2];
    const double x = __dmul_rn((double)i + 0.5, g.dx), y = __dmul_rn((double)j + 0.5, g.dx),
                 z = __dmul_rn((double)k + 0.5, g.dx);
    const int solid_before = iv_before(r.s0, r.s1, k);
    const int fluid_before = iv_before(r.f0, r.f1, k) - iv_overlap_before(r.f0, r.f1, r.s0, r.s1, k);
    auto jittered = [&](double* p) {
        const long long d = b.d + fluid_before + (r.fixed ? 0 : solid_before);
        for (int a = 0; a < 3; ++a) {
            const double u = case_uniform(g.seed, 3 * d + a);
            p[a] = __dadd_rn(p[a], __dmul_rn(__dsub_rn(__dmul_rn(2.0, u), 1.0), g.jit));
        }
    };
    if (in_solid) {
        const int idx = b.s + solid_before;
        double p[3] = {x, y, z};
        if (!r.fixed && g.jitter) jittered(p);
        const float4 q = make_float4((float)p[0], (float)p[1], (float)p[2], 0.0f);
        A.spos[idx] = q;
        A.sref[idx] = q;
        A.svel[idx] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        A.stype[idx] = r.fixed ? 1 : 0;
        A.sorig[idx] = idx;
    } else if (outside) {
        const int before = r.inside ? (k < 0 ? k + g.L : g.L + (k - g.T[2])) : (k + g.L) - solid_before;
        A.vpos[b.v + before] = make_float4((float)x, (float)y, (float)z, A.rho0);
    } else if (k >= r.f0 && k < r.f1) {
        const int idx = b.f + fluid_before;
        double p[3] = {x, y, z};
        if (g.jitter) jittered(p);
        const float2 hp = A.hydro[j];
        A.fposr[idx] = make_float4((float)p[0], (float)p[1], (float)p[2], hp.x);
        A.fvelp[idx] = make_float4(0.0f, 0.0f, 0.0f, hp.y);
        A.forig[idx] = idx;
    }
}

// ------------------------------------------------------------------ probes
// Probe::getData (src/probe.cu, commented out in the reference, 2D), in 3D:
// the Shepard average, weight (exp(-r^2/h^2) - c1) c2 as in
// solidPressureCalculate, of fluid velocity, pressure and density and of solid
// velocity and pressure (solid density 0) over the particles within the
// impact distance in the 27 cells of the probe's cell (cell lists of the last
// cell phase, current positions); (0, 0, rho0) when none is in range or the
// probe is outside the grid.  One warp per probe.
struct ProbeArgs {
    const float *pts;
    int n;
    float *out; // 5 per probe: u, v, w, p, rho
    const float4 *fposr, *fvelp;
    const int *start_f;
    const float4 *s_pos, *s_vel, *s_np;
    const int *start_s;
};
__global__ void k_probe(const DevParams P, const ProbeArgs A)
{
    const int k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (k >= A.n) return; // whole warp
    const float4 xi = make_float4(A.pts[3 * k], A.pts[3 * k + 1], A.pts[3 * k + 2], 0.0f);
    const float xa[3] = {xi.x, xi.y, xi.z};
    int c[3];
    bool inside = true;
    const int nn[3] = {P.nx, P.ny, P.nz};
    for (int a = 0; a < 3; ++a) {
        c[a] = (int)__fmul_rn(__fsub_rn(xa[a], P.cmin[a]), P.cinv[a]);
        inside = inside && c[a] >= 0 && c[a] < nn[a];
    }
    float w_sum = 0.0f, ux = 0.0f, uy = 0.0f, uz = 0.0f, p = 0.0f, rho = 0.0f;
    if (inside) {
        const int cell = (c[0] * P.ny + c[1]) * P.nz + c[2];
        auto fluid = [&](int j, float dx, float dy, float dz) {
            const float r2 = dist2(dx, dy, dz);
            if (r2 < P.R2) {
                const float w = (__expf(-r2 * P.h_inv2) - P.kc1) * P.kc2;
                const float4 q = A.fposr[j], u = A.fvelp[j];
                w_sum += w;
                ux += u.x * w;
                uy += u.y * w;
                uz += u.z * w;
                if (P.mixed) {
                    p += eos_delta(P, u.w) * w;
                    rho += fmaf(P.rho0, u.w, P.rho0) * w;
                } else {
                    p += u.w * w;
                    rho += q.w * w;
                }
            }
        };
        if (P.mixed) {
            solid_fluid_walk_m<32>(P, A.start_f, A.fposr, cell, xi, lane, fluid);
        }
        Rows rows;
        neighbor_rows(P, cell, rows);
        for (int r = 0; r < rows.count; ++r) {
            const int c0 = rows.base[r] + rows.z0, c1 = rows.base[r] + rows.z1;
            if (!P.mixed) {
                for (int j = A.start_f[c0] + lane, je = A.start_f[c1]; j < je; j += 32) {
                    const float4 q = A.fposr[j];
                    fluid(j, q.x - xi.x, q.y - xi.y, q.z - xi.z);
                }
            }
            for (int j = A.start_s[c0] + lane, je = A.start_s[c1]; j < je; j += 32) {
                const float4 q = A.s_pos[j];
                const float r2 = dist2(q.x - xi.x, q.y - xi.y, q.z - xi.z);
                if (r2 < P.R2) {
                    const float w = (__expf(-r2 * P.h_inv2) - P.kc1) * P.kc2;
                    const float4 v = A.s_vel[j];
                    w_sum += w;
                    ux += v.x * w;
                    uy += v.y * w;
                    uz += v.z * w;
                    p += A.s_np[j].w * w;
                }
            }
        }
    }
    w_sum = warp_sum(w_sum);
    ux = warp_sum(ux);
    uy = warp_sum(uy);
    uz = warp_sum(uz);
    p = warp_sum(p);
    rho = warp_sum(rho);
    if (lane) return;
    float *o = A.out + 5 * (size_t)k;
    if (w_sum != 0.0f) {
        o[0] = ux / w_sum;
        o[1] = uy / w_sum;
        o[2] = uz / w_sum;
        o[3] = p / w_sum;
        o[4] = rho / w_sum;
    } else {
        o[0] = o[1] = o[2] = o[3] = 0.0f;
        o[4] = P.rho0;
    }
}


// ------------------------------------------------ fused solid sub-steps
// All solid sub-steps of a step, for every instance of a plan, in ONE
// persistent cooperative launch: per sub-step deformation, force and update
// phases separated by grid barriers; each CTA walks the phases' virtual blocks
// (the batched kernels' block prefix tables) with a grid stride.  Instances
// with fewer sub-steps sit out the later ones.  The cooperative launch makes
// every CTA resident at once; the barrier still gives up after a bounded wait
// (FLAG_BARRIER_TIMEOUT on every instance, reported as FSIM_ETIMEOUT) instead
// of spinning for ever.
struct GridBarrier {
    unsigned count, gen;
};
constexpr unsigned kBarrierSpinLimit = 1u << 22; // x ~64 ns sleeps: about a quarter of a second and more

__device__ __forceinline__ void grid_sync(GridBarrier *b, bool &ok)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned *vgen = &b->gen;
        const unsigned g = *vgen; // read before arriving
        __threadfence();
        if (atomicAdd(&b->count, 1u) == gridDim.x - 1) {
            atomicExch(&b->count, 0u);
            __threadfence();
            atomicAdd(&b->gen, 1u);
        } else {
            unsigned spins = 0;
            while (*vgen == g) {
                if (++spins > kBarrierSpinLimit) {
                    ok = false;
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
    }
    __syncthreads();
}

struct SolidFusedArgs {
    const int *bstart_w, *bstart_t; // prefix tables: kSolidGroup lanes per particle / thread per particle
    int ninst, max_sub;
    GridBarrier *barrier;
};

template <bool MIXED>
__global__ void __launch_bounds__(kBlock, 3) kb_solid_fused(const Item<SolidArgs> *__restrict__ items,
                                                         const SolidFusedArgs F)
{
    const int total_w = F.bstart_w[F.ninst], total_t = F.bstart_t[F.ninst];
    bool ok = true;
    for (int k = 0; k < F.max_sub; ++k) {
        for (int b = blockIdx.x; b < total_w; b += gridDim.x) {
            const int inst = locate_instance(F.bstart_w, F.ninst, b);
            if (k >= items[inst].A.nsub) continue;
            const DevParams P = items[inst].P;
            solid_deform_body<MIXED>(P, items[inst].A, b - F.bstart_w[inst]);
        }
        grid_sync(F.barrier, ok);
        for (int b = blockIdx.x; b < total_w; b += gridDim.x) {
            const int inst = locate_instance(F.bstart_w, F.ninst, b);
            if (k >= items[inst].A.nsub) continue;
            const DevParams P = items[inst].P;
            solid_force_body<MIXED>(P, items[inst].A, b - F.bstart_w[inst]);
        }
        grid_sync(F.barrier, ok);
        for (int b = blockIdx.x; b < total_t; b += gridDim.x) {
            const int inst = locate_instance(F.bstart_t, F.ninst, b);
            if (k >= items[inst].A.nsub) continue;
            const DevParams P = items[inst].P;
            solid_update_body(P, items[inst].A, b - F.bstart_t[inst]);
        }
        if (k + 1 < F.max_sub) grid_sync(F.barrier, ok);
    }
    if (!ok && threadIdx.x == 0)
        for (int inst = 0; inst < F.ninst; ++inst) atomicOr(items[inst].A.flags, FLAG_BARRIER_TIMEOUT);
}

// ------------------------------------------------------- neighbour counts
__global__ void k_neighbor_counts(const DevParams P, const float4 *__restrict__ fposr, const int *__restrict__ cell_f,
                                  const int *__restrict__ start_f, const float4 *__restrict__ s_pos,
                                  const int *__restrict__ start_s, const float4 *__restrict__ v_posr,
                                  const int *__restrict__ start_v, int *__restrict__ out, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 p = fposr[i];
    Rows rows;
    neighbor_rows(P, cell_f[i], rows);
    int cf = 0, cs = 0, cv = 0;
    for (int r = 0; r < rows.count; ++r) {
        const int c0 = rows.base[r] + rows.z0, c1 = rows.base[r] + rows.z1;
        for (int j = start_f[c0]; j < start_f[c1]; ++j) {
            const float4 q = fposr[j];
            cf += dist2(q.x - p.x, q.y - p.y, q.z - p.z) < P.R2;
        }
        for (int j = start_s[c0]; j < start_s[c1]; ++j) {
            const float4 q = s_pos[j];
            cs += dist2(q.x - p.x, q.y - p.y, q.z - p.z) < P.R2;
        }
        for (int j = start_v[c0]; j < start_v[c1]; ++j) {
            const float4 q = v_posr[j];
            cv += dist2(q.x - p.x, q.y - p.y, q.z - p.z) < P.R2;
        }
    }
    out[3 * i] = cf;
    out[3 * i + 1] = cs;
    out[3 * i + 2] = cv;
}

// --------------------------------------------------- (un)permutation
// out[orig[s]] = component(s) of a float4 array: width 3 -> xyz, width 1 -> comp
__global__ void k_unpermute_f4(const float4 *__restrict__ src, const int *__restrict__ orig, int n, int comp, int width,
                               float *__restrict__ out)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const float4 v = src[s];
    const int o = orig[s];
    if (width == 3) {
        out[3 * o] = v.x;
        out[3 * o + 1] = v.y;
        out[3 * o + 2] = v.z;
    } else {
        out[o] = comp == 0 ? v.x : comp == 1 ? v.y : comp == 2 ? v.z : v.w;
    }
}
__global__ void k_unpermute_words(const int *__restrict__ src, const int *__restrict__ orig, int n, int width,
                                  int *__restrict__ out)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const int o = orig[s];
    for (int k = 0; k < width; ++k) out[width * o + k] = src[width * s + k];
}
__global__ void k_permute_in_f4(float4 *__restrict__ dst, const int *__restrict__ orig, int n, int comp, int width,
                                const float *__restrict__ in)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const int o = orig[s];
    float4 v = dst[s];
    if (width == 3) {
        v.x = in[3 * o];
        v.y = in[3 * o + 1];
        v.z = in[3 * o + 2];
    } else if (comp == 3) {
        v.w = in[o];
    }
    dst[s] = v;
}
__global__ void k_iota(int *a, int n)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < n) a[s] = s;
}
__global__ void k_pack_f4(const float *__restrict__ xyz, const float *__restrict__ w, int n, float wconst,
                          float4 *__restrict__ out)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    out[s] = make_float4(xyz[3 * s], xyz[3 * s + 1], xyz[3 * s + 2], w ? w[s] : wconst);
}

// Mixed form conversions (FP64 arithmetic, once per particle).
__device__ __forceinline__ double cell_corner(const DevParams &P, int axis, int c)
{
    return (double)P.cmin[axis] + (double)c * (double)P.cdx[axis];
}
// plain (x, y, z, rho) / (u, v, w, p) -> mixed offsets / delta; the cell of
// every particle from the FP32 cell index of its position
__global__ void k_fluid_to_mixed(const DevParams P, float4 *__restrict__ posr, float4 *__restrict__ velp,
                                 int *__restrict__ cell, int n, unsigned *flags)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const float4 p = posr[s];
    const int c = cell_index(P, p.x, p.y, p.z, flags);
    int cx, cy, cz;
    cell_xyz(P, c, cx, cy, cz);
    posr[s] = make_float4((float)((double)p.x - cell_corner(P, 0, cx)), (float)((double)p.y - cell_corner(P, 1, cy)),
                          (float)((double)p.z - cell_corner(P, 2, cz)), 0.0f);
    velp[s].w = (float)((double)p.w / (double)P.rho0 - 1.0);
    cell[s] = c;
}
// absolute positions -> offsets from the given cells (wall particles)
__global__ void k_offsets_in_cells(const DevParams P, float4 *__restrict__ pos, const int *__restrict__ cell, int n)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    float4 p = pos[s];
    int cx, cy, cz;
    cell_xyz(P, cell[s], cx, cy, cz);
    p.x = (float)((double)p.x - cell_corner(P, 0, cx));
    p.y = (float)((double)p.y - cell_corner(P, 1, cy));
    p.z = (float)((double)p.z - cell_corner(P, 2, cz));
    pos[s] = p;
}
enum MixedField { MF_POS = 0, MF_RHO = 1, MF_P = 2 };
// out[orig[s]] = absolute position / density / pressure of a mixed-form particle
__global__ void k_unpermute_mixed(const DevParams P, const float4 *__restrict__ pos, const float4 *__restrict__ velp,
                                  const int *__restrict__ cell, const int *__restrict__ orig, int n, int what,
                                  float *__restrict__ out)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const int o = orig[s];
    if (what == MF_POS) {
        const float4 p = pos[s];
        int cx, cy, cz;
        cell_xyz(P, cell[s], cx, cy, cz);
        out[3 * o] = (float)(cell_corner(P, 0, cx) + (double)p.x);
        out[3 * o + 1] = (float)(cell_corner(P, 1, cy) + (double)p.y);
        out[3 * o + 2] = (float)(cell_corner(P, 2, cz) + (double)p.z);
    } else {
        const double d = (double)velp[s].w;
        if (what == MF_RHO) {
            out[o] = (float)((double)P.rho0 * (1.0 + d));
        } else {
            const double pr = (double)P.rho2p * expm1((double)P.gamma * log1p(d));
            out[o] = (float)fmax(pr, (double)P.min_p);
        }
    }
}
// set a mixed-form position (offset from the particle's current cell) or density
__global__ void k_permute_in_mixed(const DevParams P, float4 *__restrict__ pos, float4 *__restrict__ velp,
                                   const int *__restrict__ cell, const int *__restrict__ orig, int n, int what,
                                   const float *__restrict__ in)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const int o = orig[s];
    if (what == MF_POS) {
        float4 p = pos[s];
        int cx, cy, cz;
        cell_xyz(P, cell[s], cx, cy, cz);
        p.x = (float)((double)in[3 * o] - cell_corner(P, 0, cx));
        p.y = (float)((double)in[3 * o + 1] - cell_corner(P, 1, cy));
        p.z = (float)((double)in[3 * o + 2] - cell_corner(P, 2, cz));
        pos[s] = p;
    } else {
        velp[s].w = (float)((double)in[o] / (double)P.rho0 - 1.0);
    }
}


// ------------------------------------------------- conservation (FP64)
// Per-particle terms in FP64, block sums in a fixed tree order; the host adds
// the block sums in order.  Layout of a block's terms: FSIM_CONSERVATION_N.
__device__ __forceinline__ double block_sum_d(double v, double *sh)
{
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int o = blockDim.x >> 1; o > 0; o >>= 1) {
        if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    const double r = sh[0];
    __syncthreads();
    return r;
}
// specific elastic energy of the Tait EOS, integral_rho0^rho p / rho'^2, in delta
__device__ __forceinline__ double tait_energy(const DevParams &P, double d)
{
    const double g1 = (double)P.gamma - 1.0;
    const double l = log1p(d);
    const double a = g1 != 0.0 ? expm1(g1 * l) / g1 : l;
    return (double)P.rho2p / (double)P.rho0 * (a - d / (1.0 + d));
}
__global__ void __launch_bounds__(kBlock) k_conservation_fluid(const DevParams P, const float4 *__restrict__ posr,
                                                               const float4 *__restrict__ velp,
                                                               const int *__restrict__ cell, int n, double vol,
                                                               double *__restrict__ partials)
{
    __shared__ double sh[kBlock];
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    double t[FSIM_CONSERVATION_N] = {};
    if (s < n) {
        const float4 p = posr[s], u = velp[s];
        double x = p.x, y = p.y, z = p.z, d;
        if (P.mixed) {
            int cx, cy, cz;
            cell_xyz(P, cell[s], cx, cy, cz);
            x += cell_corner(P, 0, cx);
            y += cell_corner(P, 1, cy);
            z += cell_corner(P, 2, cz);
            d = (double)u.w;
        } else {
            d = (double)p.w / (double)P.rho0 - 1.0;
        }
        const double m = (double)P.rho0 * vol;
        const double ux = u.x, uy = u.y, uz = u.z;
        t[0] = m;
        t[2] = m * ux;
        t[3] = m * uy;
        t[4] = m * uz;
        t[5] = 0.5 * m * (ux * ux + uy * uy + uz * uz);
        t[6] = -m * ((double)P.gx * x + (double)P.gy * y + (double)P.gz * z);
        t[7] = m * tait_energy(P, d);
        t[8] = (double)P.rho0 * d * vol;
    }
#pragma unroll 1
    for (int k = 0; k < FSIM_CONSERVATION_N; ++k) {
        const double r = block_sum_d(t[k], sh);
        if (threadIdx.x == 0) partials[(size_t)blockIdx.x * FSIM_CONSERVATION_N + k] = r;
    }
}
__global__ void __launch_bounds__(kBlock) k_conservation_solid(const DevParams P, const float4 *__restrict__ pos,
                                                               const float4 *__restrict__ vel,
                                                               const float *__restrict__ F, int n, double rho_s,
                                                               double vol, double *__restrict__ partials)
{
    __shared__ double sh[kBlock];
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    double t[FSIM_CONSERVATION_N] = {};
    if (s < n) {
        const float4 p = pos[s], u = vel[s];
        const double m = rho_s * vol;
        const double ux = u.x, uy = u.y, uz = u.z;
        t[1] = m;
        t[2] = m * ux;
        t[3] = m * uy;
        t[4] = m * uz;
        t[5] = 0.5 * m * (ux * ux + uy * uy + uz * uz);
        t[6] = -m * ((double)P.gx * p.x + (double)P.gy * p.y + (double)P.gz * p.z);
        double f[9], E[9];
        for (int k = 0; k < 9; ++k) f[k] = F[9 * (size_t)s + k];
        for (int a = 0; a < 3; ++a)
            for (int c = 0; c < 3; ++c)
                E[3 * a + c] = 0.5 * (f[a] * f[c] + f[3 + a] * f[3 + c] + f[6 + a] * f[6 + c] - (a == c ? 1.0 : 0.0));
        double ee = 0.0;
        for (int k = 0; k < 9; ++k) ee += E[k] * E[k];
        const double tr = E[0] + E[4] + E[8];
        t[9] = vol * ((double)P.mu_s * ee + 0.5 * (double)P.lambda * tr * tr);
    }
#pragma unroll 1
    for (int k = 0; k < FSIM_CONSERVATION_N; ++k) {
        const double r = block_sum_d(t[k], sh);
        if (threadIdx.x == 0) partials[(size_t)blockIdx.x * FSIM_CONSERVATION_N + k] = r;
    }
}
} // namespace

// =================================================================== handle
namespace {
struct Plan; // the launches of a step (or of one phase) over a set of instances

// Online autotuner of the fluid sweep's launch shape (see run_plan_step).
struct SweepTuner {
    int chosen = -1; // shape index once tuned
    int next = 0;    // next shape to time
    float ms[kSweepShapes] = {};
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int shape() const { return chosen >= 0 ? chosen : 0; }
    void release()
    {
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        e0 = e1 = nullptr;
    }
};
}

struct fsim_batch;
struct fsim_sim {
    int device = 0;
    cudaStream_t stream = nullptr;
    fsim_config cfg;
    fsim_derived der;
    DevParams P;
    int nf = 0, ns = 0, nv = 0, ncell = 0;
    bool keep = false;
    bool check_z = true; // z-cell re-check in the sweep (see k_fluid_sweep)
    // fluid
    float4 *f_posr[2] = {}, *f_velp[2] = {};
    int *f_orig[2] = {};
    int *f_cell = nullptr, *f_key = nullptr, *f_slot = nullptr, *f_tmp = nullptr;
    int *f_cnt = nullptr, *f_start = nullptr;
    float2 *f_cm = nullptr;  // mixed form: per-cell (delta, p) references of the FP16 gather
    bool mixed = false;
    float *f_drho = nullptr;
    float4 *f_dudt = nullptr;
    int f_cur = 0;
    bool f_sorted = false;   // start/cell arrays describe the order of f_cur
    bool f_deriv_ok = false; // derivative arrays are in the order of f_cur
    // solid
    float4 *s_pos[2] = {}, *s_vel[2] = {}, *s_ref[2] = {};
    int *s_type[2] = {}, *s_orig[2] = {};
    int *s_cell = nullptr, *s_key = nullptr, *s_slot = nullptr, *s_tmp = nullptr;
    int *s_cnt = nullptr, *s_start = nullptr;
    float4 *s_np = nullptr, *s_dudt = nullptr, *s_couple = nullptr;
    float *s_F = nullptr, *s_P = nullptr, *s_L = nullptr, *s_PL = nullptr, *s_AV = nullptr;
    int *s_inv = nullptr;         // sorted position of every input id (written by the gather)
    unsigned *s_cxyz = nullptr;   // packed cell coordinates, sorted order
    int *s_nbr_off = nullptr, *s_nbr_orig = nullptr; // static reference neighbours (CSR, input ids)
    float4 *s_nbr_dXw = nullptr;  // (X_j - X_i, kernel weight) per list entry
    int s_cur = 0;
    bool s_sorted = false;
    bool s_np_ok = false;    // normal + pressure are in the order of s_cur
    bool s_mech_ok = false;  // F, P, L^-1, du/dt are in the order of s_cur
    // virtual
    float4 *v_posr = nullptr, *v_velp = nullptr, *v_normal = nullptr;
    int *v_orig = nullptr, *v_cell = nullptr, *v_start = nullptr;
    // misc
    int *scan_partials = nullptr; // 2 * kMaxScanTiles
    unsigned *d_flags = nullptr;
    void *staging = nullptr;
    size_t staging_bytes = 0;
    void *bulk = nullptr;            // several fields at once (fsim_get_fields / fsim_set_fields)
    size_t bulk_bytes = 0;
    cudaStream_t copy_stream = nullptr;
    std::vector<cudaEvent_t> xfer_events;
    SweepTuner tuner;
    Plan *step_plans[2][2] = {};   // full step, by (fluid, solid) buffer parity
    Plan *phase_plans[5][2][2] = {}; // one phase, by parity
    fsim_batch *batch = nullptr;   // set while the handle belongs to a batch
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::vector<cudaEvent_t> sweep_events;
    std::vector<void *> allocations;
};

namespace {

#define CK(call)                                                                                        \
    do {                                                                                                \
        cudaError_t e_ = (call);                                                                        \
        if (e_ != cudaSuccess) {                                                                        \
            fsim_set_error("%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
            return FSIM_ECUDA;                                                                          \
        }                                                                                               \
    } while (0)

#define CK_LAUNCH()                                                                                            \
    do {                                                                                                       \
        cudaError_t e_ = cudaGetLastError();                                                                   \
        if (e_ != cudaSuccess) {                                                                               \
            fsim_set_error("kernel launch failed: %s (%s:%d)", cudaGetErrorString(e_), __FILE__, __LINE__);    \
            return FSIM_ECUDA;                                                                                 \
        }                                                                                                      \
    } while (0)

template <typename T>
fsim_status dalloc(fsim_sim *h, T **p, size_t count)
{
    *p = nullptr;
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc((void **)p, count * sizeof(T));
    if (e != cudaSuccess) {
        cudaGetLastError();
        fsim_set_error("cudaMalloc of %zu bytes failed: %s", count * sizeof(T), cudaGetErrorString(e));
        return FSIM_ENOMEM;
    }
    h->allocations.push_back((void *)*p);
    return FSIM_OK;
}

void free_plan(Plan *pl);

void free_all(fsim_sim *h)
{
    for (auto &row : h->step_plans)
        for (Plan *&pl : row) {
            free_plan(pl);
            pl = nullptr;
        }
    for (auto &ph : h->phase_plans)
        for (auto &row : ph)
            for (Plan *&pl : row) {
                free_plan(pl);
                pl = nullptr;
            }
    for (void *p : h->allocations) cudaFree(p);
    h->allocations.clear();
    for (cudaEvent_t e : h->sweep_events) cudaEventDestroy(e);
    h->sweep_events.clear();
    if (h->ev0) cudaEventDestroy(h->ev0);
    if (h->ev1) cudaEventDestroy(h->ev1);
    h->tuner.release();
    if (h->bulk) cudaFree(h->bulk);
    for (cudaEvent_t e : h->xfer_events) cudaEventDestroy(e);
    h->xfer_events.clear();
    if (h->copy_stream) cudaStreamDestroy(h->copy_stream);
    if (h->stream) cudaStreamDestroy(h->stream);
}

void fill_params(fsim_sim *h)
{
    const fsim_config &c = h->cfg;
    const fsim_derived &d = h->der;
    DevParams &P = h->P;
    std::memset(&P, 0, sizeof P);
    P.R2 = d.impact_distance_square;
    P.h = c.smoothing_length;
    P.h_inv2 = d.smoothing_length_inverse_square;
    P.kdiff = d.kernel_differential;
    P.kc1 = d.kernel_coefficient_1;
    P.kc2 = d.kernel_coefficient_2;
    P.eps_h2 = 0.01f * d.smoothing_length_square;
    P.exp2_scale = -d.smoothing_length_inverse_square * 1.4426950408889634f;
    P.c0 = c.fluid_sound_speed;
    P.c0_inv = 1.0f / c.fluid_sound_speed;
    P.rho0 = c.fluid_density;
    P.rho0_inv = d.reference_density_inverse;
    P.gamma = c.gamma;
    P.rho2p = d.coefficient_rho2p;
    P.min_p = c.min_pressure;
    P.min_rho = d.min_density;
    P.max_rho = d.max_density;
    P.mu10 = 10.0f * c.viscosity;
    P.vmax = 0.3f * c.fluid_sound_speed;
    P.viscid = c.is_viscid ? 1 : 0;
    P.rho_s_inv = 1.0f / c.solid_density;
    P.lambda = d.lambda;
    P.mu_s = d.shear_modulus;
    P.cs_s = d.solid_sound_speed;
    P.alpha = c.arti_vis_alpha;
    P.beta = c.arti_vis_beta;
    P.gx = d.gravity_vec[0];
    P.gy = d.gravity_vec[1];
    P.gz = d.gravity_vec[2];
    P.dt = c.dt;
    P.dt_sub = c.dt / (float)c.solid_sub_step;
    const float lo[3] = {c.xmin, c.ymin, c.zmin}, hi[3] = {c.xmax, c.ymax, c.zmax};
    for (int k = 0; k < 3; ++k) {
        P.dmin[k] = lo[k];
        P.dmax[k] = hi[k];
        P.cmin[k] = d.cell_min[k];
        P.cinv[k] = d.interval_inv[k];
    }
    P.nx = d.cell_number[0];
    P.ny = d.cell_number[1];
    P.nz = d.cell_number[2];
    P.ncell = d.cell_number_total;
    // mixed form
    P.mixed = c.precision == FSIM_PRECISION_MIXED ? 1 : 0;
    for (int k = 0; k < 3; ++k) {
        P.cdx[k] = d.interval[k];
        P.dlo_rel[k] = (float)((double)lo[k] - (double)d.cell_min[k]);
        P.dhi_rel[k] = (float)((double)hi[k] - (double)d.cell_min[k]);
    }
    const double rho0 = c.fluid_density;
    P.dlt_min = (float)((double)d.min_density / rho0 - 1.0);
    P.dlt_max = (float)((double)d.max_density / rho0 - 1.0);
    // FP16 unit of the gathered pressure deviation: a power of two such that
    // the largest possible deviation (EOS at the density bounds, the pressure
    // floor) stays below 2^15 units
    {
        const double g = c.gamma, b = d.coefficient_rho2p;
        const double pmax = b * (std::pow(1.0 + P.dlt_max, g) - 1.0);
        const double pmin = std::max((double)c.min_pressure, b * (std::pow(1.0 + P.dlt_min, g) - 1.0));
        const double span = std::max(pmax - pmin, 1e-30);
        const int e = (int)std::ceil(std::log2(span / 32768.0));
        P.p_unit = (float)std::ldexp(1.0, e);
        P.p_unit_inv = (float)std::ldexp(1.0, -e);
    }
}

// ---------------------------------------------------------------- plans
// A plan is the ordered list of batched launches that advance a set of
// instances by one step (or one phase), with every launch's {params, args}
// items and block prefix table in one device arena.  Buffer parities are the
// same for all instances of a plan, so the plan is fixed and a whole step is
// captured once into a CUDA graph.
enum LaunchKind {
    L_ZERO, L_HASH, L_SCAN_REDUCE, L_SCAN_PARTIALS, L_SCAN_APPLY, L_SCATTER, L_GATHER_F, L_GATHER_S,
    L_COUPLE, L_VIRT, L_SWEEP, L_DEFORM, L_FORCE, L_UPDATE,
    L_HASH_M, L_CELLREF, L_COUPLE_M, L_VIRT_M, L_DEFORM_M, L_FORCE_M, L_SOLID_FUSED
};

struct Launch {
    int kind;
    size_t items_off, table_off; // arena offsets
    int ninst, blocks, variant;
    size_t shape_table_off[kSweepShapes]; // L_SWEEP: block prefix table per launch shape
    int shape_blocks[kSweepShapes];
    size_t table2_off, barrier_off;       // L_SOLID_FUSED: thread-per-particle table, grid barrier
    int max_sub;
};

struct Plan {
    int device = 0;
    int pf = 0, ps = 0;           // buffer parities at the start
    int pf_after = 0, ps_after = 0;
    std::vector<Launch> launches;
    char *arena = nullptr;
    std::vector<char> host; // host image of the arena (one-instance launches pass items by value)
    cudaGraphExec_t graph = nullptr;
    int sweep_index = -1;         // launch index of the fluid sweep
};

void free_plan(Plan *pl)
{
    if (!pl) return;
    if (pl->graph) cudaGraphExecDestroy(pl->graph);
    if (pl->arena) cudaFree(pl->arena);
    delete pl;
}

// Host image of a plan's arena.
struct ArenaBuilder {
    std::vector<char> bytes;
    size_t put(const void *p, size_t n)
    {
        const size_t off = (bytes.size() + 255) & ~size_t(255);
        bytes.resize(off + n);
        std::memcpy(bytes.data() + off, p, n);
        return off;
    }
};

template <class Args>
void add_launch(Plan &pl, ArenaBuilder &ab, int kind, const std::vector<Item<Args>> &items,
                const std::vector<int> &blocks_per_item, int variant = 0)
{
    std::vector<int> table(items.size() + 1, 0);
    for (size_t k = 0; k < items.size(); ++k) table[k + 1] = table[k] + blocks_per_item[k];
    if (table.back() == 0) return; // nothing to do for any instance
    Launch L;
    L.kind = kind;
    L.items_off = ab.put(items.data(), sizeof(Item<Args>) * items.size());
    L.table_off = ab.put(table.data(), sizeof(int) * table.size());
    L.ninst = (int)items.size();
    L.blocks = table.back();
    L.variant = variant;
    pl.launches.push_back(L);
}

// The fluid sweep: one block prefix table per launch shape (blocks per
// instance depend on the warps per block).
void add_sweep_launch(Plan &pl, ArenaBuilder &ab, const std::vector<Item<FluidSweepArgs>> &items,
                      const std::vector<int> (&blocks)[kSweepShapes], int variant)
{
    Launch L{};
    L.kind = L_SWEEP;
    L.items_off = ab.put(items.data(), sizeof(Item<FluidSweepArgs>) * items.size());
    L.ninst = (int)items.size();
    L.variant = variant;
    for (int s = 0; s < kSweepShapes; ++s) {
        std::vector<int> table(items.size() + 1, 0);
        for (size_t k = 0; k < items.size(); ++k) table[k + 1] = table[k] + blocks[s][k];
        if (table.back() == 0) return; // no fluid in any instance
        L.shape_table_off[s] = ab.put(table.data(), sizeof(int) * table.size());
        L.shape_blocks[s] = table.back();
    }
    L.table_off = L.shape_table_off[0];
    L.blocks = L.shape_blocks[0];
    pl.launches.push_back(L);
}

// The cell phase: counting sort of fluid and solid (parity pf -> 1-pf, ps -> 1-ps).
void plan_cell(Plan &pl, ArenaBuilder &ab, const std::vector<fsim_sim *> &m, int pf, int ps)
{
    std::vector<Item<ZeroArgs>> zi;
    std::vector<Item<HashArgs>> hi;
    std::vector<Item<HashMixedArgs>> hmi;
    std::vector<Item<ScanArgs>> si;
    std::vector<Item<ScatterArgs>> ci;
    std::vector<int> zb, hb, hmb, sb, sp, cb;
    for (fsim_sim *h : m) {
        for (int sp_ = 0; sp_ < 2; ++sp_) {
            const int n = sp_ ? h->ns : h->nf;
            Item<ZeroArgs> z{h->P, ZeroArgs{sp_ ? h->s_cnt : h->f_cnt, n ? h->ncell : 0}};
            zi.push_back(z);
            zb.push_back(blocks_for(z.A.n, kBlock));
            if (!sp_ && h->mixed) {
                hmi.push_back({h->P, HashMixedArgs{h->f_posr[pf], h->f_cell, h->nf, h->f_key, h->f_slot, h->f_cnt,
                                                   h->d_flags}});
                hmb.push_back(blocks_for(n, kBlock));
            } else {
                Item<HashArgs> hh{h->P, sp_ ? HashArgs{h->s_pos[ps], h->ns, h->s_key, h->s_slot, h->s_cnt, h->d_flags}
                                            : HashArgs{h->f_posr[pf], h->nf, h->f_key, h->f_slot, h->f_cnt,
                                                       h->d_flags}};
                hi.push_back(hh);
                hb.push_back(blocks_for(n, kBlock));
            }
            Item<ScanArgs> sc{h->P, sp_ ? ScanArgs{h->s_cnt, h->s_start, h->ncell, h->scan_partials + kMaxScanTiles}
                                        : ScanArgs{h->f_cnt, h->f_start, h->ncell, h->scan_partials}};
            si.push_back(sc);
            sb.push_back(n ? blocks_for(h->ncell, kScanTile) : 0);
            sp.push_back(n ? 1 : 0);
            Item<ScatterArgs> cc{h->P, sp_ ? ScatterArgs{h->s_key, h->s_slot, h->s_start, h->s_tmp, h->ns}
                                           : ScatterArgs{h->f_key, h->f_slot, h->f_start, h->f_tmp, h->nf}};
            ci.push_back(cc);
            cb.push_back(blocks_for(n, kBlock));
        }
    }
    add_launch(pl, ab, L_ZERO, zi, zb);
    add_launch(pl, ab, L_HASH, hi, hb);
    add_launch(pl, ab, L_HASH_M, hmi, hmb);
    add_launch(pl, ab, L_SCAN_REDUCE, si, sb);
    add_launch(pl, ab, L_SCAN_PARTIALS, si, sp);
    add_launch(pl, ab, L_SCAN_APPLY, si, sb);
    add_launch(pl, ab, L_SCATTER, ci, cb);
    std::vector<Item<GatherFluidArgs>> gf;
    std::vector<Item<GatherSolidArgs>> gs;
    std::vector<int> gfb, gsb;
    for (fsim_sim *h : m) {
        gf.push_back({h->P, GatherFluidArgs{h->f_tmp, h->f_key, h->f_start, h->nf, h->f_posr[pf], h->f_velp[pf],
                                            h->f_orig[pf], h->f_posr[1 - pf], h->f_velp[1 - pf], h->f_orig[1 - pf],
                                            h->f_cell}});
        gfb.push_back(blocks_for(h->nf, kBlock));
        gs.push_back({h->P, GatherSolidArgs{h->s_tmp, h->s_key, h->s_start, h->ns, h->s_pos[ps], h->s_vel[ps],
                                            h->s_ref[ps], h->s_type[ps], h->s_orig[ps], h->s_pos[1 - ps],
                                            h->s_vel[1 - ps], h->s_ref[1 - ps], h->s_type[1 - ps], h->s_orig[1 - ps],
                                            h->s_cell, h->s_inv, h->s_cxyz}});
        gsb.push_back(blocks_for(h->ns, kBlock));
    }
    add_launch(pl, ab, L_GATHER_F, gf, gfb);
    add_launch(pl, ab, L_GATHER_S, gs, gsb);
    std::vector<Item<CellRefArgs>> cr;
    std::vector<int> crb;
    for (fsim_sim *h : m) {
        if (!h->mixed) continue;
        cr.push_back({h->P, CellRefArgs{h->f_posr[1 - pf], h->f_velp[1 - pf], h->f_start, h->f_cm, h->ncell}});
        crb.push_back(h->nf ? blocks_for(h->ncell, kBlock) : 0);
    }
    add_launch(pl, ab, L_CELLREF, cr, crb);
}

void plan_couple(Plan &pl, ArenaBuilder &ab, const std::vector<fsim_sim *> &m, int pf, int ps)
{
    std::vector<Item<CoupleArgs>> it;
    std::vector<int> nb;
    for (fsim_sim *h : m) {
        it.push_back({h->P, CoupleArgs{h->s_pos[ps], h->s_cell, h->s_start, h->f_posr[pf], h->f_velp[pf], h->f_start,
                                       h->s_np, h->ns}});
        nb.push_back(h->nf && h->ns ? blocks_for((long long)kSolidGroup * h->ns, kBlock) : 0);
    }
    add_launch(pl, ab, m.empty() || !m[0]->mixed ? L_COUPLE : L_COUPLE_M, it, nb);
}

void plan_virt(Plan &pl, ArenaBuilder &ab, const std::vector<fsim_sim *> &m, int pf)
{
    std::vector<Item<VirtArgs>> it;
    std::vector<int> nb;
    for (fsim_sim *h : m) {
        it.push_back({h->P, VirtArgs{h->v_posr, h->v_normal, h->v_cell, h->f_posr[pf], h->f_velp[pf], h->f_orig[pf],
                                     h->f_start, h->v_posr, h->v_velp, h->nv}});
        nb.push_back(blocks_for(h->nv, kBlock));
    }
    add_launch(pl, ab, m.empty() || !m[0]->mixed ? L_VIRT : L_VIRT_M, it, nb);
}

// fluid sweep + update (parity pf -> 1-pf)
void plan_fluid(Plan &pl, ArenaBuilder &ab, const std::vector<fsim_sim *> &m, int pf, int ps)
{
    std::vector<Item<FluidSweepArgs>> it;
    std::vector<int> nb[kSweepShapes];
    bool any_check = false;
    int nvisc = 0;
    for (fsim_sim *h : m) {
        FluidSweepArgs A;
        A.posr = h->f_posr[pf];
        A.velp = h->f_velp[pf];
        A.start_f = h->f_start;
        A.cell_f = h->f_cell;
        A.orig_in = h->f_orig[pf];
        A.s_pos = h->s_pos[ps];
        A.s_vel = h->s_vel[ps];
        A.s_np = h->s_np;
        A.start_s = h->s_start;
        A.v_posr = h->v_posr;
        A.v_velp = h->v_velp;
        A.start_v = h->v_start;
        A.posr_out = h->f_posr[1 - pf];
        A.velp_out = h->f_velp[1 - pf];
        A.orig_out = h->f_orig[1 - pf];
        A.drho_out = h->f_drho;
        A.dudt_out = h->f_dudt;
        A.n = h->nf;
        A.keep = h->keep ? 1 : 0;
        A.cm = h->f_cm;
        it.push_back({h->P, A});
        for (int sh = 0; sh < kSweepShapes; ++sh) nb[sh].push_back(blocks_for(h->nf, kShapeWarps[sh] * 32));
        if (h->nf) {
            any_check = any_check || h->check_z;
            nvisc += h->P.viscid ? 1 : 0;
        }
    }
    const int n_active = (int)std::count_if(m.begin(), m.end(), [](fsim_sim *h) { return h->nf > 0; });
    const int visc_mode = nvisc == 0 ? 0 : nvisc == n_active ? 1 : 2;
    const size_t before = pl.launches.size();
    const bool mixed = !m.empty() && m[0]->mixed;
    add_sweep_launch(pl, ab, it, nb, mixed ? 6 + visc_mode : (any_check ? 3 : 0) + visc_mode);
    if (pl.launches.size() > before) pl.sweep_index = (int)before;
}

// solid sub-steps (in place on parity ps; the fluid is read at parity pf):
// per-phase batched launches, or (solid_fused) one persistent cooperative
// launch for all sub-steps of all instances
// CTAs of the fused solid kernel that can be resident at once on the current
// device (a cooperative launch needs all of them resident), capped at `want`
int fused_grid(bool mixed, int want)
{
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (mixed)
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kb_solid_fused<true>, kBlock, 0);
    else
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kb_solid_fused<false>, kBlock, 0);
    const int c = std::max(1, sms * per_sm);
    return std::max(1, std::min(want, c));
}

void plan_solid(Plan &pl, ArenaBuilder &ab, const std::vector<fsim_sim *> &m, int pf, int ps)
{
    int max_sub = 0;
    for (fsim_sim *h : m)
        if (h->ns) max_sub = std::max(max_sub, h->cfg.solid_sub_step);
    if (!max_sub) return;
    std::vector<Item<SolidArgs>> it;
    std::vector<int> tw(m.size() + 1, 0), tt(m.size() + 1, 0);
    for (size_t q = 0; q < m.size(); ++q) {
        fsim_sim *h = m[q];
        SolidArgs S;
        S.pos = h->s_pos[ps];
        S.vel = h->s_vel[ps];
        S.ref = h->s_ref[ps];
        S.type = h->s_type[ps];
        S.cell = h->s_cell;
        S.start_s = h->s_start;
        S.np = h->s_np;
        S.F = h->s_F;
        S.Pk = h->s_P;
        S.L = h->s_L;
        S.PL = h->s_PL;
        S.AV = h->s_AV;
        S.dudt = h->s_dudt;
        S.couple = h->s_couple;
        S.fposr = h->f_posr[pf];
        S.fvelp = h->f_velp[pf];
        S.start_f = h->f_start;
        S.n = h->ns;
        S.orig = h->s_orig[ps];
        S.inv = h->s_inv;
        S.nbr_off = h->s_nbr_off;
        S.nbr_orig = h->s_nbr_orig;
        S.nbr_dXw = h->s_nbr_dXw;
        S.cxyz = h->s_cxyz;
        S.nsub = h->ns ? h->cfg.solid_sub_step : 0;
        S.flags = h->d_flags;
        it.push_back({h->P, S});
        tw[q + 1] = tw[q] + (h->ns ? blocks_for((long long)kSolidGroup * h->ns, kBlock) : 0);
        tt[q + 1] = tt[q] + (h->ns ? blocks_for(h->ns, kBlock) : 0);
    }
    const bool mixed = !m.empty() && m[0]->mixed;
    if (m.empty() || !m[0]->cfg.solid_fused) {
        // one batched launch per phase per sub-step; an instance takes part in
        // the sub-steps it has
        for (int k = 0; k < max_sub; ++k) {
            std::vector<int> wb, tb;
            for (fsim_sim *h : m) {
                const bool active = h->ns && k < h->cfg.solid_sub_step;
                wb.push_back(active ? blocks_for((long long)kSolidGroup * h->ns, kBlock) : 0);
                tb.push_back(active ? blocks_for(h->ns, kBlock) : 0);
            }
            add_launch(pl, ab, mixed ? L_DEFORM_M : L_DEFORM, it, wb);
            add_launch(pl, ab, mixed ? L_FORCE_M : L_FORCE, it, wb);
            add_launch(pl, ab, L_UPDATE, it, tb);
        }
        return;
    }
    Launch L{};
    L.kind = L_SOLID_FUSED;
    L.items_off = ab.put(it.data(), sizeof(Item<SolidArgs>) * it.size());
    L.table_off = ab.put(tw.data(), sizeof(int) * tw.size());
    L.table2_off = ab.put(tt.data(), sizeof(int) * tt.size());
    const GridBarrier zero{0u, 0u};
    L.barrier_off = ab.put(&zero, sizeof zero);
    L.ninst = (int)it.size();
    L.blocks = fused_grid(mixed, std::max(tw.back(), tt.back()));
    L.variant = mixed ? 1 : 0;
    L.max_sub = max_sub;
    pl.launches.push_back(L);
}

// phases: bit k = FSIM_PHASE k
fsim_status build_plan(const std::vector<fsim_sim *> &m, unsigned phases, int pf, int ps, Plan **out)
{
    *out = nullptr;
    auto *pl = new (std::nothrow) Plan;
    if (!pl) return FSIM_ENOMEM;
    pl->device = m.empty() ? 0 : m[0]->device;
    pl->pf = pf;
    pl->ps = ps;
    ArenaBuilder ab;
    if (phases & (1u << FSIM_PHASE_CELL)) {
        plan_cell(*pl, ab, m, pf, ps);
        pf ^= 1;
        ps ^= 1;
    }
    if (phases & (1u << FSIM_PHASE_COUPLE)) plan_couple(*pl, ab, m, pf, ps);
    if (phases & (1u << FSIM_PHASE_VIRT)) plan_virt(*pl, ab, m, pf);
    if (phases & (1u << FSIM_PHASE_FLUID)) {
        plan_fluid(*pl, ab, m, pf, ps);
        pf ^= 1;
    }
    if (phases & (1u << FSIM_PHASE_SOLID)) plan_solid(*pl, ab, m, pf, ps);
    pl->pf_after = pf;
    pl->ps_after = ps;
    pl->host = ab.bytes;
    if (!ab.bytes.empty()) {
        cudaError_t e = cudaMalloc((void **)&pl->arena, ab.bytes.size());
        if (e == cudaSuccess) e = cudaMemcpy(pl->arena, ab.bytes.data(), ab.bytes.size(), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            cudaGetLastError();
            fsim_set_error("plan upload failed: %s", cudaGetErrorString(e));
            free_plan(pl);
            return FSIM_ENOMEM;
        }
    }
    *out = pl;
    return FSIM_OK;
}

template <class Args>
const Item<Args> *items_of(const Plan &pl, const Launch &L)
{
    return reinterpret_cast<const Item<Args> *>(pl.arena + L.items_off);
}
template <class Args>
const Item<Args> &host_item(const Plan &pl, const Launch &L)
{
    return *reinterpret_cast<const Item<Args> *>(pl.host.data() + L.items_off);
}

#define FSIM_LAUNCH(KB, ARGS, THREADS) KB<<<g, THREADS, 0, st>>>(items_of<ARGS>(pl, L), tb, n)

// Enqueue a plan's launches; optional events around the fluid sweep.
fsim_status enqueue_plan(const Plan &pl, cudaStream_t st, int shape, cudaEvent_t sweep0 = nullptr,
                         cudaEvent_t sweep1 = nullptr)
{
    using SweepFn = void (*)(const Item<FluidSweepArgs> *, const int *, int);
    using Sweep1Fn = void (*)(const DevParams, const FluidSweepArgs);
    // [variant][shape]; variants 0-5: plain (CHECK_Z, VISCID); 6-8: mixed (VISCID)
    static const SweepFn sweeps[9][kSweepShapes] = {
        {kb_fluid_sweep<false, 0, Shape0>, kb_fluid_sweep<false, 0, Shape1>, kb_fluid_sweep<false, 0, Shape2>},
        {kb_fluid_sweep<false, 1, Shape0>, kb_fluid_sweep<false, 1, Shape1>, kb_fluid_sweep<false, 1, Shape2>},
        {kb_fluid_sweep<false, 2, Shape0>, kb_fluid_sweep<false, 2, Shape1>, kb_fluid_sweep<false, 2, Shape2>},
        {kb_fluid_sweep<true, 0, Shape0>, kb_fluid_sweep<true, 0, Shape1>, kb_fluid_sweep<true, 0, Shape2>},
        {kb_fluid_sweep<true, 1, Shape0>, kb_fluid_sweep<true, 1, Shape1>, kb_fluid_sweep<true, 1, Shape2>},
        {kb_fluid_sweep<true, 2, Shape0>, kb_fluid_sweep<true, 2, Shape1>, kb_fluid_sweep<true, 2, Shape2>},
        {kb_fluid_sweep_m<0, Shape0>, kb_fluid_sweep_m<0, Shape1>, kb_fluid_sweep_m<0, Shape2>},
        {kb_fluid_sweep_m<1, Shape0>, kb_fluid_sweep_m<1, Shape1>, kb_fluid_sweep_m<1, Shape2>},
        {kb_fluid_sweep_m<2, Shape0>, kb_fluid_sweep_m<2, Shape1>, kb_fluid_sweep_m<2, Shape2>}};
    static const Sweep1Fn sweeps1[9][kSweepShapes] = {
        {kb_fluid_sweep_1<false, 0, Shape0>, kb_fluid_sweep_1<false, 0, Shape1>, kb_fluid_sweep_1<false, 0, Shape2>},
        {kb_fluid_sweep_1<false, 1, Shape0>, kb_fluid_sweep_1<false, 1, Shape1>, kb_fluid_sweep_1<false, 1, Shape2>},
        {kb_fluid_sweep_1<false, 2, Shape0>, kb_fluid_sweep_1<false, 2, Shape1>, kb_fluid_sweep_1<false, 2, Shape2>},
        {kb_fluid_sweep_1<true, 0, Shape0>, kb_fluid_sweep_1<true, 0, Shape1>, kb_fluid_sweep_1<true, 0, Shape2>},
        {kb_fluid_sweep_1<true, 1, Shape0>, kb_fluid_sweep_1<true, 1, Shape1>, kb_fluid_sweep_1<true, 1, Shape2>},
        {kb_fluid_sweep_1<true, 2, Shape0>, kb_fluid_sweep_1<true, 2, Shape1>, kb_fluid_sweep_1<true, 2, Shape2>},
        {kb_fluid_sweep_m1<0, Shape0>, kb_fluid_sweep_m1<0, Shape1>, kb_fluid_sweep_m1<0, Shape2>},
        {kb_fluid_sweep_m1<1, Shape0>, kb_fluid_sweep_m1<1, Shape1>, kb_fluid_sweep_m1<1, Shape2>},
        {kb_fluid_sweep_m1<2, Shape0>, kb_fluid_sweep_m1<2, Shape1>, kb_fluid_sweep_m1<2, Shape2>}};
    for (size_t k = 0; k < pl.launches.size(); ++k) {
        const Launch &L = pl.launches[k];
        const int *tb = reinterpret_cast<const int *>(pl.arena + L.table_off);
        const int g = L.blocks, n = L.ninst;
        switch (L.kind) {
        case L_ZERO: FSIM_LAUNCH(kb_zero, ZeroArgs, kBlock); break;
        case L_HASH: FSIM_LAUNCH(kb_hash, HashArgs, kBlock); break;
        case L_SCAN_REDUCE: FSIM_LAUNCH(kb_scan_reduce, ScanArgs, kScanThreads); break;
        case L_SCAN_PARTIALS: FSIM_LAUNCH(kb_scan_partials, ScanArgs, kScanThreads); break;
        case L_SCAN_APPLY: FSIM_LAUNCH(kb_scan_apply, ScanArgs, kScanThreads); break;
        case L_SCATTER: FSIM_LAUNCH(kb_scatter, ScatterArgs, kBlock); break;
        case L_GATHER_F: FSIM_LAUNCH(kb_gather_fluid, GatherFluidArgs, kBlock); break;
        case L_GATHER_S: FSIM_LAUNCH(kb_gather_solid, GatherSolidArgs, kBlock); break;
        case L_COUPLE: FSIM_LAUNCH(kb_couple, CoupleArgs, kBlock); break;
        case L_VIRT: FSIM_LAUNCH(kb_virt, VirtArgs, kBlock); break;
        case L_SWEEP:
            if (sweep0) CK(cudaEventRecord(sweep0, st));
            {
                const int *tbs = reinterpret_cast<const int *>(pl.arena + L.shape_table_off[shape]);
                const int gs = L.shape_blocks[shape], thr = kShapeWarps[shape] * 32;
                if (n == 1) {
                    const Item<FluidSweepArgs> &it = host_item<FluidSweepArgs>(pl, L);
                    sweeps1[L.variant][shape]<<<gs, thr, 0, st>>>(it.P, it.A);
                } else {
                    sweeps[L.variant][shape]<<<gs, thr, 0, st>>>(items_of<FluidSweepArgs>(pl, L), tbs, n);
                }
            }
            CK_LAUNCH();
            if (sweep1) CK(cudaEventRecord(sweep1, st));
            break;
        case L_DEFORM: FSIM_LAUNCH(kb_solid_deform, SolidArgs, kBlock); break;
        case L_FORCE: FSIM_LAUNCH(kb_solid_force, SolidArgs, kBlock); break;
        case L_UPDATE: FSIM_LAUNCH(kb_solid_update, SolidArgs, kBlock); break;
        case L_HASH_M: FSIM_LAUNCH(kb_hash_mixed, HashMixedArgs, kBlock); break;
        case L_CELLREF: FSIM_LAUNCH(kb_cell_ref, CellRefArgs, kBlock); break;
        case L_COUPLE_M: FSIM_LAUNCH(kb_couple_mixed, CoupleArgs, kBlock); break;
        case L_VIRT_M: FSIM_LAUNCH(kb_virt_mixed, VirtArgs, kBlock); break;
        case L_DEFORM_M: FSIM_LAUNCH(kb_solid_deform_mixed, SolidArgs, kBlock); break;
        case L_FORCE_M: FSIM_LAUNCH(kb_solid_force_mixed, SolidArgs, kBlock); break;
        case L_SOLID_FUSED: {
            SolidFusedArgs F;
            F.bstart_w = tb;
            F.bstart_t = reinterpret_cast<const int *>(pl.arena + L.table2_off);
            F.ninst = n;
            F.max_sub = L.max_sub;
            F.barrier = reinterpret_cast<GridBarrier *>(pl.arena + L.barrier_off);
            CK(cudaMemsetAsync(F.barrier, 0, sizeof(GridBarrier), st));
            cudaLaunchConfig_t lc = {};
            lc.gridDim = dim3((unsigned)g);
            lc.blockDim = dim3(kBlock);
            lc.stream = st;
            cudaLaunchAttribute attr[1];
            attr[0].id = cudaLaunchAttributeCooperative;
            attr[0].val.cooperative = 1;
            lc.attrs = attr;
            lc.numAttrs = 1;
            const Item<SolidArgs> *items = items_of<SolidArgs>(pl, L);
            if (L.variant)
                CK(cudaLaunchKernelEx(&lc, kb_solid_fused<true>, items, F));
            else
                CK(cudaLaunchKernelEx(&lc, kb_solid_fused<false>, items, F));
            break;
        }
        default: fsim_set_error("unknown launch kind"); return FSIM_EINVAL;
        }
        CK_LAUNCH();
    }
    return FSIM_OK;
}

fsim_status capture_plan(Plan &pl, cudaStream_t st, int shape)
{
    cudaGraph_t graph = nullptr;
    CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    fsim_status s = enqueue_plan(pl, st, shape);
    cudaError_t e = cudaStreamEndCapture(st, &graph);
    if (s) {
        if (graph) cudaGraphDestroy(graph);
        return s;
    }
    if (e != cudaSuccess) {
        fsim_set_error("stream capture failed: %s", cudaGetErrorString(e));
        return FSIM_ECUDA;
    }
    e = cudaGraphInstantiate(&pl.graph, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
        pl.graph = nullptr;
        fsim_set_error("graph instantiate failed: %s", cudaGetErrorString(e));
        return FSIM_ECUDA;
    }
    return FSIM_OK;
}

// Validity bookkeeping after a plan ran on an instance.
void after_plan(fsim_sim *h, unsigned phases, const Plan &pl)
{
    h->f_cur = pl.pf_after;
    h->s_cur = pl.ps_after;
    if (phases & (1u << FSIM_PHASE_CELL)) {
        h->f_sorted = h->s_sorted = true;
        h->f_deriv_ok = h->s_np_ok = h->s_mech_ok = false;
    }
    if ((phases & (1u << FSIM_PHASE_COUPLE)) && h->nf && h->ns) h->s_np_ok = true;
    if (phases & (1u << FSIM_PHASE_FLUID)) h->f_deriv_ok = h->keep && h->nf > 0;
    if ((phases & (1u << FSIM_PHASE_SOLID)) && h->ns) h->s_mech_ok = true;
}

constexpr unsigned kAllPhases = 0x1fu;

fsim_status handle_step_plan(fsim_sim *h, Plan **out)
{
    Plan *&pl = h->step_plans[h->f_cur][h->s_cur];
    if (!pl) {
        fsim_status st = build_plan({h}, kAllPhases, h->f_cur, h->s_cur, &pl);
        if (st) return st;
    }
    *out = pl;
    return FSIM_OK;
}

// One step of a plan: while the sweep's launch shape is untuned, run launch
// by launch with the next candidate shape and time its sweep (CUDA events on
// the stream, waited for on the host); once every shape has been timed, keep
// the fastest and run the plan as a CUDA graph captured with it.
fsim_status run_plan_step(Plan &pl, cudaStream_t st, SweepTuner &t)
{
    if (t.chosen < 0 && pl.sweep_index >= 0) {
        if (!t.e0) {
            CK(cudaEventCreate(&t.e0));
            CK(cudaEventCreate(&t.e1));
        }
        const int s = t.next;
        fsim_status r = enqueue_plan(pl, st, s, t.e0, t.e1);
        if (r) return r;
        CK(cudaEventSynchronize(t.e1));
        CK(cudaEventElapsedTime(&t.ms[s], t.e0, t.e1));
        if (++t.next == kSweepShapes) {
            t.chosen = 0;
            for (int k = 1; k < kSweepShapes; ++k)
                if (t.ms[k] < t.ms[t.chosen]) t.chosen = k;
        }
        return FSIM_OK;
    }
    if (t.chosen < 0) t.chosen = 0; // no fluid: nothing to tune
    if (!pl.graph) {
        fsim_status r = capture_plan(pl, st, t.chosen);
        if (r) return r;
    }
    CK(cudaGraphLaunch(pl.graph, st));
    return FSIM_OK;
}

fsim_status run_step_graph(fsim_sim *h)
{
    Plan *pl = nullptr;
    fsim_status st = handle_step_plan(h, &pl);
    if (st) return st;
    if ((st = run_plan_step(*pl, h->stream, h->tuner))) return st;
    after_plan(h, kAllPhases, *pl);
    return FSIM_OK;
}

fsim_status check_flags(fsim_sim *h)
{
    unsigned flags = 0;
    CK(cudaMemcpyAsync(&flags, h->d_flags, sizeof flags, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    if (flags) CK(cudaMemsetAsync(h->d_flags, 0, sizeof(unsigned), h->stream));
    if (flags & FLAG_BARRIER_TIMEOUT) {
        fsim_set_error("a grid barrier of the solid sub-step kernel gave up waiting (results invalid)");
        return FSIM_ETIMEOUT;
    }
    if (flags & FLAG_OUT_OF_GRID) {
        fsim_set_error("a particle position fell outside the cell grid (clamped)");
        return FSIM_ENUMERIC;
    }
    return FSIM_OK;
}

void batch_wait(fsim_sim *h);

struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev)
    {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DeviceGuard()
    {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

// counting-sort the virtual particles once (walls are static), with the same
// batched sort kernels run as a one-instance plan over temporary arrays
// vpos_host: 3 floats per wall particle in host memory; or vpos_dev: float4
// (x, y, z, rho0) per wall particle already on the device (consumed)
fsim_status sort_virtual(fsim_sim *h, const float *vpos_host, float4 *vpos_dev = nullptr)
{
    const int n = h->nv;
    float *d_xyz = nullptr;
    float4 *tmp_pos = nullptr;
    int *key = nullptr, *slot = nullptr, *tmp = nullptr, *cnt = nullptr, *orig0 = nullptr;
    fsim_status st;
    if ((st = dalloc(h, &d_xyz, vpos_dev ? 1 : 3 * (size_t)n)) || (st = dalloc(h, &tmp_pos, n)) ||
        (st = dalloc(h, &key, n)) || (st = dalloc(h, &slot, n)) || (st = dalloc(h, &tmp, n)) ||
        (st = dalloc(h, &cnt, h->ncell)) || (st = dalloc(h, &orig0, n)))
        return st;
    if (vpos_dev) {
        CK(cudaMemcpyAsync(tmp_pos, vpos_dev, sizeof(float4) * n, cudaMemcpyDeviceToDevice, h->stream));
    } else {
        CK(cudaMemcpyAsync(d_xyz, vpos_host, sizeof(float) * 3 * n, cudaMemcpyHostToDevice, h->stream));
        k_pack_f4<<<blocks_for(n, kBlock), kBlock, 0, h->stream>>>(d_xyz, nullptr, n, h->P.rho0, tmp_pos);
    }
    k_iota<<<blocks_for(n, kBlock), kBlock, 0, h->stream>>>(orig0, n);
    CK_LAUNCH();
    Plan pl;
    ArenaBuilder ab;
    add_launch(pl, ab, L_ZERO, std::vector<Item<ZeroArgs>>{{h->P, ZeroArgs{cnt, h->ncell}}},
               {blocks_for(h->ncell, kBlock)});
    add_launch(pl, ab, L_HASH, std::vector<Item<HashArgs>>{{h->P, HashArgs{tmp_pos, n, key, slot, cnt, h->d_flags}}},
               {blocks_for(n, kBlock)});
    const std::vector<Item<ScanArgs>> sc{{h->P, ScanArgs{cnt, h->v_start, h->ncell, h->scan_partials}}};
    add_launch(pl, ab, L_SCAN_REDUCE, sc, {blocks_for(h->ncell, kScanTile)});
    add_launch(pl, ab, L_SCAN_PARTIALS, sc, {1});
    add_launch(pl, ab, L_SCAN_APPLY, sc, {blocks_for(h->ncell, kScanTile)});
    add_launch(pl, ab, L_SCATTER, std::vector<Item<ScatterArgs>>{{h->P, ScatterArgs{key, slot, h->v_start, tmp, n}}},
               {blocks_for(n, kBlock)});
    // the fluid gather with a dummy velocity stream
    add_launch(pl, ab, L_GATHER_F,
               std::vector<Item<GatherFluidArgs>>{{h->P, GatherFluidArgs{tmp, key, h->v_start, n, tmp_pos, tmp_pos,
                                                                         orig0, h->v_posr, h->v_velp, h->v_orig,
                                                                         h->v_cell}}},
               {blocks_for(n, kBlock)});
    pl.host = ab.bytes;
    CK(cudaMalloc((void **)&pl.arena, ab.bytes.size()));
    cudaError_t e = cudaMemcpy(pl.arena, ab.bytes.data(), ab.bytes.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && (st = enqueue_plan(pl, h->stream, 0)) == FSIM_OK) {
        e = cudaMemsetAsync(h->v_velp, 0, sizeof(float4) * n, h->stream);
        k_virt_normal<<<blocks_for(n, kBlock), kBlock, 0, h->stream>>>(h->P, h->v_posr, h->v_cell, h->v_start,
                                                                        h->v_normal, n);
        if (e == cudaSuccess) e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    }
    cudaFree(pl.arena);
    pl.arena = nullptr;
    if (e != cudaSuccess) {
        fsim_set_error("sorting the wall particles failed: %s", cudaGetErrorString(e));
        return FSIM_ECUDA;
    }
    if (st) return st;
    // temporaries are released now
    void *tmps[] = {d_xyz, tmp_pos, key, slot, tmp, cnt, orig0};
    for (void *p : tmps) {
        cudaFree(p);
        for (auto it = h->allocations.begin(); it != h->allocations.end(); ++it)
            if (*it == p) {
                h->allocations.erase(it);
                break;
            }
    }
    return FSIM_OK;
}

// Static reference-configuration neighbour lists of the solid: for every
// input id i, the ids j != i with |X_j - X_i|^2 < (2h)^2, the squared distance
// formed as the device forms it (fmaf(dz, dz, fmaf(dy, dy, dx * dx)) in FP32).
// Binned on a host grid of cell size >= 2h; list entries are in increasing j.
fsim_status build_solid_neighbors(fsim_sim *h, const float *ref)
{
    const int ns = h->ns;
    const float R2 = h->P.R2;
    const double cs = std::sqrt((double)R2) * 1.0001 + 1e-12;
    float lo[3] = {ref[0], ref[1], ref[2]}, hi[3] = {ref[0], ref[1], ref[2]};
    for (int i = 0; i < ns; ++i)
        for (int a = 0; a < 3; ++a) {
            lo[a] = std::min(lo[a], ref[3 * i + a]);
            hi[a] = std::max(hi[a], ref[3 * i + a]);
        }
    int nb[3];
    for (int a = 0; a < 3; ++a) nb[a] = std::max(1, std::min(1024, (int)((hi[a] - lo[a]) / cs) + 1));
    auto bin = [&](int i, int a) {
        const int b = (int)((ref[3 * i + a] - lo[a]) / cs);
        return std::min(nb[a] - 1, std::max(0, b));
    };
    const size_t nbins = (size_t)nb[0] * nb[1] * nb[2];
    std::vector<int> bstart(nbins + 1, 0), order(ns);
    std::vector<int> key(ns);
    for (int i = 0; i < ns; ++i) {
        key[i] = (bin(i, 0) * nb[1] + bin(i, 1)) * nb[2] + bin(i, 2);
        ++bstart[key[i] + 1];
    }
    for (size_t b = 0; b < nbins; ++b) bstart[b + 1] += bstart[b];
    {
        std::vector<int> fill(bstart.begin(), bstart.end() - 1);
        for (int i = 0; i < ns; ++i) order[fill[key[i]]++] = i; // increasing i within a bin
    }
    std::vector<int> off(ns + 1, 0), nbr;
    std::vector<float4> dXw;
    std::vector<int> cand;
    for (int i = 0; i < ns; ++i) {
        const int bx = bin(i, 0), by = bin(i, 1), bz = bin(i, 2);
        cand.clear();
        for (int x = std::max(0, bx - 1); x <= std::min(nb[0] - 1, bx + 1); ++x)
            for (int y = std::max(0, by - 1); y <= std::min(nb[1] - 1, by + 1); ++y)
                for (int z = std::max(0, bz - 1); z <= std::min(nb[2] - 1, bz + 1); ++z) {
                    const int b = (x * nb[1] + y) * nb[2] + z;
                    for (int k = bstart[b]; k < bstart[b + 1]; ++k) cand.push_back(order[k]);
                }
        std::sort(cand.begin(), cand.end());
        for (int j : cand) {
            if (j == i) continue;
            const float dx = ref[3 * j] - ref[3 * i], dy = ref[3 * j + 1] - ref[3 * i + 1],
                        dz = ref[3 * j + 2] - ref[3 * i + 2];
            const float r2 = std::fmaf(dz, dz, std::fmaf(dy, dy, dx * dx));
            if (r2 < R2) {
                nbr.push_back(j);
                dXw.push_back(make_float4(dx, dy, dz, 0.0f));
            }
        }
        off[i + 1] = (int)nbr.size();
    }
    const size_t ne = nbr.size();
    fsim_status st;
    if ((st = dalloc(h, &h->s_nbr_off, (size_t)ns + 1)) || (st = dalloc(h, &h->s_nbr_orig, ne)) ||
        (st = dalloc(h, &h->s_nbr_dXw, ne)))
        return st;
    CK(cudaMemcpy(h->s_nbr_off, off.data(), sizeof(int) * (ns + 1), cudaMemcpyHostToDevice));
    if (ne) {
        CK(cudaMemcpy(h->s_nbr_orig, nbr.data(), sizeof(int) * ne, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(h->s_nbr_dXw, dXw.data(), sizeof(float4) * ne, cudaMemcpyHostToDevice));
        k_solid_pair_weights<<<blocks_for((long long)ne, kBlock), kBlock, 0, h->stream>>>(h->P, h->s_nbr_dXw, (int)ne);
        CK_LAUNCH();
    }
    return FSIM_OK;
}

// Stream, events and every device array of a handle whose counts are set.
fsim_status alloc_state(fsim_sim *h)
{
    const int nf = h->nf, ns = h->ns, nv = h->nv, nc = h->ncell;
    CK(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
    CK(cudaEventCreate(&h->ev0));
    CK(cudaEventCreate(&h->ev1));
    fsim_status st;
    if ((st = dalloc(h, &h->d_flags, 1))) return st;
    if ((st = dalloc(h, &h->scan_partials, 2 * kMaxScanTiles))) return st;
    CK(cudaMemsetAsync(h->d_flags, 0, sizeof(unsigned), h->stream));
    // fluid
    for (int b = 0; b < 2; ++b) {
        if ((st = dalloc(h, &h->f_posr[b], nf)) || (st = dalloc(h, &h->f_velp[b], nf)) ||
            (st = dalloc(h, &h->f_orig[b], nf)))
            return st;
    }
    if ((st = dalloc(h, &h->f_cell, nf)) || (st = dalloc(h, &h->f_key, nf)) || (st = dalloc(h, &h->f_slot, nf)) ||
        (st = dalloc(h, &h->f_tmp, nf)) || (st = dalloc(h, &h->f_cnt, nc)) || (st = dalloc(h, &h->f_start, nc + 1)))
        return st;
    if (h->keep && ((st = dalloc(h, &h->f_drho, nf)) || (st = dalloc(h, &h->f_dudt, nf)))) return st;
    if (h->mixed && (st = dalloc(h, &h->f_cm, nc))) return st;
    // solid
    for (int b = 0; b < 2; ++b) {
        if ((st = dalloc(h, &h->s_pos[b], ns)) || (st = dalloc(h, &h->s_vel[b], ns)) ||
            (st = dalloc(h, &h->s_ref[b], ns)) || (st = dalloc(h, &h->s_type[b], ns)) ||
            (st = dalloc(h, &h->s_orig[b], ns)))
            return st;
    }
    if ((st = dalloc(h, &h->s_cell, ns)) || (st = dalloc(h, &h->s_key, ns)) || (st = dalloc(h, &h->s_slot, ns)) ||
        (st = dalloc(h, &h->s_tmp, ns)) || (st = dalloc(h, &h->s_cnt, nc)) || (st = dalloc(h, &h->s_start, nc + 1)) ||
        (st = dalloc(h, &h->s_np, ns)) || (st = dalloc(h, &h->s_dudt, ns)) || (st = dalloc(h, &h->s_couple, ns)) ||
        (st = dalloc(h, &h->s_F, 9 * (size_t)ns)) || (st = dalloc(h, &h->s_P, 9 * (size_t)ns)) ||
        (st = dalloc(h, &h->s_L, 9 * (size_t)ns)) || (st = dalloc(h, &h->s_PL, 9 * (size_t)ns)) ||
        (st = dalloc(h, &h->s_AV, 9 * (size_t)ns)) || (st = dalloc(h, &h->s_inv, ns)) ||
        (st = dalloc(h, &h->s_cxyz, ns)))
        return st;
    // virtual
    if ((st = dalloc(h, &h->v_posr, nv)) || (st = dalloc(h, &h->v_velp, nv)) || (st = dalloc(h, &h->v_normal, nv)) ||
        (st = dalloc(h, &h->v_orig, nv)) || (st = dalloc(h, &h->v_cell, nv)) || (st = dalloc(h, &h->v_start, nc + 1)))
        return st;
    // staging for field copies (input order)
    size_t words = 3 * (size_t)nf;
    if (9 * (size_t)ns > words) words = 9 * (size_t)ns;
    if (3 * (size_t)nv > words) words = 3 * (size_t)nv;
    h->staging_bytes = 4 * (words ? words : 1);
    if ((st = dalloc(h, (char **)&h->staging, h->staging_bytes))) return st;

    // empty cell structures are valid before the first cell phase
    CK(cudaMemsetAsync(h->f_cell, 0, sizeof(int) * (nf ? nf : 1), h->stream));
    CK(cudaMemsetAsync(h->f_start, 0, sizeof(int) * (nc + 1), h->stream));
    CK(cudaMemsetAsync(h->s_start, 0, sizeof(int) * (nc + 1), h->stream));
    CK(cudaMemsetAsync(h->v_start, 0, sizeof(int) * (nc + 1), h->stream));
    CK(cudaMemsetAsync(h->s_np, 0, sizeof(float4) * (ns ? ns : 1), h->stream));
    return FSIM_OK;
}

fsim_status create_impl(fsim_sim *h, const fsim_particles *p)
{
    const int nf = p->n_fluid, ns = p->n_solid, nv = p->n_virt;
    fsim_status st = alloc_state(h);
    if (st) return st;
    float *stg = (float *)h->staging;
    if (nf) {
        CK(cudaMemcpyAsync(stg, p->fluid_pos, sizeof(float) * 3 * nf, cudaMemcpyHostToDevice, h->stream));
        float *d_rho = nullptr;
        if ((st = dalloc(h, &d_rho, nf))) return st;
        CK(cudaMemcpyAsync(d_rho, p->fluid_rho, sizeof(float) * nf, cudaMemcpyHostToDevice, h->stream));
        k_pack_f4<<<blocks_for(nf, kBlock), kBlock, 0, h->stream>>>(stg, d_rho, nf, 0.0f, h->f_posr[0]);
        CK(cudaMemcpyAsync(d_rho, p->fluid_p, sizeof(float) * nf, cudaMemcpyHostToDevice, h->stream));
        CK(cudaStreamSynchronize(h->stream));
        CK(cudaMemcpyAsync(stg, p->fluid_vel, sizeof(float) * 3 * nf, cudaMemcpyHostToDevice, h->stream));
        k_pack_f4<<<blocks_for(nf, kBlock), kBlock, 0, h->stream>>>(stg, d_rho, nf, 0.0f, h->f_velp[0]);
        k_iota<<<blocks_for(nf, kBlock), kBlock, 0, h->stream>>>(h->f_orig[0], nf);
        if (h->mixed)
            k_fluid_to_mixed<<<blocks_for(nf, kBlock), kBlock, 0, h->stream>>>(h->P, h->f_posr[0], h->f_velp[0],
                                                                               h->f_cell, nf, h->d_flags);
        CK_LAUNCH();
        CK(cudaStreamSynchronize(h->stream));
        cudaFree(d_rho);
        h->allocations.pop_back();
    }
    if (ns) {
        CK(cudaMemcpyAsync(stg, p->solid_pos, sizeof(float) * 3 * ns, cudaMemcpyHostToDevice, h->stream));
        k_pack_f4<<<blocks_for(ns, kBlock), kBlock, 0, h->stream>>>(stg, nullptr, ns, 0.0f, h->s_pos[0]);
        CK(cudaStreamSynchronize(h->stream));
        CK(cudaMemcpyAsync(stg, p->solid_vel, sizeof(float) * 3 * ns, cudaMemcpyHostToDevice, h->stream));
        k_pack_f4<<<blocks_for(ns, kBlock), kBlock, 0, h->stream>>>(stg, nullptr, ns, 0.0f, h->s_vel[0]);
        CK(cudaStreamSynchronize(h->stream));
        CK(cudaMemcpyAsync(stg, p->solid_ref_pos, sizeof(float) * 3 * ns, cudaMemcpyHostToDevice, h->stream));
        k_pack_f4<<<blocks_for(ns, kBlock), kBlock, 0, h->stream>>>(stg, nullptr, ns, 0.0f, h->s_ref[0]);
        CK(cudaMemcpyAsync(h->s_type[0], p->solid_type, sizeof(int) * ns, cudaMemcpyHostToDevice, h->stream));
        k_iota<<<blocks_for(ns, kBlock), kBlock, 0, h->stream>>>(h->s_orig[0], ns);
        CK_LAUNCH();
        CK(cudaStreamSynchronize(h->stream));
        // F = L = I, P = 0 until the first solid phase (include/host_data.cuh:95-97)
        std::vector<float> eye(9 * (size_t)ns, 0.0f);
        for (int i = 0; i < ns; ++i) eye[9 * i] = eye[9 * i + 4] = eye[9 * i + 8] = 1.0f;
        CK(cudaMemcpy(h->s_F, eye.data(), sizeof(float) * 9 * ns, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(h->s_L, eye.data(), sizeof(float) * 9 * ns, cudaMemcpyHostToDevice));
        CK(cudaMemset(h->s_P, 0, sizeof(float) * 9 * ns));
        CK(cudaMemset(h->s_dudt, 0, sizeof(float4) * ns));
        CK(cudaMemset(h->s_couple, 0, sizeof(float4) * ns));
        h->s_mech_ok = true; // initial values, in input order (= s_orig[0])
        h->s_np_ok = true;
        if ((st = build_solid_neighbors(h, p->solid_ref_pos))) return st;
    }
    if (nv && (st = sort_virtual(h, p->virt_pos))) return st;
    if (nv && h->mixed) {
        k_offsets_in_cells<<<blocks_for(nv, kBlock), kBlock, 0, h->stream>>>(h->P, h->v_posr, h->v_cell, nv);
        CK_LAUNCH();
    }
    CK(cudaStreamSynchronize(h->stream));
    return check_flags(h);
}

} // namespace

// =================================================================== C ABI
namespace {
// A handle with its configuration, derived constants, device parameters and
// counts set and checked; nothing allocated on the device yet.
fsim_status new_handle(const fsim_config *cfg, int nf, int ns, int nv, int device, fsim_sim **out)
{
    *out = nullptr;
    if (cfg->solid_sub_step < 1 || !(cfg->dt > 0.0f)) {
        fsim_set_error("dt must be > 0 and solid_sub_step >= 1");
        return FSIM_EINVAL;
    }
    auto *h = new (std::nothrow) fsim_sim;
    if (!h) return FSIM_ENOMEM;
    h->cfg = *cfg;
    fsim_status st = fsim_derive(cfg, &h->der);
    if (st) {
        delete h;
        return st;
    }
    if (blocks_for(h->der.cell_number_total, kScanTile) > kMaxScanTiles) {
        fsim_set_error("cell grid of %d cells exceeds the supported %d", h->der.cell_number_total,
                       kMaxScanTiles * kScanTile);
        delete h;
        return FSIM_EINVAL;
    }
    if (device < 0) {
        if (cudaGetDevice(&device) != cudaSuccess) {
            fsim_set_error("no CUDA device");
            delete h;
            return FSIM_ECUDA;
        }
    }
    h->device = device;
    fill_params(h);
    h->nf = nf;
    h->ns = ns;
    h->nv = nv;
    h->ncell = h->der.cell_number_total;
    h->keep = cfg->keep_derivatives != 0;
    h->mixed = h->P.mixed != 0;
    if (h->mixed && (h->nf > kIndexMask || h->nv > kIndexMask)) {
        fsim_set_error("the mixed form takes at most %d fluid and %d wall particles", kIndexMask, kIndexMask);
        delete h;
        return FSIM_EINVAL;
    }
    if (h->ns && (h->P.nx >= 2048 || h->P.ny >= 1024 || h->P.nz >= 2048)) {
        fsim_set_error("cell grid %d x %d x %d too large for a solid (limit 2047 x 1023 x 2047)", h->P.nx, h->P.ny,
                       h->P.nz);
        delete h;
        return FSIM_EINVAL;
    }
    // The union-of-rows sweep needs no z-cell check when the z spacing exceeds
    // the impact distance by more than FP32 rounding of the cell coordinate
    // (about 2.4e-7 * nz cells, doubled here, plus slack) can eat; keep it otherwise.
    {
        const double R = std::sqrt((double)h->der.impact_distance_square);
        const double margin = (double)h->der.interval[2] / R - 1.0;
        h->check_z = !(margin > 8e-7 * h->der.cell_number[2] + 1e-4);
    }
    *out = h;
    return FSIM_OK;
}
} // namespace

extern "C" fsim_status fsim_create(const fsim_config *cfg, const fsim_particles *p, int device, fsim_handle *out)
{
    if (!cfg || !p || !out) return FSIM_EINVAL;
    *out = nullptr;
    if (p->n_fluid < 0 || p->n_solid < 0 || p->n_virt < 0 || (p->n_fluid && (!p->fluid_pos || !p->fluid_vel ||
                                                                             !p->fluid_rho || !p->fluid_p)) ||
        (p->n_solid && (!p->solid_pos || !p->solid_vel || !p->solid_ref_pos || !p->solid_type)) ||
        (p->n_virt && !p->virt_pos)) {
        fsim_set_error("invalid particle arrays");
        return FSIM_EINVAL;
    }
    fsim_sim *h = nullptr;
    fsim_status st = new_handle(cfg, p->n_fluid, p->n_solid, p->n_virt, device, &h);
    if (st) return st;
    DeviceGuard guard(h->device);
    st = create_impl(h, p);
    if (st) {
        free_all(h);
        delete h;
        return st;
    }
    *out = h;
    return FSIM_OK;
}

extern "C" fsim_status fsim_destroy(fsim_handle h)
{
    if (!h) return FSIM_OK;
    if (h->batch) {
        fsim_set_error("destroy the batch before its members");
        return FSIM_EINVAL;
    }
    DeviceGuard guard(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    free_all(h);
    delete h;
    return FSIM_OK;
}

extern "C" fsim_status fsim_step(fsim_handle h, int nsteps)
{
    if (!h || nsteps < 0) return FSIM_EINVAL;
    if (h->batch) {
        fsim_set_error("the handle belongs to a batch; step it through the batch");
        return FSIM_EINVAL;
    }
    DeviceGuard guard(h->device);
    for (int k = 0; k < nsteps; ++k) {
        fsim_status st = run_step_graph(h);
        if (st) return st;
    }
    return FSIM_OK;
}

extern "C" fsim_status fsim_sync(fsim_handle h)
{
    if (!h) return FSIM_EINVAL;
    if (h->batch) batch_wait(h);
    DeviceGuard guard(h->device);
    CK(cudaStreamSynchronize(h->stream));
    return check_flags(h);
}

extern "C" fsim_status fsim_run_phase(fsim_handle h, int phase)
{
    if (!h) return FSIM_EINVAL;
    if (phase < FSIM_PHASE_CELL || phase > FSIM_PHASE_SOLID) {
        fsim_set_error("unknown phase %d", phase);
        return FSIM_EINVAL;
    }
    if (phase != FSIM_PHASE_CELL && (!h->f_sorted || !h->s_sorted)) {
        fsim_set_error("run FSIM_PHASE_CELL first");
        return FSIM_EINVAL;
    }
    if (h->batch) {
        fsim_set_error("the handle belongs to a batch; step it through the batch");
        return FSIM_EINVAL;
    }
    DeviceGuard guard(h->device);
    Plan *&pl = h->phase_plans[phase][h->f_cur][h->s_cur];
    if (!pl) {
        fsim_status st = build_plan({h}, 1u << phase, h->f_cur, h->s_cur, &pl);
        if (st) return st;
    }
    fsim_status st = enqueue_plan(*pl, h->stream, h->tuner.shape());
    if (st) return st;
    after_plan(h, 1u << phase, *pl);
    return FSIM_OK;
}

extern "C" int fsim_field_width(int field)
{
    switch (field) {
    case FSIM_FLUID_POS: case FSIM_FLUID_VEL: case FSIM_FLUID_DU_DT:
    case FSIM_SOLID_POS: case FSIM_SOLID_VEL: case FSIM_SOLID_REF_POS: case FSIM_SOLID_NORMAL:
    case FSIM_SOLID_DU_DT: case FSIM_SOLID_COUPLE_DUDT:
    case FSIM_VIRT_POS: case FSIM_VIRT_NORMAL: case FSIM_VIRT_VEL:
        return 3;
    case FSIM_FLUID_RHO: case FSIM_FLUID_P: case FSIM_FLUID_DRHO_DT: case FSIM_FLUID_CELL_ID:
    case FSIM_SOLID_TYPE: case FSIM_SOLID_P: case FSIM_SOLID_CELL_ID:
    case FSIM_VIRT_P: case FSIM_VIRT_RHO: case FSIM_VIRT_CELL_ID:
        return 1;
    case FSIM_SOLID_F: case FSIM_SOLID_PK1: case FSIM_SOLID_LINV:
        return 9;
    default: return 0;
    }
}

static int field_count(fsim_sim *h, int field)
{
    if (field < 10) return h->nf;
    if (field < 30) return h->ns;
    return h->nv;
}

namespace {
// Field size check shared by the getters and setters.
fsim_status check_field_bytes(fsim_sim *h, int field, size_t bytes, int *count)
{
    const int width = fsim_field_width(field);
    if (!width) {
        fsim_set_error("unknown field %d", field);
        return FSIM_EINVAL;
    }
    const int n = field_count(h, field);
    if (bytes != (size_t)n * width * 4) {
        fsim_set_error("field %d needs %zu bytes, got %zu", field, (size_t)n * width * 4, bytes);
        return FSIM_EINVAL;
    }
    *count = n;
    return FSIM_OK;
}

// Enqueue on the handle's stream the kernel that writes `field` in input
// order into device memory `stg` (n = the field's particle count > 0).
fsim_status enqueue_unpermute(fsim_sim *h, int field, int n, float *stg)
{
    const int g = blocks_for(n, kBlock);
    const int *forig = h->f_orig[h->f_cur];
    const int *sorig = h->s_orig[h->s_cur];
    if (h->mixed && (field == FSIM_FLUID_POS || field == FSIM_FLUID_RHO || field == FSIM_FLUID_P ||
                     field == FSIM_VIRT_POS)) {
        if (field == FSIM_VIRT_POS)
            k_unpermute_mixed<<<g, kBlock, 0, h->stream>>>(h->P, h->v_posr, h->v_velp, h->v_cell, h->v_orig, n, MF_POS,
                                                            stg);
        else
            k_unpermute_mixed<<<g, kBlock, 0, h->stream>>>(h->P, h->f_posr[h->f_cur], h->f_velp[h->f_cur], h->f_cell,
                                                            forig, n,
                                                            field == FSIM_FLUID_POS   ? MF_POS
                                                            : field == FSIM_FLUID_RHO ? MF_RHO
                                                                                      : MF_P,
                                                            stg);
        CK_LAUNCH();
        return FSIM_OK;
    }
    switch (field) {
    case FSIM_FLUID_POS: k_unpermute_f4<<<g, kBlock, 0, h->stream>>>(h->f_posr[h->f_cur], forig, n, 0, 3, stg); break;
    case FSIM_FLUID_RHO: k_unpermute_f4<<<g, kBlock, 0, h->stream>>>(h->f_posr[h->f_cur], forig, n, 3, 1, stg); break;
    case FSIM_FLUID_VEL: k_unpermute_f4<<<g, kBlock, 0, h->stream>>>(h->f_velp[h->f_cur], forig, n, 0, 3, stg); break;
    case FSIM_FLUID_P: k_unpermute_f4<<<g, kBlock, 0, h->stream>>>(h->f_velp[h->f_cur], forig, n, 3, 1, stg); break;
    case FSIM_FLUID_DRHO_DT:
    case FSIM_FLUID_DU_DT:
        if (!h->f_deriv_ok) {
            fsim_set_error("derivatives unavailable (set keep_derivatives and run the fluid phase)");
            return FSIM_EINVAL;
        }
        if (field == FSIM_FLUID_DU_DT)
            k_unpermute_f4<<<g, kBlock, 0, h->stream>>>(h->f_dudt, forig, n, 0, 3, stg);
        else
            k_unpermute_words<<<g, kBlock, 0, h->stream>>>((const int *)h->f_drho, forig, n, 1, (int *)stg);
        break;
    case FSIM_FLUID_CELL_ID:
        if (!h->f_sorted) {
            fsim_set_error("cell ids unavailable before the first cell phase");
            return FSIM_EINVAL;
        }
        k_unpermute_words<<<g, kBlock, 0, h->stream>>>(h->f_cell, forig, n, 1, (int *)stg);
        break;
    case FSIM_SOLID_POS: k_unpermute_f4<<<g, kBlock, 0, h->stream>>>(h->s_pos[h->s_cur], sorig, n, 0, 3, stg); break;
    case FSIM_SOLID_VEL: k_unpermute_f4<<<g, kBlock, 0, h->stream>>>(h->s_vel[h->s_cur], sorig, n, 0, 3, stg); break;
    case FSIM_SOLID_REF_POS:
        k_unpermute_f4<<<g, kBlock, 0, h->stream>>>(h->s_ref[h->s_cur], sorig, n, 0, 3, stg);
        break;
    case FSIM_SOLID_TYPE:
        k_unpermute_words<<<g, kBlock, 0, h->stream>>>(h->s_type[h->s_cur], sorig, n, 1, (int *)stg);
        break;
    case FSIM_SOLID_CELL_ID:
        if (!h->s_sorted) {
            fsim_set_error("cell ids unavailable before the first cell phase");
            return FSIM_EINVAL;
        }
        k_unpermute_words<<<g, kBlock, 0, h->stream>>>(h->s_cell, sorig, n, 1, (int *)stg);
        break;
    case FSIM_SOLID_NORMAL:
    case FSIM_SOLID_P:
        if (!h->s_np_ok) {
            fsim_set_error("solid normal/pressure are stale after a cell phase; run the coupling phase first");
            return FSIM_EINVAL;
        }
        if (field == FSIM_SOLID_NORMAL) k_unpermute_f4<<<g, kBlock, 0, h->stream>>>(h->s_np, sorig, n, 0, 3, stg);
        else k_unpermute_f4<<<g, kBlock, 0, h->stream>>>(h->s_np, sorig, n, 3, 1, stg);
        break;
    case FSIM_SOLID_DU_DT:
    case FSIM_SOLID_COUPLE_DUDT:
    case FSIM_SOLID_F:
    case FSIM_SOLID_PK1:
    case FSIM_SOLID_LINV:
        if (!h->s_mech_ok) {
            fsim_set_error("solid stress products are stale after a cell phase; run the solid phase first");
            return FSIM_EINVAL;
        }
        if (field == FSIM_SOLID_DU_DT) k_unpermute_f4<<<g, kBlock, 0, h->stream>>>(h->s_dudt, sorig, n, 0, 3, stg);
        else if (field == FSIM_SOLID_COUPLE_DUDT)
            k_unpermute_f4<<<g, kBlock, 0, h->stream>>>(h->s_couple, sorig, n, 0, 3, stg);
        else {
            const float *src = field == FSIM_SOLID_F ? h->s_F : field == FSIM_SOLID_PK1 ? h->s_P : h->s_L;
            k_unpermute_words<<<g, kBlock, 0, h->stream>>>((const int *)src, sorig, n, 9, (int *)stg);
        }
        break;
    case FSIM_VIRT_POS: k_unpermute_f4<<<g, kBlock, 0, h->stream>>>(h->v_posr, h->v_orig, n, 0, 3, stg); break;
    case FSIM_VIRT_RHO: k_unpermute_f4<<<g, kBlock, 0, h->stream>>>(h->v_posr, h->v_orig, n, 3, 1, stg); break;
    case FSIM_VIRT_VEL: k_unpermute_f4<<<g, kBlock, 0, h->stream>>>(h->v_velp, h->v_orig, n, 0, 3, stg); break;
    case FSIM_VIRT_P: k_unpermute_f4<<<g, kBlock, 0, h->stream>>>(h->v_velp, h->v_orig, n, 3, 1, stg); break;
    case FSIM_VIRT_NORMAL: k_unpermute_f4<<<g, kBlock, 0, h->stream>>>(h->v_normal, h->v_orig, n, 0, 3, stg); break;
    case FSIM_VIRT_CELL_ID:
        k_unpermute_words<<<g, kBlock, 0, h->stream>>>(h->v_cell, h->v_orig, n, 1, (int *)stg);
        break;
    default: return FSIM_EINVAL;
    }
    CK_LAUNCH();
    return FSIM_OK;
}
} // namespace

extern "C" fsim_status fsim_get_field(fsim_handle h, int field, void *dst, size_t bytes)
{
    if (!h || (!dst && bytes)) return FSIM_EINVAL;
    if (h->batch) batch_wait(h);
    int n = 0;
    fsim_status st = check_field_bytes(h, field, bytes, &n);
    if (st) return st;
    if (n == 0) return FSIM_OK;
    DeviceGuard guard(h->device);
    float *stg = (float *)h->staging;
    if ((st = enqueue_unpermute(h, field, n, stg))) return st;
    CK(cudaMemcpyAsync(dst, stg, bytes, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return FSIM_OK;
}

namespace {
// The destination of a settable field; FSIM_EINVAL for the others.
fsim_status set_target(fsim_sim *h, int field, float4 **dst, const int **orig, int *comp)
{
    switch (field) {
    case FSIM_FLUID_POS: *dst = h->f_posr[h->f_cur]; *comp = 0; break;
    case FSIM_FLUID_RHO: *dst = h->f_posr[h->f_cur]; *comp = 3; break;
    case FSIM_FLUID_VEL: *dst = h->f_velp[h->f_cur]; *comp = 0; break;
    case FSIM_FLUID_P: *dst = h->f_velp[h->f_cur]; *comp = 3; break;
    case FSIM_SOLID_POS: *dst = h->s_pos[h->s_cur]; *comp = 0; break;
    case FSIM_SOLID_VEL: *dst = h->s_vel[h->s_cur]; *comp = 0; break;
    default: fsim_set_error("field %d is not settable", field); return FSIM_EINVAL;
    }
    *orig = field < 10 ? h->f_orig[h->f_cur] : h->s_orig[h->s_cur];
    if (h->mixed && field == FSIM_FLUID_P) {
        fsim_set_error("in the mixed form the fluid pressure is the EOS of the density; set FSIM_FLUID_RHO");
        return FSIM_EINVAL;
    }
    return FSIM_OK;
}

// Enqueue on the handle's stream the kernel that scatters `field` (input
// order, device memory `stg`) into the state (n > 0).
fsim_status enqueue_permute_in(fsim_sim *h, int field, int n, const float *stg)
{
    float4 *dst = nullptr;
    const int *orig = nullptr;
    int comp = 0;
    fsim_status st = set_target(h, field, &dst, &orig, &comp);
    if (st) return st;
    const int width = fsim_field_width(field);
    if (h->mixed && (field == FSIM_FLUID_POS || field == FSIM_FLUID_RHO))
        k_permute_in_mixed<<<blocks_for(n, kBlock), kBlock, 0, h->stream>>>(
            h->P, h->f_posr[h->f_cur], h->f_velp[h->f_cur], h->f_cell, orig, n,
            field == FSIM_FLUID_POS ? MF_POS : MF_RHO, stg);
    else
        k_permute_in_f4<<<blocks_for(n, kBlock), kBlock, 0, h->stream>>>(dst, orig, n, comp, width, stg);
    CK_LAUNCH();
    return FSIM_OK;
}
} // namespace

extern "C" fsim_status fsim_set_field(fsim_handle h, int field, const void *src, size_t bytes)
{
    if (!h || (!src && bytes)) return FSIM_EINVAL;
    if (h->batch) batch_wait(h);
    float4 *dst = nullptr;
    const int *orig = nullptr;
    int comp = 0, n = 0;
    fsim_status st = set_target(h, field, &dst, &orig, &comp);
    if (st) return st;
    if ((st = check_field_bytes(h, field, bytes, &n))) return st;
    if (n == 0) return FSIM_OK;
    DeviceGuard guard(h->device);
    CK(cudaMemcpyAsync(h->staging, src, bytes, cudaMemcpyHostToDevice, h->stream));
    if ((st = enqueue_permute_in(h, field, n, (const float *)h->staging))) return st;
    if (h->batch) CK(cudaStreamSynchronize(h->stream)); // the batch stream must see it
    return FSIM_OK;
}

namespace {
// Device buffer for several fields at once, grown on demand; a copy stream
// and events so that copies overlap the (un)permute kernels.
fsim_status bulk_reserve(fsim_sim *h, size_t bytes, int nev)
{
    if (bytes > h->bulk_bytes) {
        if (h->bulk) cudaFree(h->bulk);
        h->bulk = nullptr;
        h->bulk_bytes = 0;
        cudaError_t e = cudaMalloc(&h->bulk, bytes);
        if (e != cudaSuccess) {
            cudaGetLastError();
            fsim_set_error("cudaMalloc of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
            return FSIM_ENOMEM;
        }
        h->bulk_bytes = bytes;
    }
    if (!h->copy_stream) CK(cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking));
    while ((int)h->xfer_events.size() < nev) {
        cudaEvent_t e;
        CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        h->xfer_events.push_back(e);
    }
    return FSIM_OK;
}
} // namespace

extern "C" fsim_status fsim_get_fields(fsim_handle h, int nfields, const int *fields, void *const *dst,
                                       const size_t *bytes)
{
    if (!h || nfields < 0 || (nfields && (!fields || !dst || !bytes))) return FSIM_EINVAL;
    if (h->batch) batch_wait(h);
    std::vector<int> counts(nfields);
    size_t total = 0;
    for (int k = 0; k < nfields; ++k) {
        fsim_status st = check_field_bytes(h, fields[k], bytes[k], &counts[k]);
        if (st) return st;
        if (bytes[k] && !dst[k]) return FSIM_EINVAL;
        total += (bytes[k] + 255) & ~size_t(255);
    }
    DeviceGuard guard(h->device);
    fsim_status st = bulk_reserve(h, total, nfields);
    if (st) return st;
    size_t off = 0;
    for (int k = 0; k < nfields; ++k) {
        if (!counts[k]) continue;
        float *stg = reinterpret_cast<float *>(static_cast<char *>(h->bulk) + off);
        if ((st = enqueue_unpermute(h, fields[k], counts[k], stg))) return st;
        CK(cudaEventRecord(h->xfer_events[k], h->stream));
        CK(cudaStreamWaitEvent(h->copy_stream, h->xfer_events[k], 0));
        CK(cudaMemcpyAsync(dst[k], stg, bytes[k], cudaMemcpyDeviceToHost, h->copy_stream));
        off += (bytes[k] + 255) & ~size_t(255);
    }
    CK(cudaStreamSynchronize(h->copy_stream));
    return FSIM_OK;
}

extern "C" fsim_status fsim_set_fields(fsim_handle h, int nfields, const int *fields, const void *const *src,
                                       const size_t *bytes)
{
    if (!h || nfields < 0 || (nfields && (!fields || !src || !bytes))) return FSIM_EINVAL;
    if (h->batch) batch_wait(h);
    std::vector<int> counts(nfields);
    size_t total = 0;
    for (int k = 0; k < nfields; ++k) {
        float4 *d;
        const int *o;
        int c;
        fsim_status st = set_target(h, fields[k], &d, &o, &c);
        if (st) return st;
        if ((st = check_field_bytes(h, fields[k], bytes[k], &counts[k]))) return st;
        if (bytes[k] && !src[k]) return FSIM_EINVAL;
        total += (bytes[k] + 255) & ~size_t(255);
    }
    DeviceGuard guard(h->device);
    fsim_status st = bulk_reserve(h, total, nfields);
    if (st) return st;
    // the copies start after the handle's queued work (they overwrite the bulk buffer)
    CK(cudaEventRecord(h->ev1, h->stream));
    CK(cudaStreamWaitEvent(h->copy_stream, h->ev1, 0));
    size_t off = 0;
    for (int k = 0; k < nfields; ++k) {
        if (!counts[k]) continue;
        float *stg = reinterpret_cast<float *>(static_cast<char *>(h->bulk) + off);
        CK(cudaMemcpyAsync(stg, src[k], bytes[k], cudaMemcpyHostToDevice, h->copy_stream));
        CK(cudaEventRecord(h->xfer_events[k], h->copy_stream));
        CK(cudaStreamWaitEvent(h->stream, h->xfer_events[k], 0));
        if ((st = enqueue_permute_in(h, fields[k], counts[k], stg))) return st;
        off += (bytes[k] + 255) & ~size_t(255);
    }
    CK(cudaStreamSynchronize(h->copy_stream)); // the host buffers may be reused on return
    if (h->batch) CK(cudaStreamSynchronize(h->stream));
    return FSIM_OK;
}

extern "C" fsim_status fsim_probe(fsim_handle h, const float *points, int n, float *out)
{
    if (!h || n < 0 || (n && (!points || !out))) return FSIM_EINVAL;
    if (h->batch) batch_wait(h);
    if (!h->f_sorted || !h->s_sorted) {
        fsim_set_error("run FSIM_PHASE_CELL (or a step) first");
        return FSIM_EINVAL;
    }
    if (!n) return FSIM_OK;
    DeviceGuard guard(h->device);
    float *d = nullptr;
    CK(cudaMalloc((void **)&d, sizeof(float) * 8 * (size_t)n));
    ProbeArgs A;
    A.pts = d;
    A.n = n;
    A.out = d + 3 * (size_t)n;
    A.fposr = h->f_posr[h->f_cur];
    A.fvelp = h->f_velp[h->f_cur];
    A.start_f = h->f_start;
    A.s_pos = h->s_pos[h->s_cur];
    A.s_vel = h->s_vel[h->s_cur];
    A.s_np = h->s_np;
    A.start_s = h->s_start;
    cudaError_t e = cudaMemcpyAsync(d, points, sizeof(float) * 3 * n, cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) {
        k_probe<<<blocks_for(32ll * n, kBlock), kBlock, 0, h->stream>>>(h->P, A);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(out, A.out, sizeof(float) * 5 * n, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    cudaFree(d);
    if (e != cudaSuccess) {
        fsim_set_error("probe failed: %s", cudaGetErrorString(e));
        return FSIM_ECUDA;
    }
    return FSIM_OK;
}

extern "C" fsim_status fsim_neighbor_counts(fsim_handle h, int *out, size_t bytes)
{
    if (!h || (!out && bytes)) return FSIM_EINVAL;
    if (h->batch) batch_wait(h);
    if (bytes != (size_t)h->nf * 3 * 4) {
        fsim_set_error("neighbor counts need %zu bytes", (size_t)h->nf * 12);
        return FSIM_EINVAL;
    }
    if (!h->f_sorted) {
        fsim_set_error("run FSIM_PHASE_CELL first");
        return FSIM_EINVAL;
    }
    if (h->mixed) {
        fsim_set_error("neighbour counts are a check of the plain form's FP32 pair set");
        return FSIM_EINVAL;
    }
    if (!h->nf) return FSIM_OK;
    DeviceGuard guard(h->device);
    int *d_counts = (int *)h->staging; // 3 * nf words fit the staging buffer
    const int g = blocks_for(h->nf, kBlock);
    k_neighbor_counts<<<g, kBlock, 0, h->stream>>>(h->P, h->f_posr[h->f_cur], h->f_cell, h->f_start,
                                                    h->s_pos[h->s_cur], h->s_start, h->v_posr, h->v_start, d_counts,
                                                    h->nf);
    CK_LAUNCH();
    // reorder to input order in place is not possible; copy sorted and unpermute on the host
    std::vector<int> sorted(3 * (size_t)h->nf), orig(h->nf);
    CK(cudaMemcpyAsync(sorted.data(), d_counts, bytes, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaMemcpyAsync(orig.data(), h->f_orig[h->f_cur], sizeof(int) * h->nf, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    for (int s = 0; s < h->nf; ++s)
        for (int k = 0; k < 3; ++k) out[3 * orig[s] + k] = sorted[3 * s + k];
    return FSIM_OK;
}

extern "C" fsim_status fsim_get_cells(fsim_handle h, int species, int *cell_start, size_t start_bytes, int *ids,
                                      size_t ids_bytes)
{
    if (!h || species < 0 || species > 2) return FSIM_EINVAL;
    if (h->batch) batch_wait(h);
    const int n = species == 0 ? h->nf : species == 1 ? h->ns : h->nv;
    if (start_bytes != (size_t)(h->ncell + 1) * 4 || ids_bytes != (size_t)n * 4 || !cell_start || (n && !ids)) {
        fsim_set_error("fsim_get_cells: wrong buffer sizes");
        return FSIM_EINVAL;
    }
    if ((species == 0 && !h->f_sorted) || (species == 1 && !h->s_sorted)) {
        fsim_set_error("run FSIM_PHASE_CELL first");
        return FSIM_EINVAL;
    }
    DeviceGuard guard(h->device);
    const int *start = species == 0 ? h->f_start : species == 1 ? h->s_start : h->v_start;
    const int *orig = species == 0 ? h->f_orig[h->f_cur] : species == 1 ? h->s_orig[h->s_cur] : h->v_orig;
    CK(cudaMemcpyAsync(cell_start, start, start_bytes, cudaMemcpyDeviceToHost, h->stream));
    if (n) CK(cudaMemcpyAsync(ids, orig, ids_bytes, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return FSIM_OK;
}

namespace {
fsim_status write_vtk(fsim_handle h, const char *out_dir, int file_step, bool binary)
{
    if (!h || !out_dir) return FSIM_EINVAL;
    std::vector<float> fpos(3 * (size_t)h->nf), fvel(3 * (size_t)h->nf), frho(h->nf), fp(h->nf);
    std::vector<float> spos(3 * (size_t)h->ns), svel(3 * (size_t)h->ns), sp(h->ns), snormal(3 * (size_t)h->ns);
    std::vector<float> vpos(3 * (size_t)h->nv), vnormal(3 * (size_t)h->nv), vp(h->nv);
    fsim_status st;
    if ((st = fsim_get_field(h, FSIM_FLUID_POS, fpos.data(), fpos.size() * 4)) ||
        (st = fsim_get_field(h, FSIM_FLUID_VEL, fvel.data(), fvel.size() * 4)) ||
        (st = fsim_get_field(h, FSIM_FLUID_RHO, frho.data(), frho.size() * 4)) ||
        (st = fsim_get_field(h, FSIM_FLUID_P, fp.data(), fp.size() * 4)) ||
        (st = fsim_get_field(h, FSIM_SOLID_POS, spos.data(), spos.size() * 4)) ||
        (st = fsim_get_field(h, FSIM_SOLID_VEL, svel.data(), svel.size() * 4)) ||
        (st = fsim_get_field(h, FSIM_VIRT_POS, vpos.data(), vpos.size() * 4)) ||
        (st = fsim_get_field(h, FSIM_VIRT_NORMAL, vnormal.data(), vnormal.size() * 4)) ||
        (st = fsim_get_field(h, FSIM_VIRT_P, vp.data(), vp.size() * 4)))
        return st;
    if (h->ns && h->s_np_ok) {
        if ((st = fsim_get_field(h, FSIM_SOLID_P, sp.data(), sp.size() * 4)) ||
            (st = fsim_get_field(h, FSIM_SOLID_NORMAL, snormal.data(), snormal.size() * 4)))
            return st;
    }
    VtkHostState vs;
    vs.n_fluid = h->nf;
    vs.n_solid = h->ns;
    vs.n_virt = h->nv;
    vs.fpos = fpos.data();
    vs.fvel = fvel.data();
    vs.frho = frho.data();
    vs.fp = fp.data();
    vs.spos = spos.data();
    vs.svel = svel.data();
    vs.sp = sp.data();
    vs.snormal = snormal.data();
    vs.solid_density = h->cfg.solid_density;
    vs.vpos = vpos.data();
    vs.vnormal = vnormal.data();
    vs.vp = vp.data();
    return fsim_write_vtk_host(out_dir, file_step, vs, binary);
}
} // namespace

extern "C" fsim_status fsim_write_vtk(fsim_handle h, const char *out_dir, int file_step)
{
    return write_vtk(h, out_dir, file_step, false);
}

extern "C" fsim_status fsim_write_vtk_binary(fsim_handle h, const char *out_dir, int file_step)
{
    return write_vtk(h, out_dir, file_step, true);
}

extern "C" fsim_status fsim_time_steps(fsim_handle h, int nsteps, float *ms)
{
    if (!h || nsteps < 0 || !ms) return FSIM_EINVAL;
    if (h->batch) {
        fsim_set_error("the handle belongs to a batch; time the batch");
        return FSIM_EINVAL;
    }
    DeviceGuard guard(h->device);
    // capture outside the timed region
    fsim_status st;
    CK(cudaEventRecord(h->ev0, h->stream));
    for (int k = 0; k < nsteps; ++k)
        if ((st = run_step_graph(h))) return st;
    CK(cudaEventRecord(h->ev1, h->stream));
    CK(cudaEventSynchronize(h->ev1));
    CK(cudaEventElapsedTime(ms, h->ev0, h->ev1));
    return check_flags(h);
}

extern "C" fsim_status fsim_time_sweep(fsim_handle h, int nsteps, float *total_ms, float *sweep_ms)
{
    if (!h || nsteps < 0 || !total_ms || !sweep_ms) return FSIM_EINVAL;
    if (h->batch) {
        fsim_set_error("the handle belongs to a batch; time the batch");
        return FSIM_EINVAL;
    }
    DeviceGuard guard(h->device);
    while ((int)h->sweep_events.size() < 2 * nsteps) {
        cudaEvent_t e;
        CK(cudaEventCreate(&e));
        h->sweep_events.push_back(e);
    }
    fsim_status st = FSIM_OK;
    CK(cudaEventRecord(h->ev0, h->stream));
    for (int k = 0; k < nsteps; ++k) {
        Plan *pl = nullptr;
        if ((st = handle_step_plan(h, &pl))) return st;
        if ((st = enqueue_plan(*pl, h->stream, h->tuner.shape(), h->sweep_events[2 * k], h->sweep_events[2 * k + 1])))
            return st;
        after_plan(h, kAllPhases, *pl);
    }
    CK(cudaEventRecord(h->ev1, h->stream));
    CK(cudaEventSynchronize(h->ev1));
    CK(cudaEventElapsedTime(total_ms, h->ev0, h->ev1));
    float sum = 0.0f;
    if (h->nf) {
        for (int k = 0; k < nsteps; ++k) {
            float t = 0.0f;
            CK(cudaEventElapsedTime(&t, h->sweep_events[2 * k], h->sweep_events[2 * k + 1]));
            sum += t;
        }
    }
    *sweep_ms = sum;
    return check_flags(h);
}

extern "C" fsim_status fsim_launches_per_step(fsim_handle h, int *n)
{
    if (!h || !n) return FSIM_EINVAL;
    DeviceGuard guard(h->device);
    Plan *pl = nullptr;
    fsim_status st = handle_step_plan(h, &pl);
    if (st) return st;
    *n = (int)pl->launches.size();
    return FSIM_OK;
}

extern "C" fsim_status fsim_conservation(fsim_handle h, double *out, int n_out)
{
    if (!h || !out || n_out < 1) return FSIM_EINVAL;
    if (h->batch) batch_wait(h);
    DeviceGuard guard(h->device);
    const int bf = blocks_for(h->nf, kBlock), bs = blocks_for(h->ns, kBlock);
    const size_t words = (size_t)(bf + bs) * FSIM_CONSERVATION_N;
    double *d_part = nullptr;
    CK(cudaMalloc((void **)&d_part, sizeof(double) * (words ? words : 1)));
    const double vol = (double)h->der.particle_volume;
    cudaError_t e = cudaSuccess;
    if (bf)
        k_conservation_fluid<<<bf, kBlock, 0, h->stream>>>(h->P, h->f_posr[h->f_cur], h->f_velp[h->f_cur], h->f_cell,
                                                            h->nf, vol, d_part);
    if (bs)
        k_conservation_solid<<<bs, kBlock, 0, h->stream>>>(h->P, h->s_pos[h->s_cur], h->s_vel[h->s_cur], h->s_F, h->ns,
                                                            (double)h->cfg.solid_density, vol,
                                                            d_part + (size_t)bf * FSIM_CONSERVATION_N);
    e = cudaGetLastError();
    std::vector<double> part(words);
    if (e == cudaSuccess && words)
        e = cudaMemcpyAsync(part.data(), d_part, sizeof(double) * words, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    cudaFree(d_part);
    if (e != cudaSuccess) {
        fsim_set_error("conservation sums failed: %s", cudaGetErrorString(e));
        return FSIM_ECUDA;
    }
    double tot[FSIM_CONSERVATION_N] = {};
    for (int b = 0; b < bf + bs; ++b)
        for (int k = 0; k < FSIM_CONSERVATION_N; ++k) tot[k] += part[(size_t)b * FSIM_CONSERVATION_N + k];
    for (int k = 0; k < n_out && k < FSIM_CONSERVATION_N; ++k) out[k] = tot[k];
    for (int k = FSIM_CONSERVATION_N; k < n_out; ++k) out[k] = 0.0;
    return FSIM_OK;
}

// =================================================================== snapshots
// Binary snapshot of an instance: a fixed header, then the device arrays that
// define the state in their current (cell-sorted) order, so that an instance
// restored from it continues bit for bit like the original.  Per-step products
// (cell starts, solid stress, derivatives) are recomputed by the next step.
namespace {
struct SnapHeader {
    char magic[8];
    uint32_t version, config_bytes;
    int64_t step;
    int32_t n_fluid, n_solid, n_virt, ncell;
    uint64_t payload_bytes;
    fsim_config cfg;
};
constexpr char kSnapMagic[8] = {'F', 'S', 'I', 'M', 'S', 'N', 'P', '1'};
constexpr size_t kSnapHeaderBytes = 512; // header padded; arrays start 16-byte aligned
static_assert(sizeof(SnapHeader) <= kSnapHeaderBytes, "snapshot header");

struct SnapArray {
    void *dev;
    size_t bytes;
};
std::vector<SnapArray> snap_arrays(fsim_sim *h, int pf, int ps)
{
    const size_t nf = h->nf, ns = h->ns, nv = h->nv, nc = h->ncell;
    return {{h->f_posr[pf], 16 * nf}, {h->f_velp[pf], 16 * nf}, {h->f_orig[pf], 4 * nf},   {h->f_cell, 4 * nf},
            {h->s_pos[ps], 16 * ns},  {h->s_vel[ps], 16 * ns},  {h->s_ref[ps], 16 * ns},   {h->s_type[ps], 4 * ns},
            {h->s_orig[ps], 4 * ns},  {h->v_posr, 16 * nv},     {h->v_velp, 16 * nv},      {h->v_normal, 16 * nv},
            {h->v_orig, 4 * nv},      {h->v_cell, 4 * nv},      {h->v_start, 4 * (nc + 1)}};
}
size_t snap_payload(fsim_sim *h)
{
    size_t b = 0;
    for (const SnapArray &a : snap_arrays(h, 0, 0)) b += (a.bytes + 15) & ~size_t(15);
    return b;
}
} // namespace

extern "C" fsim_status fsim_snapshot_bytes(fsim_handle h, size_t *bytes)
{
    if (!h || !bytes) return FSIM_EINVAL;
    *bytes = kSnapHeaderBytes + snap_payload(h);
    return FSIM_OK;
}

extern "C" fsim_status fsim_snapshot_save(fsim_handle h, long long step, void *buf, size_t bytes)
{
    if (!h || !buf) return FSIM_EINVAL;
    if (h->batch) batch_wait(h);
    const size_t need = kSnapHeaderBytes + snap_payload(h);
    if (bytes != need) {
        fsim_set_error("a snapshot of this instance takes %zu bytes, got %zu", need, bytes);
        return FSIM_EINVAL;
    }
    DeviceGuard guard(h->device);
    SnapHeader hd;
    std::memset(&hd, 0, sizeof hd);
    std::memcpy(hd.magic, kSnapMagic, 8);
    hd.version = 1;
    hd.config_bytes = sizeof(fsim_config);
    hd.step = step;
    hd.n_fluid = h->nf;
    hd.n_solid = h->ns;
    hd.n_virt = h->nv;
    hd.ncell = h->ncell;
    hd.payload_bytes = need - kSnapHeaderBytes;
    hd.cfg = h->cfg;
    char *out = static_cast<char *>(buf);
    std::memset(out, 0, kSnapHeaderBytes);
    std::memcpy(out, &hd, sizeof hd);
    size_t off = kSnapHeaderBytes;
    for (const SnapArray &a : snap_arrays(h, h->f_cur, h->s_cur)) {
        if (a.bytes) CK(cudaMemcpyAsync(out + off, a.dev, a.bytes, cudaMemcpyDeviceToHost, h->stream));
        const size_t padded = (a.bytes + 15) & ~size_t(15);
        if (padded > a.bytes) std::memset(out + off + a.bytes, 0, padded - a.bytes);
        off += padded;
    }
    CK(cudaStreamSynchronize(h->stream));
    return FSIM_OK;
}

extern "C" fsim_status fsim_snapshot_load(const void *buf, size_t bytes, int device, fsim_handle *out,
                                          long long *step)
{
    if (!buf || !out) return FSIM_EINVAL;
    *out = nullptr;
    SnapHeader hd;
    if (bytes < kSnapHeaderBytes) {
        fsim_set_error("snapshot too short");
        return FSIM_EIO;
    }
    std::memcpy(&hd, buf, sizeof hd);
    if (std::memcmp(hd.magic, kSnapMagic, 8) || hd.version != 1 || hd.config_bytes != sizeof(fsim_config) ||
        hd.n_fluid < 0 || hd.n_solid < 0 || hd.n_virt < 0) {
        fsim_set_error("not a version-1 fluidsim snapshot");
        return FSIM_EIO;
    }
    fsim_sim *h = nullptr;
    fsim_status st = new_handle(&hd.cfg, hd.n_fluid, hd.n_solid, hd.n_virt, device, &h);
    if (st) return st;
    if (h->ncell != hd.ncell || bytes != kSnapHeaderBytes + snap_payload(h) ||
        hd.payload_bytes != bytes - kSnapHeaderBytes) {
        fsim_set_error("snapshot size does not match its header");
        delete h;
        return FSIM_EIO;
    }
    DeviceGuard guard(h->device);
    if ((st = alloc_state(h))) {
        free_all(h);
        delete h;
        return st;
    }
    const char *in = static_cast<const char *>(buf);
    size_t off = kSnapHeaderBytes;
    const int ns = h->ns;
    std::vector<float> ref(3 * (size_t)ns);
    const char *ref_src = nullptr, *orig_src = nullptr;
    cudaError_t e = cudaSuccess;
    for (const SnapArray &a : snap_arrays(h, 0, 0)) {
        if (a.bytes && e == cudaSuccess) e = cudaMemcpy(a.dev, in + off, a.bytes, cudaMemcpyHostToDevice);
        if (a.dev == h->s_ref[0]) ref_src = in + off;
        if (a.dev == h->s_orig[0]) orig_src = in + off;
        off += (a.bytes + 15) & ~size_t(15);
    }
    if (e != cudaSuccess) {
        fsim_set_error("snapshot upload failed: %s", cudaGetErrorString(e));
        free_all(h);
        delete h;
        return FSIM_ECUDA;
    }
    // solid: F = L = I, P = 0 until the next solid phase; static neighbour lists
    // from the reference positions in input order
    if (ns) {
        for (int k = 0; k < ns; ++k) {
            int o;
            float r[4];
            std::memcpy(&o, orig_src + 4 * (size_t)k, 4);
            std::memcpy(r, ref_src + 16 * (size_t)k, 16);
            if (o < 0 || o >= ns) {
                fsim_set_error("corrupt snapshot (solid ids)");
                free_all(h);
                delete h;
                return FSIM_EIO;
            }
            std::memcpy(&ref[3 * (size_t)o], r, 12);
        }
        std::vector<float> eye(9 * (size_t)ns, 0.0f);
        for (int i = 0; i < ns; ++i) eye[9 * i] = eye[9 * i + 4] = eye[9 * i + 8] = 1.0f;
        e = cudaMemcpy(h->s_F, eye.data(), sizeof(float) * 9 * ns, cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(h->s_L, eye.data(), sizeof(float) * 9 * ns, cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemset(h->s_P, 0, sizeof(float) * 9 * ns);
        if (e == cudaSuccess) e = cudaMemset(h->s_dudt, 0, sizeof(float4) * ns);
        if (e == cudaSuccess) e = cudaMemset(h->s_couple, 0, sizeof(float4) * ns);
        if (e != cudaSuccess || (st = build_solid_neighbors(h, ref.data()))) {
            if (!st) fsim_set_error("snapshot restore failed: %s", cudaGetErrorString(e));
            free_all(h);
            delete h;
            return st ? st : FSIM_ECUDA;
        }
    }
    cudaStreamSynchronize(h->stream);
    h->f_cur = h->s_cur = 0;
    h->f_sorted = h->s_sorted = false;
    h->f_deriv_ok = h->s_np_ok = h->s_mech_ok = false;
    if (step) *step = hd.step;
    *out = h;
    return FSIM_OK;
}

extern "C" fsim_status fsim_snapshot_write(fsim_handle h, long long step, const char *path)
{
    if (!h || !path) return FSIM_EINVAL;
    size_t n = 0;
    fsim_status st = fsim_snapshot_bytes(h, &n);
    if (st) return st;
    std::vector<char> buf(n);
    if ((st = fsim_snapshot_save(h, step, buf.data(), n))) return st;
    FILE *f = std::fopen(path, "wb");
    if (!f) {
        fsim_set_error("cannot open %s for writing", path);
        return FSIM_EIO;
    }
    const bool ok = std::fwrite(buf.data(), 1, n, f) == n;
    if (std::fclose(f) != 0 || !ok) {
        fsim_set_error("writing %s failed", path);
        return FSIM_EIO;
    }
    return FSIM_OK;
}

extern "C" fsim_status fsim_snapshot_read(const char *path, int device, fsim_handle *out, long long *step)
{
    if (!path || !out) return FSIM_EINVAL;
    FILE *f = std::fopen(path, "rb");
    if (!f) {
        fsim_set_error("cannot open %s", path);
        return FSIM_EIO;
    }
    std::vector<char> buf;
    char chunk[1 << 16];
    size_t got;
    while ((got = std::fread(chunk, 1, sizeof chunk, f)) > 0) buf.insert(buf.end(), chunk, chunk + got);
    std::fclose(f);
    return fsim_snapshot_load(buf.data(), buf.size(), device, out, step);
}

// =================================================================== case on the device
namespace {
fsim_status case_geometry(const fsim_case *cs, CaseGeom &g)
{
    if (!(cs->dx > 0.0f) || cs->tank_n[0] <= 0 || cs->tank_n[1] <= 0 || cs->tank_n[2] <= 0 || cs->virt_layers < 0 ||
        cs->solid_fixed_layers < 0) {
        fsim_set_error("invalid case description");
        return FSIM_EINVAL;
    }
    for (int a = 0; a < 3; ++a) {
        g.T[a] = cs->tank_n[a];
        g.FN[a] = cs->fluid_n[a];
        g.SL[a] = cs->solid_lo[a];
        g.SN[a] = cs->solid_n[a];
    }
    g.fixed_layers = cs->solid_fixed_layers;
    g.L = cs->virt_layers;
    g.has_solid = cs->solid_n[0] > 0 && cs->solid_n[1] > 0 && cs->solid_n[2] > 0;
    g.dx = cs->dx;
    g.jit = (double)cs->jitter * (double)cs->dx;
    g.jitter = g.jit > 0.0;
    g.seed = cs->seed;
    const double sites = (double)(g.T[0] + 2 * g.L) * (g.T[1] + 2 * g.L) * (g.T[2] + 2 * g.L);
    if (sites > 2e9) {
        fsim_set_error("case lattice too large");
        return FSIM_EINVAL;
    }
    return FSIM_OK;
}

// per-row bases and the totals
void case_rows(const CaseGeom &g, std::vector<RowBase> &base, long long tot[4])
{
    const int ni = g.T[0] + 2 * g.L, nj = g.T[1] + 2 * g.L;
    base.resize((size_t)ni * nj);
    tot[0] = tot[1] = tot[2] = tot[3] = 0;
    for (int i = -g.L; i < g.T[0] + g.L; ++i)
        for (int j = -g.L; j < g.T[1] + g.L; ++j) {
            RowIv r;
            case_row(g, i, j, r);
            int c[4];
            case_row_counts(g, r, c);
            RowBase &b = base[(size_t)(i + g.L) * nj + (j + g.L)];
            b.f = (int)tot[0];
            b.s = (int)tot[1];
            b.v = (int)tot[2];
            b.pad = 0;
            b.d = tot[3];
            for (int a = 0; a < 4; ++a) tot[a] += c[a];
        }
}
} // namespace

extern "C" fsim_status fsim_case_counts(const fsim_case *cs, int *n_fluid, int *n_solid, int *n_virt)
{
    if (!cs || !n_fluid || !n_solid || !n_virt) return FSIM_EINVAL;
    CaseGeom g;
    fsim_status st = case_geometry(cs, g);
    if (st) return st;
    std::vector<RowBase> base;
    long long tot[4];
    case_rows(g, base, tot);
    if (tot[0] > INT_MAX || tot[1] > INT_MAX || tot[2] > INT_MAX) {
        fsim_set_error("case too large");
        return FSIM_EINVAL;
    }
    *n_fluid = (int)tot[0];
    *n_solid = (int)tot[1];
    *n_virt = (int)tot[2];
    return FSIM_OK;
}

extern "C" fsim_status fsim_create_case(const fsim_config *cfg, const fsim_case *cs, int device, fsim_handle *out)
{
    if (!cfg || !cs || !out) return FSIM_EINVAL;
    *out = nullptr;
    CaseGeom g;
    fsim_status st = case_geometry(cs, g);
    if (st) return st;
    std::vector<RowBase> base;
    long long tot[4];
    case_rows(g, base, tot);
    if (tot[0] > INT_MAX || tot[1] > INT_MAX || tot[2] > INT_MAX) {
        fsim_set_error("case too large");
        return FSIM_EINVAL;
    }
    // hydrostatic (rho, p) per fluid lattice row, as fsim_case_generate computes them
    std::vector<float2> hydro(g.FN[1] > 0 ? g.FN[1] : 1, make_float2(cfg->fluid_density, 0.0f));
    if (cs->hydrostatic) {
        const double rho0 = cfg->fluid_density, c0 = cfg->fluid_sound_speed, gam = cfg->gamma, gr = cfg->gravity;
        const double H = g.FN[1] * g.dx, p2rho = gam / (rho0 * c0 * c0);
        for (int j = 0; j < g.FN[1]; ++j) {
            const double y = (j + 0.5) * g.dx;
            const double p = rho0 * gr * (H - y);
            const double rho = rho0 * std::pow(p * p2rho + 1.0, 1.0 / gam);
            hydro[j] = make_float2((float)rho, (float)p);
        }
    }
    fsim_sim *h = nullptr;
    if ((st = new_handle(cfg, (int)tot[0], (int)tot[1], (int)tot[2], device, &h))) return st;
    DeviceGuard guard(h->device);
    auto fail = [&](fsim_status code) {
        free_all(h);
        delete h;
        return code;
    };
    if ((st = alloc_state(h))) return fail(st);
    RowBase *d_base = nullptr;
    float2 *d_hydro = nullptr;
    float4 *d_vpos = nullptr;
    if ((st = dalloc(h, &d_base, base.size())) || (st = dalloc(h, &d_hydro, hydro.size())) ||
        (st = dalloc(h, &d_vpos, (size_t)h->nv)))
        return fail(st);
    CK(cudaMemcpyAsync(d_base, base.data(), sizeof(RowBase) * base.size(), cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(d_hydro, hydro.data(), sizeof(float2) * hydro.size(), cudaMemcpyHostToDevice, h->stream));
    CaseGenArgs A;
    A.g = g;
    A.base = d_base;
    A.hydro = d_hydro;
    A.rho0 = h->P.rho0;
    A.fposr = h->f_posr[0];
    A.fvelp = h->f_velp[0];
    A.forig = h->f_orig[0];
    A.spos = h->s_pos[0];
    A.svel = h->s_vel[0];
    A.sref = h->s_ref[0];
    A.stype = h->s_type[0];
    A.sorig = h->s_orig[0];
    A.vpos = d_vpos;
    A.nsite = (long long)(g.T[0] + 2 * g.L) * (g.T[1] + 2 * g.L) * (g.T[2] + 2 * g.L);
    k_case_generate<<<blocks_for(A.nsite, kBlock), kBlock, 0, h->stream>>>(A);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        fsim_set_error("case generation failed: %s", cudaGetErrorString(e));
        return fail(FSIM_ECUDA);
    }
    const int nf = h->nf, ns = h->ns;
    if (nf && h->mixed) {
        k_fluid_to_mixed<<<blocks_for(nf, kBlock), kBlock, 0, h->stream>>>(h->P, h->f_posr[0], h->f_velp[0],
                                                                           h->f_cell, nf, h->d_flags);
        CK(cudaGetLastError());
    }
    if (ns) {
        std::vector<float4> ref4(ns);
        CK(cudaMemcpyAsync(ref4.data(), h->s_ref[0], sizeof(float4) * ns, cudaMemcpyDeviceToHost, h->stream));
        CK(cudaStreamSynchronize(h->stream));
        std::vector<float> ref(3 * (size_t)ns);
        for (int k = 0; k < ns; ++k) {
            ref[3 * k] = ref4[k].x;
            ref[3 * k + 1] = ref4[k].y;
            ref[3 * k + 2] = ref4[k].z;
        }
        std::vector<float> eye(9 * (size_t)ns, 0.0f);
        for (int k = 0; k < ns; ++k) eye[9 * k] = eye[9 * k + 4] = eye[9 * k + 8] = 1.0f;
        CK(cudaMemcpy(h->s_F, eye.data(), sizeof(float) * 9 * ns, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(h->s_L, eye.data(), sizeof(float) * 9 * ns, cudaMemcpyHostToDevice));
        CK(cudaMemset(h->s_P, 0, sizeof(float) * 9 * ns));
        CK(cudaMemset(h->s_dudt, 0, sizeof(float4) * ns));
        CK(cudaMemset(h->s_couple, 0, sizeof(float4) * ns));
        h->s_mech_ok = h->s_np_ok = true;
        if ((st = build_solid_neighbors(h, ref.data()))) return fail(st);
    }
    if (h->nv) {
        if ((st = sort_virtual(h, nullptr, d_vpos))) return fail(st);
        if (h->mixed) {
            k_offsets_in_cells<<<blocks_for(h->nv, kBlock), kBlock, 0, h->stream>>>(h->P, h->v_posr, h->v_cell,
                                                                                     h->nv);
            CK(cudaGetLastError());
        }
    }
    // generation temporaries are released now
    CK(cudaStreamSynchronize(h->stream));
    void *tmps[] = {d_base, d_hydro, d_vpos};
    for (void *p : tmps) {
        cudaFree(p);
        for (auto it = h->allocations.begin(); it != h->allocations.end(); ++it)
            if (*it == p) {
                h->allocations.erase(it);
                break;
            }
    }
    if ((st = check_flags(h))) return fail(st);
    *out = h;
    return FSIM_OK;
}

extern "C" fsim_status fsim_counts(fsim_handle h, int *nf, int *ns, int *nv)
{
    if (!h) return FSIM_EINVAL;
    if (nf) *nf = h->nf;
    if (ns) *ns = h->ns;
    if (nv) *nv = h->nv;
    return FSIM_OK;
}

extern "C" fsim_status fsim_get_derived(fsim_handle h, fsim_derived *out)
{
    if (!h || !out) return FSIM_EINVAL;
    *out = h->der;
    return FSIM_OK;
}

extern "C" fsim_status fsim_host_alloc(size_t bytes, void **out)
{
    if (!out) return FSIM_EINVAL;
    *out = nullptr;
    cudaError_t e = cudaMallocHost(out, bytes ? bytes : 1);
    if (e != cudaSuccess) {
        cudaGetLastError();
        fsim_set_error("cudaMallocHost(%zu) failed: %s", bytes, cudaGetErrorString(e));
        return FSIM_ENOMEM;
    }
    return FSIM_OK;
}

extern "C" fsim_status fsim_host_free(void *p)
{
    if (p) cudaFreeHost(p);
    return FSIM_OK;
}

// =================================================================== batches
struct fsim_batch;
namespace {
} // namespace
struct fsim_batch {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    SweepTuner tuner;
    std::vector<fsim_sim *> members;
    Plan *plans[2][2] = {}; // by (fluid, solid) parity of the members
};

namespace {

void batch_wait(fsim_sim *h) { cudaStreamSynchronize(h->batch->stream); }

// Bring a member to buffer parities (pf, ps) by copying its current state
// into the other buffers (same order, so cell structures stay valid).
fsim_status set_parity(fsim_sim *h, int pf, int ps)
{
    if (h->f_cur != pf && h->nf) {
        const int a = h->f_cur, b = pf;
        CK(cudaMemcpyAsync(h->f_posr[b], h->f_posr[a], sizeof(float4) * h->nf, cudaMemcpyDeviceToDevice, h->stream));
        CK(cudaMemcpyAsync(h->f_velp[b], h->f_velp[a], sizeof(float4) * h->nf, cudaMemcpyDeviceToDevice, h->stream));
        CK(cudaMemcpyAsync(h->f_orig[b], h->f_orig[a], sizeof(int) * h->nf, cudaMemcpyDeviceToDevice, h->stream));
    }
    h->f_cur = pf;
    if (h->s_cur != ps && h->ns) {
        const int a = h->s_cur, b = ps;
        CK(cudaMemcpyAsync(h->s_pos[b], h->s_pos[a], sizeof(float4) * h->ns, cudaMemcpyDeviceToDevice, h->stream));
        CK(cudaMemcpyAsync(h->s_vel[b], h->s_vel[a], sizeof(float4) * h->ns, cudaMemcpyDeviceToDevice, h->stream));
        CK(cudaMemcpyAsync(h->s_ref[b], h->s_ref[a], sizeof(float4) * h->ns, cudaMemcpyDeviceToDevice, h->stream));
        CK(cudaMemcpyAsync(h->s_type[b], h->s_type[a], sizeof(int) * h->ns, cudaMemcpyDeviceToDevice, h->stream));
        CK(cudaMemcpyAsync(h->s_orig[b], h->s_orig[a], sizeof(int) * h->ns, cudaMemcpyDeviceToDevice, h->stream));
    }
    h->s_cur = ps;
    CK(cudaStreamSynchronize(h->stream));
    return FSIM_OK;
}

void free_batch(fsim_batch *b)
{
    for (auto &row : b->plans)
        for (Plan *&pl : row) {
            free_plan(pl);
            pl = nullptr;
        }
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    b->tuner.release();
    if (b->stream) cudaStreamDestroy(b->stream);
}

fsim_status batch_step_once(fsim_batch *b)
{
    if (b->members.empty()) return FSIM_OK;
    const int pf = b->members[0]->f_cur, ps = b->members[0]->s_cur;
    Plan *&pl = b->plans[pf][ps];
    if (!pl) {
        fsim_status st = build_plan(b->members, kAllPhases, pf, ps, &pl);
        if (st) return st;
    }
    fsim_status st = run_plan_step(*pl, b->stream, b->tuner);
    if (st) return st;
    for (fsim_sim *h : b->members) after_plan(h, kAllPhases, *pl);
    return FSIM_OK;
}

fsim_status batch_check_flags(fsim_batch *b)
{
    CK(cudaStreamSynchronize(b->stream));
    fsim_status worst = FSIM_OK;
    for (fsim_sim *h : b->members) {
        fsim_status st = check_flags(h);
        if (st && !worst) worst = st;
    }
    return worst;
}

} // namespace

extern "C" fsim_status fsim_batch_create(fsim_handle *members, int n, fsim_batch_t *out)
{
    if (!members || n < 1 || !out) return FSIM_EINVAL;
    *out = nullptr;
    for (int k = 0; k < n; ++k) {
        if (!members[k] || members[k]->batch || members[k]->device != members[0]->device) {
            fsim_set_error("batch members must be distinct standalone handles on one device");
            return FSIM_EINVAL;
        }
        if (members[k]->mixed != members[0]->mixed ||
            members[k]->cfg.solid_fused != members[0]->cfg.solid_fused) {
            fsim_set_error("batch members must share the precision form and the solid launch form");
            return FSIM_EINVAL;
        }
        for (int j = 0; j < k; ++j)
            if (members[j] == members[k]) {
                fsim_set_error("a handle appears twice in the batch");
                return FSIM_EINVAL;
            }
    }
    auto *b = new (std::nothrow) fsim_batch;
    if (!b) return FSIM_ENOMEM;
    b->device = members[0]->device;
    DeviceGuard guard(b->device);
    fsim_status st = FSIM_OK;
    cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&b->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&b->ev1);
    if (e != cudaSuccess) {
        fsim_set_error("batch stream/event creation failed: %s", cudaGetErrorString(e));
        free_batch(b);
        delete b;
        return FSIM_ECUDA;
    }
    const int ps = members[0]->s_cur;
    for (int k = 0; k < n && !st; ++k) st = set_parity(members[k], 0, ps);
    if (st) {
        free_batch(b);
        delete b;
        return st;
    }
    b->members.assign(members, members + n);
    for (fsim_sim *h : b->members) h->batch = b;
    *out = b;
    return FSIM_OK;
}

extern "C" fsim_status fsim_batch_step(fsim_batch_t b, int nsteps)
{
    if (!b || nsteps < 0) return FSIM_EINVAL;
    DeviceGuard guard(b->device);
    for (int k = 0; k < nsteps; ++k) {
        fsim_status st = batch_step_once(b);
        if (st) return st;
    }
    return FSIM_OK;
}

extern "C" fsim_status fsim_batch_sync(fsim_batch_t b)
{
    if (!b) return FSIM_EINVAL;
    DeviceGuard guard(b->device);
    return batch_check_flags(b);
}

namespace {
void drop_batch_plans(fsim_batch *b)
{
    for (auto &row : b->plans)
        for (Plan *&pl : row) {
            free_plan(pl);
            pl = nullptr;
        }
}
} // namespace

extern "C" fsim_status fsim_batch_add(fsim_batch_t b, fsim_handle h)
{
    if (!b || !h) return FSIM_EINVAL;
    if (h->batch || h->device != b->device) {
        fsim_set_error("a batch member must be a standalone handle on the batch's device");
        return FSIM_EINVAL;
    }
    if (!b->members.empty() && (h->mixed != b->members[0]->mixed ||
                                h->cfg.solid_fused != b->members[0]->cfg.solid_fused)) {
        fsim_set_error("batch members must share the precision form and the solid launch form");
        return FSIM_EINVAL;
    }
    DeviceGuard guard(b->device);
    CK(cudaStreamSynchronize(b->stream));
    CK(cudaStreamSynchronize(h->stream));
    const int pf = b->members.empty() ? 0 : b->members[0]->f_cur;
    const int ps = b->members.empty() ? h->s_cur : b->members[0]->s_cur;
    fsim_status st = set_parity(h, pf, ps);
    if (st) return st;
    drop_batch_plans(b); // rebuilt (and recaptured) at the next step; the tuned sweep shape is kept
    b->members.push_back(h);
    h->batch = b;
    return FSIM_OK;
}

extern "C" fsim_status fsim_batch_remove(fsim_batch_t b, fsim_handle h)
{
    if (!b || !h) return FSIM_EINVAL;
    auto it = std::find(b->members.begin(), b->members.end(), h);
    if (it == b->members.end()) {
        fsim_set_error("the handle is not a member of this batch");
        return FSIM_EINVAL;
    }
    DeviceGuard guard(b->device);
    CK(cudaStreamSynchronize(b->stream));
    drop_batch_plans(b);
    b->members.erase(it);
    h->batch = nullptr;
    return FSIM_OK;
}

extern "C" fsim_status fsim_batch_sync_members(fsim_batch_t b, int *status, int n)
{
    if (!b || (n && !status) || n != (int)b->members.size()) return FSIM_EINVAL;
    DeviceGuard guard(b->device);
    CK(cudaStreamSynchronize(b->stream));
    for (int k = 0; k < n; ++k) status[k] = check_flags(b->members[k]);
    return FSIM_OK;
}

extern "C" fsim_status fsim_batch_time_steps(fsim_batch_t b, int nsteps, float *ms)
{
    if (!b || nsteps < 0 || !ms) return FSIM_EINVAL;
    DeviceGuard guard(b->device);
    CK(cudaEventRecord(b->ev0, b->stream));
    for (int k = 0; k < nsteps; ++k) {
        fsim_status st = batch_step_once(b);
        if (st) return st;
    }
    CK(cudaEventRecord(b->ev1, b->stream));
    CK(cudaEventSynchronize(b->ev1));
    CK(cudaEventElapsedTime(ms, b->ev0, b->ev1));
    return batch_check_flags(b);
}

extern "C" fsim_status fsim_batch_launches_per_step(fsim_batch_t b, int *n)
{
    if (!b || !n) return FSIM_EINVAL;
    *n = 0;
    if (b->members.empty()) return FSIM_OK;
    DeviceGuard guard(b->device);
    const int pf = b->members[0]->f_cur, ps = b->members[0]->s_cur;
    Plan *&pl = b->plans[pf][ps];
    if (!pl) {
        fsim_status st = build_plan(b->members, kAllPhases, pf, ps, &pl);
        if (st) return st;
    }
    *n = (int)pl->launches.size();
    return FSIM_OK;
}

namespace {
fsim_status report_tuning(const SweepTuner &t, int *chosen, float *ms, int n)
{
    if (!chosen || (n > 0 && !ms) || n < 0) return FSIM_EINVAL;
    *chosen = t.chosen;
    for (int k = 0; k < n; ++k) ms[k] = k < kSweepShapes && k < t.next ? t.ms[k] : 0.0f;
    return FSIM_OK;
}
} // namespace

extern "C" fsim_status fsim_sweep_tuning(fsim_handle h, int *chosen, float *ms, int n)
{
    if (!h) return FSIM_EINVAL;
    return report_tuning(h->tuner, chosen, ms, n);
}

extern "C" fsim_status fsim_batch_sweep_tuning(fsim_batch_t b, int *chosen, float *ms, int n)
{
    if (!b) return FSIM_EINVAL;
    return report_tuning(b->tuner, chosen, ms, n);
}

extern "C" fsim_status fsim_batch_destroy(fsim_batch_t b)
{
    if (!b) return FSIM_OK;
    DeviceGuard guard(b->device);
    cudaStreamSynchronize(b->stream);
    for (fsim_sim *h : b->members) h->batch = nullptr;
    free_batch(b);
    delete b;
    return FSIM_OK;
}

extern "C" fsim_status fsim_estimate_bytes(const fsim_config *cfg, int n_fluid, int n_solid, int n_virt,
                                           size_t *out)
{
    if (!cfg || !out || n_fluid < 0 || n_solid < 0 || n_virt < 0) return FSIM_EINVAL;
    fsim_derived d;
    fsim_status st = fsim_derive(cfg, &d);
    if (st) return st;
    const size_t nf = n_fluid, ns = n_solid, nv = n_virt, nc = d.cell_number_total;
    size_t b = 0;
    b += nf * (2 * 2 * sizeof(float4) + 2 * sizeof(int) + 4 * sizeof(int)); // state x2, orig x2, cell/key/slot/tmp
    if (cfg->keep_derivatives) b += nf * (sizeof(float) + sizeof(float4));
    b += ns * (2 * 3 * sizeof(float4) + 2 * 2 * sizeof(int) + 4 * sizeof(int)); // state x2, cell/key/slot/tmp
    b += ns * (3 * sizeof(float4) + 5 * 9 * sizeof(float) + 2 * sizeof(int));  // per-step products, inv, cells
    {
        // static solid neighbour lists: lattice count within 2h, plus slack
        const double r = std::sqrt((double)d.impact_distance_square) / (double)cfg->particle_diameter;
        const size_t per = (size_t)(4.18879 * r * r * r * 1.25) + 8;
        b += ns * per * (sizeof(int) + sizeof(float4)) + (ns + 1) * sizeof(int);
    }
    b += nv * (3 * sizeof(float4) + 2 * sizeof(int));
    b += nc * sizeof(int) * 2 + (nc + 1) * sizeof(int) * 3; // counts, starts
    if (cfg->precision == FSIM_PRECISION_MIXED) b += nc * sizeof(float2); // per-cell references
    b += 2 * kMaxScanTiles * sizeof(int) + sizeof(unsigned);
    size_t words = 3 * nf;
    if (9 * ns > words) words = 9 * ns;
    if (3 * nv > words) words = 3 * nv;
    b += 4 * (words ? words : 1);
    b += 64 * 1024; // plans and allocation granularity
    *out = b;
    return FSIM_OK;
}
