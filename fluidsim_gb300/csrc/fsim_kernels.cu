// fsim_kernels.cu — the sm_103a kernels of the library and the launcher of
// plans; the host side is fsim_sim.cu.
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
#include "fsim_types.h"

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

using namespace fsim_rt;

namespace {

constexpr unsigned kFull = 0xffffffffu; // all lanes of a warp

// Device-side index checks, compiled in only with -DFSIM_DEVICE_CHECKS (a
// debugging build): a failed check records its site bit in g_check_sites and
// skips the access instead of reading or writing out of bounds.
#ifdef FSIM_DEVICE_CHECKS
__device__ unsigned g_check_sites;
#define FSIM_DCHECK(cond, bit, skip)                                                                          \
    if (!(cond)) {                                                                                            \
        atomicOr(&g_check_sites, (bit));                                                                      \
        skip;                                                                                                 \
    }
#else
#define FSIM_DCHECK(cond, bit, skip)
#endif

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

// The same kernel in two more launch forms whose parameters sit in the constant
// bank: one instance by value (NAME_1), and up to ParamBlock<ARGS>::kMax
// instances as one __grid_constant__ parameter block (NAME_p).  Only for
// bodies whose arithmetic spells out every rounding, so that all forms agree.
#define FSIM_BATCHED_KERNEL_P(NAME, ARGS, BODY, BOUNDS)                                                    \
    FSIM_BATCHED_KERNEL(NAME, ARGS, BODY, BOUNDS)                                                         \
    __global__ void __launch_bounds__(BOUNDS) NAME##_1(const DevParams P, const ARGS A)                   \
    {                                                                                                     \
        BODY(P, A, (int)blockIdx.x);                                                                      \
    }                                                                                                     \
    __global__ void __launch_bounds__(BOUNDS) NAME##_p(const __grid_constant__ ParamBlock<ARGS> B)        \
    {                                                                                                     \
        const int inst = locate_instance(B.bstart, B.n, blockIdx.x);                                      \
        BODY(B.it[inst].P, B.it[inst].A, (int)blockIdx.x - B.bstart[inst]);                               \
    }

// ------------------------------------------------------- counting sort
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

// the element blocks an item's block `blk` covers: blk, blk + grid, ... (all of
// them when the item is launched with one block per element block)
#define FSIM_ELEMENT_BLOCKS(A, blk, b)                                                                     \
    for (int b = (blk), nb_ = blocks_for((A).n, (int)blockDim.x), st_ = (A).grid ? (A).grid : nb_; b < nb_; \
         b += st_)

__device__ __forceinline__ void hash_body(const DevParams &P, const HashArgs &A, int blk)
{
    if (A.gate && !*A.gate) return; // uniform per block
    FSIM_ELEMENT_BLOCKS(A, blk, b)
    {
        const int s = b * blockDim.x + threadIdx.x;
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
}
FSIM_BATCHED_KERNEL(kb_hash, HashArgs, hash_body, kBlock)

__device__ __forceinline__ void zero_body(const DevParams &, const ZeroArgs &A, int blk)
{
    if (A.gate && !*A.gate) return;
    FSIM_ELEMENT_BLOCKS(A, blk, b)
    {
        const int s = b * blockDim.x + threadIdx.x;
        if (s < A.n) A.p[s] = 0;
    }
}
FSIM_BATCHED_KERNEL(kb_zero, ZeroArgs, zero_body, kBlock)

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
    if (J.gate && !*J.gate) return; // uniform per block
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
    if (J.gate && !*J.gate) return;
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
    if (J.gate && !*J.gate) return;
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

__device__ __forceinline__ void scatter_body(const DevParams &, const ScatterArgs &A, int blk)
{
    if (A.gate && !*A.gate) return;
    FSIM_ELEMENT_BLOCKS(A, blk, b)
    {
        const int s = b * blockDim.x + threadIdx.x;
        if (s >= A.n) continue;
        const int c = A.key[s];
        FSIM_DCHECK(A.start[c] + A.slot[s] >= 0 && A.start[c] + A.slot[s] < A.n, 8192u, continue);
        A.tmp[A.start[c] + A.slot[s]] = s;
        if (A.reset) A.reset[c] = 0; // the counts are spent: zero for the next sort
    }
}
FSIM_BATCHED_KERNEL(kb_scatter, ScatterArgs, scatter_body, kBlock)

// Rank inside the cell by previous position: the new order is sorted by
// (cell, previous sorted position), a stable and deterministic order.  The
// scan costs the cell's count per particle, so a cell of more than
// kStableRankMax particles (only out-of-grid input clamped into a boundary
// cell, or a smoothing length of several particle spacings, makes one) keeps
// the scatter's order and raises FLAG_CELL_OVERFULL: bounded work, and the
// step reports the failure.
__device__ __forceinline__ int stable_dst(const int *__restrict__ tmp, const int *__restrict__ key,
                                          const int *__restrict__ start, int d, int &src, int &cell,
                                          unsigned *flags, int n)
{
    src = tmp[d];
    FSIM_DCHECK(src >= 0 && src < n, 4096u, {
        src = d;
        cell = key[d];
        return d;
    });
    (void)n;
    cell = key[src];
    const int b = start[cell], e = start[cell + 1];
    if (e - b > kStableRankMax) {
        if (d == b && flags) atomicOr(flags, FLAG_CELL_OVERFULL);
        return d;
    }
    int rank = 0;
    for (int t = b; t < e; ++t) rank += tmp[t] < src;
    return b + rank;
}

__device__ __forceinline__ void gather_fluid_body(const DevParams &, const GatherFluidArgs &A, int blk)
{
    const int d = blk * blockDim.x + threadIdx.x;
    if (d >= A.n) return;
    if (A.gate && !*A.gate) {
        // neighbour-list step without a rebuild: the order stays, the state
        // moves to the other buffer unpermuted
        const float4 p = A.posr_in[d], v = A.velp_in[d];
        A.posr_out[d] = p;
        A.velp_out[d] = v;
        A.orig_out[d] = A.orig_in[d];
        if (A.icell_out) A.icell_out[d] = A.icell_in[d];
        if (A.rec_out) {
            A.rec_out[2 * (size_t)d] = p;
            A.rec_out[2 * (size_t)d + 1] = v;
        }
        return;
    }
    int src, cell;
    const int dst = stable_dst(A.tmp, A.key, A.start, d, src, cell, A.flags, A.n);
    FSIM_DCHECK(dst >= 0 && dst < A.n && src >= 0 && src < A.n, 8u, return);
    const float4 p = A.posr_in[src], v = A.velp_in[src];
    A.posr_out[dst] = p;
    A.velp_out[dst] = v;
    A.orig_out[dst] = A.orig_in[src];
    A.cell_out[dst] = cell;
    if (A.x0_out) A.x0_out[dst] = A.x0_in ? A.x0_in[src] : p;
    if (A.icell_out) A.icell_out[dst] = A.icell_in[src];
    if (A.rec_out) {
        A.rec_out[2 * (size_t)dst] = p;
        A.rec_out[2 * (size_t)dst + 1] = v;
    }
}
FSIM_BATCHED_KERNEL(kb_gather_fluid, GatherFluidArgs, gather_fluid_body, kBlock)

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
    if (A.gate && !*A.gate) { // no rebuild: unpermuted copy (inv stays valid)
        A.pos_out[d] = A.pos_in[d];
        A.vel_out[d] = A.vel_in[d];
        A.ref_out[d] = A.ref_in[d];
        A.type_out[d] = A.type_in[d];
        A.orig_out[d] = A.orig_in[d];
        return;
    }
    int src, cell;
    const int dst = stable_dst(A.tmp, A.key, A.start, d, src, cell, A.flags, A.n);
    FSIM_DCHECK(dst >= 0 && dst < A.n && src >= 0 && src < A.n, 16u, return);
    const float4 p = A.pos_in[src];
    A.pos_out[dst] = p;
    A.vel_out[dst] = A.vel_in[src];
    A.ref_out[dst] = A.ref_in[src];
    A.type_out[dst] = A.type_in[src];
    const int o = A.orig_in[src];
    A.orig_out[dst] = o;
    A.cell_out[dst] = cell;
    A.inv_out[o] = dst;
    if (A.cxyz_out) A.cxyz_out[dst] = pack_cell(P, cell);
    if (A.x0_out) A.x0_out[dst] = p;
}
FSIM_BATCHED_KERNEL(kb_gather_solid, GatherSolidArgs, gather_solid_body, kBlock)

// Neighbour-list instances: the per-step cell index.  Slot d of the scatter
// holds particle slot src = tmp[d] of cell `cell`; its rank among the cell's
// slots (in increasing slot order, as stable_dst ranks) places it in ids.
__device__ __forceinline__ void rank_body(const DevParams &P, const RankArgs &A, int blk)
{
    const int d = blk * blockDim.x + threadIdx.x;
    if (d >= A.n) return;
    int src, cell;
    const int dst = stable_dst(A.tmp, A.key, A.start, d, src, cell, A.flags, A.n);
    FSIM_DCHECK(dst >= 0 && dst < A.n && src >= 0 && src < A.n, 4u, return);
    A.ids[dst] = src;
    A.cell_out[src] = cell;
    if (A.cxyz_out) A.cxyz_out[src] = pack_cell(P, cell);
    if (A.pos_out) A.pos_out[dst] = A.pos_in[src];
}
FSIM_BATCHED_KERNEL(kb_rank, RankArgs, rank_body, kBlock)

// ------------------------------------------------------------ EOS
// densityToPressure (src/fluid.cu:16-24): Tait EOS, floored at min_pressure.
// The accurate powf, not the fast-math __powf that the reference's release
// build compiles it to: (rho/rho0)^gamma - 1 is a cancellation near rho0, and
// __powf's log2 approximation has an absolute error there that is large next
// to the small difference (it dominated the pressure error against FP64 in the
// reference build and in a first version of this kernel alike).  Once per
// particle per step, so its cost is negligible.
__device__ __forceinline__ float tait_pressure(const DevParams &P, float rho)
{
    const float p = (powf(rho * P.rho0_inv, P.gamma) - 1.0f) * P.rho2p;
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

// fluidUpdate (src/fluid.cu:234-269) applied to the sums of one particle: NaN
// scrub, Euler step with the old velocity, density clamp, EOS, position clamp,
// speed cap; writes the integrated state into the other buffer.
__device__ __forceinline__ float4 fluid_update_store(const DevParams &P, const FluidSweepArgs &A, int i, float4 pr,
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
    const float4 xr = make_float4(x, y, z, rho);
    A.posr_out[i] = xr;
    A.velp_out[i] = make_float4(ux, uy, uz, p);
    A.orig_out[i] = A.orig_in[i];
    if (A.keep) {
        A.drho_out[i] = drho;
        A.dudt_out[i] = make_float4(ax, ay, az, 0.0f);
    }
    return xr;
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
static_assert(kShapeWarps[0] == Shape0::warps && kShapeWarps[1] == Shape1::warps &&
                  kShapeWarps[2] == Shape2::warps,
              "fsim_types.h restates the sweep shapes");

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

template <int SP, bool CHECK_Z, int VISCID, class SH, bool KAHAN = false, bool BITS = false>
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
                if (BITS && j + SH::chunk <= je) {
                    // BITS (the batched sweep): a full chunk's hits as bits,
                    // appended afterwards in candidate order -- one predicated
                    // OR per candidate instead of a predicated append; the same
                    // list.  Measured faster in the batched kernel (ensemble step
                    // 5.67 -> 5.55 ms) and slower in the one-instance kernel,
                    // whose 16-candidate chunk then needs 62 registers.
                    unsigned bits = 0;
#pragma unroll
                    for (int c = 0; c < SH::chunk; ++c) {
                        const float4 q = pos[j + c]; // same address in every lane: a broadcast
                        const float r2 = dist2(q.x - pr.x, q.y - pr.y, q.z - pr.z);
                        bool hit = in && r2 < P.R2;
                        if (CHECK_Z && hit) {
                            const int czj = (int)__fmul_rn(__fsub_rn(q.z, P.cmin[2]), P.cinv[2]);
                            hit = abs(czj - cz) <= 1;
                        }
                        if (hit) bits |= 1u << c;
                    }
                    while (bits) {
                        const int c = __ffs(bits) - 1;
                        bits &= bits - 1;
                        lst[cnt++][lane] = j + c;
                    }
                    j += SH::chunk;
                } else {
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
    }
    flush_list<SP, VISCID, KAHAN>(P, A, lst, lane, cnt, pr, vp, acc);
}

template <bool CHECK_Z, int VISCID, class SH, bool BITS = false>
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
        gather_species<kFluid, CHECK_Z, VISCID, SH, false, BITS>(P, A, lst, lane, cnt, in, cz, cx, cy, z0, z1, pr, vp,
                                                                acc);
        gather_species<kVirt, CHECK_Z, VISCID, SH, false, BITS>(P, A, lst, lane, cnt, in, cz, cx, cy, z0, z1, pr, vp,
                                                               acc);
        gather_species<kSolid, CHECK_Z, VISCID, SH, false, BITS>(P, A, lst, lane, cnt, in, cz, cx, cy, z0, z1, pr, vp,
                                                                acc);
    }
    if (valid) fluid_update_store(P, A, i, pr, vp, acc);
}

template <bool CHECK_Z, int VISCID, class SH>
__global__ void __launch_bounds__(SH::warps * 32) kb_fluid_sweep(const Item<FluidSweepArgs> *__restrict__ items,
                                                                 const int *__restrict__ bstart, int ninst)
{
    const int inst = locate_instance(bstart, ninst, blockIdx.x);
    const DevParams P = items[inst].P;
    fluid_sweep_body<CHECK_Z, VISCID, SH, true>(P, items[inst].A, (int)blockIdx.x - bstart[inst]);
}

// The one-instance sweep takes {params, args} by value: kernel parameters live
// in the constant bank, where its hot loops read them without extra loads.
template <bool CHECK_Z, int VISCID, class SH>
__global__ void __launch_bounds__(SH::warps * 32) kb_fluid_sweep_1(const DevParams P, const FluidSweepArgs A)
{
    fluid_sweep_body<CHECK_Z, VISCID, SH>(P, A, (int)blockIdx.x);
}

// The batched sweep with its instances' {params, args} passed by value: one
// kernel parameter block (in the constant bank, like the one-instance
// sweep's), up to kSweepParamItems instances.
template <bool CHECK_Z, int VISCID, class SH>
__global__ void __launch_bounds__(SH::warps * 32) kb_fluid_sweep_p(const __grid_constant__ SweepBatchParams B)
{
    const int inst = locate_instance(B.bstart, B.n, blockIdx.x);
    const Item<FluidSweepArgs> &it = B.it[inst];
    fluid_sweep_body<CHECK_Z, VISCID, SH, true>(it.P, it.A, (int)blockIdx.x - B.bstart[inst]);
}

// ------------------------------------------------------- fluid neighbour lists
// Neighbour-list instances advance the fluid with per-particle lists that
// are kept for many steps (a Verlet list): the list of particle i holds every
// fluid, wall and solid particle within the list radius Rs = R + skin of i
// when the list was built.  While no particle has moved more than (Rs - R) / 2
// since the build, every pair within the impact distance R is in the lists,
// so the sweep finds exactly the reference's pair set (src/fluid.cu:169-232:
// 27 cells of side >= R, then r^2 < R^2) with no cell walk.  The particles
// keep the order of the last build between builds; the other phases walk a
// per-step cell index (kb_rank) instead.

// One block per instance at the start of every step: rebuild when forced or
// when the largest displacement since the last build (fluid: accumulated by
// the last sweep; solid: measured here) exceeds the allowance.
__device__ __forceinline__ void nl_decide_body(const DevParams &, const NlDecideArgs &A, int blk)
{
    __shared__ unsigned wmax[kBlock / 32];
    unsigned m = 0;
    for (int i = blk * blockDim.x + threadIdx.x; i < A.ns; i += A.nblocks * blockDim.x) {
        const float4 p = A.s_pos[i], o = A.s_x0[i];
        m = max(m, __float_as_uint(dist2(p.x - o.x, p.y - o.y, p.z - o.z)));
    }
    m = __reduce_max_sync(kFull, m);
    if ((threadIdx.x & 31) == 0) wmax[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x) return;
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) m = max(m, wmax[w]);
    NlState &S = *A.nl;
    if (m) atomicMax(&S.maxd2, m); // NaN bits compare above every distance
    __threadfence();
    if (atomicAdd(&S.ticket, 1u) != (unsigned)A.nblocks - 1u) return;
    // the last block: every block's maximum (and the last sweep's) is in maxd2
    __threadfence();
    const float d2 = __uint_as_float(atomicMax(&S.maxd2, 0u));
    const int rb = S.force || !(d2 <= A.move2);
    S.rebuild = rb;
    S.force = 0;
    S.maxd2 = 0u; // this step's sweep accumulates afresh (against the new x0 if rebuilt)
    S.ticket = 0u;
    if (rb) {
        S.builds += 1;
        S.overflow = 0;
    }
}
FSIM_BATCHED_KERNEL(kb_nl_decide, NlDecideArgs, nl_decide_body, kBlock)

// The list build: the sweep's warp-uniform candidate stream (a warp's lanes of
// one cell row walk the union of their 9 neighbour rows) over the list grid,
// testing r^2 < Rs^2; hits collect in a per-lane shared-memory list that is
// appended to the lane's global list in candidate order.  Per particle: its
// fluid, then wall, then solid candidates, in row order -- the order in which
// the stream sweep sums them.
constexpr int kNlBuildWarps = kNlBuildThreads / 32, kNlBuildCap = 32, kNlBuildChunk = 8;

// Append a lane's pending hits lst[0..cnt) to its list in whole groups of
// kNlGroup entries (two 16-byte stores: a full sector); the remainder stays
// pending at the front.  `tot` counts the entries stored so far; the final
// flush stores the last partial group padded with -1 and makes `tot` exact.
__device__ __forceinline__ void nl_flush(const NlBuildArgs &A, int (*lst)[32], int lane, int i, int &cnt, int &tot,
                                         bool last)
{
    const int full = last ? (cnt + kNlGroup - 1) / kNlGroup : cnt / kNlGroup;
    const int mfull = __reduce_max_sync(kFull, full);
    for (int g = 0; g < mfull; ++g) {
        const int grp = tot / kNlGroup + g;
        if (g < full && grp * kNlGroup < A.cap) {
            int v[kNlGroup];
#pragma unroll
            for (int q = 0; q < kNlGroup; ++q) {
                const int k = g * kNlGroup + q;
                v[q] = k < cnt ? lst[k][lane] : -1;
            }
            int4 *dst = reinterpret_cast<int4 *>(A.list + ((size_t)grp * A.n + i) * kNlGroup);
            __stcs(dst, make_int4(v[0], v[1], v[2], v[3])); // streaming: keep the positions in L2
            __stcs(dst + 1, make_int4(v[4], v[5], v[6], v[7]));
        }
    }
    if (last) {
        tot += cnt;
        cnt = 0;
        return;
    }
    const int rem = cnt - full * kNlGroup; // < kNlGroup; moves down from index >= kNlGroup (or stays put)
    for (int q = 0; q < rem; ++q) lst[q][lane] = lst[full * kNlGroup + q][lane];
    tot += full * kNlGroup;
    cnt = rem;
}

template <int SP>
__device__ __forceinline__ void nl_gather(const DevParams &P, const NlBuildArgs &A, int (*lst)[32], int lane, int i,
                                          int &cnt, int &tot, bool in, int cx, int cy, int z0, int z1, float4 pr)
{
    const int *start = SP == 0 ? A.start_f : SP == 1 ? A.start_v : A.start_s;
    const float4 *pos = SP == 0 ? A.posr : SP == 1 ? A.v_posr : A.s_pos;
    const int tag = (int)((unsigned)SP << kNlSpeciesShift);
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
                if (__reduce_max_sync(kFull, cnt) > kNlBuildCap - kNlBuildChunk)
                    nl_flush(A, lst, lane, i, cnt, tot, false);
                const int jend = min(j + kNlBuildChunk, je);
#pragma unroll 4
                for (; j < jend; ++j) {
                    FSIM_DCHECK(j < (SP == 0 ? A.n : SP == 1 ? A.nv : A.ns), 2u, continue);
                    const float4 q = pos[j]; // same address in every lane: a broadcast
                    const float r2 = dist2(q.x - pr.x, q.y - pr.y, q.z - pr.z);
                    if (in && r2 < A.R2s) lst[cnt++][lane] = j | tag;
                }
            }
        }
    }
}

__device__ __forceinline__ void nl_build_block(const DevParams &P, const NlBuildArgs &A, int blk);

__device__ __forceinline__ void nl_build_body(const DevParams &P, const NlBuildArgs &A, int blk)
{
    if (!A.nl->rebuild) return; // uniform per block
    FSIM_ELEMENT_BLOCKS(A, blk, b) nl_build_block(P, A, b);
}

__device__ __forceinline__ void nl_build_block(const DevParams &P, const NlBuildArgs &A, int blk)
{
    __shared__ int lists[kNlBuildWarps][kNlBuildCap][32];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int i = (blk * kNlBuildWarps + warp) * 32 + lane;
    const bool valid = i < A.n;
    int(*lst)[32] = lists[warp];
    const float4 pr = valid ? A.posr[i] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const int cell = valid ? A.cell_f[i] : 0;
    const int row = cell / P.nz, cz = cell - row * P.nz;
    int cnt = 0, tot = 0;
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
        nl_gather<0>(P, A, lst, lane, i, cnt, tot, in, cx, cy, z0, z1, pr);
        nl_gather<1>(P, A, lst, lane, i, cnt, tot, in, cx, cy, z0, z1, pr);
        nl_gather<2>(P, A, lst, lane, i, cnt, tot, in, cx, cy, z0, z1, pr);
    }
    nl_flush(A, lst, lane, i, cnt, tot, true);
    if (valid) {
        A.cnt[i] = tot;
        if (tot > A.cap) {
            atomicAdd(&A.nl->overflow, 1);
            atomicOr(A.flags, FLAG_LIST_OVERFLOW);
        }
    }
}
FSIM_BATCHED_KERNEL(kb_nl_build, NlBuildArgs, nl_build_body, kNlBuildWarps * 32)

// The list sweep: one thread per particle walks its list, tests r^2 < R^2
// and sums the Riemann pair terms in list order (fluid, then wall, then solid
// candidates, as the stream sweep sums them), then fluidUpdate
// (src/fluid.cu:234-269) as in the stream sweep; the particle's squared
// displacement since the build goes into the instance's running maximum.
// One 32-byte (position, velocity) record with a single 256-bit load through
// the read-only path (32-byte aligned: records start on 256-byte allocations).
__device__ __forceinline__ void load_record(const float4 *p, float4 &a, float4 &b)
{
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
        : "l"(p));
}

template <int VISCID, bool CHECK>
__device__ __forceinline__ void fluid_sweep_nl_pairs(const DevParams &P, const FluidSweepArgs &A, int i, float4 pr,
                                                     float4 vp, PairAcc &acc)
{
    const int m = min(A.nl_cnt[i], A.nl_cap);
    const int4 *__restrict__ l = reinterpret_cast<const int4 *>(A.nl_list) + (size_t)i * (kNlGroup / 4);
    const size_t stride = (size_t)A.n * (kNlGroup / 4); // int4 per group row
    const unsigned ci = CHECK ? A.nl_cxyz_f[i] : 0u;
    for (int k0 = 0; k0 < m; k0 += kNlGroup) {
        // one group: a whole 32-byte sector of the lane's list, read once per
        // sweep, so loaded evict-first: the lists (1.6 GB at the 4M case) would
        // otherwise push the neighbour records out of L1 and L2
        const int4 a = __ldcs(l + (size_t)(k0 / kNlGroup) * stride), b = __ldcs(l + (size_t)(k0 / kNlGroup) * stride + 1);
        const int grp[kNlGroup] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
#pragma unroll
        for (int q = 0; q < kNlGroup; ++q) {
            if (k0 + q >= m) break;
            const unsigned e = (unsigned)grp[q];
            const int sp = (int)(e >> kNlSpeciesShift), j = (int)(e & kNlIndexMask);
            FSIM_DCHECK(sp == 0 ? j < A.n : sp == 1 ? j < A.nl_nv : sp == 2 && j < A.nl_ns, 1u, continue);
            if (sp == 2) {
                const float4 q4 = A.s_pos[j];
                const float dx = q4.x - pr.x, dy = q4.y - pr.y, dz = q4.z - pr.z;
                const float r2 = dist2(dx, dy, dz);
                if (r2 < P.R2 && (!CHECK || cells_adjacent(ci, A.nl_cxyz_s[j]))) {
                    const float4 np = A.s_np[j], sv = A.s_vel[j];
                    const float k2 = 2.0f * ((vp.x - sv.x) * np.x + (vp.y - sv.y) * np.y + (vp.z - sv.z) * np.z);
                    riemann_pair<false, VISCID>(P, dx, dy, dz, r2, vp.x, vp.y, vp.z, pr.w, vp.w, vp.x - k2 * np.x,
                                                vp.y - k2 * np.y, vp.z - k2 * np.z, pr.w, np.w, false, acc);
                }
            } else if (sp == 1) {
                const float4 q4 = A.v_posr[j];
                const float dx = q4.x - pr.x, dy = q4.y - pr.y, dz = q4.z - pr.z;
                const float r2 = dist2(dx, dy, dz);
                if (r2 < P.R2 && (!CHECK || cells_adjacent(ci, A.nl_cxyz_v[j]))) {
                    const float4 u = A.v_velp[j];
                    riemann_pair<true, VISCID>(P, dx, dy, dz, r2, vp.x, vp.y, vp.z, pr.w, vp.w, u.x, u.y, u.z, q4.w,
                                               u.w, true, acc);
                }
            } else {
                float4 q4, u;
                load_record(A.rec + 2 * (size_t)j, q4, u); // position and velocity: one sector
                const float dx = q4.x - pr.x, dy = q4.y - pr.y, dz = q4.z - pr.z;
                const float r2 = dist2(dx, dy, dz);
                if (r2 < P.R2 && (!CHECK || cells_adjacent(ci, A.nl_cxyz_f[j]))) {
                    riemann_pair<true, VISCID>(P, dx, dy, dz, r2, vp.x, vp.y, vp.z, pr.w, vp.w, u.x, u.y, u.z, q4.w,
                                               u.w, false, acc);
                }
            }
        }
    }
}

template <int VISCID>
__device__ __forceinline__ void fluid_sweep_nl_body(const DevParams &P, const FluidSweepArgs &A, int blk)
{
    const int i = blk * blockDim.x + threadIdx.x;
    const bool valid = i < A.n;
    unsigned d2bits = 0u;
    if (valid) {
        const float4 pr = A.posr[i], vp = A.velp[i];
        PairAcc acc = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
        if (A.nl_cxyz_f) fluid_sweep_nl_pairs<VISCID, true>(P, A, i, pr, vp, acc);
        else fluid_sweep_nl_pairs<VISCID, false>(P, A, i, pr, vp, acc);
        const float4 x = fluid_update_store(P, A, i, pr, vp, acc);
        const float4 o = A.x0[i];
        d2bits = __float_as_uint(dist2(x.x - o.x, x.y - o.y, x.z - o.z));
    }
    const unsigned wmax = __reduce_max_sync(kFull, d2bits);
    if ((threadIdx.x & 31) == 0 && wmax) atomicMax(&A.nl->maxd2, wmax);
}

// launch shapes of the list sweep: threads per block, minimum blocks per SM
template <int BS, int MINB>
struct NlShape {
    static constexpr int threads = BS, min_blocks = MINB;
};
using NlShape0 = NlShape<128, 16>; // at most 32 registers: 16 blocks (64 warps) per SM
using NlShape1 = NlShape<128, 12>; // at most 40 registers: 12 blocks (48 warps) per SM
using NlShape2 = NlShape<256, 5>;  // at most 51 registers: 5 blocks (40 warps) per SM
static_assert(kShapeWarps[0] * 32 == NlShape0::threads && kShapeWarps[1] * 32 == NlShape1::threads &&
                  kShapeWarps[2] * 32 == NlShape2::threads,
              "list-sweep shapes follow the block sizes of fsim_types.h");

template <int VISCID, class SH>
__global__ void __launch_bounds__(SH::threads, SH::min_blocks) kb_fluid_sweep_nl_1(const DevParams P,
                                                                                   const FluidSweepArgs A)
{
    fluid_sweep_nl_body<VISCID>(P, A, (int)blockIdx.x);
}
template <int VISCID, class SH>
__global__ void __launch_bounds__(SH::threads, SH::min_blocks)
    kb_fluid_sweep_nl(const Item<FluidSweepArgs> *__restrict__ items, const int *__restrict__ bstart, int ninst)
{
    const int inst = locate_instance(bstart, ninst, blockIdx.x);
    fluid_sweep_nl_body<VISCID>(items[inst].P, items[inst].A, (int)blockIdx.x - bstart[inst]);
}
template <int VISCID, class SH>
__global__ void __launch_bounds__(SH::threads, SH::min_blocks) kb_fluid_sweep_nl_p(const __grid_constant__ SweepBatchParams B)
{
    const int inst = locate_instance(B.bstart, B.n, blockIdx.x);
    const Item<FluidSweepArgs> &it = B.it[inst];
    fluid_sweep_nl_body<VISCID>(it.P, it.A, (int)blockIdx.x - B.bstart[inst]);
}

// ------------------------------------------------------- virtual particles
// getVirtData (src/virt.cu:9-75): nearest fluid particle's rho, hydrostatically
// corrected p and velocity mirrored about the (static) wall normal.  Ties in
// distance go to the smaller input id.
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
        for (int t = A.start_f[rows.base[r] + rows.z0], te = A.start_f[rows.base[r] + rows.z1]; t < te; ++t) {
            // with the index's position copy, the particle id only for a new best
            const float4 q = A.fpos_t ? A.fpos_t[t] : A.fposr[A.ids_f ? A.ids_f[t] : t];
            const float d2 = dist2(q.x - xi.x, q.y - xi.y, q.z - xi.z);
            if (d2 <= best) {
                const int j = A.ids_f ? A.ids_f[t] : t;
                FSIM_DCHECK(j >= 0 && j < A.nf, 32u, continue);
                const int o = A.forig[j];
                if (d2 < best || o < best_orig) {
                    best = d2;
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

template <int G = kSolidGroup>
__device__ __forceinline__ float group_sum(float v)
{
#pragma unroll
    for (int o = 1; o < G; o <<= 1) v += __shfl_xor_sync(kFull, v, o);
    return v;
}

// ------------------------------------------------------- fluid-solid coupling
// solidCoupleUpdate (src/solid.cu:262-344): solid normal from the solid
// neighbours' kernel gradients, solid pressure as the Shepard average of the
// fluid pressure.  kCoupleGroup lanes per solid particle.
__device__ __forceinline__ void couple_body(const DevParams &P, const CoupleArgs &A, int blk)
{
    const int t = blk * blockDim.x + threadIdx.x;
    const int i = t / kCoupleGroup, g = t % kCoupleGroup;
    const bool valid = i < A.n;
    float nx = 0.0f, ny = 0.0f, nz = 0.0f, psum = 0.0f, wsum = 0.0f;
    if (valid) {
        const float4 xi = A.s_pos[i];
        Rows rows;
        neighbor_rows(P, A.s_cell[i], rows);
        for (int r = 0; r < rows.count; ++r) {
            const int c0 = rows.base[r] + rows.z0, c1 = rows.base[r] + rows.z1;
            for (int tf = A.start_f[c0] + g, te = A.start_f[c1]; tf < te; tf += kCoupleGroup) {
                const float4 q = A.fpos_t ? A.fpos_t[tf] : A.fposr[A.ids_f ? A.ids_f[tf] : tf];
                const float dx = q.x - xi.x, dy = q.y - xi.y, dz = q.z - xi.z;
                const float r2 = dist2(dx, dy, dz);
                if (r2 < P.R2) {
                    const int j = A.ids_f ? A.ids_f[tf] : tf;
                    FSIM_DCHECK(j >= 0 && j < A.nf, 64u, continue);
                    const float w = (__expf(-r2 * P.h_inv2) - P.kc1) * P.kc2;
                    wsum += w;
                    psum += A.fvelp[j].w * w;
                }
            }
            for (int ts = A.start_s[c0] + g, te = A.start_s[c1]; ts < te; ts += kCoupleGroup) {
                const int j = A.ids_s ? A.ids_s[ts] : ts;
                FSIM_DCHECK(j >= 0 && j < A.n, 128u, continue);
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
    nx = group_sum<kCoupleGroup>(nx);
    ny = group_sum<kCoupleGroup>(ny);
    nz = group_sum<kCoupleGroup>(nz);
    psum = group_sum<kCoupleGroup>(psum);
    wsum = group_sum<kCoupleGroup>(wsum);
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
__device__ __forceinline__ void cell_ref_body(const DevParams &P, const CellRefArgs &A, int blk)
{
    // kCellRefLanes lanes per cell (a cell holds ~18 particles at the
    // benchmark spacing, and most cells of the grid are empty), each summing
    // every kCellRefLanes-th particle; then a butterfly over the lanes
    const int t = blk * blockDim.x + threadIdx.x;
    const int c = t / kCellRefLanes, sub = t % kCellRefLanes;
    int b = 0, e = 0;
    if (c < A.ncell) {
        b = A.start[c];
        e = A.start[c + 1];
    }
    float sd = 0.0f, sp = 0.0f;
    for (int k = b + sub; k < e; k += kCellRefLanes) {
        const float d = A.velp[A.ids ? A.ids[k] : k].w;
        sd += d;
        sp += eos_delta(P, d);
    }
#pragma unroll
    for (int o = kCellRefLanes / 2; o > 0; o >>= 1) {
        sd += __shfl_xor_sync(kFull, sd, o);
        sp += __shfl_xor_sync(kFull, sp, o);
    }
    if (b == e) return; // never read: no particle refers to an empty cell
    const float inv_n = 1.0f / (float)(e - b);
    const float dm = sd * inv_n, pm = sp * inv_n;
    if (sub == 0) A.cm[c] = make_float2(dm, pm);
    if (A.ids) return; // neighbour-list instances: kb_mixed_records, in slot order
    float *w = reinterpret_cast<float *>(A.posr);
    for (int j = b + sub; j < e; j += kCellRefLanes) {
        const float d = A.velp[j].w;
        w[4 * (size_t)j + 3] = __uint_as_float(half2_bits((d - dm) * kDeltaScale, (eos_delta(P, d) - pm) * P.p_unit_inv));
    }
}
FSIM_BATCHED_KERNEL(kb_cell_ref, CellRefArgs, cell_ref_body, kBlock)

// Neighbour-list instances: every slot's FP16 gather pair against its cell's
// references (the same expression as kb_cell_ref's), and its 32-byte record
// for the list sweep (offset, FP16 pair | velocity, packed cell).
__device__ __forceinline__ void mixed_records_body(const DevParams &P, const CellRefArgs &A, int blk)
{
    const int i = blk * blockDim.x + threadIdx.x;
    if (i >= A.n) return;
    const float4 v = A.velp[i];
    float4 p = A.posr[i];
    const float2 ref = A.cm[A.cell[i]];
    p.w = __uint_as_float(half2_bits((v.w - ref.x) * kDeltaScale, (eos_delta(P, v.w) - ref.y) * P.p_unit_inv));
    A.posr[i] = p;
    A.rec[2 * (size_t)i] = p;
    A.rec[2 * (size_t)i + 1] = make_float4(v.x, v.y, v.z, __uint_as_float(A.cxyz[i]));
}
FSIM_BATCHED_KERNEL(kb_mixed_records, CellRefArgs, mixed_records_body, kBlock)

// Own particle of the mixed sweep.
struct OwnMixed {
    float bx, by, bz; // offset + one cell: the list's cell code b in {0,1,2} gives offset - (b - 1) cell
    int cbase;        // linear cell of code (0, 0, 0)
    float rho, p;
};
// The own offset (plus one cell, `ob`) shifted by `o` in {-1, 0, 1} cells:
// what a pair subtracts from the offset of a neighbour in the cell `o` away.
// Every mixed-form pair test and pair term rounds it this one way.
__device__ __forceinline__ float shifted(float ob, int o, float cdx) { return fmaf(-(float)(o + 1), cdx, ob); }
// Cell codes (o + 1 per axis, each in {0, 1, 2} for neighbouring cells) of a
// pair from packed coordinates (x | y << 11 | z << 21): with cb = kCellBias -
// c_i, the fields of c_j + cb are the codes when the cells are neighbours;
// otherwise some field exceeds 2 (a field below -1 wraps to at least 3 in its
// own bits, given fewer than 2^11, 2^10, 2^11 cells per axis, and any borrow
// it passes up only shows where a field has already failed).
constexpr unsigned kCellBias = 1u | (1u << 11) | (1u << 21);
__device__ __forceinline__ bool cell_codes(unsigned cj, unsigned cb, int &bx, int &by, int &bz)
{
    const unsigned d = cj + cb;
    bx = (int)(d & 0x7ffu);
    by = (int)((d >> 11) & 0x3ffu);
    bz = (int)(d >> 21);
    return bx <= 2 && by <= 2 && bz <= 2;
}

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
        const float psx = shifted(o.bx, ox, P.cdx[0]);
        for (int oy = -1; oy <= 1; ++oy) {
            const int y = cy + oy;
            if (y < 0 || y >= P.ny) continue;
            const float psy = shifted(o.by, oy, P.cdx[1]);
            const int rb = (x * P.ny + y) * P.nz;
            const unsigned code_xy = (unsigned)(ox + 1) | ((unsigned)(oy + 1) << 2);
            int j = start[rb + z0];
            for (int z = z0; z < z1; ++z) {
                const int je = start[rb + z + 1];
                const int dzc = z - cz;
                const bool inz = in && dzc >= -1 && dzc <= 1;
                const float psz = shifted(o.bz, dzc, P.cdx[2]);
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
__device__ __forceinline__ float4 fluid_update_store_m(const DevParams &P, const FluidSweepArgs &A, int i, float4 off,
                                                       float4 vp, float rho, const PairAcc &acc, int cx, int cy,
                                                       int cz)
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
    return make_float4(x, y, z, 0.0f);
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

// Absolute FP32 position of a mixed-form particle at offset `off` from the
// corner of cell (cx, cy, cz) (the sweep's position of the fluid particle for
// its solid pairs; the list build's positions).
__device__ __forceinline__ float4 mixed_abs(const DevParams &P, float4 off, int cx, int cy, int cz, float w)
{
    return make_float4(__fadd_rn(fmaf((float)cx, P.cdx[0], P.cmin[0]), off.x),
                       __fadd_rn(fmaf((float)cy, P.cdx[1], P.cmin[1]), off.y),
                       __fadd_rn(fmaf((float)cz, P.cdx[2], P.cmin[2]), off.z), w);
}
__device__ __forceinline__ void unpack_cell(unsigned c, int &cx, int &cy, int &cz)
{
    cx = (int)(c & 0x7ffu);
    cy = (int)((c >> 11) & 0x3ffu);
    cz = (int)(c >> 21);
}

// Neighbour lists in the mixed form.  The particles keep the order of the last
// list build between builds; each step re-bins every offset to the cell it now
// lies in (in place), and the per-step cell index (kb_rank) gives every
// particle's cell and packed cell coordinates.  A fluid neighbour's record
// (32 bytes, written by kb_mixed_records after the per-cell references) is
//   (offset x y z, FP16 (delta, p) deviations | u v w, packed cell)
// and a pair is taken exactly as the mixed cell walk takes it: the two cells
// are neighbours, and r^2 < R^2 with the offset of i shifted by the cell
// difference (`shifted`), so both sum bit-identical pair terms (in list order).
template <int VISCID>
__device__ __forceinline__ void fluid_sweep_nlm_pairs(const DevParams &P, const FluidSweepArgs &A, int i,
                                                      const OwnMixed &o, float4 pa, float4 vp, unsigned ci,
                                                      PairAcc &acc)
{
    const unsigned cb = kCellBias - ci;
    const int m = min(A.nl_cnt[i], A.nl_cap);
    const int4 *__restrict__ l = reinterpret_cast<const int4 *>(A.nl_list) + (size_t)i * (kNlGroup / 4);
    const size_t stride = (size_t)A.n * (kNlGroup / 4);
    const int nynz = P.ny * P.nz;
    for (int k0 = 0; k0 < m; k0 += kNlGroup) {
        const int4 a = __ldcs(l + (size_t)(k0 / kNlGroup) * stride), b = __ldcs(l + (size_t)(k0 / kNlGroup) * stride + 1);
        const int grp[kNlGroup] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
#pragma unroll
        for (int q = 0; q < kNlGroup; ++q) {
            if (k0 + q >= m) break;
            const unsigned e = (unsigned)grp[q];
            const int sp = (int)(e >> kNlSpeciesShift), j = (int)(e & kNlIndexMask);
            FSIM_DCHECK(sp == 0 ? j < A.n : sp == 1 ? j < A.nl_nv : sp == 2 && j < A.nl_ns, 1u, continue);
            if (sp == 2) {
                const float4 q4 = A.s_pos[j];
                const float dx = q4.x - pa.x, dy = q4.y - pa.y, dz = q4.z - pa.z;
                const float r2 = dist2(dx, dy, dz);
                if (r2 < P.R2 && cells_adjacent(ci, A.nl_cxyz_s[j])) {
                    const float4 np = A.s_np[j], sv = A.s_vel[j];
                    const float k2 = __fmul_rn(2.0f, fmaf(__fsub_rn(vp.z, sv.z), np.z,
                                                          fmaf(__fsub_rn(vp.y, sv.y), np.y,
                                                               __fmul_rn(__fsub_rn(vp.x, sv.x), np.x))));
                    riemann_pair<false, VISCID, true>(P, dx, dy, dz, r2, vp.x, vp.y, vp.z, o.rho, o.p,
                                                      fmaf(-k2, np.x, vp.x), fmaf(-k2, np.y, vp.y),
                                                      fmaf(-k2, np.z, vp.z), o.rho, np.w, false, acc);
                }
                continue;
            }
            float4 q4, u;
            unsigned cj;
            if (sp == 1) {
                q4 = A.v_posr[j];
                u = A.v_velp[j];
                cj = A.nl_cxyz_v[j];
            } else {
                load_record(A.rec + 2 * (size_t)j, q4, u);
                cj = __float_as_uint(u.w);
            }
            int bx, by, bz;
            if (!cell_codes(cj, cb, bx, by, bz)) continue;
            // = shifted(o.b*, b* - 1, cdx)
            const float dx = q4.x - fmaf(-(float)bx, P.cdx[0], o.bx);
            const float dy = q4.y - fmaf(-(float)by, P.cdx[1], o.by);
            const float dz = q4.z - fmaf(-(float)bz, P.cdx[2], o.bz);
            const float r2 = dist2(dx, dy, dz);
            if (!(r2 < P.R2)) continue;
            float rhoj, pj;
            if (sp == 0) {
                const float2 ref = A.cm[o.cbase + bx * nynz + by * P.nz + bz];
                const float2 dev = half2_floats(q4.w);
                rhoj = fmaf(P.rho0, fmaf(dev.x, kDeltaUnit, ref.x), P.rho0);
                pj = fmaf(dev.y, P.p_unit, ref.y);
            } else {
                rhoj = q4.w;
                pj = u.w;
            }
            riemann_pair<true, VISCID, true>(P, dx, dy, dz, r2, vp.x, vp.y, vp.z, o.rho, o.p, u.x, u.y, u.z, rhoj, pj,
                                             sp == 1, acc);
        }
    }
}

template <int VISCID>
__device__ __forceinline__ void fluid_sweep_nlm_body(const DevParams &P, const FluidSweepArgs &A, int blk)
{
    const int i = blk * blockDim.x + threadIdx.x;
    const bool valid = i < A.n;
    unsigned d2bits = 0u;
    if (valid) {
        const float4 off = A.posr[i], vp = A.velp[i];
        const unsigned ci = A.nl_cxyz_f[i];
        int cx, cy, cz;
        unpack_cell(ci, cx, cy, cz);
        OwnMixed o;
        o.bx = __fadd_rn(off.x, P.cdx[0]);
        o.by = __fadd_rn(off.y, P.cdx[1]);
        o.bz = __fadd_rn(off.z, P.cdx[2]);
        o.cbase = A.cell_f[i] - P.ny * P.nz - P.nz - 1;
        o.rho = fmaf(P.rho0, vp.w, P.rho0);
        o.p = eos_delta(P, vp.w);
        const float4 pa = mixed_abs(P, off, cx, cy, cz, o.rho);
        PairAcc acc = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
        fluid_sweep_nlm_pairs<VISCID>(P, A, i, o, pa, vp, ci, acc);
        const float4 x = mixed_abs(P, fluid_update_store_m(P, A, i, off, vp, o.rho, acc, cx, cy, cz), cx, cy, cz,
                                   0.0f);
        const float4 x0 = A.x0[i];
        d2bits = __float_as_uint(dist2(x.x - x0.x, x.y - x0.y, x.z - x0.z));
    }
    const unsigned wmax = __reduce_max_sync(kFull, d2bits);
    if ((threadIdx.x & 31) == 0 && wmax) atomicMax(&A.nl->maxd2, wmax);
}

// launch shapes of the mixed list sweep (more registers than the plain one)
using NlmShape0 = NlShape<128, 8>;  // at most 64 registers
using NlmShape1 = NlShape<128, 10>; // at most 48 registers (a few spills)
using NlmShape2 = NlShape<256, 3>;  // at most 85 registers
static_assert(NlmShape0::threads == NlShape0::threads && NlmShape1::threads == NlShape1::threads &&
                  NlmShape2::threads == NlShape2::threads,
              "mixed list-sweep shapes use the block sizes of the plain ones");

template <int VISCID, class SH>
__global__ void __launch_bounds__(SH::threads, SH::min_blocks) kb_fluid_sweep_nlm_1(const DevParams P,
                                                                                    const FluidSweepArgs A)
{
    fluid_sweep_nlm_body<VISCID>(P, A, (int)blockIdx.x);
}
template <int VISCID, class SH>
__global__ void __launch_bounds__(SH::threads, SH::min_blocks)
    kb_fluid_sweep_nlm(const Item<FluidSweepArgs> *__restrict__ items, const int *__restrict__ bstart, int ninst)
{
    const int inst = locate_instance(bstart, ninst, blockIdx.x);
    fluid_sweep_nlm_body<VISCID>(items[inst].P, items[inst].A, (int)blockIdx.x - bstart[inst]);
}
template <int VISCID, class SH>
__global__ void __launch_bounds__(SH::threads, SH::min_blocks)
    kb_fluid_sweep_nlm_p(const __grid_constant__ SweepBatchParams B)
{
    const int inst = locate_instance(B.bstart, B.n, blockIdx.x);
    const Item<FluidSweepArgs> &it = B.it[inst];
    fluid_sweep_nlm_body<VISCID>(it.P, it.A, (int)blockIdx.x - B.bstart[inst]);
}

// Neighbour-list instances in the mixed form, on a rebuild: every particle's
// absolute position from its cell and offset (the list grid's sort key and, in
// the new order, the positions of the build).
__device__ __forceinline__ void mixed_abs_body(const DevParams &P, const MixedAbsArgs &A, int blk)
{
    if (A.gate && !*A.gate) return; // uniform per block
    FSIM_ELEMENT_BLOCKS(A, blk, b)
    {
        const int s = b * blockDim.x + threadIdx.x;
        if (s >= A.n) continue;
        int cx, cy, cz;
        cell_xyz(P, A.cell[s], cx, cy, cz);
        A.out[s] = mixed_abs(P, A.posr[s], cx, cy, cz, 0.0f);
    }
}
FSIM_BATCHED_KERNEL(kb_mixed_abs, MixedAbsArgs, mixed_abs_body, kBlock)

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
                for (int t = A.start_f[rb + z], te = A.start_f[rb + z + 1]; t < te; ++t) {
                    const float4 q = A.fpos_t ? A.fpos_t[t] : A.fposr[A.ids_f ? A.ids_f[t] : t];
                    const float d2 = dist2(q.x - psx, q.y - psy, q.z - psz);
                    if (d2 <= best) {
                        const int j = A.ids_f ? A.ids_f[t] : t;
                        FSIM_DCHECK(j >= 0 && j < A.nf, 32u, continue);
                        const int o = A.forig[j];
                        if (d2 < best || o < best_orig) {
                            best = d2;
                            best_j = j;
                            best_orig = o;
                            bsx = psx;
                            bsy = psy;
                            bsz = psz;
                        }
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
__device__ __forceinline__ void fluid_rel(const DevParams &P, const RowMixed &R, int t, float sz0, float4 q, float &dx,
                                          float &dy, float &dz)
{
    const int k = (t >= R.b1) + (t >= R.b2);
    dx = q.x - R.sx;
    dy = q.y - R.sy;
    dz = q.z - fmaf(-(float)k, P.cdx[2], sz0);
}

// A candidate's particle id, read from the cell index only when asked for (a
// walk that tests positions in index order needs it for the hits alone).
struct SlotId {
    const int *ids;
    int t;
    __device__ __forceinline__ operator int() const { return ids ? ids[t] : t; }
};

// The mixed-form row walk of a solid particle: calls f(j, q, dx, dy, dz) for
// every fluid candidate of the 27 cells of solid cell `cell`, lanes of a group
// of `G` taking every G-th candidate of a row.  `ids`: the per-step cell index
// of a neighbour-list instance (slot t of the walk is particle ids[t]), else
// nullptr (slot = particle).
template <int G, class F>
__device__ __forceinline__ void solid_fluid_walk_m(const DevParams &P, const int *__restrict__ start_f,
                                                   const int *__restrict__ ids, const float4 *__restrict__ fposr,
                                                   int cell, float4 xi, int g, F &&f,
                                                   const float4 *__restrict__ fpos_t = nullptr)
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
            for (int t = start_f[rb + z0] + g, te = start_f[rb + z1]; t < te; t += G) {
                const float4 q = fpos_t ? fpos_t[t] : fposr[ids ? ids[t] : t];
                float dx, dy, dz;
                fluid_rel(P, R, t, sz0, q, dx, dy, dz);
                f(SlotId{ids, t}, dx, dy, dz);
            }
        }
    }
}

// solidCoupleUpdate (src/solid.cu:262-344) in the mixed form.
__device__ __forceinline__ void couple_mixed_body(const DevParams &P, const CoupleArgs &A, int blk)
{
    const int t = blk * blockDim.x + threadIdx.x;
    const int i = t / kCoupleGroup, g = t % kCoupleGroup;
    const bool valid = i < A.n;
    float nx = 0.0f, ny = 0.0f, nz = 0.0f, psum = 0.0f, wsum = 0.0f;
    if (valid) {
        const float4 xi = A.s_pos[i];
        solid_fluid_walk_m<kCoupleGroup>(P, A.start_f, A.ids_f, A.fposr, A.s_cell[i], xi, g,
                                        [&](SlotId s, float dx, float dy, float dz) {
                                            const float r2 = dist2(dx, dy, dz);
                                            if (r2 < P.R2) {
                                                const int j = s;
                                                const float w = (__expf(-r2 * P.h_inv2) - P.kc1) * P.kc2;
                                                wsum += w;
                                                psum += eos_delta(P, A.fvelp[j].w) * w;
                                            }
                                        },
                                        A.fpos_t);
        Rows rows;
        neighbor_rows(P, A.s_cell[i], rows);
        for (int r = 0; r < rows.count; ++r) {
            const int c0 = rows.base[r] + rows.z0, c1 = rows.base[r] + rows.z1;
            for (int ts = A.start_s[c0] + g, te = A.start_s[c1]; ts < te; ts += kCoupleGroup) {
                const float4 q = A.s_pos[A.ids_s ? A.ids_s[ts] : ts];
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
    nx = group_sum<kCoupleGroup>(nx);
    ny = group_sum<kCoupleGroup>(ny);
    nz = group_sum<kCoupleGroup>(nz);
    psum = group_sum<kCoupleGroup>(psum);
    wsum = group_sum<kCoupleGroup>(wsum);
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

// The list entries resolved once per step (the cells and the sort order are
// fixed for the step's sub-steps): the sorted slot of each entry's neighbour,
// or -1 where its current cell is not adjacent to the owner's.  The sub-steps
// then read one index per entry instead of a chain of three loads.
__device__ __forceinline__ void solid_slots_body(const DevParams &, const SolidArgs &S, int blk)
{
    const int e = blk * blockDim.x + threadIdx.x;
    if (e >= S.ne) return;
    const int i = S.inv[S.nbr_owner[e]], j = S.inv[S.nbr_orig[e]];
    S.nbr_slot[e] = cells_adjacent(S.cxyz[i], S.cxyz[j]) ? j : -1;
}
FSIM_BATCHED_KERNEL(kb_solid_slots, SolidArgs, solid_slots_body, kBlock)

// Kernel weight of a reference-configuration pair from X_j - X_i.  X_j - X_i
// is formed from the sorted reference positions (static, a few hundred KB,
// cache-resident) instead of being stored per list entry: the same FP32
// difference the list was built from, for 4 B per entry instead of 20.
__device__ __forceinline__ float solid_pair_weight(const DevParams &P, float dx, float dy, float dz)
{
    return __fmul_rn(__expf(__fmul_rn(-dist2(dx, dy, dz), P.h_inv2)), P.kdiff);
}

// solidDeformationCalculate (src/solid.cu:10-79): F and L over the
// reference-configuration neighbours, L^-1 (identity when singular),
// F <- F L^-1, Green strain, St-Venant-Kirchhoff 2nd Piola, P = F S.
// Also stores P L^-1 and cof(F) L^-1 (= det(F) F^-T L^-1) for the force sweep.
// MIXED: L^-1 is formed in FP64 (cofactors, determinant, division) and rounded.
// RESOLVE (the step's first sub-step): each list entry's neighbour slot is
// resolved here, as kb_solid_slots would, and stored for the later sub-steps.
// FORM_L (the step's first sub-step): L and its inverse are formed and stored;
// the later sub-steps read the inverse back (L depends on the reference
// configuration and the step's neighbour set only).
template <bool MIXED, bool RESOLVE = false, bool FORM_L = RESOLVE>
__device__ __forceinline__ void solid_deform_body(const DevParams &P, const SolidArgs &S, int blk)
{
    const int t = blk * blockDim.x + threadIdx.x;
    const int i = t / kSolidGroup, g = t % kSolidGroup;
    const bool valid = i < S.n;
    M3 F, L;
#pragma unroll
    for (int k = 0; k < 9; ++k) F.m[k] = L.m[k] = 0.0f;
    if (valid) {
        const float4 xi = S.pos[i], ri = S.ref[i];
        const int o = S.orig[i];
        const unsigned ci = RESOLVE ? S.cxyz[i] : 0u;
        for (int e = S.nbr_off[o] + g, ee = S.nbr_off[o + 1]; e < ee; e += kSolidGroup) {
            int j;
            if (RESOLVE) {
                const int jj = S.inv[S.nbr_orig[e]];
                FSIM_DCHECK(jj >= 0 && jj < S.n, 512u, {
                    S.nbr_slot[e] = -1;
                    continue;
                });
                j = cells_adjacent(ci, S.cxyz[jj]) ? jj : -1;
                S.nbr_slot[e] = j;
            } else {
                j = S.nbr_slot[e];
            }
            if (j < 0) continue;
            const float4 xj = S.pos[j], rj = S.ref[j];
            const float dx[3] = {xj.x - xi.x, xj.y - xi.y, xj.z - xi.z};
            const float dX[3] = {__fsub_rn(rj.x, ri.x), __fsub_rn(rj.y, ri.y), __fsub_rn(rj.z, ri.z)};
            const float w = solid_pair_weight(P, dX[0], dX[1], dX[2]);
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                // roundings spelled out: the instantiations compute alike
                const float ra = __fmul_rn(dx[a], w), la = __fmul_rn(dX[a], w);
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    F.m[3 * a + c] = fmaf(ra, dX[c], F.m[3 * a + c]);
                    if (FORM_L) L.m[3 * a + c] = fmaf(la, dX[c], L.m[3 * a + c]);
                }
            }
        }
    }
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        F.m[k] = group_sum(F.m[k]);
        if (FORM_L) L.m[k] = group_sum(L.m[k]);
    }
    if (!valid || g) return;
    M3 Linv;
    if (!FORM_L) {
#pragma unroll
        for (int k = 0; k < 9; ++k) Linv.m[k] = S.L[9 * i + k];
    } else if (MIXED) {
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
        if (FORM_L) S.L[9 * i + k] = Linv.m[k];
        S.AV[9 * i + k] = AV.m[k];
    }
    float4 *pl = reinterpret_cast<float4 *>(S.PL + kPLStride * i);
    pl[0] = make_float4(PL.m[0], PL.m[1], PL.m[2], PL.m[3]);
    pl[1] = make_float4(PL.m[4], PL.m[5], PL.m[6], PL.m[7]);
    pl[2] = make_float4(PL.m[8], 0.0f, 0.0f, 0.0f);
}
FSIM_BATCHED_KERNEL(kb_solid_deform, SolidArgs, solid_deform_body<false>, kBlock)
FSIM_BATCHED_KERNEL(kb_solid_deform_mixed, SolidArgs, solid_deform_body<true>, kBlock)
FSIM_BATCHED_KERNEL(kb_solid_deform_resolve, SolidArgs, (solid_deform_body<false, true>), kBlock)
FSIM_BATCHED_KERNEL(kb_solid_deform_mixed_resolve, SolidArgs, (solid_deform_body<true, true>), kBlock)

// solidForceCalculate (src/solid.cu:81-207): fluid traction over the fluid
// neighbours (current configuration, fluid already advanced; candidates from
// the 27 cells of the step-start cell) plus stress divergence and artificial
// viscosity over the reference-configuration solid neighbours.
// MIXED: fluid positions are cell offsets, fluid (rho, p) come from delta.
//
// Fluid lists (plain form, FLIST): the fluid does not move during a step's
// sub-steps and the candidates come from the step's cells, so sub-step 0
// (FLIST 1) walks the 27 cells and records, per lane, the candidates within
// (R + d)(1 + 1e-5) of the particle; later sub-steps (FLIST 2) walk only that
// list while the particle is within d of where it was recorded (then every
// dropped candidate is farther than R, with room for FP32 rounding).  A lane
// keeps exactly the candidates it walked, in the same order, so the sums are
// those of the full walk (FLIST 0) bit for bit; an overflowing list (count -1)
// or a larger displacement falls back to the walk.  Every rounding of the
// sums is spelled out so that the three instantiations compute alike.
template <bool MIXED, int FLIST = 0>
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
            const float w = __fmul_rn(__expf(__fmul_rn(-r2, P.h_inv2)), P.kdiff);
            const float k2 = __fmul_rn(2.0f, fmaf(__fsub_rn(u.z, vi.z), ni.z,
                                                  fmaf(__fsub_rn(u.y, vi.y), ni.y,
                                                       __fmul_rn(__fsub_rn(u.x, vi.x), ni.x))));
            const float inv_r = r2 > 0.0f ? rsqrtf(r2) : 0.0f;
            const float du = __fmul_rn(__fmul_rn(-k2, fmaf(ni.z, dz, fmaf(ni.y, dy, __fmul_rn(ni.x, dx)))), inv_r);
            float ps = __fmul_rn(0.5f, __fadd_rn(ni.w, pj));
            if (du >= 0.0f) ps = fmaf(__fmul_rn(__fmul_rn(0.5f, rhoj), du), P.c0, ps);
            const float f = __fmul_rn(__fmul_rn(-2.0f, ps), __fmul_rn(P.rho_s_inv, w));
            cx = fmaf(f, dx, cx);
            cy = fmaf(f, dy, cy);
            cz = fmaf(f, dz, cz);
        };
        if (MIXED) {
            solid_fluid_walk_m<kSolidGroup>(P, S.start_f, S.ids_f, S.fposr, S.cell[i], xi, g,
                                            [&](SlotId s, float dx, float dy, float dz) {
                                                const float r2 = dist2(dx, dy, dz);
                                                if (r2 < P.R2) {
                                                    const float4 u = S.fvelp[(int)s];
                                                    traction(dx, dy, dz, r2, u, fmaf(P.rho0, u.w, P.rho0),
                                                             eos_delta(P, u.w));
                                                }
                                            });
        }
        bool walk = !MIXED;
        const int T = kSolidGroup * S.n; // stride of the entry-major lane lists
        if (!MIXED && FLIST == 2) {
            const float4 o = S.fl_org[i];
            const int c = S.fl_cnt[t];
            if (c >= 0 && dist2(xi.x - o.x, xi.y - o.y, xi.z - o.z) < P.fl_move2) {
                walk = false;
                for (int e = 0; e < c; ++e) {
                    const int j = S.fl[(size_t)e * T + t];
                    FSIM_DCHECK(j >= 0 && j < S.nf, 1024u, continue);
                    const float4 q = S.fposr[j];
                    const float dx = q.x - xi.x, dy = q.y - xi.y, dz = q.z - xi.z;
                    const float r2 = dist2(dx, dy, dz);
                    if (r2 < P.R2) {
                        const float4 u = S.fvelp[j];
                        traction(dx, dy, dz, r2, u, q.w, u.w);
                    }
                }
            }
        }
        if (walk) {
            Rows rows;
            neighbor_rows(P, S.cell[i], rows);
            int nrec = 0;
            for (int r = 0; r < rows.count; ++r) {
                const int c0 = rows.base[r] + rows.z0, c1 = rows.base[r] + rows.z1;
                for (int tf = S.start_f[c0] + g, te = S.start_f[c1]; tf < te; tf += kSolidGroup) {
                    const int j = S.ids_f ? S.ids_f[tf] : tf;
                    FSIM_DCHECK(j >= 0 && j < S.nf, 256u, continue);
                    const float4 q = S.fposr[j];
                    const float dx = q.x - xi.x, dy = q.y - xi.y, dz = q.z - xi.z;
                    const float r2 = dist2(dx, dy, dz);
                    if (FLIST == 1 && r2 < P.fl_build2) {
                        if (nrec < kFluidListCap) S.fl[(size_t)nrec * T + t] = j;
                        ++nrec;
                    }
                    if (r2 < P.R2) {
                        const float4 u = S.fvelp[j];
                        traction(dx, dy, dz, r2, u, q.w, u.w);
                    }
                }
            }
            if (FLIST == 1) {
                S.fl_cnt[t] = nrec <= kFluidListCap ? nrec : -1;
                if (g == 0) S.fl_org[i] = xi;
            }
        }
        // solidSolidForce (src/solid.cu:119-157)
        float PLi[9], AVi[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) {
            PLi[k] = S.PL[kPLStride * i + k];
            AVi[k] = S.AV[9 * i + k];
        }
        const float4 ri = S.ref[i];
        const int o = S.orig[i];
        for (int e = S.nbr_off[o] + g, ee = S.nbr_off[o + 1]; e < ee; e += kSolidGroup) {
            const int j = S.nbr_slot[e];
            if (j < 0) continue;
            FSIM_DCHECK(j < S.n, 2048u, continue);
            const float4 rj = S.ref[j];
            const float dX = __fsub_rn(rj.x, ri.x), dY = __fsub_rn(rj.y, ri.y), dZ = __fsub_rn(rj.z, ri.z);
            const float w = solid_pair_weight(P, dX, dY, dZ);
            const float4 *plj = reinterpret_cast<const float4 *>(S.PL + kPLStride * j);
            const float4 q0 = plj[0], q1 = plj[1], q2 = plj[2];
            const float PLj[9] = {q0.x, q0.y, q0.z, q0.w, q1.x, q1.y, q1.z, q1.w, q2.x};
            const float ws = __fmul_rn(w, P.rho_s_inv);
            auto row3 = [&](float a0, float a1, float a2) {
                return fmaf(a2, dZ, fmaf(a1, dY, __fmul_rn(a0, dX)));
            };
            ax = fmaf(row3(__fadd_rn(PLj[0], PLi[0]), __fadd_rn(PLj[1], PLi[1]), __fadd_rn(PLj[2], PLi[2])), ws, ax);
            ay = fmaf(row3(__fadd_rn(PLj[3], PLi[3]), __fadd_rn(PLj[4], PLi[4]), __fadd_rn(PLj[5], PLi[5])), ws, ay);
            az = fmaf(row3(__fadd_rn(PLj[6], PLi[6]), __fadd_rn(PLj[7], PLi[7]), __fadd_rn(PLj[8], PLi[8])), ws, az);
            const float4 xj = S.pos[j], vj = S.vel[j];
            const float ddx = __fsub_rn(xj.x, xi.x), ddy = __fsub_rn(xj.y, xi.y), ddz = __fsub_rn(xj.z, xi.z);
            const float dvdx = fmaf(__fsub_rn(vj.z, vi.z), ddz,
                                    fmaf(__fsub_rn(vj.y, vi.y), ddy, __fmul_rn(__fsub_rn(vj.x, vi.x), ddx)));
            const float nu = __fdiv_rn(__fmul_rn(P.h, dvdx),
                                       __fadd_rn(fmaf(ddz, ddz, fmaf(ddy, ddy, __fmul_rn(ddx, ddx))), P.eps_h2));
            const float visc = __fmul_rn(fmaf(__fmul_rn(P.alpha, nu), P.cs_s, -__fmul_rn(__fmul_rn(P.beta, nu), nu)), w);
            ax = fmaf(row3(AVi[0], AVi[1], AVi[2]), visc, ax);
            ay = fmaf(row3(AVi[3], AVi[4], AVi[5]), visc, ay);
            az = fmaf(row3(AVi[6], AVi[7], AVi[8]), visc, az);
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
    S.dudt[i] = make_float4(__fadd_rn(ax, cx), __fadd_rn(ay, cy), __fadd_rn(az, cz), 0.0f);
}
FSIM_BATCHED_KERNEL_P(kb_solid_force, SolidArgs, solid_force_body<false>, kBlock)
FSIM_BATCHED_KERNEL_P(kb_solid_force_record, SolidArgs, (solid_force_body<false, 1>), kBlock)
FSIM_BATCHED_KERNEL_P(kb_solid_force_listed, SolidArgs, (solid_force_body<false, 2>), kBlock)
FSIM_BATCHED_KERNEL(kb_solid_force_mixed, SolidArgs, solid_force_body<true>, kBlock)

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
// per-row particle counts: fluid, solid, virtual, jitter-drawing sites

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
            solid_fluid_walk_m<32>(P, A.start_f, A.ids_f, A.fposr, cell, xi, lane, fluid);
        }
        Rows rows;
        neighbor_rows(P, cell, rows);
        for (int r = 0; r < rows.count; ++r) {
            const int c0 = rows.base[r] + rows.z0, c1 = rows.base[r] + rows.z1;
            if (!P.mixed) {
                for (int t = A.start_f[c0] + lane, te = A.start_f[c1]; t < te; t += 32) {
                    const int j = A.ids_f ? A.ids_f[t] : t;
                    const float4 q = A.fposr[j];
                    fluid(j, q.x - xi.x, q.y - xi.y, q.z - xi.z);
                }
            }
            for (int t = A.start_s[c0] + lane, te = A.start_s[c1]; t < te; t += 32) {
                const int j = A.ids_s ? A.ids_s[t] : t;
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
constexpr unsigned kBarrierSpinLimit = 1u << 22; // x ~64 ns sleeps: about a quarter of a second and more

// `limit`: polls before giving up (kBarrierSpinLimit unless the configuration
// asks for fewer, gb300_barrier_wait_polls)
__device__ __forceinline__ void grid_sync(GridBarrier *b, bool &ok, unsigned limit)
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
                if (++spins > limit) {
                    ok = false;
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
    }
    // thread 0 alone waited: every thread of the CTA learns whether it gave up
    ok = __syncthreads_and(ok) != 0;
}

struct SolidFusedArgs {
    const int *bstart_w, *bstart_t; // prefix tables: kSolidGroup lanes per particle / thread per particle
    int ninst, max_sub;
    GridBarrier *barrier;
    unsigned polls; // barrier wait limit
};

template <bool MIXED>
__global__ void __launch_bounds__(kBlock, 3) kb_solid_fused(const Item<SolidArgs> *__restrict__ items,
                                                         const SolidFusedArgs F)
{
    const int total_w = F.bstart_w[F.ninst], total_t = F.bstart_t[F.ninst];
    bool ok = true;
    // a CTA whose wait gave up leaves at once (the CTAs still waiting for it
    // give up in turn after their own bounded wait)
    for (int k = 0; k < F.max_sub && ok; ++k) {
        for (int b = blockIdx.x; b < total_w; b += gridDim.x) {
            const int inst = locate_instance(F.bstart_w, F.ninst, b);
            if (k >= items[inst].A.nsub) continue;
            const DevParams P = items[inst].P;
            if (k == 0) solid_deform_body<MIXED, false, true>(P, items[inst].A, b - F.bstart_w[inst]);
            else solid_deform_body<MIXED>(P, items[inst].A, b - F.bstart_w[inst]);
        }
        grid_sync(F.barrier, ok, F.polls);
        if (!ok) break;
        for (int b = blockIdx.x; b < total_w; b += gridDim.x) {
            const int inst = locate_instance(F.bstart_w, F.ninst, b);
            if (k >= items[inst].A.nsub) continue;
            const DevParams P = items[inst].P;
            solid_force_body<MIXED>(P, items[inst].A, b - F.bstart_w[inst]);
        }
        grid_sync(F.barrier, ok, F.polls);
        if (!ok) break;
        for (int b = blockIdx.x; b < total_t; b += gridDim.x) {
            const int inst = locate_instance(F.bstart_t, F.ninst, b);
            if (k >= items[inst].A.nsub) continue;
            const DevParams P = items[inst].P;
            solid_update_body(P, items[inst].A, b - F.bstart_t[inst]);
        }
        if (k + 1 < F.max_sub) grid_sync(F.barrier, ok, F.polls);
    }
    if (!ok && threadIdx.x == 0)
        for (int inst = 0; inst < F.ninst; ++inst) atomicOr(items[inst].A.flags, FLAG_BARRIER_TIMEOUT);
}

// ------------------------------------------------------- neighbour counts
// Per fluid particle: fluid, solid and wall particles within the impact
// distance in its 27 cells.  Neighbour-list instances pass their per-step cell
// indices (ids_f, ids_s) and the list grid Pv of the walls, whose cells are
// then located from the particle's position.
__global__ void k_neighbor_counts(const DevParams P, const DevParams Pv, const float4 *__restrict__ fposr,
                                  const int *__restrict__ cell_f, const int *__restrict__ start_f,
                                  const int *__restrict__ ids_f, const float4 *__restrict__ s_pos,
                                  const int *__restrict__ start_s, const int *__restrict__ ids_s,
                                  const float4 *__restrict__ v_posr, const int *__restrict__ start_v,
                                  int *__restrict__ out, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 p = fposr[i];
    Rows rows;
    neighbor_rows(P, cell_f[i], rows);
    int cf = 0, cs = 0, cv = 0;
    for (int r = 0; r < rows.count; ++r) {
        const int c0 = rows.base[r] + rows.z0, c1 = rows.base[r] + rows.z1;
        for (int t = start_f[c0]; t < start_f[c1]; ++t) {
            const float4 q = fposr[ids_f ? ids_f[t] : t];
            cf += dist2(q.x - p.x, q.y - p.y, q.z - p.z) < P.R2;
        }
        for (int t = start_s[c0]; t < start_s[c1]; ++t) {
            const float4 q = s_pos[ids_s ? ids_s[t] : t];
            cs += dist2(q.x - p.x, q.y - p.y, q.z - p.z) < P.R2;
        }
    }
    Rows vrows;
    neighbor_rows(Pv, ids_f ? cell_index(Pv, p.x, p.y, p.z, nullptr) : cell_f[i], vrows);
    for (int r = 0; r < vrows.count; ++r) {
        const int c0 = vrows.base[r] + vrows.z0, c1 = vrows.base[r] + vrows.z1;
        for (int j = start_v[c0]; j < start_v[c1]; ++j) {
            const float4 q = v_posr[j];
            cv += dist2(q.x - p.x, q.y - p.y, q.z - p.z) < P.R2;
        }
    }
    out[3 * i] = cf;
    out[3 * i + 1] = cs;
    out[3 * i + 2] = cv;
}

// The same counts of a neighbour-list instance, from its lists (which hold
// every pair within the impact distance while no rebuild is due).
__global__ void k_neighbor_counts_nl(const DevParams P, const float4 *__restrict__ fposr, const int *__restrict__ list,
                                     const int *__restrict__ cnt, int cap, const float4 *__restrict__ s_pos,
                                     const float4 *__restrict__ v_posr, int *__restrict__ out, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 p = fposr[i];
    int c[3] = {0, 0, 0};
    const int m = min(cnt[i], cap);
    for (int k = 0; k < m; ++k) {
        const unsigned e = (unsigned)list[((size_t)(k / kNlGroup) * n + i) * kNlGroup + k % kNlGroup];
        const int sp = (int)(e >> kNlSpeciesShift), j = (int)(e & kNlIndexMask);
        const float4 q = sp == 0 ? fposr[j] : sp == 1 ? v_posr[j] : s_pos[j];
        if (dist2(q.x - p.x, q.y - p.y, q.z - p.z) < P.R2) ++c[sp == 0 ? 0 : sp == 2 ? 1 : 2];
    }
    out[3 * i] = c[0];
    out[3 * i + 1] = c[1];
    out[3 * i + 2] = c[2];
}

// The counts in the mixed form: pairs as the mixed sweep's cell walk takes
// them (fluid and wall candidates of the 27 cells, r^2 < R^2 with the
// particle's offset shifted by the cell difference; solid candidates of the 27
// cells within R of the absolute position).  Walls lie on the walked grid
// (v_cxyz == nullptr, offsets from the walked cell) or, in a neighbour-list
// instance, on the list grid Pv with their impact-grid cells in v_cxyz.
__global__ void k_neighbor_counts_mixed(const DevParams P, const DevParams Pv, const float4 *__restrict__ fposr,
                                        const int *__restrict__ cell_f, const int *__restrict__ start_f,
                                        const int *__restrict__ ids_f, const float4 *__restrict__ s_pos,
                                        const int *__restrict__ start_s, const int *__restrict__ ids_s,
                                        const float4 *__restrict__ v_posr, const int *__restrict__ start_v,
                                        const unsigned *__restrict__ v_cxyz, int *__restrict__ out, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 off = fposr[i];
    int cx, cy, cz;
    cell_xyz(P, cell_f[i], cx, cy, cz);
    const float4 pa = mixed_abs(P, off, cx, cy, cz, 0.0f);
    const float obx = __fadd_rn(off.x, P.cdx[0]), oby = __fadd_rn(off.y, P.cdx[1]), obz = __fadd_rn(off.z, P.cdx[2]);
    int cf = 0, cs = 0, cv = 0;
    for (int ox = -1; ox <= 1; ++ox)
        for (int oy = -1; oy <= 1; ++oy)
            for (int oz = -1; oz <= 1; ++oz) {
                const int x = cx + ox, y = cy + oy, z = cz + oz;
                if (x < 0 || x >= P.nx || y < 0 || y >= P.ny || z < 0 || z >= P.nz) continue;
                const int c = (x * P.ny + y) * P.nz + z;
                const float psx = shifted(obx, ox, P.cdx[0]), psy = shifted(oby, oy, P.cdx[1]),
                            psz = shifted(obz, oz, P.cdx[2]);
                for (int t = start_f[c]; t < start_f[c + 1]; ++t) {
                    const float4 q = fposr[ids_f ? ids_f[t] : t];
                    cf += dist2(q.x - psx, q.y - psy, q.z - psz) < P.R2;
                }
                for (int t = start_s[c]; t < start_s[c + 1]; ++t) {
                    const float4 q = s_pos[ids_s ? ids_s[t] : t];
                    cs += dist2(q.x - pa.x, q.y - pa.y, q.z - pa.z) < P.R2;
                }
                if (!v_cxyz)
                    for (int j = start_v[c]; j < start_v[c + 1]; ++j) {
                        const float4 q = v_posr[j];
                        cv += dist2(q.x - psx, q.y - psy, q.z - psz) < P.R2;
                    }
            }
    if (v_cxyz) {
        Rows vrows;
        neighbor_rows(Pv, cell_index(Pv, pa.x, pa.y, pa.z, nullptr), vrows);
        for (int r = 0; r < vrows.count; ++r) {
            const int c0 = vrows.base[r] + vrows.z0, c1 = vrows.base[r] + vrows.z1;
            for (int j = start_v[c0]; j < start_v[c1]; ++j) {
                int jx, jy, jz;
                unpack_cell(v_cxyz[j], jx, jy, jz);
                const int ox = jx - cx, oy = jy - cy, oz = jz - cz;
                if (abs(ox) > 1 || abs(oy) > 1 || abs(oz) > 1) continue;
                const float4 q = v_posr[j];
                cv += dist2(q.x - shifted(obx, ox, P.cdx[0]), q.y - shifted(oby, oy, P.cdx[1]),
                            q.z - shifted(obz, oz, P.cdx[2])) < P.R2;
            }
        }
    }
    out[3 * i] = cf;
    out[3 * i + 1] = cs;
    out[3 * i + 2] = cv;
}

// The same counts of a mixed-form neighbour-list instance from its lists,
// with the list sweep's pair rule.
__global__ void k_neighbor_counts_nlm(const DevParams P, const float4 *__restrict__ fposr,
                                      const int *__restrict__ cell_f, const unsigned *__restrict__ cxyz_f,
                                      const int *__restrict__ list, const int *__restrict__ cnt, int cap,
                                      const float4 *__restrict__ s_pos, const unsigned *__restrict__ cxyz_s,
                                      const float4 *__restrict__ v_posr, const unsigned *__restrict__ cxyz_v,
                                      int *__restrict__ out, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 off = fposr[i];
    int cx, cy, cz;
    cell_xyz(P, cell_f[i], cx, cy, cz);
    const float4 pa = mixed_abs(P, off, cx, cy, cz, 0.0f);
    const float obx = __fadd_rn(off.x, P.cdx[0]), oby = __fadd_rn(off.y, P.cdx[1]), obz = __fadd_rn(off.z, P.cdx[2]);
    const unsigned ci = cxyz_f[i];
    int c[3] = {0, 0, 0};
    const int m = min(cnt[i], cap);
    for (int k = 0; k < m; ++k) {
        const unsigned e = (unsigned)list[((size_t)(k / kNlGroup) * n + i) * kNlGroup + k % kNlGroup];
        const int sp = (int)(e >> kNlSpeciesShift), j = (int)(e & kNlIndexMask);
        if (sp == 2) {
            const float4 q = s_pos[j];
            if (dist2(q.x - pa.x, q.y - pa.y, q.z - pa.z) < P.R2 && cells_adjacent(ci, cxyz_s[j])) ++c[1];
            continue;
        }
        const float4 q = sp == 0 ? fposr[j] : v_posr[j];
        int jx, jy, jz;
        unpack_cell(sp == 0 ? cxyz_f[j] : cxyz_v[j], jx, jy, jz);
        const int ox = jx - cx, oy = jy - cy, oz = jz - cz;
        if (abs(ox) > 1 || abs(oy) > 1 || abs(oz) > 1) continue;
        if (dist2(q.x - shifted(obx, ox, P.cdx[0]), q.y - shifted(oby, oy, P.cdx[1]),
                  q.z - shifted(obz, oz, P.cdx[2])) < P.R2)
            ++c[sp == 0 ? 0 : 2];
    }
    out[3 * i] = c[0];
    out[3 * i + 1] = c[1];
    out[3 * i + 2] = c[2];
}

// (posr, velp) records of every fluid slot (after fields were set from the
// host); the mixed form (cxyz != nullptr) carries the packed cell in place of
// the density deviation
__global__ void k_pack_records(const float4 *__restrict__ posr, const float4 *__restrict__ velp,
                               const unsigned *__restrict__ cxyz, int n, float4 *__restrict__ rec)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 v = velp[i];
    if (cxyz) v.w = __uint_as_float(cxyz[i]);
    rec[2 * (size_t)i] = posr[i];
    rec[2 * (size_t)i + 1] = v;
}

// dst[t] = src[ids[t]]: positions set from the host, into the per-step
// index's order (between the cell phase and the walks that read it)
__global__ void k_gather_f4(const int *__restrict__ ids, const float4 *__restrict__ src, int n,
                            float4 *__restrict__ dst)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) dst[t] = src[ids[t]];
}

// Positions set from the host: fold their squared displacement since the last
// list build into the instance's running maximum (the next step's decision).
// Mixed form (cell != nullptr): posr holds offsets from the cells.
__global__ void k_nl_displacement(const DevParams P, const float4 *__restrict__ posr, const int *__restrict__ cell,
                                  const float4 *__restrict__ x0, int n, NlState *__restrict__ nl)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned d2 = 0u;
    if (i < n) {
        float4 p = posr[i];
        if (cell) {
            int cx, cy, cz;
            cell_xyz(P, cell[i], cx, cy, cz);
            p = mixed_abs(P, p, cx, cy, cz, 0.0f);
        }
        const float4 o = x0[i];
        d2 = __float_as_uint(dist2(p.x - o.x, p.y - o.y, p.z - o.z));
    }
    d2 = __reduce_max_sync(kFull, d2);
    if ((threadIdx.x & 31) == 0 && d2) atomicMax(&nl->maxd2, d2);
}

// cell index of every position (the wall particles' impact-grid cells), and
// optionally its packed coordinates
__global__ void k_cells_of(const DevParams P, const float4 *__restrict__ pos, int n, int *__restrict__ out,
                           unsigned *__restrict__ packed)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 p = pos[i];
    const int c = cell_index(P, p.x, p.y, p.z, nullptr);
    out[i] = c;
    if (packed) packed[i] = pack_cell(P, c);
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

namespace fsim_rt {

#define FSIM_LAUNCH(KB, ARGS, THREADS) KB<<<g, THREADS, 0, st>>>(items_of<ARGS>(pl, L), tb, n)
// one instance by value; up to ParamBlock<ARGS>::kMax as a parameter block; else the item array
#define FSIM_LAUNCH_P(KB, ARGS, THREADS)                                                                    \
    if (n == 1) {                                                                                          \
        const Item<ARGS> &it1 = host_item<ARGS>(pl, L);                                                    \
        KB##_1<<<g, THREADS, 0, st>>>(it1.P, it1.A);                                                       \
    } else if (n <= ParamBlock<ARGS>::kMax) {                                                              \
        static thread_local ParamBlock<ARGS> B;                                                            \
        B.n = n;                                                                                           \
        std::memcpy(B.bstart, pl.host.data() + L.table_off, sizeof(int) * (n + 1));                        \
        std::memcpy(B.it, pl.host.data() + L.items_off, sizeof(Item<ARGS>) * n);                           \
        KB##_p<<<g, THREADS, 0, st>>>(B);                                                                  \
    } else {                                                                                               \
        KB<<<g, THREADS, 0, st>>>(items_of<ARGS>(pl, L), tb, n);                                           \
    }

// Enqueue a plan's launches; optional events around the fluid sweep.
fsim_status enqueue_plan(const Plan &pl, cudaStream_t st, int shape_arg, cudaEvent_t sweep0, cudaEvent_t sweep1,
                         const cudaEvent_t *per_launch, unsigned sweep_flags, const cudaEvent_t *tune_ev,
                         int tune_rounds)
{
    using SweepFn = void (*)(const Item<FluidSweepArgs> *, const int *, int);
    using Sweep1Fn = void (*)(const DevParams, const FluidSweepArgs);
    using SweepPFn = void (*)(const SweepBatchParams);
    static const SweepPFn sweepsp[6][kSweepShapes] = {
        {kb_fluid_sweep_p<false, 0, Shape0>, kb_fluid_sweep_p<false, 0, Shape1>, kb_fluid_sweep_p<false, 0, Shape2>},
        {kb_fluid_sweep_p<false, 1, Shape0>, kb_fluid_sweep_p<false, 1, Shape1>, kb_fluid_sweep_p<false, 1, Shape2>},
        {kb_fluid_sweep_p<false, 2, Shape0>, kb_fluid_sweep_p<false, 2, Shape1>, kb_fluid_sweep_p<false, 2, Shape2>},
        {kb_fluid_sweep_p<true, 0, Shape0>, kb_fluid_sweep_p<true, 0, Shape1>, kb_fluid_sweep_p<true, 0, Shape2>},
        {kb_fluid_sweep_p<true, 1, Shape0>, kb_fluid_sweep_p<true, 1, Shape1>, kb_fluid_sweep_p<true, 1, Shape2>},
        {kb_fluid_sweep_p<true, 2, Shape0>, kb_fluid_sweep_p<true, 2, Shape1>, kb_fluid_sweep_p<true, 2, Shape2>}};
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
    // list sweep [VISCID][shape], the variants kSweepNlVariant + VISCID
    static const Sweep1Fn nl1[3][kSweepShapes] = {
        {kb_fluid_sweep_nl_1<0, NlShape0>, kb_fluid_sweep_nl_1<0, NlShape1>, kb_fluid_sweep_nl_1<0, NlShape2>},
        {kb_fluid_sweep_nl_1<1, NlShape0>, kb_fluid_sweep_nl_1<1, NlShape1>, kb_fluid_sweep_nl_1<1, NlShape2>},
        {kb_fluid_sweep_nl_1<2, NlShape0>, kb_fluid_sweep_nl_1<2, NlShape1>, kb_fluid_sweep_nl_1<2, NlShape2>}};
    static const SweepPFn nlp[3][kSweepShapes] = {
        {kb_fluid_sweep_nl_p<0, NlShape0>, kb_fluid_sweep_nl_p<0, NlShape1>, kb_fluid_sweep_nl_p<0, NlShape2>},
        {kb_fluid_sweep_nl_p<1, NlShape0>, kb_fluid_sweep_nl_p<1, NlShape1>, kb_fluid_sweep_nl_p<1, NlShape2>},
        {kb_fluid_sweep_nl_p<2, NlShape0>, kb_fluid_sweep_nl_p<2, NlShape1>, kb_fluid_sweep_nl_p<2, NlShape2>}};
    static const SweepFn nlb[3][kSweepShapes] = {
        {kb_fluid_sweep_nl<0, NlShape0>, kb_fluid_sweep_nl<0, NlShape1>, kb_fluid_sweep_nl<0, NlShape2>},
        {kb_fluid_sweep_nl<1, NlShape0>, kb_fluid_sweep_nl<1, NlShape1>, kb_fluid_sweep_nl<1, NlShape2>},
        {kb_fluid_sweep_nl<2, NlShape0>, kb_fluid_sweep_nl<2, NlShape1>, kb_fluid_sweep_nl<2, NlShape2>}};
    // mixed-form list sweep, the variants kSweepNlMixedVariant + VISCID
    static const Sweep1Fn nlm1[3][kSweepShapes] = {
        {kb_fluid_sweep_nlm_1<0, NlmShape0>, kb_fluid_sweep_nlm_1<0, NlmShape1>, kb_fluid_sweep_nlm_1<0, NlmShape2>},
        {kb_fluid_sweep_nlm_1<1, NlmShape0>, kb_fluid_sweep_nlm_1<1, NlmShape1>, kb_fluid_sweep_nlm_1<1, NlmShape2>},
        {kb_fluid_sweep_nlm_1<2, NlmShape0>, kb_fluid_sweep_nlm_1<2, NlmShape1>, kb_fluid_sweep_nlm_1<2, NlmShape2>}};
    static const SweepPFn nlmp[3][kSweepShapes] = {
        {kb_fluid_sweep_nlm_p<0, NlmShape0>, kb_fluid_sweep_nlm_p<0, NlmShape1>, kb_fluid_sweep_nlm_p<0, NlmShape2>},
        {kb_fluid_sweep_nlm_p<1, NlmShape0>, kb_fluid_sweep_nlm_p<1, NlmShape1>, kb_fluid_sweep_nlm_p<1, NlmShape2>},
        {kb_fluid_sweep_nlm_p<2, NlmShape0>, kb_fluid_sweep_nlm_p<2, NlmShape1>, kb_fluid_sweep_nlm_p<2, NlmShape2>}};
    static const SweepFn nlmb[3][kSweepShapes] = {
        {kb_fluid_sweep_nlm<0, NlmShape0>, kb_fluid_sweep_nlm<0, NlmShape1>, kb_fluid_sweep_nlm<0, NlmShape2>},
        {kb_fluid_sweep_nlm<1, NlmShape0>, kb_fluid_sweep_nlm<1, NlmShape1>, kb_fluid_sweep_nlm<1, NlmShape2>},
        {kb_fluid_sweep_nlm<2, NlmShape0>, kb_fluid_sweep_nlm<2, NlmShape1>, kb_fluid_sweep_nlm<2, NlmShape2>}};
    for (size_t k = 0; k < pl.launches.size(); ++k) {
        const Launch &L = pl.launches[k];
        const int *tb = reinterpret_cast<const int *>(pl.arena + L.table_off);
        const int g = L.blocks, n = L.ninst;
        if (per_launch) CK(cudaEventRecord(per_launch[2 * k], st));
        switch (L.kind) {
        case L_ZERO: FSIM_LAUNCH(kb_zero, ZeroArgs, kBlock); break;
        case L_HASH: FSIM_LAUNCH(kb_hash, HashArgs, kBlock); break;
        case L_SCAN_REDUCE: FSIM_LAUNCH(kb_scan_reduce, ScanArgs, kScanThreads); break;
        case L_SCAN_PARTIALS: FSIM_LAUNCH(kb_scan_partials, ScanArgs, kScanThreads); break;
        case L_SCAN_APPLY: FSIM_LAUNCH(kb_scan_apply, ScanArgs, kScanThreads); break;
        case L_SCATTER: FSIM_LAUNCH(kb_scatter, ScatterArgs, kBlock); break;
        case L_GATHER_F: FSIM_LAUNCH(kb_gather_fluid, GatherFluidArgs, kBlock); break;
        case L_GATHER_S: FSIM_LAUNCH(kb_gather_solid, GatherSolidArgs, kBlock); break;
        case L_RANK_F:
        case L_RANK_S: FSIM_LAUNCH(kb_rank, RankArgs, kBlock); break;
        case L_NL_DECIDE: FSIM_LAUNCH(kb_nl_decide, NlDecideArgs, kBlock); break;
        case L_NL_BUILD: FSIM_LAUNCH(kb_nl_build, NlBuildArgs, kNlBuildWarps * 32); break;
        case L_MIXED_ABS: FSIM_LAUNCH(kb_mixed_abs, MixedAbsArgs, kBlock); break;
        case L_MIXED_REC: FSIM_LAUNCH(kb_mixed_records, CellRefArgs, kBlock); break;
        case L_COUPLE: FSIM_LAUNCH(kb_couple, CoupleArgs, kBlock); break;
        case L_VIRT: FSIM_LAUNCH(kb_virt, VirtArgs, kBlock); break;
        case L_SWEEP:
            if (sweep0) CK(cudaEventRecordWithFlags(sweep0, st, sweep_flags));
            for (int tr = 0; tr < (tune_ev ? tune_rounds * kSweepShapes : 1); ++tr) {
                const int shape = tune_ev ? tr % kSweepShapes : shape_arg;
                if (tune_ev) CK(cudaEventRecord(tune_ev[2 * tr], st));
                const int *tbs = reinterpret_cast<const int *>(pl.arena + L.shape_table_off[shape]);
                const int gs = L.shape_blocks[shape], thr = kShapeWarps[shape] * 32;
                if (L.variant >= kSweepNlVariant) {
                    const bool mx = L.variant >= kSweepNlMixedVariant;
                    const int v = L.variant - (mx ? kSweepNlMixedVariant : kSweepNlVariant);
                    if (n == 1) {
                        const Item<FluidSweepArgs> &it = host_item<FluidSweepArgs>(pl, L);
                        (mx ? nlm1 : nl1)[v][shape]<<<gs, thr, 0, st>>>(it.P, it.A);
                    } else if (n <= kSweepParamItems) {
                        static thread_local SweepBatchParams B;
                        B.n = n;
                        std::memcpy(B.bstart, pl.host.data() + L.shape_table_off[shape], sizeof(int) * (n + 1));
                        std::memcpy(B.it, pl.host.data() + L.items_off, sizeof(Item<FluidSweepArgs>) * n);
                        (mx ? nlmp : nlp)[v][shape]<<<gs, thr, 0, st>>>(B);
                    } else {
                        (mx ? nlmb : nlb)[v][shape]<<<gs, thr, 0, st>>>(items_of<FluidSweepArgs>(pl, L), tbs, n);
                    }
                } else if (n == 1) {
                    const Item<FluidSweepArgs> &it = host_item<FluidSweepArgs>(pl, L);
                    sweeps1[L.variant][shape]<<<gs, thr, 0, st>>>(it.P, it.A);
                } else if (L.variant < 6 && n <= kSweepParamItems) {
                    static thread_local SweepBatchParams B;
                    B.n = n;
                    std::memcpy(B.bstart, pl.host.data() + L.shape_table_off[shape], sizeof(int) * (n + 1));
                    std::memcpy(B.it, pl.host.data() + L.items_off, sizeof(Item<FluidSweepArgs>) * n);
                    sweepsp[L.variant][shape]<<<gs, thr, 0, st>>>(B);
                } else {
                    sweeps[L.variant][shape]<<<gs, thr, 0, st>>>(items_of<FluidSweepArgs>(pl, L), tbs, n);
                }
                CK_LAUNCH();
                if (tune_ev) CK(cudaEventRecord(tune_ev[2 * tr + 1], st));
            }
            if (sweep1) CK(cudaEventRecordWithFlags(sweep1, st, sweep_flags));
            break;
        case L_DEFORM: FSIM_LAUNCH(kb_solid_deform, SolidArgs, kBlock); break;
        case L_FORCE: { FSIM_LAUNCH_P(kb_solid_force, SolidArgs, kBlock); } break;
        case L_FORCE_RECORD: { FSIM_LAUNCH_P(kb_solid_force_record, SolidArgs, kBlock); } break;
        case L_FORCE_LISTED: { FSIM_LAUNCH_P(kb_solid_force_listed, SolidArgs, kBlock); } break;
        case L_UPDATE: FSIM_LAUNCH(kb_solid_update, SolidArgs, kBlock); break;
        case L_SOLID_SLOTS: FSIM_LAUNCH(kb_solid_slots, SolidArgs, kBlock); break;
        case L_DEFORM_R: FSIM_LAUNCH(kb_solid_deform_resolve, SolidArgs, kBlock); break;
        case L_DEFORM_M_R: FSIM_LAUNCH(kb_solid_deform_mixed_resolve, SolidArgs, kBlock); break;
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
            F.polls = L.polls ? L.polls : kBarrierSpinLimit;
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
        if (per_launch) CK(cudaEventRecord(per_launch[2 * k + 1], st));
    }
    return FSIM_OK;
}

int launch_phase(int kind)
{
    switch (kind) {
    case L_COUPLE: case L_COUPLE_M: return FSIM_PHASE_COUPLE;
    case L_VIRT: case L_VIRT_M: return FSIM_PHASE_VIRT;
    case L_SWEEP: return FSIM_PHASE_FLUID;
    case L_DEFORM: case L_FORCE: case L_UPDATE: case L_DEFORM_M: case L_FORCE_M: case L_SOLID_FUSED:
    case L_SOLID_SLOTS: case L_FORCE_RECORD: case L_FORCE_LISTED: case L_DEFORM_R: case L_DEFORM_M_R:
        return FSIM_PHASE_SOLID;
    default: return FSIM_PHASE_CELL;
    }
}

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

void launch_k_pack_f4(int grid, cudaStream_t st, const float *xyz, const float *w, int n, float wconst, float4 *out)
{
    k_pack_f4<<<grid, kBlock, 0, st>>>(xyz, w, n, wconst, out);
}

void launch_k_iota(int grid, cudaStream_t st, int *a, int n)
{
    k_iota<<<grid, kBlock, 0, st>>>(a, n);
}

void launch_k_virt_normal(int grid, cudaStream_t st, const DevParams P, const float4 *v_posr, const int *v_cell, const int *start_v, float4 *v_normal, int n)
{
    k_virt_normal<<<grid, kBlock, 0, st>>>(P, v_posr, v_cell, start_v, v_normal, n);
}

void launch_k_fluid_to_mixed(int grid, cudaStream_t st, const DevParams P, float4 *posr, float4 *velp, int *cell, int n, unsigned *flags)
{
    k_fluid_to_mixed<<<grid, kBlock, 0, st>>>(P, posr, velp, cell, n, flags);
}

void launch_k_offsets_in_cells(int grid, cudaStream_t st, const DevParams P, float4 *pos, const int *cell, int n)
{
    k_offsets_in_cells<<<grid, kBlock, 0, st>>>(P, pos, cell, n);
}

void launch_k_unpermute_mixed(int grid, cudaStream_t st, const DevParams P, const float4 *pos, const float4 *velp, const int *cell, const int *orig, int n, int what, float *out)
{
    k_unpermute_mixed<<<grid, kBlock, 0, st>>>(P, pos, velp, cell, orig, n, what, out);
}

void launch_k_unpermute_f4(int grid, cudaStream_t st, const float4 *src, const int *orig, int n, int comp, int width, float *out)
{
    k_unpermute_f4<<<grid, kBlock, 0, st>>>(src, orig, n, comp, width, out);
}

void launch_k_unpermute_words(int grid, cudaStream_t st, const int *src, const int *orig, int n, int width, int *out)
{
    k_unpermute_words<<<grid, kBlock, 0, st>>>(src, orig, n, width, out);
}

void launch_k_permute_in_mixed(int grid, cudaStream_t st, const DevParams P, float4 *pos, float4 *velp, const int *cell, const int *orig, int n, int what, const float *in)
{
    k_permute_in_mixed<<<grid, kBlock, 0, st>>>(P, pos, velp, cell, orig, n, what, in);
}

void launch_k_permute_in_f4(int grid, cudaStream_t st, float4 *dst, const int *orig, int n, int comp, int width, const float *in)
{
    k_permute_in_f4<<<grid, kBlock, 0, st>>>(dst, orig, n, comp, width, in);
}

void launch_k_probe(int grid, cudaStream_t st, const DevParams P, const ProbeArgs A)
{
    k_probe<<<grid, kBlock, 0, st>>>(P, A);
}

void launch_k_neighbor_counts(int grid, cudaStream_t st, const DevParams P, const DevParams Pv, const float4 *fposr, const int *cell_f, const int *start_f, const int *ids_f, const float4 *s_pos, const int *start_s, const int *ids_s, const float4 *v_posr, const int *start_v, int *out, int n)
{
    k_neighbor_counts<<<grid, kBlock, 0, st>>>(P, Pv, fposr, cell_f, start_f, ids_f, s_pos, start_s, ids_s, v_posr, start_v, out, n);
}

void launch_k_neighbor_counts_nl(int grid, cudaStream_t st, const DevParams P, const float4 *fposr, const int *list, const int *cnt, int cap, const float4 *s_pos, const float4 *v_posr, int *out, int n)
{
    k_neighbor_counts_nl<<<grid, kBlock, 0, st>>>(P, fposr, list, cnt, cap, s_pos, v_posr, out, n);
}

void launch_k_neighbor_counts_mixed(int grid, cudaStream_t st, const DevParams P, const DevParams Pv, const float4 *fposr, const int *cell_f, const int *start_f, const int *ids_f, const float4 *s_pos, const int *start_s, const int *ids_s, const float4 *v_posr, const int *start_v, const unsigned *v_cxyz, int *out, int n)
{
    k_neighbor_counts_mixed<<<grid, kBlock, 0, st>>>(P, Pv, fposr, cell_f, start_f, ids_f, s_pos, start_s, ids_s, v_posr, start_v, v_cxyz, out, n);
}

void launch_k_neighbor_counts_nlm(int grid, cudaStream_t st, const DevParams P, const float4 *fposr, const int *cell_f, const unsigned *cxyz_f, const int *list, const int *cnt, int cap, const float4 *s_pos, const unsigned *cxyz_s, const float4 *v_posr, const unsigned *cxyz_v, int *out, int n)
{
    k_neighbor_counts_nlm<<<grid, kBlock, 0, st>>>(P, fposr, cell_f, cxyz_f, list, cnt, cap, s_pos, cxyz_s, v_posr, cxyz_v, out, n);
}

void launch_k_gather_f4(int grid, cudaStream_t st, const int *ids, const float4 *src, int n, float4 *dst)
{
    k_gather_f4<<<grid, kBlock, 0, st>>>(ids, src, n, dst);
}

void launch_k_pack_records(int grid, cudaStream_t st, const float4 *posr, const float4 *velp, const unsigned *cxyz, int n, float4 *rec)
{
    k_pack_records<<<grid, kBlock, 0, st>>>(posr, velp, cxyz, n, rec);
}

void launch_k_nl_displacement(int grid, cudaStream_t st, const DevParams P, const float4 *posr, const int *cell, const float4 *x0, int n, NlState *nl)
{
    k_nl_displacement<<<grid, kBlock, 0, st>>>(P, posr, cell, x0, n, nl);
}

void launch_k_cells_of(int grid, cudaStream_t st, const DevParams P, const float4 *pos, int n, int *out, unsigned *packed)
{
    k_cells_of<<<grid, kBlock, 0, st>>>(P, pos, n, out, packed);
}

void launch_k_conservation_fluid(int grid, cudaStream_t st, const DevParams P, const float4 *posr, const float4 *velp, const int *cell, int n, double vol, double *partials)
{
    k_conservation_fluid<<<grid, kBlock, 0, st>>>(P, posr, velp, cell, n, vol, partials);
}

void launch_k_conservation_solid(int grid, cudaStream_t st, const DevParams P, const float4 *pos, const float4 *vel, const float *F, int n, double rho_s, double vol, double *partials)
{
    k_conservation_solid<<<grid, kBlock, 0, st>>>(P, pos, vel, F, n, rho_s, vol, partials);
}

void launch_k_case_generate(int grid, cudaStream_t st, const CaseGenArgs A)
{
    k_case_generate<<<grid, kBlock, 0, st>>>(A);
}

} // namespace fsim_rt

#ifdef FSIM_DEVICE_CHECKS
// debugging build only: the check sites that failed since the last call (bit
// per site, see FSIM_DCHECK), cleared by the call
extern "C" int fsim_debug_check_sites(unsigned *out)
{
    unsigned zero = 0;
    if (cudaMemcpyFromSymbol(out, g_check_sites, sizeof(unsigned)) != cudaSuccess) return 1;
    return cudaMemcpyToSymbol(g_check_sites, &zero, sizeof(unsigned)) != cudaSuccess;
}
#endif
static_assert(sizeof(fsim_rt::ParamBlock<fsim_rt::SolidArgs>) <= 32764, "parameter block size");
static_assert(fsim_rt::ParamBlock<fsim_rt::SolidArgs>::kMax >= 64, "a 64-instance ensemble fits");
