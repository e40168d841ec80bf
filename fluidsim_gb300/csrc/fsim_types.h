// fsim_types.h — what the device kernels (fsim_kernels.cu) and the host side
// of the library (fsim_sim.cu) share: the device parameters of an instance,
// the argument block of every batched launch, the plans that list a step's
// launches, and the launch entry points of fsim_kernels.cu.  Internal; not
// part of the public ABI (include/fluidsim.h).
#pragma once

#include "fsim_internal.h"

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <vector>

namespace fsim_rt {

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
    // solid force fluid lists: recording radius^2, allowed displacement^2
    float fl_build2, fl_move2;
};

// Per-instance state of the fluid neighbour lists, in device memory.  The
// sweep and the list-decision kernel own it; the host only forces a rebuild
// (after it changed positions) and reads the counters.
struct NlState {
    unsigned maxd2;   // largest squared displacement since the last build (float bits; >= 0)
    int rebuild;      // this step rebuilds (set by the decision kernel at the start of the step)
    int force;        // the next step rebuilds whatever the displacement
    int builds;       // list builds so far
    int overflow;     // particles whose list exceeded the capacity at the last build
    unsigned ticket;  // blocks of the decision kernel done this step
    int pad[2];
};

// per-instance error flags (device word, read by check_flags)
enum : unsigned { FLAG_OUT_OF_GRID = 1u, FLAG_BARRIER_TIMEOUT = 2u, FLAG_CELL_OVERFULL = 4u, FLAG_LIST_OVERFLOW = 8u };
// A cell's particles are ordered by their previous sorted position with a scan
// over the cell; cells above this count keep the scatter's order instead (the
// scan's cost grows with the square of the count) and raise FLAG_CELL_OVERFULL.
constexpr int kStableRankMax = 1024;

constexpr int kBlock = 256;         // threads per block of the element-wise and solid kernels
constexpr int kScanThreads = 1024;  // cell-count scan: threads per block
constexpr int kScanItems = 4;       //   and counts per thread
constexpr int kScanTile = kScanThreads * kScanItems;
constexpr int kMaxScanTiles = 16384; // cell grids up to 67M cells
constexpr int kFluidListCap = 48;   // fluid list entries per solid lane
constexpr int kPLStride = 12;       // floats per particle of the solid's P L^-1 array (16-byte rows)
constexpr int kCellRefLanes = 8;    // lanes per cell of the mixed form's per-cell references (a power of two)

__host__ __device__ inline int blocks_for(long long n, int b) { return (int)((n + b - 1) / b); }

// One instance's share of a batched launch: its parameters and buffers.
template <class Args>
struct Item {
    DevParams P;
    Args A;
};

// ---- argument blocks of the batched kernels (one Item per instance)
// cell phase: hash (plain / mixed), count reset, scans, scatter, gathers
// `gate` (neighbour-list instances): when set, the kernel runs only in steps
// whose *gate is non-zero (a list rebuild); the other steps skip it.  `grid`
// (0: one block per blockDim.x elements): the blocks launched for the item,
// each looping over the element blocks -- a small grid, so that a gated launch
// that has nothing to do costs little.
struct HashArgs {
    const float4 *pos;
    int n;
    int *key, *slot, *cnt;
    unsigned *flags;
    const int *gate;
    int grid;
};

struct ZeroArgs {
    int *p;
    int n;
    const int *gate;
    int grid;
};

struct ScanArgs {
    const int *in;
    int *out;
    int n;
    int *partial;
    const int *gate;
};

struct ScatterArgs {
    const int *key, *slot, *start;
    int *tmp;
    int n;
    const int *gate;
    int grid;
    // the sort's cell counts, which the hash filled and the scan has read:
    // zeroed here cell by cell (every counted cell holds a particle), so that
    // the next sort needs no zeroing launch (nullptr: left as they are)
    int *reset;
};

// With a gate, a step that does not rebuild copies the state unpermuted; a
// step that does also records the new positions in x0_out.
struct GatherFluidArgs {
    const int *tmp, *key, *start;
    int n;
    const float4 *posr_in, *velp_in;
    const int *orig_in;
    float4 *posr_out, *velp_out;
    int *orig_out, *cell_out;
    unsigned *flags;
    const int *gate;
    float4 *x0_out;
    float4 *rec_out; // neighbour-list instances: (posr, velp) of every slot side by side (32 bytes)
    // mixed-form neighbour-list instances: x0_out takes x0_in (absolute
    // positions in the old order) instead of posr, and every particle's
    // impact-grid cell moves along from icell_in to icell_out
    const float4 *x0_in;
    const int *icell_in;
    int *icell_out;
};

// mixed-form neighbour-list instances, on a rebuild: absolute positions
// (cell corner + offset) of every fluid particle
struct MixedAbsArgs {
    const float4 *posr;
    const int *cell;
    float4 *out;
    int n;
    const int *gate;
    int grid;
};

struct GatherSolidArgs {
    const int *tmp, *key, *start;
    int n;
    const float4 *pos_in, *vel_in, *ref_in;
    const int *type_in, *orig_in;
    float4 *pos_out, *vel_out, *ref_out;
    int *type_out, *orig_out, *cell_out;
    int *inv_out;       // sorted position of every input id
    unsigned *cxyz_out; // cell coordinates packed x | y << 11 | z << 21 (nullptr: not written)
    unsigned *flags;
    const int *gate;
    float4 *x0_out;
};

// Neighbour-list instances: the per-step cell index over the (unmoved)
// particles of the impact-distance grid.  ids[start[c] .. start[c+1]) are the
// slots of cell c in increasing slot order; cell_out[slot] is the slot's cell
// and (solid) cxyz_out[slot] its packed coordinates.
struct RankArgs {
    const int *tmp, *key, *start;
    int n;
    int *ids, *cell_out;
    unsigned *cxyz_out;
    unsigned *flags;
    // fluid: pos_out[slot] = pos_in[ids[slot]], the positions in index order
    // that the wall and coupling walks test (nullptr: not written)
    const float4 *pos_in;
    float4 *pos_out;
};

// list decision: `nblocks` blocks per instance share the solid's displacement;
// the last one to finish decides
struct NlDecideArgs {
    NlState *nl;
    const float4 *s_pos, *s_x0; // the solid's step-start positions and their values at the last build
    int ns;
    float move2; // squared displacement allowed since the build: ((Rs - R) / 2 - rounding slack)^2
    int nblocks;
};

// list build: every fluid particle's candidates within the list radius among
// fluid, wall and solid particles of its 27 cells of the list grid (whose
// cells are at least the list radius), in cell-row order; entry = index |
// species << kNlSpeciesShift, in groups of kNlGroup: entry e of particle i at
// ((e / kNlGroup) * n + i) * kNlGroup + e % kNlGroup, so that a lane writes and
// reads a whole 32-byte sector per group and a warp's group is 1 KB contiguous
struct NlBuildArgs {
    const float4 *posr;       // fluid positions at the build (sorted on the list grid)
    const int *cell_f, *start_f;
    const float4 *v_posr;
    const int *start_v;
    const float4 *s_pos;
    const int *start_s;
    int n, cap;
    int *list, *cnt;
    NlState *nl;
    unsigned *flags;
    float R2s; // list radius^2
    int nv, ns;
    int grid;  // blocks launched (each loops over warps of particles; 0: one block per 4 warps)
};
constexpr int kNlSpeciesShift = 30; // list entry: index | species << 30 (0 fluid, 1 wall, 2 solid)
constexpr int kNlGroup = 8;         // list entries per 32-byte group (the capacity is a multiple)
constexpr int kNlIndexMask = (1 << kNlSpeciesShift) - 1;

// fused fluid sweep + update (plain and mixed)
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
    // neighbour-list sweep: the lists, the positions of the last build and the
    // instance's list state (largest displacement since the build)
    const int *nl_list, *nl_cnt;
    int nl_cap, nl_nv, nl_ns; // list capacity; wall and solid counts
    const float4 *x0;
    NlState *nl;
    // where the impact grid's cells are too close to the impact distance for
    // r < R to imply neighbouring cells under FP32 rounding: the packed
    // impact-grid cell of every fluid, wall and solid slot (else nullptr), and
    // a pair also needs neighbouring cells, as in the reference's cell walk
    const unsigned *nl_cxyz_f, *nl_cxyz_v, *nl_cxyz_s;
    // the step-start (posr, velp) of every fluid slot side by side: one
    // 32-byte sector per fluid neighbour, fetched with one 256-bit load
    const float4 *rec;
};

// The cell walks below take `ids_*`: nullptr when the particles are sorted by
// the walked grid (slot = position in the cell order), else the slots of the
// per-step cell index (RankArgs) of a neighbour-list instance.

// wall particles' data from their nearest fluid particle
struct VirtArgs {
    const float4 *v_posr_in, *v_normal;
    const int *v_cell;
    const float4 *fposr, *fvelp;
    const int *forig, *start_f;
    float4 *v_posr, *v_velp;
    int n, nf;
    const int *ids_f;
    const float4 *fpos_t; // with ids_f: fposr[ids_f[t]] for every index slot t
};

// solid normal and Shepard pressure
struct CoupleArgs {
    const float4 *s_pos;
    const int *s_cell, *start_s;
    const float4 *fposr, *fvelp;
    const int *start_f;
    float4 *s_np;
    int n, nf;
    const int *ids_f, *ids_s;
    const float4 *fpos_t; // with ids_f: fposr[ids_f[t]] for every index slot t
};

// mixed form: re-binning hash, per-cell references of the FP16 gather
struct HashMixedArgs {
    float4 *pos;
    const int *cell_old;
    int n;
    int *key, *slot, *cnt;
    unsigned *flags;
};

struct CellRefArgs {
    float4 *posr;
    const float4 *velp;
    const int *start;
    float2 *cm;
    int ncell;
    // neighbour-list instances: the per-step cell index (slots ids[start[c] ..
    // start[c+1]) of cell c; kb_cell_ref then only forms cm), and for
    // kb_mixed_records the fluid slots, their cells and packed cell
    // coordinates, and the records the list sweep reads
    const int *ids;
    int n;
    const int *cell;
    const unsigned *cxyz;
    float4 *rec;
};

// solid sub-step kernels (deformation, force, update, fused)
struct SolidArgs {
    float4 *pos, *vel;
    const float4 *ref;
    const int *type, *cell;
    const int *ids_f;      // per-step fluid cell index of a neighbour-list instance (else nullptr)
    const float4 *np;
    float *F, *Pk, *L, *AV; // 9 floats per particle, row-major
    float *PL;              // kPLStride floats per particle (9 used): three 16-byte loads per neighbour
    float4 *dudt, *couple;
    const float4 *fposr, *fvelp;
    const int *start_f;
    int n, nf;             // solid and fluid particles
    // static reference-configuration neighbours (CSR over input ids)
    const int *orig, *inv, *nbr_off, *nbr_orig;
    const int *nbr_owner;  // input id of each entry's particle
    // fluid candidates of each solid lane within the recording radius (plain
    // form, entry-major: entry e of lane t at e * (kSolidGroup * n) + t), their
    // counts (-1: overflow) and where each particle was when they were recorded
    int *fl, *fl_cnt;
    float4 *fl_org;
    int *nbr_slot;         // this step: sorted slot of each entry's neighbour, -1 if its cell is not adjacent
    int ne;                // list entries
    int nsub;              // this instance's solid sub-steps per step
    const unsigned *cxyz;
    unsigned *flags;       // this instance's error flags
};

// a batched kernel's instances passed by value as one kernel parameter block
// (at most 32,764 bytes of kernel parameters)
template <class ARGS>
struct ParamBlock {
    static constexpr int kMax = (32764 - 16) / (int)(sizeof(Item<ARGS>) + sizeof(int));
    int n;
    int bstart[kMax + 1];
    Item<ARGS> it[kMax];
};

// the batched sweep's instances passed by value as one kernel parameter block
// (at most 32,764 bytes of kernel parameters)
constexpr int kSweepParamItems = 64;
struct SweepBatchParams {
    int n;
    int bstart[kSweepParamItems + 1];
    Item<FluidSweepArgs> it[kSweepParamItems];
};
static_assert(sizeof(SweepBatchParams) <= 32764, "kernel parameter limit");

// ---- device case generator (fsim_create_case): lattice rows and their bases
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

// point probes (fsim_probe)
struct ProbeArgs {
    const float *pts;
    int n;
    float *out; // 5 per probe: u, v, w, p, rho
    const float4 *fposr, *fvelp;
    const int *start_f;
    const float4 *s_pos, *s_vel, *s_np;
    const int *start_s;
    const int *ids_f, *ids_s;
};

// grid barrier of the fused solid kernel
struct GridBarrier {
    unsigned count, gen;
};

// what the mixed-form field (un)permutes move
enum MixedField { MF_POS = 0, MF_RHO = 1, MF_P = 2 };

// lanes per solid particle in the solid sweeps, and in the coupling (whose
// walks over the fluid of 27 cells are longer: more lanes measured faster
// there, slower in the solid sweeps)
constexpr int kSolidGroup = 4;
constexpr int kCoupleGroup = 8;

// mixed sweep: neighbour-list entry = particle index | 6-bit cell code << kCodeShift
constexpr int kCodeShift = 26;                   // neighbour-list entry = j | cell code << 26

constexpr int kIndexMask = (1 << kCodeShift) - 1;

// launch shapes of the fluid sweep the autotuner chooses among
constexpr int kSweepShapes = 3;

constexpr int kShapeWarps[kSweepShapes] = {4, 4, 8}; // warps per block of sweep shapes 0..2

// L_SWEEP variants: 0-5 stream sweep (CHECK_Z * 3 + VISCID mode), 6-8 mixed
// form (6 + VISCID mode), 9-11 list sweep (kSweepNlVariant + VISCID mode),
// 12-14 mixed-form list sweep (kSweepNlMixedVariant + VISCID mode)
constexpr int kSweepNlVariant = 9;
constexpr int kSweepNlMixedVariant = 12;
// threads per block of the list build
constexpr int kNlBuildThreads = 128;

// ---------------------------------------------------------------- plans
// A plan is the ordered list of batched launches that advance a set of
// instances by one step (or one phase), with every launch's {params, args}
// items and block prefix tables in one device arena.
enum LaunchKind {
    L_ZERO, L_HASH, L_SCAN_REDUCE, L_SCAN_PARTIALS, L_SCAN_APPLY, L_SCATTER, L_GATHER_F, L_GATHER_S,
    L_COUPLE, L_VIRT, L_SWEEP, L_DEFORM, L_FORCE, L_UPDATE,
    L_HASH_M, L_CELLREF, L_COUPLE_M, L_VIRT_M, L_DEFORM_M, L_FORCE_M, L_SOLID_FUSED, L_SOLID_SLOTS,
    L_FORCE_RECORD, L_FORCE_LISTED, L_DEFORM_R, L_DEFORM_M_R,
    L_NL_DECIDE, L_NL_BUILD, L_RANK_F, L_RANK_S, L_MIXED_ABS, L_MIXED_REC
};

struct Launch {
    int kind;
    size_t items_off, table_off; // arena offsets
    int ninst, blocks, variant;
    size_t shape_table_off[kSweepShapes]; // L_SWEEP: block prefix table per launch shape
    int shape_blocks[kSweepShapes];
    size_t table2_off, barrier_off;       // L_SOLID_FUSED: thread-per-particle table, grid barrier
    int max_sub;
    unsigned polls;                       // L_SOLID_FUSED: barrier wait limit, 0 = the default
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
    // the same step graph with event nodes around the sweep, for timing the
    // sweep inside graph replays: two executable copies (consecutive replays
    // alternate, so an event update never touches the copy just launched)
    // and the nodes whose events each replay sets
    cudaGraph_t tgraph = nullptr;
    cudaGraphExec_t texec[2] = {nullptr, nullptr};
    cudaGraphNode_t tnode[2] = {nullptr, nullptr};
    cudaEvent_t tev[2] = {nullptr, nullptr}; // the events at capture
    int tnext = 0;
};

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

// ------------------------------------------------------ host error checks
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

// ---------------------------------------------- entry points of the kernels
// Enqueue a plan's launches on `st`, the fluid sweep with launch shape
// `shape`; optional events around the sweep (recorded with sweep_flags:
// cudaEventRecordExternal makes them event nodes of a captured graph).
// per_launch: 2 events per launch, recorded before and after it.
// tune_ev (the autotuner): instead of one sweep, tune_rounds rounds of one
// sweep per launch shape, round r shape s between tune_ev[2 (r S + s)] and
// tune_ev[2 (r S + s) + 1] (S = kSweepShapes).
fsim_status enqueue_plan(const Plan &pl, cudaStream_t st, int shape, cudaEvent_t sweep0 = nullptr,
                         cudaEvent_t sweep1 = nullptr, const cudaEvent_t *per_launch = nullptr,
                         unsigned sweep_flags = cudaEventRecordDefault, const cudaEvent_t *tune_ev = nullptr,
                         int tune_rounds = 0);
// the FSIM_PHASE_* a launch kind belongs to
int launch_phase(int kind);
// CTAs of the fused solid kernel that fit on the current device at once (<= want)
int fused_grid(bool mixed, int want);
// One launch of a utility kernel (kBlock threads per block) on `st`.
void launch_k_pack_f4(int grid, cudaStream_t st, const float *xyz, const float *w, int n, float wconst, float4 *out);
void launch_k_iota(int grid, cudaStream_t st, int *a, int n);
void launch_k_virt_normal(int grid, cudaStream_t st, const DevParams P, const float4 *v_posr, const int *v_cell, const int *start_v, float4 *v_normal, int n);
void launch_k_fluid_to_mixed(int grid, cudaStream_t st, const DevParams P, float4 *posr, float4 *velp, int *cell, int n, unsigned *flags);
void launch_k_offsets_in_cells(int grid, cudaStream_t st, const DevParams P, float4 *pos, const int *cell, int n);
void launch_k_unpermute_mixed(int grid, cudaStream_t st, const DevParams P, const float4 *pos, const float4 *velp, const int *cell, const int *orig, int n, int what, float *out);
void launch_k_unpermute_f4(int grid, cudaStream_t st, const float4 *src, const int *orig, int n, int comp, int width, float *out);
void launch_k_unpermute_words(int grid, cudaStream_t st, const int *src, const int *orig, int n, int width, int *out);
void launch_k_permute_in_mixed(int grid, cudaStream_t st, const DevParams P, float4 *pos, float4 *velp, const int *cell, const int *orig, int n, int what, const float *in);
void launch_k_permute_in_f4(int grid, cudaStream_t st, float4 *dst, const int *orig, int n, int comp, int width, const float *in);
void launch_k_probe(int grid, cudaStream_t st, const DevParams P, const ProbeArgs A);
void launch_k_neighbor_counts(int grid, cudaStream_t st, const DevParams P, const DevParams Pv, const float4 *fposr, const int *cell_f, const int *start_f, const int *ids_f, const float4 *s_pos, const int *start_s, const int *ids_s, const float4 *v_posr, const int *start_v, int *out, int n);
void launch_k_neighbor_counts_nl(int grid, cudaStream_t st, const DevParams P, const float4 *fposr, const int *list, const int *cnt, int cap, const float4 *s_pos, const float4 *v_posr, int *out, int n);
void launch_k_neighbor_counts_mixed(int grid, cudaStream_t st, const DevParams P, const DevParams Pv, const float4 *fposr, const int *cell_f, const int *start_f, const int *ids_f, const float4 *s_pos, const int *start_s, const int *ids_s, const float4 *v_posr, const int *start_v, const unsigned *v_cxyz, int *out, int n);
void launch_k_neighbor_counts_nlm(int grid, cudaStream_t st, const DevParams P, const float4 *fposr, const int *cell_f, const unsigned *cxyz_f, const int *list, const int *cnt, int cap, const float4 *s_pos, const unsigned *cxyz_s, const float4 *v_posr, const unsigned *cxyz_v, int *out, int n);
void launch_k_gather_f4(int grid, cudaStream_t st, const int *ids, const float4 *src, int n, float4 *dst);
void launch_k_pack_records(int grid, cudaStream_t st, const float4 *posr, const float4 *velp, const unsigned *cxyz, int n, float4 *rec);
void launch_k_nl_displacement(int grid, cudaStream_t st, const DevParams P, const float4 *posr, const int *cell, const float4 *x0, int n, NlState *nl);
void launch_k_cells_of(int grid, cudaStream_t st, const DevParams P, const float4 *pos, int n, int *out, unsigned *packed);
void launch_k_conservation_fluid(int grid, cudaStream_t st, const DevParams P, const float4 *posr, const float4 *velp, const int *cell, int n, double vol, double *partials);
void launch_k_conservation_solid(int grid, cudaStream_t st, const DevParams P, const float4 *pos, const float4 *vel, const float *F, int n, double rho_s, double vol, double *partials);
void launch_k_case_generate(int grid, cudaStream_t st, const CaseGenArgs A);

} // namespace fsim_rt
