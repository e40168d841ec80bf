// fsim_sim.cu — the host side of the simulation half of the C ABI
// (include/fluidsim.h): handles and their device memory, plans (the launch
// lists of a step, captured into CUDA graphs), batches, field I/O, snapshots
// and the device-side case generator driver.  The kernels are in
// fsim_kernels.cu; what both share is in fsim_types.h.
#include "fsim_types.h"

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

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
// NVTX range over an API call (visible to Nsight tools; free without them)
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
};
} // namespace

// =================================================================== handle
namespace {

// Online autotuner of the fluid sweep's launch shape (see run_plan_step).
constexpr int kTuneRounds = 2; // each shape is timed this many times; the fastest time counts
struct SweepTuner {
    int chosen = -1; // shape index once tuned
    int next = 0;    // shapes timed
    float ms[kSweepShapes] = {};
    cudaEvent_t ev[2 * kSweepShapes * kTuneRounds] = {};
    int shape() const { return chosen >= 0 ? chosen : 0; }
    void release()
    {
        for (cudaEvent_t &e : ev) {
            if (e) cudaEventDestroy(e);
            e = nullptr;
        }
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
    int *s_nbr_owner = nullptr;   // input id of each entry's particle
    int *s_fl = nullptr, *s_fl_cnt = nullptr; // solid force fluid lists (per lane) and counts
    float4 *s_fl_org = nullptr;   // where each solid particle was when its lists were recorded
    int *s_nbr_slot = nullptr;    // per step: sorted slot of each entry's neighbour (-1: cells not adjacent)
    int s_ne = 0;                 // list entries
    int s_cur = 0;
    bool s_sorted = false;
    bool s_np_ok = false;    // normal + pressure are in the order of s_cur
    bool s_mech_ok = false;  // F, P, L^-1, du/dt are in the order of s_cur
    // virtual
    float4 *v_posr = nullptr, *v_velp = nullptr, *v_normal = nullptr;
    int *v_orig = nullptr, *v_cell = nullptr, *v_start = nullptr;
    // fluid neighbour lists (nl): particles sorted on the list grid Pl (cells of
    // at least the list radius) at every list build and left in that order in
    // between; per step an index of the impact grid (f_start/f_ids, s_start/
    // s_ids; f_cell/s_cell/s_cxyz per slot) serves the other phases.  Walls are
    // sorted on the list grid (v_cell, v_start); v_icell is their impact-grid cell.
    bool nl = false;
    bool nl_check = false;        // pairs also need neighbouring impact-grid cells (f_cxyz, v_icxyz, s_cxyz)
    unsigned *f_cxyz = nullptr, *v_icxyz = nullptr;
    DevParams Pl;                 // the list grid's parameters (else unused)
    int ncell_l = 0, nl_cap = 0;
    float nl_R2s = 0.0f, nl_move2 = 0.0f;
    int *nl_list = nullptr, *nl_cnt = nullptr;
    NlState *nl_state = nullptr;
    float4 *f_x0 = nullptr, *s_x0 = nullptr;
    int *f_ids = nullptr, *f_lcell = nullptr, *f_lcnt = nullptr, *f_lstart = nullptr;
    int *s_ids = nullptr, *s_lcell = nullptr, *s_lcnt = nullptr, *s_lstart = nullptr;
    int *v_icell = nullptr;
    float4 *f_rec = nullptr;      // (posr, velp) per slot, 32 bytes: the list sweep's neighbour records
    // mixed form with lists: f_cell is every slot's impact-grid cell (its
    // offset's cell), carried through a rebuild's gather in f_cell2; the walls'
    // absolute positions for the build (their v_posr are offsets from v_icell)
    int *f_cell2 = nullptr;
    float4 *v_abs = nullptr;
    float4 *f_spos = nullptr;     // fluid positions in the per-step index's order (the wall and coupling walks)
    bool rec_live = false;        // a cell phase wrote f_rec and the fluid phase has not run yet
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
    std::vector<std::pair<void *, size_t>> allocations; // the instance's device arrays and their bytes
    // creation temporaries, freed at the instance's first step or batch entry
    // rather than during creation: cudaFree waits for the whole device, and a
    // server creates instances while a batch runs
    std::vector<void *> deferred;
};

namespace {

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
    h->allocations.emplace_back((void *)*p, count * sizeof(T));
    return FSIM_OK;
}

// a temporary that dalloc made: no longer part of the instance, freed by
// flush_deferred (at the first step or batch entry, or with the instance)
void release(fsim_sim *h, void *p)
{
    h->deferred.push_back(p);
    for (auto it = h->allocations.begin(); it != h->allocations.end(); ++it)
        if (it->first == p) {
            h->allocations.erase(it);
            return;
        }
}

void flush_deferred(fsim_sim *h)
{
    for (void *p : h->deferred) cudaFree(p);
    h->deferred.clear();
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
    for (auto &a : h->allocations) cudaFree(a.first);
    h->allocations.clear();
    flush_deferred(h);
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
    {
        // solid force fluid lists: a particle may move 0.1 R within a step
        // before its list is bypassed; the list keeps candidates within
        // 1.1 R (1 + 1e-5), which covers the FP32 rounding of both tests
        const double R = std::sqrt((double)P.R2), dmove = 0.1 * R, rb = (R + dmove) * (1.0 + 1e-5);
        P.fl_move2 = (float)(dmove * dmove);
        P.fl_build2 = (float)(rb * rb);
    }
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

void free_plan(Plan *pl)
{
    if (!pl) return;
    if (pl->graph) cudaGraphExecDestroy(pl->graph);
    for (int k = 0; k < 2; ++k) {
        if (pl->texec[k]) cudaGraphExecDestroy(pl->texec[k]);
        if (pl->tev[k]) cudaEventDestroy(pl->tev[k]);
    }
    if (pl->tgraph) cudaGraphDestroy(pl->tgraph);
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

// The cell phase of neighbour-list instances (parity pf -> 1-pf, ps -> 1-ps):
// the list decision; on a rebuild, the counting sort of fluid and solid on the
// list grid, else an unpermuted copy; the per-step impact-grid index; on a
// rebuild, the list build.
// Blocks a gated launch gets per instance at most (8 per SM of a GB300; the
// list build, whose blocks carry uneven work, 32 per SM): each loops over its
// element blocks when its instance rebuilds and returns at once when it does
// not.  A grid shared by a batch's instances (equally, or in proportion to
// their particles) measured slower: in a batch some member rebuilds in most
// steps, and its sort and build then ran on a fraction of the GPU.
constexpr int kGatedGrid = 8 * 152, kGatedBuildGrid = 32 * 152;

int gated_grid(int grid, long long n, int block)
{
    return n > 0 ? (int)std::min<long long>(grid, blocks_for(n, block)) : 0;
}

void plan_cell_nl(Plan &pl, ArenaBuilder &ab, const std::vector<fsim_sim *> &m, int pf, int ps)
{
    std::vector<Item<NlDecideArgs>> di;
    std::vector<int> db;
    for (fsim_sim *h : m) {
        const int nb = std::min(64, std::max(1, blocks_for(h->ns, kBlock)));
        NlDecideArgs a{h->nl_state, h->s_pos[ps], h->s_x0, h->ns, h->nl_move2, nb};
        Item<NlDecideArgs> it{h->P, a};
        di.push_back(it);
        db.push_back(nb);
    }
    add_launch(pl, ab, L_NL_DECIDE, di, db);
    // mixed form: the absolute positions the list grid sorts by (into f_rec,
    // which the cell references overwrite later in the phase)
    const bool mixed = !m.empty() && m[0]->mixed;
    if (mixed) {
        std::vector<Item<MixedAbsArgs>> ai;
        std::vector<int> abk;
        for (fsim_sim *h : m) {
            const int ag = gated_grid(kGatedGrid, h->nf, kBlock);
            const Item<MixedAbsArgs> it{h->P, MixedAbsArgs{h->f_posr[pf], h->f_cell, h->f_rec, h->nf,
                                                           &h->nl_state->rebuild, ag}};
            ai.push_back(it);
            abk.push_back(ag);
        }
        add_launch(pl, ab, L_MIXED_ABS, ai, abk);
    }
    // list-grid sort, run only when the decision says rebuild
    std::vector<Item<ZeroArgs>> zi;
    std::vector<Item<HashArgs>> hi;
    std::vector<Item<ScanArgs>> si;
    std::vector<Item<ScatterArgs>> ci;
    std::vector<int> zb, hb, sb, sp, cb;
    for (fsim_sim *h : m) {
        const int *gate = &h->nl_state->rebuild;
        for (int s_ = 0; s_ < 2; ++s_) {
            const int n = s_ ? h->ns : h->nf;
            int *lcnt = s_ ? h->s_lcnt : h->f_lcnt, *lstart = s_ ? h->s_lstart : h->f_lstart;
            const int zn = n ? h->ncell_l : 0, zg = gated_grid(kGatedGrid, zn, kBlock);
            const Item<ZeroArgs> z{h->Pl, ZeroArgs{lcnt, zn, gate, zg}};
            zi.push_back(z);
            zb.push_back(zg);
            const int hg = gated_grid(kGatedGrid, n, kBlock);
            const float4 *fpos = mixed ? h->f_rec : h->f_posr[pf];
            const HashArgs ha = s_ ? HashArgs{h->s_pos[ps], h->ns, h->s_key, h->s_slot, lcnt, h->d_flags, gate, hg}
                                   : HashArgs{fpos, h->nf, h->f_key, h->f_slot, lcnt, h->d_flags, gate, hg};
            const Item<HashArgs> hh{h->Pl, ha};
            hi.push_back(hh);
            hb.push_back(hg);
            const Item<ScanArgs> sc{h->Pl,
                                    ScanArgs{lcnt, lstart, h->ncell_l, h->scan_partials + (s_ ? kMaxScanTiles : 0), gate}};
            si.push_back(sc);
            sb.push_back(n ? blocks_for(h->ncell_l, kScanTile) : 0);
            sp.push_back(n ? 1 : 0);
            const ScatterArgs ca = s_ ? ScatterArgs{h->s_key, h->s_slot, lstart, h->s_tmp, h->ns, gate, hg}
                                      : ScatterArgs{h->f_key, h->f_slot, lstart, h->f_tmp, h->nf, gate, hg};
            const Item<ScatterArgs> cc{h->Pl, ca};
            ci.push_back(cc);
            cb.push_back(hg);
        }
    }
    add_launch(pl, ab, L_ZERO, zi, zb);
    add_launch(pl, ab, L_HASH, hi, hb);
    add_launch(pl, ab, L_SCAN_REDUCE, si, sb);
    add_launch(pl, ab, L_SCAN_PARTIALS, si, sp);
    add_launch(pl, ab, L_SCAN_APPLY, si, sb);
    add_launch(pl, ab, L_SCATTER, ci, cb);
    std::vector<Item<GatherFluidArgs>> gf;
    std::vector<Item<GatherSolidArgs>> gs;
    std::vector<int> gfb, gsb;
    for (fsim_sim *h : m) {
        const int *gate = &h->nl_state->rebuild;
        const GatherFluidArgs fa{h->f_tmp,          h->f_key,           h->f_lstart,        h->nf,
                                 h->f_posr[pf],     h->f_velp[pf],      h->f_orig[pf],      h->f_posr[1 - pf],
                                 h->f_velp[1 - pf], h->f_orig[1 - pf],  h->f_lcell,         h->d_flags,
                                 gate,              h->f_x0,            mixed ? nullptr : h->f_rec,
                                 mixed ? h->f_rec : nullptr,            mixed ? h->f_cell : nullptr,
                                 mixed ? h->f_cell2 : nullptr};
        const Item<GatherFluidArgs> fi{h->Pl, fa};
        gf.push_back(fi);
        gfb.push_back(blocks_for(h->nf, kBlock));
        const GatherSolidArgs sa{h->s_tmp, h->s_key, h->s_lstart, h->ns, h->s_pos[ps], h->s_vel[ps], h->s_ref[ps],
                                 h->s_type[ps], h->s_orig[ps], h->s_pos[1 - ps], h->s_vel[1 - ps], h->s_ref[1 - ps],
                                 h->s_type[1 - ps], h->s_orig[1 - ps], h->s_lcell, h->s_inv, nullptr, h->d_flags,
                                 gate, h->s_x0};
        const Item<GatherSolidArgs> sg{h->Pl, sa};
        gs.push_back(sg);
        gsb.push_back(blocks_for(h->ns, kBlock));
    }
    add_launch(pl, ab, L_GATHER_F, gf, gfb);
    add_launch(pl, ab, L_GATHER_S, gs, gsb);
    // the per-step impact-grid index of the particles as they now lie
    zi.clear();
    hi.clear();
    si.clear();
    ci.clear();
    zb.clear();
    hb.clear();
    sb.clear();
    sp.clear();
    cb.clear();
    std::vector<Item<RankArgs>> ri;
    std::vector<Item<HashMixedArgs>> hmi;
    std::vector<int> rb, hmb;
    for (fsim_sim *h : m) {
        for (int s_ = 0; s_ < 2; ++s_) {
            const int n = s_ ? h->ns : h->nf;
            int *cnt = s_ ? h->s_cnt : h->f_cnt, *start = s_ ? h->s_start : h->f_start;
            if (!s_ && mixed) {
                // the mixed form re-bins every offset to its cell (in place)
                const Item<HashMixedArgs> hm{h->P, HashMixedArgs{h->f_posr[1 - pf], h->f_cell2, h->nf, h->f_key,
                                                                 h->f_slot, cnt, h->d_flags}};
                hmi.push_back(hm);
                hmb.push_back(blocks_for(n, kBlock));
            } else {
                const HashArgs ha = s_ ? HashArgs{h->s_pos[1 - ps], h->ns, h->s_key, h->s_slot, cnt, h->d_flags,
                                                  nullptr}
                                       : HashArgs{h->f_posr[1 - pf], h->nf, h->f_key, h->f_slot, cnt, h->d_flags,
                                                  nullptr};
                const Item<HashArgs> hh{h->P, ha};
                hi.push_back(hh);
                hb.push_back(blocks_for(n, kBlock));
            }
            const Item<ScanArgs> sc{h->P,
                                    ScanArgs{cnt, start, h->ncell, h->scan_partials + (s_ ? kMaxScanTiles : 0), nullptr}};
            si.push_back(sc);
            sb.push_back(n ? blocks_for(h->ncell, kScanTile) : 0);
            sp.push_back(n ? 1 : 0);
            // the scatter zeroes the counts again (set to zero at creation)
            const ScatterArgs ca = s_ ? ScatterArgs{h->s_key, h->s_slot, start, h->s_tmp, h->ns, nullptr, 0, cnt}
                                      : ScatterArgs{h->f_key, h->f_slot, start, h->f_tmp, h->nf, nullptr, 0, cnt};
            const Item<ScatterArgs> cc{h->P, ca};
            ci.push_back(cc);
            cb.push_back(blocks_for(n, kBlock));
            const RankArgs ra = s_ ? RankArgs{h->s_tmp, h->s_key, start, h->ns, h->s_ids, h->s_cell, h->s_cxyz,
                                              h->d_flags, nullptr, nullptr}
                                   : RankArgs{h->f_tmp, h->f_key, start, h->nf, h->f_ids, h->f_cell, h->f_cxyz,
                                              h->d_flags, h->f_posr[1 - pf], h->f_spos};
            const Item<RankArgs> rr{h->P, ra};
            ri.push_back(rr);
            rb.push_back(blocks_for(n, kBlock));
        }
    }
    add_launch(pl, ab, L_HASH, hi, hb);
    add_launch(pl, ab, L_HASH_M, hmi, hmb);
    add_launch(pl, ab, L_SCAN_REDUCE, si, sb);
    add_launch(pl, ab, L_SCAN_PARTIALS, si, sp);
    add_launch(pl, ab, L_SCAN_APPLY, si, sb);
    add_launch(pl, ab, L_SCATTER, ci, cb);
    add_launch(pl, ab, L_RANK_F, ri, rb);
    if (mixed) {
        // per-cell references, then per slot the FP16 gather pair and the
        // sweep's record
        std::vector<Item<CellRefArgs>> cr;
        std::vector<int> crb, rcb;
        for (fsim_sim *h : m) {
            const CellRefArgs ca{h->f_posr[1 - pf], h->f_velp[1 - pf], h->f_start, h->f_cm, h->ncell,
                                 h->f_ids,          h->nf,             h->f_cell,  h->f_cxyz, h->f_rec};
            const Item<CellRefArgs> c{h->P, ca};
            cr.push_back(c);
            crb.push_back(h->nf ? blocks_for((long long)kCellRefLanes * h->ncell, kBlock) : 0);
            rcb.push_back(blocks_for(h->nf, kBlock));
        }
        add_launch(pl, ab, L_CELLREF, cr, crb);
        add_launch(pl, ab, L_MIXED_REC, cr, rcb);
    }
    // the list build (runs only on a rebuild)
    std::vector<Item<NlBuildArgs>> bi;
    std::vector<int> bb;
    for (fsim_sim *h : m) {
        const int bg = gated_grid(kGatedBuildGrid, h->nf, kNlBuildThreads);
        const NlBuildArgs ba{h->f_x0,   h->f_lcell,  h->f_lstart, mixed ? h->v_abs : h->v_posr, h->v_start,
                             h->s_x0,   h->s_lstart, h->nf,       h->nl_cap,  h->nl_list,
                             h->nl_cnt, h->nl_state, h->d_flags,  h->nl_R2s,  h->nv,
                             h->ns,     bg};
        const Item<NlBuildArgs> bt{h->Pl, ba};
        bi.push_back(bt);
        bb.push_back(bg);
    }
    add_launch(pl, ab, L_NL_BUILD, bi, bb);
}

// The cell phase: counting sort of fluid and solid (parity pf -> 1-pf, ps -> 1-ps).
void plan_cell(Plan &pl, ArenaBuilder &ab, const std::vector<fsim_sim *> &m, int pf, int ps)
{
    if (!m.empty() && m[0]->nl) {
        plan_cell_nl(pl, ab, m, pf, ps);
        return;
    }
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
                                            h->f_cell, h->d_flags}});
        gfb.push_back(blocks_for(h->nf, kBlock));
        gs.push_back({h->P, GatherSolidArgs{h->s_tmp, h->s_key, h->s_start, h->ns, h->s_pos[ps], h->s_vel[ps],
                                            h->s_ref[ps], h->s_type[ps], h->s_orig[ps], h->s_pos[1 - ps],
                                            h->s_vel[1 - ps], h->s_ref[1 - ps], h->s_type[1 - ps], h->s_orig[1 - ps],
                                            h->s_cell, h->s_inv, h->s_cxyz, h->d_flags}});
        gsb.push_back(blocks_for(h->ns, kBlock));
    }
    add_launch(pl, ab, L_GATHER_F, gf, gfb);
    add_launch(pl, ab, L_GATHER_S, gs, gsb);
    std::vector<Item<CellRefArgs>> cr;
    std::vector<int> crb;
    for (fsim_sim *h : m) {
        if (!h->mixed) continue;
        cr.push_back({h->P, CellRefArgs{h->f_posr[1 - pf], h->f_velp[1 - pf], h->f_start, h->f_cm, h->ncell}});
        crb.push_back(h->nf ? blocks_for((long long)kCellRefLanes * h->ncell, kBlock) : 0);
    }
    add_launch(pl, ab, L_CELLREF, cr, crb);
}

void plan_couple(Plan &pl, ArenaBuilder &ab, const std::vector<fsim_sim *> &m, int pf, int ps)
{
    std::vector<Item<CoupleArgs>> it;
    std::vector<int> nb;
    for (fsim_sim *h : m) {
        const CoupleArgs ca{h->s_pos[ps], h->s_cell,  h->s_start, h->f_posr[pf], h->f_velp[pf],
                            h->f_start,   h->s_np,    h->ns,      h->nf,         h->nl ? h->f_ids : nullptr,
                            h->nl ? h->s_ids : nullptr,           h->nl ? h->f_spos : nullptr};
        const Item<CoupleArgs> ci{h->P, ca};
        it.push_back(ci);
        nb.push_back(h->nf && h->ns ? blocks_for((long long)kCoupleGroup * h->ns, kBlock) : 0);
    }
    add_launch(pl, ab, m.empty() || !m[0]->mixed ? L_COUPLE : L_COUPLE_M, it, nb);
}

void plan_virt(Plan &pl, ArenaBuilder &ab, const std::vector<fsim_sim *> &m, int pf)
{
    std::vector<Item<VirtArgs>> it;
    std::vector<int> nb;
    for (fsim_sim *h : m) {
        const VirtArgs va{h->v_posr,      h->v_normal, h->nl ? h->v_icell : h->v_cell, h->f_posr[pf],
                          h->f_velp[pf],  h->f_orig[pf], h->f_start, h->v_posr, h->v_velp, h->nv, h->nf,
                          h->nl ? h->f_ids : nullptr, h->nl ? h->f_spos : nullptr};
        const Item<VirtArgs> vi{h->P, va};
        it.push_back(vi);
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
        A.nl_list = h->nl_list;
        A.nl_cnt = h->nl_cnt;
        A.nl_cap = h->nl_cap;
        A.nl_nv = h->nv;
        A.nl_ns = h->ns;
        A.x0 = h->f_x0;
        A.nl = h->nl_state;
        A.nl_cxyz_f = h->nl_check ? h->f_cxyz : nullptr; // (always in the mixed form)
        A.nl_cxyz_v = h->nl_check ? h->v_icxyz : nullptr;
        A.nl_cxyz_s = h->nl_check ? h->s_cxyz : nullptr;
        A.rec = h->f_rec;
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
    const bool mixed = !m.empty() && m[0]->mixed, nl = !m.empty() && m[0]->nl;
    add_sweep_launch(pl, ab, it, nb,
                     nl ? (mixed ? kSweepNlMixedVariant : kSweepNlVariant) + visc_mode
                        : mixed ? 6 + visc_mode : (any_check ? 3 : 0) + visc_mode);
    if (pl.launches.size() > before) pl.sweep_index = (int)before;
}

// solid sub-steps (in place on parity ps; the fluid is read at parity pf):
// per-phase batched launches, or (solid_fused) one persistent cooperative
// launch for all sub-steps of all instances

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
        S.nf = h->nf;
        S.orig = h->s_orig[ps];
        S.inv = h->s_inv;
        S.nbr_off = h->s_nbr_off;
        S.nbr_orig = h->s_nbr_orig;
        S.nbr_owner = h->s_nbr_owner;
        S.nbr_slot = h->s_nbr_slot;
        S.fl = h->s_fl;
        S.fl_cnt = h->s_fl_cnt;
        S.fl_org = h->s_fl_org;
        S.ne = h->s_ne;
        S.cxyz = h->s_cxyz;
        S.nsub = h->ns ? h->cfg.solid_sub_step : 0;
        S.flags = h->d_flags;
        S.ids_f = h->nl ? h->f_ids : nullptr;
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
            // sub-step 0 also resolves the step's list slots for the later sub-steps
            add_launch(pl, ab, mixed ? (k == 0 ? L_DEFORM_M_R : L_DEFORM_M) : (k == 0 ? L_DEFORM_R : L_DEFORM), it,
                       wb);
            // plain form: sub-step 0 records each lane's fluid list, later sub-steps walk it
            const bool lists = !mixed && !m[0]->cfg.solid_full_walk;
            add_launch(pl, ab, mixed ? L_FORCE_M : !lists ? L_FORCE : k == 0 ? L_FORCE_RECORD : L_FORCE_LISTED, it,
                       wb);
            add_launch(pl, ab, L_UPDATE, it, tb);
        }
        return;
    }
    {
        std::vector<int> eb;
        for (fsim_sim *h : m) eb.push_back(h->ns ? blocks_for(h->s_ne, kBlock) : 0);
        add_launch(pl, ab, L_SOLID_SLOTS, it, eb);
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
    // the longest wait any member allows (0 = the kernel's default)
    L.polls = 0;
    for (fsim_sim *h : m) {
        if (h->cfg.barrier_wait_polls <= 0) {
            L.polls = 0;
            break;
        }
        L.polls = std::max(L.polls, (unsigned)h->cfg.barrier_wait_polls);
    }
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

// The step graph with event nodes around the sweep (see Plan::tgraph).
fsim_status capture_timed_plan(Plan &pl, cudaStream_t st, int shape)
{
    for (int k = 0; k < 2; ++k)
        if (!pl.tev[k]) CK(cudaEventCreate(&pl.tev[k]));
    CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    fsim_status s = enqueue_plan(pl, st, shape, pl.tev[0], pl.tev[1], nullptr, cudaEventRecordExternal);
    cudaError_t e = cudaStreamEndCapture(st, &pl.tgraph);
    if (s) return s;
    if (e != cudaSuccess) {
        fsim_set_error("stream capture failed: %s", cudaGetErrorString(e));
        return FSIM_ECUDA;
    }
    size_t n = 0;
    CK(cudaGraphGetNodes(pl.tgraph, nullptr, &n));
    std::vector<cudaGraphNode_t> nodes(n);
    CK(cudaGraphGetNodes(pl.tgraph, nodes.data(), &n));
    for (cudaGraphNode_t nd : nodes) {
        cudaGraphNodeType type;
        CK(cudaGraphNodeGetType(nd, &type));
        if (type != cudaGraphNodeTypeEventRecord) continue;
        cudaEvent_t ev = nullptr;
        CK(cudaGraphEventRecordNodeGetEvent(nd, &ev));
        for (int k = 0; k < 2; ++k)
            if (ev == pl.tev[k]) pl.tnode[k] = nd;
    }
    if (!pl.tnode[0] || !pl.tnode[1]) {
        fsim_set_error("the captured step graph has no event nodes around the sweep");
        return FSIM_ECUDA;
    }
    for (int k = 0; k < 2; ++k) CK(cudaGraphInstantiate(&pl.texec[k], pl.tgraph, 0));
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
    if (phases & (1u << FSIM_PHASE_CELL)) h->rec_live = true;
    if (phases & (1u << FSIM_PHASE_FLUID)) h->rec_live = false;
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
// by launch and, in place of the one sweep, sweep kTuneRounds times with every
// candidate shape, timing each (CUDA events on the stream, waited for on the
// host).  A sweep is a pure function of its input buffer (it writes the other
// buffer; its running displacement maximum is idempotent) and the shapes give
// bit-identical results, so the step's outcome is the same.  Then keep the
// fastest shape and run the plan as a CUDA graph captured with it.
fsim_status run_plan_step(Plan &pl, cudaStream_t st, SweepTuner &t)
{
    if (t.chosen < 0 && pl.sweep_index >= 0) {
        for (cudaEvent_t &e : t.ev)
            if (!e) CK(cudaEventCreate(&e));
        fsim_status r = enqueue_plan(pl, st, 0, nullptr, nullptr, nullptr, cudaEventRecordDefault, t.ev, kTuneRounds);
        if (r) return r;
        CK(cudaEventSynchronize(t.ev[2 * kSweepShapes * kTuneRounds - 1]));
        for (int s_ = 0; s_ < kSweepShapes; ++s_) {
            t.ms[s_] = 0.0f;
            for (int r_ = 0; r_ < kTuneRounds; ++r_) {
                const int k = 2 * (r_ * kSweepShapes + s_);
                float ms = 0.0f;
                CK(cudaEventElapsedTime(&ms, t.ev[k], t.ev[k + 1]));
                if (r_ == 0 || ms < t.ms[s_]) t.ms[s_] = ms;
            }
        }
        t.next = kSweepShapes;
        t.chosen = 0;
        for (int k = 1; k < kSweepShapes; ++k)
            if (t.ms[k] < t.ms[t.chosen]) t.chosen = k;
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
    if (flags & FLAG_LIST_OVERFLOW) {
        fsim_set_error("a fluid particle has more than %d neighbour-list candidates (results invalid); "
                       "lower gb300_neighbor_skin or set it to 0", h->nl_cap);
        return FSIM_ENUMERIC;
    }
    if (flags & FLAG_CELL_OVERFULL) {
        fsim_set_error("a cell holds more than %d particles of one species (order inside it not kept)",
                       kStableRankMax);
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
    // neighbour-list instances keep their walls on the list grid (the list
    // build walks them there) and note each wall's impact-grid cell
    const DevParams &G = h->nl ? h->Pl : h->P;
    const int gcells = h->nl ? h->ncell_l : h->ncell;
    if ((st = dalloc(h, &d_xyz, vpos_dev ? 1 : 3 * (size_t)n)) || (st = dalloc(h, &tmp_pos, n)) ||
        (st = dalloc(h, &key, n)) || (st = dalloc(h, &slot, n)) || (st = dalloc(h, &tmp, n)) ||
        (st = dalloc(h, &cnt, gcells)) || (st = dalloc(h, &orig0, n)))
        return st;
    if (vpos_dev) {
        CK(cudaMemcpyAsync(tmp_pos, vpos_dev, sizeof(float4) * n, cudaMemcpyDeviceToDevice, h->stream));
    } else {
        CK(cudaMemcpyAsync(d_xyz, vpos_host, sizeof(float) * 3 * n, cudaMemcpyHostToDevice, h->stream));
        launch_k_pack_f4(blocks_for(n, kBlock), h->stream, d_xyz, nullptr, n, h->P.rho0, tmp_pos);
    }
    launch_k_iota(blocks_for(n, kBlock), h->stream, orig0, n);
    CK_LAUNCH();
    Plan pl;
    ArenaBuilder ab;
    add_launch(pl, ab, L_ZERO, std::vector<Item<ZeroArgs>>{{G, ZeroArgs{cnt, gcells, nullptr}}},
               {blocks_for(gcells, kBlock)});
    add_launch(pl, ab, L_HASH,
               std::vector<Item<HashArgs>>{{G, HashArgs{tmp_pos, n, key, slot, cnt, h->d_flags, nullptr}}},
               {blocks_for(n, kBlock)});
    const std::vector<Item<ScanArgs>> sc{{G, ScanArgs{cnt, h->v_start, gcells, h->scan_partials, nullptr}}};
    add_launch(pl, ab, L_SCAN_REDUCE, sc, {blocks_for(gcells, kScanTile)});
    add_launch(pl, ab, L_SCAN_PARTIALS, sc, {1});
    add_launch(pl, ab, L_SCAN_APPLY, sc, {blocks_for(gcells, kScanTile)});
    add_launch(pl, ab, L_SCATTER,
               std::vector<Item<ScatterArgs>>{{G, ScatterArgs{key, slot, h->v_start, tmp, n, nullptr}}},
               {blocks_for(n, kBlock)});
    // the fluid gather with a dummy velocity stream
    add_launch(pl, ab, L_GATHER_F,
               std::vector<Item<GatherFluidArgs>>{{G, GatherFluidArgs{tmp, key, h->v_start, n, tmp_pos, tmp_pos,
                                                                      orig0, h->v_posr, h->v_velp, h->v_orig,
                                                                      h->v_cell, h->d_flags, nullptr, nullptr}}},
               {blocks_for(n, kBlock)});
    pl.host = ab.bytes;
    CK(cudaMalloc((void **)&pl.arena, ab.bytes.size()));
    cudaError_t e = cudaMemcpy(pl.arena, ab.bytes.data(), ab.bytes.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && (st = enqueue_plan(pl, h->stream, 0)) == FSIM_OK) {
        e = cudaMemsetAsync(h->v_velp, 0, sizeof(float4) * n, h->stream);
        // the normal sums the walls within R: any grid of cells >= R finds them
        launch_k_virt_normal(blocks_for(n, kBlock), h->stream, G, h->v_posr, h->v_cell, h->v_start, h->v_normal, n);
        if (h->nl) launch_k_cells_of(blocks_for(n, kBlock), h->stream, h->P, h->v_posr, n, h->v_icell, h->v_icxyz);
        if (e == cudaSuccess) e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    }
    h->deferred.push_back(pl.arena);
    pl.arena = nullptr;
    if (e != cudaSuccess) {
        fsim_set_error("sorting the wall particles failed: %s", cudaGetErrorString(e));
        return FSIM_ECUDA;
    }
    if (st) return st;
    // temporaries are released now
    void *tmps[] = {d_xyz, tmp_pos, key, slot, tmp, cnt, orig0};
    for (void *p : tmps) release(h, p);
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
            if (r2 < R2) nbr.push_back(j);
        }
        off[i + 1] = (int)nbr.size();
    }
    const size_t ne = nbr.size();
    if (ne > (size_t)INT_MAX) {
        fsim_set_error("%zu solid neighbour entries exceed the index range", ne);
        return FSIM_EINVAL;
    }
    h->s_ne = (int)ne;
    std::vector<int> owner(ne);
    for (int i = 0; i < ns; ++i)
        for (int e = off[i]; e < off[i + 1]; ++e) owner[e] = i;
    fsim_status st;
    if ((st = dalloc(h, &h->s_nbr_off, (size_t)ns + 1)) || (st = dalloc(h, &h->s_nbr_orig, ne)) ||
        (st = dalloc(h, &h->s_nbr_owner, ne)) || (st = dalloc(h, &h->s_nbr_slot, ne)))
        return st;
    CK(cudaMemcpy(h->s_nbr_off, off.data(), sizeof(int) * (ns + 1), cudaMemcpyHostToDevice));
    if (ne) {
        CK(cudaMemcpy(h->s_nbr_orig, nbr.data(), sizeof(int) * ne, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(h->s_nbr_owner, owner.data(), sizeof(int) * ne, cudaMemcpyHostToDevice));
    }
    return FSIM_OK;
}

// The mixed form keeps the walls' positions as offsets from their impact-grid
// cells; a neighbour-list instance also keeps their absolute positions, which
// its list build walks on the list grid.
fsim_status walls_to_mixed(fsim_sim *h)
{
    if (h->nl) CK(cudaMemcpyAsync(h->v_abs, h->v_posr, sizeof(float4) * h->nv, cudaMemcpyDeviceToDevice, h->stream));
    launch_k_offsets_in_cells(blocks_for(h->nv, kBlock), h->stream, h->P, h->v_posr, h->nl ? h->v_icell : h->v_cell,
                              h->nv);
    CK_LAUNCH();
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
        (st = dalloc(h, &h->s_L, 9 * (size_t)ns)) || (st = dalloc(h, &h->s_PL, (size_t)kPLStride * ns)) ||
        (st = dalloc(h, &h->s_AV, 9 * (size_t)ns)) || (st = dalloc(h, &h->s_inv, ns)) ||
        (st = dalloc(h, &h->s_cxyz, ns)) ||
        (st = dalloc(h, &h->s_fl, (size_t)kFluidListCap * kSolidGroup * ns)) ||
        (st = dalloc(h, &h->s_fl_cnt, (size_t)kSolidGroup * ns)) || (st = dalloc(h, &h->s_fl_org, ns)))
        return st;
    // virtual
    if ((st = dalloc(h, &h->v_posr, nv)) || (st = dalloc(h, &h->v_velp, nv)) || (st = dalloc(h, &h->v_normal, nv)) ||
        (st = dalloc(h, &h->v_orig, nv)) || (st = dalloc(h, &h->v_cell, nv)) || (st = dalloc(h, &h->v_start, nc + 1)))
        return st;
    // fluid neighbour lists
    if (h->nl) {
        const int ncl = h->ncell_l;
        if ((st = dalloc(h, &h->nl_list, (size_t)h->nl_cap * nf)) || (st = dalloc(h, &h->nl_cnt, nf)) ||
            (st = dalloc(h, &h->nl_state, 1)) || (st = dalloc(h, &h->f_x0, nf)) || (st = dalloc(h, &h->s_x0, ns)) ||
            (st = dalloc(h, &h->f_ids, nf)) || (st = dalloc(h, &h->f_lcell, nf)) ||
            (st = dalloc(h, &h->f_lcnt, ncl)) || (st = dalloc(h, &h->f_lstart, ncl + 1)) ||
            (st = dalloc(h, &h->s_ids, ns)) || (st = dalloc(h, &h->s_lcell, ns)) ||
            (st = dalloc(h, &h->s_lcnt, ncl)) || (st = dalloc(h, &h->s_lstart, ncl + 1)) ||
            (st = dalloc(h, &h->v_icell, nv)) || (st = dalloc(h, &h->f_rec, 2 * (size_t)nf)) ||
            (st = dalloc(h, &h->f_spos, nf)))
            return st;
        if (h->nl_check && ((st = dalloc(h, &h->f_cxyz, nf)) || (st = dalloc(h, &h->v_icxyz, nv)))) return st;
        if (h->mixed && ((st = dalloc(h, &h->f_cell2, nf)) || (st = dalloc(h, &h->v_abs, nv)))) return st;
        NlState init{};
        init.force = 1; // the first step builds
        CK(cudaMemcpyAsync(h->nl_state, &init, sizeof init, cudaMemcpyHostToDevice, h->stream));
        CK(cudaMemsetAsync(h->nl_cnt, 0, sizeof(int) * (nf ? nf : 1), h->stream));
        CK(cudaMemsetAsync(h->f_x0, 0, sizeof(float4) * (nf ? nf : 1), h->stream));
        CK(cudaMemsetAsync(h->s_x0, 0, sizeof(float4) * (ns ? ns : 1), h->stream));
        CK(cudaMemsetAsync(h->f_lstart, 0, sizeof(int) * (ncl + 1), h->stream));
        CK(cudaMemsetAsync(h->s_lstart, 0, sizeof(int) * (ncl + 1), h->stream));
        // the per-step cell index starts from zero counts; each sort's scatter
        // leaves them zero again
        CK(cudaMemsetAsync(h->f_cnt, 0, sizeof(int) * nc, h->stream));
        CK(cudaMemsetAsync(h->s_cnt, 0, sizeof(int) * nc, h->stream));
        CK(cudaStreamSynchronize(h->stream)); // `init` leaves scope
    }
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
        launch_k_pack_f4(blocks_for(nf, kBlock), h->stream, stg, d_rho, nf, 0.0f, h->f_posr[0]);
        CK(cudaMemcpyAsync(d_rho, p->fluid_p, sizeof(float) * nf, cudaMemcpyHostToDevice, h->stream));
        CK(cudaStreamSynchronize(h->stream));
        CK(cudaMemcpyAsync(stg, p->fluid_vel, sizeof(float) * 3 * nf, cudaMemcpyHostToDevice, h->stream));
        launch_k_pack_f4(blocks_for(nf, kBlock), h->stream, stg, d_rho, nf, 0.0f, h->f_velp[0]);
        launch_k_iota(blocks_for(nf, kBlock), h->stream, h->f_orig[0], nf);
        if (h->mixed)
            launch_k_fluid_to_mixed(blocks_for(nf, kBlock), h->stream, h->P, h->f_posr[0], h->f_velp[0],
                                                                               h->f_cell, nf, h->d_flags);
        CK_LAUNCH();
        CK(cudaStreamSynchronize(h->stream));
        release(h, d_rho);
    }
    if (ns) {
        CK(cudaMemcpyAsync(stg, p->solid_pos, sizeof(float) * 3 * ns, cudaMemcpyHostToDevice, h->stream));
        launch_k_pack_f4(blocks_for(ns, kBlock), h->stream, stg, nullptr, ns, 0.0f, h->s_pos[0]);
        CK(cudaStreamSynchronize(h->stream));
        CK(cudaMemcpyAsync(stg, p->solid_vel, sizeof(float) * 3 * ns, cudaMemcpyHostToDevice, h->stream));
        launch_k_pack_f4(blocks_for(ns, kBlock), h->stream, stg, nullptr, ns, 0.0f, h->s_vel[0]);
        CK(cudaStreamSynchronize(h->stream));
        CK(cudaMemcpyAsync(stg, p->solid_ref_pos, sizeof(float) * 3 * ns, cudaMemcpyHostToDevice, h->stream));
        launch_k_pack_f4(blocks_for(ns, kBlock), h->stream, stg, nullptr, ns, 0.0f, h->s_ref[0]);
        CK(cudaMemcpyAsync(h->s_type[0], p->solid_type, sizeof(int) * ns, cudaMemcpyHostToDevice, h->stream));
        launch_k_iota(blocks_for(ns, kBlock), h->stream, h->s_orig[0], ns);
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
    if (nv && h->mixed && (st = walls_to_mixed(h))) return st;
    CK(cudaStreamSynchronize(h->stream));
    return check_flags(h);
}

} // namespace

// =================================================================== C ABI
namespace {
// Fluid neighbour lists (cfg.neighbor_skin > 0, both forms): list radius
// Rs = R (1 + skin); a step rebuilds once any particle has moved more than
// (Rs - R) / 2 less a rounding allowance since the last build, so that every
// pair within R is in the lists.  The reference pairs particles within R in
// neighbouring cells; where every cell side exceeds R by more than the FP32
// rounding of the cell coordinate (the stream sweep's z re-check rule, here
// on all three axes) that is the set {r < R}, else (nl_check) the list sweep
// also compares the pair's packed cell coordinates.  The list grid has cells
// of at least Rs (1 + 1e-3) on the reference grid's origin.
void setup_lists(fsim_sim *h)
{
    h->nl = false;
    h->nl_check = false;
    const double skin = h->cfg.neighbor_skin;
    if (!(skin > 0.0) || h->nf > kNlIndexMask || h->nv > kNlIndexMask || h->ns > kNlIndexMask) return;
    const double R = std::sqrt((double)h->der.impact_distance_square);
    for (int a = 0; a < 3; ++a) {
        const double margin = (double)h->der.interval[a] / R - 1.0;
        if (!(margin > 8e-7 * h->der.cell_number[a] + 1e-4)) h->nl_check = true;
    }
    // the mixed form's pair positions come from cell differences: it always
    // compares cell coordinates
    if (h->mixed) h->nl_check = true;
    // packed coordinates (x | y << 11 | z << 21) for the check
    if (h->nl_check && (h->P.nx >= 2048 || h->P.ny >= 1024 || h->P.nz >= 2048)) return;
    const double Rs = R * (1.0 + skin);
    double maxabs = 0.0;
    for (int a = 0; a < 3; ++a)
        maxabs = std::max(maxabs, std::max(std::fabs((double)h->der.cell_min[a]), std::fabs((double)h->der.cell_max[a])));
    // positions and their differences carry FP32 rounding of the coordinates
    const double slack = 16.0 * std::ldexp(maxabs, -23) + 1e-3 * (Rs - R);
    const double move = 0.5 * (Rs - R) - slack;
    if (!(move > 0.0)) return;
    DevParams Pl = h->P;
    int n[3];
    for (int a = 0; a < 3; ++a) {
        const double L = (double)h->der.cell_max[a] - (double)h->der.cell_min[a];
        n[a] = std::max(1, (int)std::floor(L / (Rs * (1.0 + 1e-3))));
        Pl.cinv[a] = (float)(n[a] / L);
        Pl.cdx[a] = (float)(L / n[a]);
        // the cells must still hold Rs with the FP32 inverse the kernels use
        if (!(1.0 / (double)Pl.cinv[a] >= Rs * (1.0 + 5e-4))) return;
    }
    Pl.nx = n[0];
    Pl.ny = n[1];
    Pl.nz = n[2];
    Pl.ncell = n[0] * n[1] * n[2];
    h->Pl = Pl;
    h->ncell_l = Pl.ncell;
    h->nl_R2s = (float)(Rs * Rs);
    h->nl_move2 = (float)(move * move);
    // list capacity: 1.5x a full sphere of radius Rs at the particle spacing
    const double dx = h->cfg.particle_diameter;
    const double full = 4.0 / 3.0 * 3.14159265358979 * std::pow(Rs / dx, 3.0);
    h->nl_cap = ((int)std::ceil(1.5 * full) + 16 + kNlGroup - 1) & ~(kNlGroup - 1); // whole groups
    h->nl = true;
}

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
    setup_lists(h);
    *out = h;
    return FSIM_OK;
}
} // namespace

extern "C" fsim_status fsim_create(const fsim_config *cfg, const fsim_particles *p, int device, fsim_handle *out)
{
    NvtxRange nvtx_("fsim_create");
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
    NvtxRange nvtx_("fsim_step");
    if (!h || nsteps < 0) return FSIM_EINVAL;
    if (h->batch) {
        fsim_set_error("the handle belongs to a batch; step it through the batch");
        return FSIM_EINVAL;
    }
    DeviceGuard guard(h->device);
    flush_deferred(h);
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
    NvtxRange nvtx_("fsim_run_phase");
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
    flush_deferred(h);
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
            launch_k_unpermute_mixed(g, h->stream, h->P, h->v_posr, h->v_velp, h->nl ? h->v_icell : h->v_cell,
                                     h->v_orig, n, MF_POS, stg);
        else
            launch_k_unpermute_mixed(g, h->stream, h->P, h->f_posr[h->f_cur], h->f_velp[h->f_cur], h->f_cell,
                                                            forig, n,
                                                            field == FSIM_FLUID_POS   ? MF_POS
                                                            : field == FSIM_FLUID_RHO ? MF_RHO
                                                                                      : MF_P,
                                                            stg);
        CK_LAUNCH();
        return FSIM_OK;
    }
    switch (field) {
    case FSIM_FLUID_POS: launch_k_unpermute_f4(g, h->stream, h->f_posr[h->f_cur], forig, n, 0, 3, stg); break;
    case FSIM_FLUID_RHO: launch_k_unpermute_f4(g, h->stream, h->f_posr[h->f_cur], forig, n, 3, 1, stg); break;
    case FSIM_FLUID_VEL: launch_k_unpermute_f4(g, h->stream, h->f_velp[h->f_cur], forig, n, 0, 3, stg); break;
    case FSIM_FLUID_P: launch_k_unpermute_f4(g, h->stream, h->f_velp[h->f_cur], forig, n, 3, 1, stg); break;
    case FSIM_FLUID_DRHO_DT:
    case FSIM_FLUID_DU_DT:
        if (!h->f_deriv_ok) {
            fsim_set_error("derivatives unavailable (set keep_derivatives and run the fluid phase)");
            return FSIM_EINVAL;
        }
        if (field == FSIM_FLUID_DU_DT)
            launch_k_unpermute_f4(g, h->stream, h->f_dudt, forig, n, 0, 3, stg);
        else
            launch_k_unpermute_words(g, h->stream, (const int *)h->f_drho, forig, n, 1, (int *)stg);
        break;
    case FSIM_FLUID_CELL_ID:
        if (!h->f_sorted) {
            fsim_set_error("cell ids unavailable before the first cell phase");
            return FSIM_EINVAL;
        }
        launch_k_unpermute_words(g, h->stream, h->f_cell, forig, n, 1, (int *)stg);
        break;
    case FSIM_SOLID_POS: launch_k_unpermute_f4(g, h->stream, h->s_pos[h->s_cur], sorig, n, 0, 3, stg); break;
    case FSIM_SOLID_VEL: launch_k_unpermute_f4(g, h->stream, h->s_vel[h->s_cur], sorig, n, 0, 3, stg); break;
    case FSIM_SOLID_REF_POS:
        launch_k_unpermute_f4(g, h->stream, h->s_ref[h->s_cur], sorig, n, 0, 3, stg);
        break;
    case FSIM_SOLID_TYPE:
        launch_k_unpermute_words(g, h->stream, h->s_type[h->s_cur], sorig, n, 1, (int *)stg);
        break;
    case FSIM_SOLID_CELL_ID:
        if (!h->s_sorted) {
            fsim_set_error("cell ids unavailable before the first cell phase");
            return FSIM_EINVAL;
        }
        launch_k_unpermute_words(g, h->stream, h->s_cell, sorig, n, 1, (int *)stg);
        break;
    case FSIM_SOLID_NORMAL:
    case FSIM_SOLID_P:
        if (!h->s_np_ok) {
            fsim_set_error("solid normal/pressure are stale after a cell phase; run the coupling phase first");
            return FSIM_EINVAL;
        }
        if (field == FSIM_SOLID_NORMAL) launch_k_unpermute_f4(g, h->stream, h->s_np, sorig, n, 0, 3, stg);
        else launch_k_unpermute_f4(g, h->stream, h->s_np, sorig, n, 3, 1, stg);
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
        if (field == FSIM_SOLID_DU_DT) launch_k_unpermute_f4(g, h->stream, h->s_dudt, sorig, n, 0, 3, stg);
        else if (field == FSIM_SOLID_COUPLE_DUDT)
            launch_k_unpermute_f4(g, h->stream, h->s_couple, sorig, n, 0, 3, stg);
        else {
            const float *src = field == FSIM_SOLID_F ? h->s_F : field == FSIM_SOLID_PK1 ? h->s_P : h->s_L;
            launch_k_unpermute_words(g, h->stream, (const int *)src, sorig, n, 9, (int *)stg);
        }
        break;
    case FSIM_VIRT_POS: launch_k_unpermute_f4(g, h->stream, h->v_posr, h->v_orig, n, 0, 3, stg); break;
    case FSIM_VIRT_RHO: launch_k_unpermute_f4(g, h->stream, h->v_posr, h->v_orig, n, 3, 1, stg); break;
    case FSIM_VIRT_VEL: launch_k_unpermute_f4(g, h->stream, h->v_velp, h->v_orig, n, 0, 3, stg); break;
    case FSIM_VIRT_P: launch_k_unpermute_f4(g, h->stream, h->v_velp, h->v_orig, n, 3, 1, stg); break;
    case FSIM_VIRT_NORMAL: launch_k_unpermute_f4(g, h->stream, h->v_normal, h->v_orig, n, 0, 3, stg); break;
    case FSIM_VIRT_CELL_ID:
        launch_k_unpermute_words(g, h->stream, h->nl ? h->v_icell : h->v_cell, h->v_orig, n, 1, (int *)stg);
        break;
    default: return FSIM_EINVAL;
    }
    CK_LAUNCH();
    return FSIM_OK;
}
} // namespace

extern "C" fsim_status fsim_get_field(fsim_handle h, int field, void *dst, size_t bytes)
{
    NvtxRange nvtx_("fsim_get_field");
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
// order, device memory `stg`) into the state (n > 0).  New fluid positions of
// a neighbour-list instance count as displacement since the last list build
// (the next step rebuilds if they moved too far); the solid's are measured at
// the next step's decision anyway.
fsim_status enqueue_permute_in(fsim_sim *h, int field, int n, const float *stg)
{
    float4 *dst = nullptr;
    const int *orig = nullptr;
    int comp = 0;
    fsim_status st = set_target(h, field, &dst, &orig, &comp);
    if (st) return st;
    const int width = fsim_field_width(field);
    if (h->mixed && (field == FSIM_FLUID_POS || field == FSIM_FLUID_RHO))
        launch_k_permute_in_mixed(blocks_for(n, kBlock), h->stream, 
            h->P, h->f_posr[h->f_cur], h->f_velp[h->f_cur], h->f_cell, orig, n,
            field == FSIM_FLUID_POS ? MF_POS : MF_RHO, stg);
    else
        launch_k_permute_in_f4(blocks_for(n, kBlock), h->stream, dst, orig, n, comp, width, stg);
    CK_LAUNCH();
    if (h->nl && field == FSIM_FLUID_POS) {
        launch_k_nl_displacement(blocks_for(n, kBlock), h->stream, h->P, dst, h->mixed ? h->f_cell : nullptr, h->f_x0,
                                 n, h->nl_state);
        CK_LAUNCH();
    }
    if (h->nl && field == FSIM_FLUID_POS && h->f_sorted) { // the index's position copy follows the state
        launch_k_gather_f4(blocks_for(n, kBlock), h->stream, h->f_ids, h->f_posr[h->f_cur], n, h->f_spos);
        CK_LAUNCH();
    }
    if (h->nl && field < 10 && h->rec_live) { // between the cell and fluid phases: records follow the state
        launch_k_pack_records(blocks_for(n, kBlock), h->stream, h->f_posr[h->f_cur], h->f_velp[h->f_cur],
                              h->mixed ? h->f_cxyz : nullptr, n, h->f_rec);
        CK_LAUNCH();
    }
    return FSIM_OK;
}
} // namespace

extern "C" fsim_status fsim_set_field(fsim_handle h, int field, const void *src, size_t bytes)
{
    NvtxRange nvtx_("fsim_set_field");
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
    NvtxRange nvtx_("fsim_get_fields");
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
    NvtxRange nvtx_("fsim_set_fields");
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
    NvtxRange nvtx_("fsim_probe");
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
    A.ids_f = h->nl ? h->f_ids : nullptr;
    A.ids_s = h->nl ? h->s_ids : nullptr;
    cudaError_t e = cudaMemcpyAsync(d, points, sizeof(float) * 3 * n, cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) {
        launch_k_probe(blocks_for(32ll * n, kBlock), h->stream, h->P, A);
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
    if (!h->nf) return FSIM_OK;
    DeviceGuard guard(h->device);
    int *d_counts = (int *)h->staging; // 3 * nf words fit the staging buffer
    const int g = blocks_for(h->nf, kBlock);
    if (h->mixed)
        launch_k_neighbor_counts_mixed(g, h->stream, h->P, h->nl ? h->Pl : h->P, h->f_posr[h->f_cur], h->f_cell,
                                       h->f_start, h->nl ? h->f_ids : nullptr, h->s_pos[h->s_cur], h->s_start,
                                       h->nl ? h->s_ids : nullptr, h->v_posr, h->v_start,
                                       h->nl ? h->v_icxyz : nullptr, d_counts, h->nf);
    else
        launch_k_neighbor_counts(g, h->stream, h->P, h->nl ? h->Pl : h->P, h->f_posr[h->f_cur], h->f_cell,
                                 h->f_start, h->nl ? h->f_ids : nullptr, h->s_pos[h->s_cur], h->s_start,
                                 h->nl ? h->s_ids : nullptr, h->v_posr, h->v_start, d_counts, h->nf);
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

namespace {
// fsim_get_cells of a neighbour-list instance: its particles lie in list-grid
// order, so the impact-grid cells come from the per-step index (fluid, solid)
// or from each wall's cell; the ids of a cell are listed in increasing input id.
fsim_status get_cells_nl(fsim_sim *h, int species, int n, int *cell_start, int *ids)
{
    std::vector<int> cell(n), orig(n);
    if (n) {
        const int *c = species == 0 ? h->f_cell : species == 1 ? h->s_cell : h->v_icell;
        const int *o = species == 0 ? h->f_orig[h->f_cur] : species == 1 ? h->s_orig[h->s_cur] : h->v_orig;
        CK(cudaMemcpyAsync(cell.data(), c, sizeof(int) * n, cudaMemcpyDeviceToHost, h->stream));
        CK(cudaMemcpyAsync(orig.data(), o, sizeof(int) * n, cudaMemcpyDeviceToHost, h->stream));
        CK(cudaStreamSynchronize(h->stream));
    }
    std::vector<int> by_input(n);
    for (int s = 0; s < n; ++s) by_input[orig[s]] = cell[s];
    std::fill(cell_start, cell_start + h->ncell + 1, 0);
    for (int i = 0; i < n; ++i) ++cell_start[by_input[i] + 1];
    for (int c = 0; c < h->ncell; ++c) cell_start[c + 1] += cell_start[c];
    std::vector<int> fill(cell_start, cell_start + h->ncell);
    for (int i = 0; i < n; ++i) ids[fill[by_input[i]]++] = i;
    return FSIM_OK;
}
} // namespace

extern "C" fsim_status fsim_list_stats(fsim_handle h, int *enabled, int *builds, int *capacity, int *check)
{
    if (!h) return FSIM_EINVAL;
    if (h->batch) batch_wait(h);
    int b = 0;
    if (h->nl) {
        DeviceGuard guard(h->device);
        NlState st;
        CK(cudaMemcpyAsync(&st, h->nl_state, sizeof st, cudaMemcpyDeviceToHost, h->stream));
        CK(cudaStreamSynchronize(h->stream));
        b = st.builds;
    }
    if (enabled) *enabled = h->nl ? 1 : 0;
    if (builds) *builds = b;
    if (capacity) *capacity = h->nl ? h->nl_cap : 0;
    if (check) *check = h->nl_check ? 1 : 0;
    return FSIM_OK;
}

extern "C" fsim_status fsim_list_counts(fsim_handle h, int *out, size_t bytes)
{
    if (!h || (!out && bytes)) return FSIM_EINVAL;
    if (h->batch) batch_wait(h);
    if (!h->nl) {
        fsim_set_error("the instance has no neighbour lists");
        return FSIM_EINVAL;
    }
    if (bytes != (size_t)h->nf * 3 * 4) {
        fsim_set_error("list counts need %zu bytes", (size_t)h->nf * 12);
        return FSIM_EINVAL;
    }
    if (!h->f_sorted) {
        fsim_set_error("run FSIM_PHASE_CELL first");
        return FSIM_EINVAL;
    }
    if (!h->nf) return FSIM_OK;
    DeviceGuard guard(h->device);
    int *d_counts = (int *)h->staging; // 3 * nf words fit the staging buffer
    if (h->mixed)
        launch_k_neighbor_counts_nlm(blocks_for(h->nf, kBlock), h->stream, h->P, h->f_posr[h->f_cur], h->f_cell,
                                     h->f_cxyz, h->nl_list, h->nl_cnt, h->nl_cap, h->s_pos[h->s_cur], h->s_cxyz,
                                     h->v_posr, h->v_icxyz, d_counts, h->nf);
    else
        launch_k_neighbor_counts_nl(blocks_for(h->nf, kBlock), h->stream, h->P, h->f_posr[h->f_cur], h->nl_list,
                                    h->nl_cnt, h->nl_cap, h->s_pos[h->s_cur], h->v_posr, d_counts, h->nf);
    CK_LAUNCH();
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
    if (h->nl) return get_cells_nl(h, species, n, cell_start, ids);
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
    NvtxRange nvtx_("fsim_write_vtk");
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
    flush_deferred(h);
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
    flush_deferred(h);
    while ((int)h->sweep_events.size() < 2 * nsteps) {
        cudaEvent_t e;
        CK(cudaEventCreate(&e));
        h->sweep_events.push_back(e);
    }
    fsim_status st = FSIM_OK;
    // once the sweep shape is tuned: the step graphs themselves (with event
    // nodes around the sweep), else launch by launch with the tuner's shape
    const bool graphs = h->tuner.chosen >= 0 && h->nf > 0;
    if (graphs) {
        // capture outside the timed region: a step flips the buffer parities
        // the same way every time, so consecutive steps use two plans
        const int f0 = h->f_cur, s0 = h->s_cur;
        for (int k = 0; k < 2; ++k) {
            Plan *pl = nullptr;
            if ((st = handle_step_plan(h, &pl))) return st;
            if (!pl->tgraph && (st = capture_timed_plan(*pl, h->stream, h->tuner.chosen))) return st;
            h->f_cur = pl->pf_after;
            h->s_cur = pl->ps_after;
        }
        h->f_cur = f0;
        h->s_cur = s0;
    }
    CK(cudaEventRecord(h->ev0, h->stream));
    for (int k = 0; k < nsteps; ++k) {
        Plan *pl = nullptr;
        if ((st = handle_step_plan(h, &pl))) return st;
        if (graphs) {
            if (!pl->tgraph && (st = capture_timed_plan(*pl, h->stream, h->tuner.chosen))) return st;
            cudaGraphExec_t ex = pl->texec[pl->tnext];
            pl->tnext ^= 1;
            CK(cudaGraphExecEventRecordNodeSetEvent(ex, pl->tnode[0], h->sweep_events[2 * k]));
            CK(cudaGraphExecEventRecordNodeSetEvent(ex, pl->tnode[1], h->sweep_events[2 * k + 1]));
            CK(cudaGraphLaunch(ex, h->stream));
        } else if ((st = enqueue_plan(*pl, h->stream, h->tuner.shape(), h->sweep_events[2 * k],
                                      h->sweep_events[2 * k + 1]))) {
            return st;
        }
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

extern "C" fsim_status fsim_time_phases(fsim_handle h, int nsteps, float *ms, int n)
{
    NvtxRange nvtx_("fsim_time_phases");
    if (!h || nsteps < 0 || !ms || n < 1) return FSIM_EINVAL;
    if (h->batch) {
        fsim_set_error("the handle belongs to a batch");
        return FSIM_EINVAL;
    }
    DeviceGuard guard(h->device);
    flush_deferred(h);
    double tot[5] = {0, 0, 0, 0, 0};
    std::vector<cudaEvent_t> ev;
    fsim_status st = FSIM_OK;
    for (int k = 0; k < nsteps && !st; ++k) {
        Plan *pl = nullptr;
        if ((st = handle_step_plan(h, &pl))) break;
        const size_t need = 2 * pl->launches.size();
        while (ev.size() < need) {
            cudaEvent_t e;
            if (cudaEventCreate(&e) != cudaSuccess) {
                st = FSIM_ECUDA;
                break;
            }
            ev.push_back(e);
        }
        if (st || (st = enqueue_plan(*pl, h->stream, h->tuner.shape(), nullptr, nullptr, ev.data()))) break;
        after_plan(h, kAllPhases, *pl);
        if (cudaEventSynchronize(ev[need - 1]) != cudaSuccess) {
            st = FSIM_ECUDA;
            break;
        }
        for (size_t q = 0; q < pl->launches.size(); ++q) {
            float t = 0.0f;
            cudaEventElapsedTime(&t, ev[2 * q], ev[2 * q + 1]);
            tot[launch_phase(pl->launches[q].kind)] += t;
        }
    }
    for (cudaEvent_t e : ev) cudaEventDestroy(e);
    if (st) return st;
    for (int p = 0; p < n; ++p) ms[p] = p < 5 ? (float)tot[p] : 0.0f;
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
        launch_k_conservation_fluid(bf, h->stream, h->P, h->f_posr[h->f_cur], h->f_velp[h->f_cur], h->f_cell,
                                                            h->nf, vol, d_part);
    if (bs)
        launch_k_conservation_solid(bs, h->stream, h->P, h->s_pos[h->s_cur], h->s_vel[h->s_cur], h->s_F, h->ns,
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
// A neighbour-list instance also saves what its lists were built from (the
// positions and list-grid cells of the last build, the particles' order then)
// and its list state; loading rebuilds the same lists from them.
std::vector<SnapArray> snap_arrays(fsim_sim *h, int pf, int ps)
{
    const size_t nf = h->nf, ns = h->ns, nv = h->nv, nc = h->ncell;
    std::vector<SnapArray> a = {
        {h->f_posr[pf], 16 * nf}, {h->f_velp[pf], 16 * nf}, {h->f_orig[pf], 4 * nf},   {h->f_cell, 4 * nf},
        {h->s_pos[ps], 16 * ns},  {h->s_vel[ps], 16 * ns},  {h->s_ref[ps], 16 * ns},   {h->s_type[ps], 4 * ns},
        {h->s_orig[ps], 4 * ns},  {h->v_posr, 16 * nv},     {h->v_velp, 16 * nv},      {h->v_normal, 16 * nv},
        {h->v_orig, 4 * nv},      {h->v_cell, 4 * nv},      {h->v_start, 4 * (nc + 1)}};
    if (h->nl) {
        const size_t ncl = h->ncell_l;
        const std::vector<SnapArray> b = {{h->f_x0, 16 * nf},           {h->f_lcell, 4 * nf},
                                          {h->f_lstart, 4 * (ncl + 1)}, {h->s_x0, 16 * ns},
                                          {h->s_lcell, 4 * ns},         {h->s_lstart, 4 * (ncl + 1)},
                                          {h->s_inv, 4 * ns},           {h->nl_state, sizeof(NlState)}};
        a.insert(a.end(), b.begin(), b.end());
        if (h->mixed) a.push_back({h->v_abs, 16 * nv});
    }
    return a;
}

// Build the lists from the saved build state (positions and cells of the last
// build) without deciding or sorting, then restore the saved list state.
fsim_status nl_restore(fsim_sim *h)
{
    NlState saved;
    CK(cudaMemcpy(&saved, h->nl_state, sizeof saved, cudaMemcpyDeviceToHost));
    NlState now = saved;
    now.rebuild = 1;
    CK(cudaMemcpy(h->nl_state, &now, sizeof now, cudaMemcpyHostToDevice));
    const float4 *vpos = h->mixed ? h->v_abs : h->v_posr; // absolute wall positions
    if (h->nv) {
        launch_k_cells_of(blocks_for(h->nv, kBlock), h->stream, h->P, vpos, h->nv, h->v_icell, h->v_icxyz);
        CK_LAUNCH();
    }
    Plan pl;
    ArenaBuilder ab;
    add_launch(pl, ab, L_NL_BUILD,
               std::vector<Item<NlBuildArgs>>{{h->Pl, NlBuildArgs{h->f_x0, h->f_lcell, h->f_lstart, vpos,
                                                                  h->v_start, h->s_x0, h->s_lstart, h->nf, h->nl_cap,
                                                                  h->nl_list, h->nl_cnt, h->nl_state, h->d_flags,
                                                                  h->nl_R2s, h->nv, h->ns}}},
               {blocks_for(h->nf, kNlBuildThreads)});
    pl.host = ab.bytes;
    CK(cudaMalloc((void **)&pl.arena, ab.bytes.size()));
    cudaError_t e = cudaMemcpy(pl.arena, ab.bytes.data(), ab.bytes.size(), cudaMemcpyHostToDevice);
    fsim_status st = FSIM_OK;
    if (e == cudaSuccess) st = enqueue_plan(pl, h->stream, 0);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    cudaFree(pl.arena);
    pl.arena = nullptr;
    if (e != cudaSuccess) {
        fsim_set_error("rebuilding the neighbour lists failed: %s", cudaGetErrorString(e));
        return FSIM_ECUDA;
    }
    if (st) return st;
    CK(cudaMemcpy(h->nl_state, &saved, sizeof saved, cudaMemcpyHostToDevice));
    return FSIM_OK;
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
    NvtxRange nvtx_("fsim_snapshot_save");
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
    hd.version = 2;
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
    NvtxRange nvtx_("fsim_snapshot_load");
    if (!buf || !out) return FSIM_EINVAL;
    *out = nullptr;
    SnapHeader hd;
    if (bytes < kSnapHeaderBytes) {
        fsim_set_error("snapshot too short");
        return FSIM_EIO;
    }
    std::memcpy(&hd, buf, sizeof hd);
    if (std::memcmp(hd.magic, kSnapMagic, 8) || hd.version != 2 || hd.config_bytes != sizeof(fsim_config) ||
        hd.n_fluid < 0 || hd.n_solid < 0 || hd.n_virt < 0) {
        fsim_set_error("not a version-2 fluidsim snapshot");
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
    if (h->nl && (st = nl_restore(h))) {
        free_all(h);
        delete h;
        return st;
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
    NvtxRange nvtx_("fsim_create_case");
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
    launch_k_case_generate(blocks_for(A.nsite, kBlock), h->stream, A);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        fsim_set_error("case generation failed: %s", cudaGetErrorString(e));
        return fail(FSIM_ECUDA);
    }
    const int nf = h->nf, ns = h->ns;
    if (nf && h->mixed) {
        launch_k_fluid_to_mixed(blocks_for(nf, kBlock), h->stream, h->P, h->f_posr[0], h->f_velp[0],
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
        if (h->mixed && (st = walls_to_mixed(h))) return fail(st);
    }
    // generation temporaries are released now
    CK(cudaStreamSynchronize(h->stream));
    void *tmps[] = {d_base, d_hydro, d_vpos};
    for (void *p : tmps) release(h, p);
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
        if (members[k]->mixed != members[0]->mixed || members[k]->nl != members[0]->nl ||
            members[k]->cfg.solid_fused != members[0]->cfg.solid_fused ||
            members[k]->cfg.solid_full_walk != members[0]->cfg.solid_full_walk) {
            fsim_set_error("batch members must share the precision form, the neighbour search (lists or cell "
                           "walk) and the solid launch form");
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
    for (fsim_sim *h : b->members) {
        flush_deferred(h);
        h->batch = b;
    }
    *out = b;
    return FSIM_OK;
}

extern "C" fsim_status fsim_batch_step(fsim_batch_t b, int nsteps)
{
    NvtxRange nvtx_("fsim_batch_step");
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
    if (!b->members.empty() && (h->mixed != b->members[0]->mixed || h->nl != b->members[0]->nl ||
                                h->cfg.solid_fused != b->members[0]->cfg.solid_fused ||
                                h->cfg.solid_full_walk != b->members[0]->cfg.solid_full_walk)) {
        fsim_set_error("batch members must share the precision form, the neighbour search (lists or cell walk) "
                       "and the solid launch form");
        return FSIM_EINVAL;
    }
    DeviceGuard guard(b->device);
    flush_deferred(h);
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

extern "C" fsim_status fsim_device_bytes(fsim_handle h, size_t *bytes)
{
    if (!h || !bytes) return FSIM_EINVAL;
    size_t b = 0;
    for (const auto &a : h->allocations) b += a.second;
    *bytes = b;
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
    b += ns * (3 * sizeof(float4) + (4 * 9 + kPLStride) * sizeof(float) + 2 * sizeof(int)); // per-step products, inv, cells
    b += ns * (kSolidGroup * (kFluidListCap + 1) * sizeof(int) + sizeof(float4)); // force fluid lists
    {
        // static solid neighbour lists (id, owner, per-step slot):
        // lattice count within 2h, plus slack
        const double r = std::sqrt((double)d.impact_distance_square) / (double)cfg->particle_diameter;
        const size_t per = (size_t)(4.18879 * r * r * r * 1.25) + 8;
        b += ns * per * 3 * sizeof(int) + (ns + 1) * sizeof(int);
    }
    b += nv * (3 * sizeof(float4) + 2 * sizeof(int));
    b += nc * sizeof(int) * 2 + (nc + 1) * sizeof(int) * 3; // counts, starts
    if (cfg->precision == FSIM_PRECISION_MIXED) b += nc * sizeof(float2); // per-cell references
    if (cfg->neighbor_skin > 0.0f) {
        // fluid neighbour lists (as setup_lists sizes them) and the list-grid
        // sort, build state and per-step index (at most as many cells as nc):
        // lists, list counts, ids, list cells, packed cells; x0, the 32-byte
        // records and the positions in the index's order; the mixed form's
        // carried cells and absolute wall positions
        const double rs = std::sqrt((double)d.impact_distance_square) * (1.0 + cfg->neighbor_skin) /
                          (double)cfg->particle_diameter;
        const size_t cap = (((size_t)std::ceil(1.5 * 4.18879 * rs * rs * rs) + 16 + kNlGroup - 1) & ~size_t(kNlGroup - 1));
        b += nf * (cap + 4) * sizeof(int) + nf * 4 * sizeof(float4);
        b += ns * (sizeof(float4) + 2 * sizeof(int)) + nv * 2 * sizeof(int);
        if (cfg->precision == FSIM_PRECISION_MIXED) b += nf * sizeof(int) + nv * sizeof(float4);
        b += nc * sizeof(int) * 2 + (nc + 1) * sizeof(int) * 2 + sizeof(NlState);
    }
    b += 2 * kMaxScanTiles * sizeof(int) + sizeof(unsigned);
    size_t words = 3 * nf;
    if (9 * ns > words) words = 9 * ns;
    if (3 * nv > words) words = 3 * nv;
    b += 4 * (words ? words : 1);
    b += 64 * 1024; // plans and allocation granularity
    *out = b;
    return FSIM_OK;
}

