// Host half of the reference build (test infrastructure only).
//
// The reference's device code (oracle/refcuda/ref_device.cu: its unmodified
// src/{memory_copy,pair,fluid,virt,solid}.cu) is compiled into a device image
// by oracle/build.py.  This file is the host program around it, written here
// because the reference's own host code is Windows-only (windows.h, MSVC
// syntax) and cannot travel without its sources.  It does what the
// reference's host does for one run, in the same order:
//
//   Sim::initiate (include/sim.cuh:33-43)      initial values of every array as
//       Fluid/Solid/Virt_Host_List::addList (include/host_data.cuh:20-38,
//       79-101,147-163) sets them; the 27-neighbour cell table of
//       Sim::createCell (src/sim.cu:153-236); the initial linked cell lists of
//       Sim::fillCell (src/sim.cu:256-302, each particle appended at the tail
//       of its cell's list in input order);
//   MemoryCopy::copyConstant (src/memory_copy.cu:8-12)   the Parameter and
//       Data_Pointer images copied into the image's dev_par / dev_data;
//   DeviceCalculation::calculation (src/calculation.cu:20-35)   per step
//       particleCellUpdate, fillCell, coupleCalculation, virtUpdate,
//       fluidCalculation, solidCalculation with the reference's launch shapes
//       (n / thread_num + 1 blocks of thread_num threads, src/pair.cu:53-69,
//       192-206, src/fluid.cu:271-283, src/virt.cu:77-86,
//       src/solid.cu:241-260,330-344) and a device synchronisation after every
//       launch, as the reference does.
//
// The Parameter mirror below follows include/parameter.h:17-49 and the member
// classes it holds (include/physics.h, properties.h, domain.h, sim_time.h,
// kernel.h); the Data_Pointer mirror follows include/data_pointer.cuh:7-47 and
// Cell include/cell.cuh:11-20.  ref_layout() reports the mirror's offsets so a
// test can compare them with the reference headers, and create() checks the
// sizes against the image's own symbols.
#include <cuda_runtime.h>

#include <stddef.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "fluidsim.h"

namespace {

struct RPhysics { float gravity[3]; };
struct RFluidProps {
    int number;
    float sound_speed, reference_density, reference_density_inverse;
    float gamma, viscosity, gamma_inv, coefficient_p2rho, coefficient_rho2p;
    float min_pressure, min_density, max_density;
    bool is_fluid_viscid;
};
struct RSolidProps {
    int number;
    float reference_density, youngs_modulus, poisson_ratio;
    float lambda, nu, bulk_modulus;
    float artificial_viscocity[2], sound_speed;
};
struct RVirtProps { int number; };
struct RDomain {
    float cell_min[3], cell_max[3], domain_min[3], domain_max[3];
    int cell_number[3];
    float interval[3], interval_inv[3];
    int cell_number_total;
};
struct RTime {
    float dt, current_time;
    int istart, iend, i, file_step, solid_sub_step, result_interval, sort_every_step;
};
struct RKernel {
    float smoothing_length, particle_diameter, particle_volume, diameter_square;
    int thread_num;
    float smoothing_length_square, smoothing_length_inverse, smoothing_length_inverse_square;
    float impact_length_hsml_ratio, impact_distance_square;
    float kernel_coefficient_1, kernel_coefficient_2, kernel_differential;
};
struct RParameter {
    RPhysics physics;
    RFluidProps fluid;
    RSolidProps solid;
    RVirtProps virt;
    RDomain domain;
    RTime time;
    RKernel kernel;
};

// vec3 = 3 floats, mat3 = 9 floats (column-major), enums = int
struct RFluidData {
    float *position, *velocity;
    float *density, *pressure, *color;
    int *cell_id, *next_id, *next_id_previous;
    float *du_dt;
    float *drho_dt;
};
struct RSolidData {
    float *position, *reference_position, *velocity;
    int *solid_type;
    float *pressure;
    int *cell_id, *next_id, *next_id_previous;
    float *deformation, *stress_1st_piola, *correction;
    float *du_dt;
    float *couple_dudt;
    float *normal;
};
struct RVirtData {
    float *position, *normal, *velocity;
    float *pressure, *density;
    int *virt_type;
    int *cell_id, *next_id, *next_id_previous;
};
struct RCell {
    int neighbor_cell_id[27];
    int fluid_start_id, solid_start_id, virt_start_id;
    int fluid_start_id_previous, solid_start_id_previous, virt_start_id_previous;
};
struct RDataPointer {
    RFluidData fluid;
    RSolidData solid;
    RVirtData virt;
    RCell *cell;
};

enum { K_FILL_FLUID, K_FILL_SOLID, K_FILL_VIRT, K_COPY_LIST, K_FILL_LIST, K_COUPLE, K_VIRT, K_FLUID_PAIR,
       K_FLUID_UPDATE, K_SOLID_DEFORM, K_SOLID_FORCE, K_SOLID_UPDATE, K_COUNT };
// Itanium-mangled names of the reference's argument-less __global__ functions.
const char *const kKernelNames[K_COUNT] = {
    "_Z15fillFluidCellIDv", "_Z15fillSolidCellIDv", "_Z14fillVirtCellIDv", "_Z12copyCellListv",
    "_Z12fillCellListv", "_Z17solidCoupleUpdatev", "_Z11getVirtDatav", "_Z13findFluidPairv",
    "_Z11fluidUpdatev", "_Z25solidDeformationCalculatev", "_Z19solidForceCalculatev", "_Z11solidUpdatev"};

thread_local std::string g_error;

int fail(const std::string &msg)
{
    g_error = msg;
    return 1;
}

#define RCHECK(call)                                                                              \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess)                                                                    \
            return fail(std::string(#call) + ": " + cudaGetErrorString(e_));                      \
    } while (0)

}  // namespace

struct ref_sim {
    cudaLibrary_t lib = nullptr;
    cudaKernel_t kernels[K_COUNT] = {};
    RParameter par;
    RDataPointer data;
    std::vector<void *> allocations;
    int nf = 0, ns = 0, nv = 0, ncell = 0, threads = 32, sub_steps = 1;
    cudaEvent_t ev[2] = {nullptr, nullptr};
};

namespace {

template <typename T>
int alloc_copy(ref_sim *s, T **dst, size_t count, const T *init)
{
    *dst = nullptr;
    if (count == 0)
        return 0;
    void *p = nullptr;
    RCHECK(cudaMalloc(&p, count * sizeof(T)));
    s->allocations.push_back(p);
    *dst = static_cast<T *>(p);
    if (init)
        RCHECK(cudaMemcpy(p, init, count * sizeof(T), cudaMemcpyHostToDevice));
    return 0;
}

// One launch of n / thread_num + 1 blocks; sync = the reference's
// cudaDeviceSynchronize after it (particleCellUpdate synchronises once after
// its three launches, every other phase after each launch).
int launch(ref_sim *s, int k, int n, bool sync = true)
{
    dim3 grid(n / s->threads + 1), block(s->threads);
    RCHECK(cudaLaunchKernel(reinterpret_cast<const void *>(s->kernels[k]), grid, block, nullptr, 0, 0));
    if (sync)
        RCHECK(cudaDeviceSynchronize());
    else
        RCHECK(cudaGetLastError());
    return 0;
}

// The step's phases (src/calculation.cu:25-31); ids follow FSIM_PHASE_*.
int run_phase(ref_sim *s, int phase)
{
    switch (phase) {
    case FSIM_PHASE_CELL:  // particleCellUpdate + fillCell
        if (launch(s, K_FILL_FLUID, s->nf, false) || launch(s, K_FILL_SOLID, s->ns, false) ||
            launch(s, K_FILL_VIRT, s->nv))
            return 1;
        return launch(s, K_COPY_LIST, s->ncell) || launch(s, K_FILL_LIST, s->ncell);
    case FSIM_PHASE_COUPLE:
        if (s->nf == 0 || s->ns == 0)
            return 0;
        return launch(s, K_COUPLE, s->ns);
    case FSIM_PHASE_VIRT:
        if (s->nv == 0)
            return 0;
        return launch(s, K_VIRT, s->nv);
    case FSIM_PHASE_FLUID:
        if (s->nf == 0)
            return 0;
        return launch(s, K_FLUID_PAIR, s->nf) || launch(s, K_FLUID_UPDATE, s->nf);
    case FSIM_PHASE_SOLID:
        if (s->ns == 0)
            return 0;
        for (int i = 0; i < s->sub_steps; ++i)
            if (launch(s, K_SOLID_DEFORM, s->ns) || launch(s, K_SOLID_FORCE, s->ns) ||
                launch(s, K_SOLID_UPDATE, s->ns))
                return 1;
        return 0;
    default:
        return fail("unknown phase");
    }
}

int run_steps(ref_sim *s, int n)
{
    for (int i = 0; i < n; ++i)
        for (int p = FSIM_PHASE_CELL; p <= FSIM_PHASE_SOLID; ++p)
            if (run_phase(s, p))
                return 1;
    return 0;
}

// Sim::getCellID (src/sim.cu:238-254), with a range check the reference lacks.
int cell_of(const RParameter &par, const float *x)
{
    const RDomain &d = par.domain;
    int nx = (int)((x[0] - d.cell_min[0]) * d.interval_inv[0]);
    int ny = (int)((x[1] - d.cell_min[1]) * d.interval_inv[1]);
    int nz = (int)((x[2] - d.cell_min[2]) * d.interval_inv[2]);
    if (nx < 0 || ny < 0 || nz < 0 || nx >= d.cell_number[0] || ny >= d.cell_number[1] || nz >= d.cell_number[2])
        return -1;
    return nx * d.cell_number[1] * d.cell_number[2] + ny * d.cell_number[2] + nz;
}

// Initial lists: particle i appended at the tail of its cell's list in input
// order (what Sim::fillCell's walk to the tail produces).
int initial_lists(const RParameter &par, int n, const float *pos, size_t start_field, std::vector<RCell> &cells,
                  std::vector<int> &next)
{
    next.assign(n, -1);
    std::vector<int> tail(cells.size(), -1);
    for (int i = 0; i < n; ++i) {
        int c = cell_of(par, pos + 3 * (size_t)i);
        if (c < 0)
            return fail("a particle lies outside the cell grid");
        int *head = reinterpret_cast<int *>(reinterpret_cast<char *>(&cells[c]) + start_field);
        if (*head == -1)
            *head = i;
        else
            next[tail[c]] = i;
        tail[c] = i;
    }
    return 0;
}

}  // namespace

extern "C" {

const char *ref_last_error(void) { return g_error.c_str(); }

// Byte offsets of the mirror's members, in the order the layout test lists
// them (sizes last).
int ref_layout(long long *out, int cap)
{
    const long long v[] = {
        (long long)offsetof(RParameter, physics), (long long)offsetof(RParameter, fluid),
        (long long)offsetof(RParameter, solid), (long long)offsetof(RParameter, virt),
        (long long)offsetof(RParameter, domain), (long long)offsetof(RParameter, time),
        (long long)offsetof(RParameter, kernel),
        (long long)offsetof(RFluidProps, is_fluid_viscid), (long long)offsetof(RSolidProps, sound_speed),
        (long long)offsetof(RDomain, cell_number_total), (long long)offsetof(RTime, sort_every_step),
        (long long)offsetof(RKernel, thread_num), (long long)offsetof(RKernel, kernel_differential),
        (long long)offsetof(RDataPointer, solid), (long long)offsetof(RDataPointer, virt),
        (long long)offsetof(RDataPointer, cell), (long long)offsetof(RSolidData, normal),
        (long long)offsetof(RVirtData, next_id_previous), (long long)offsetof(RCell, virt_start_id_previous),
        (long long)sizeof(RParameter), (long long)sizeof(RDataPointer), (long long)sizeof(RCell)};
    int n = (int)(sizeof(v) / sizeof(v[0]));
    for (int i = 0; i < n && i < cap; ++i)
        out[i] = v[i];
    return n;
}

int ref_create(const char *image_path, const fsim_config *cfg, const fsim_derived *d, const fsim_particles *p,
               int device, ref_sim **out)
{
    *out = nullptr;
    if (!image_path || !cfg || !d || !p)
        return fail("null argument");
    if (cfg->thread_num <= 0 || cfg->solid_sub_step <= 0)
        return fail("thread_num and solid_sub_step must be positive");
    if (device >= 0)
        RCHECK(cudaSetDevice(device));
    RCHECK(cudaFree(nullptr));
    ref_sim *s = new ref_sim();
    *out = s;
    RCHECK(cudaLibraryLoadFromFile(&s->lib, image_path, nullptr, nullptr, 0, nullptr, nullptr, 0));
    for (int k = 0; k < K_COUNT; ++k)
        RCHECK(cudaLibraryGetKernel(&s->kernels[k], s->lib, kKernelNames[k]));
    for (int e = 0; e < 2; ++e)
        RCHECK(cudaEventCreate(&s->ev[e]));

    s->nf = p->n_fluid;
    s->ns = p->n_solid;
    s->nv = p->n_virt;
    s->threads = cfg->thread_num;
    s->sub_steps = cfg->solid_sub_step;
    s->ncell = d->cell_number_total;

    // Parameter, as Parameter::initiate leaves it (src/parameter.cpp:9-34)
    RParameter &par = s->par;
    memset(&par, 0, sizeof(par));
    for (int i = 0; i < 3; ++i)
        par.physics.gravity[i] = d->gravity_vec[i];
    par.fluid.number = s->nf;
    par.fluid.sound_speed = cfg->fluid_sound_speed;
    par.fluid.reference_density = cfg->fluid_density;
    par.fluid.reference_density_inverse = d->reference_density_inverse;
    par.fluid.gamma = cfg->gamma;
    par.fluid.viscosity = cfg->viscosity;
    par.fluid.gamma_inv = d->gamma_inv;
    par.fluid.coefficient_p2rho = d->coefficient_p2rho;
    par.fluid.coefficient_rho2p = d->coefficient_rho2p;
    par.fluid.min_pressure = cfg->min_pressure;
    par.fluid.min_density = d->min_density;
    par.fluid.max_density = d->max_density;
    par.fluid.is_fluid_viscid = cfg->is_viscid != 0;
    par.solid.number = s->ns;
    par.solid.reference_density = cfg->solid_density;
    par.solid.youngs_modulus = cfg->youngs_modulus;
    par.solid.poisson_ratio = cfg->poisson_ratio;
    par.solid.lambda = d->lambda;
    par.solid.nu = d->shear_modulus;
    par.solid.bulk_modulus = d->bulk_modulus;
    par.solid.artificial_viscocity[0] = cfg->arti_vis_alpha;
    par.solid.artificial_viscocity[1] = cfg->arti_vis_beta;
    par.solid.sound_speed = d->solid_sound_speed;
    par.virt.number = s->nv;
    const float dmin[3] = {cfg->xmin, cfg->ymin, cfg->zmin}, dmax[3] = {cfg->xmax, cfg->ymax, cfg->zmax};
    for (int i = 0; i < 3; ++i) {
        par.domain.cell_min[i] = d->cell_min[i];
        par.domain.cell_max[i] = d->cell_max[i];
        par.domain.domain_min[i] = dmin[i];
        par.domain.domain_max[i] = dmax[i];
        par.domain.cell_number[i] = d->cell_number[i];
        par.domain.interval[i] = d->interval[i];
        par.domain.interval_inv[i] = d->interval_inv[i];
    }
    par.domain.cell_number_total = d->cell_number_total;
    par.time.dt = cfg->dt;
    par.time.istart = cfg->istart;
    par.time.iend = cfg->iend;
    par.time.i = cfg->istart;
    par.time.current_time = (float)cfg->istart * cfg->dt;
    par.time.result_interval = cfg->result_interval;
    par.time.file_step = cfg->result_interval > 0 ? cfg->istart / cfg->result_interval : 0;
    par.time.solid_sub_step = cfg->solid_sub_step;
    par.time.sort_every_step = cfg->sort_every_step;
    par.kernel.smoothing_length = cfg->smoothing_length;
    par.kernel.particle_diameter = cfg->particle_diameter;
    par.kernel.particle_volume = d->particle_volume;
    par.kernel.diameter_square = cfg->particle_diameter * cfg->particle_diameter;
    par.kernel.thread_num = cfg->thread_num;
    par.kernel.smoothing_length_square = d->smoothing_length_square;
    par.kernel.smoothing_length_inverse = d->smoothing_length_inverse;
    par.kernel.smoothing_length_inverse_square = d->smoothing_length_inverse_square;
    par.kernel.impact_length_hsml_ratio = cfg->impact_length_hsml_ratio;
    par.kernel.impact_distance_square = d->impact_distance_square;
    par.kernel.kernel_coefficient_1 = d->kernel_coefficient_1;
    par.kernel.kernel_coefficient_2 = d->kernel_coefficient_2;
    par.kernel.kernel_differential = d->kernel_differential;

    // cells: Sim::createCell's table; neighbour n of cell (i, j, k) for
    // di = n / 9 - 1 visits (dj, dk) in this order, -1 beyond the grid
    static const int kRow[9][2] = {{-1, -1}, {-1, 1}, {1, -1}, {1, 1}, {0, -1}, {0, 1}, {-1, 0}, {1, 0}, {0, 0}};
    const int cx = d->cell_number[0], cy = d->cell_number[1], cz = d->cell_number[2];
    if (cx <= 0 || cy <= 0 || cz <= 0 || (long long)cx * cy * cz != d->cell_number_total)
        return fail("bad cell grid");
    std::vector<RCell> cells((size_t)s->ncell);
    for (int i = 0; i < cx; ++i)
        for (int j = 0; j < cy; ++j)
            for (int k = 0; k < cz; ++k) {
                RCell &c = cells[((size_t)i * cy + j) * cz + k];
                for (int n = 0; n < 27; ++n) {
                    int ii = i + n / 9 - 1, jj = j + kRow[n % 9][0], kk = k + kRow[n % 9][1];
                    bool in = ii >= 0 && ii < cx && jj >= 0 && jj < cy && kk >= 0 && kk < cz;
                    c.neighbor_cell_id[n] = in ? (ii * cy + jj) * cz + kk : -1;
                }
                c.fluid_start_id = c.solid_start_id = c.virt_start_id = -1;
                c.fluid_start_id_previous = c.solid_start_id_previous = c.virt_start_id_previous = -1;
            }
    std::vector<int> fnext, snext, vnext;
    if (initial_lists(par, s->nf, p->fluid_pos, offsetof(RCell, fluid_start_id), cells, fnext) ||
        initial_lists(par, s->ns, p->solid_pos, offsetof(RCell, solid_start_id), cells, snext) ||
        initial_lists(par, s->nv, p->virt_pos, offsetof(RCell, virt_start_id), cells, vnext))
        return 1;

    // particle arrays with addList's initial values
    RDataPointer &dp = s->data;
    memset(&dp, 0, sizeof(dp));
    const size_t nf = s->nf, ns = s->ns, nv = s->nv;
    std::vector<float> zeros3(3 * std::max(nf, std::max(ns, nv)), 0.0f), zeros1(std::max(nf, std::max(ns, nv)), 0.0f);
    std::vector<int> minus1(std::max(nf, std::max(ns, nv)), -1);
    std::vector<float> ident(9 * ns, 0.0f), rho0(nv, cfg->fluid_density);
    for (size_t i = 0; i < ns; ++i)
        ident[9 * i + 0] = ident[9 * i + 4] = ident[9 * i + 8] = 1.0f;
    if (alloc_copy(s, &dp.fluid.position, 3 * nf, p->fluid_pos) ||
        alloc_copy(s, &dp.fluid.velocity, 3 * nf, p->fluid_vel) ||
        alloc_copy(s, &dp.fluid.density, nf, p->fluid_rho) || alloc_copy(s, &dp.fluid.pressure, nf, p->fluid_p) ||
        alloc_copy(s, &dp.fluid.color, nf, zeros1.data()) || alloc_copy(s, &dp.fluid.cell_id, nf, minus1.data()) ||
        alloc_copy(s, &dp.fluid.next_id, nf, fnext.data()) ||
        alloc_copy(s, &dp.fluid.next_id_previous, nf, minus1.data()) ||
        alloc_copy(s, &dp.fluid.du_dt, 3 * nf, zeros3.data()) || alloc_copy(s, &dp.fluid.drho_dt, nf, zeros1.data()))
        return 1;
    if (alloc_copy(s, &dp.solid.position, 3 * ns, p->solid_pos) ||
        alloc_copy(s, &dp.solid.reference_position, 3 * ns, p->solid_ref_pos) ||
        alloc_copy(s, &dp.solid.velocity, 3 * ns, p->solid_vel) ||
        alloc_copy(s, &dp.solid.solid_type, ns, p->solid_type) ||
        alloc_copy(s, &dp.solid.pressure, ns, zeros1.data()) || alloc_copy(s, &dp.solid.cell_id, ns, minus1.data()) ||
        alloc_copy(s, &dp.solid.next_id, ns, snext.data()) ||
        alloc_copy(s, &dp.solid.next_id_previous, ns, minus1.data()) ||
        alloc_copy(s, &dp.solid.deformation, 9 * ns, ident.data()) ||
        alloc_copy<float>(s, &dp.solid.stress_1st_piola, 9 * ns, nullptr) ||
        alloc_copy(s, &dp.solid.correction, 9 * ns, ident.data()) ||
        alloc_copy(s, &dp.solid.du_dt, 3 * ns, zeros3.data()) ||
        alloc_copy(s, &dp.solid.couple_dudt, 3 * ns, zeros3.data()) ||
        alloc_copy(s, &dp.solid.normal, 3 * ns, zeros3.data()))
        return 1;
    if (ns) {
        RCHECK(cudaMemset(dp.solid.stress_1st_piola, 0, 9 * ns * sizeof(float)));
    }
    std::vector<int> vtype(nv, 0);
    if (p->virt_type)
        for (size_t i = 0; i < nv; ++i)
            vtype[i] = p->virt_type[i];
    if (alloc_copy(s, &dp.virt.position, 3 * nv, p->virt_pos) ||
        alloc_copy(s, &dp.virt.normal, 3 * nv, zeros3.data()) ||
        alloc_copy(s, &dp.virt.velocity, 3 * nv, zeros3.data()) ||
        alloc_copy(s, &dp.virt.pressure, nv, zeros1.data()) || alloc_copy(s, &dp.virt.density, nv, rho0.data()) ||
        alloc_copy(s, &dp.virt.virt_type, nv, vtype.data()) || alloc_copy(s, &dp.virt.cell_id, nv, minus1.data()) ||
        alloc_copy(s, &dp.virt.next_id, nv, vnext.data()) ||
        alloc_copy(s, &dp.virt.next_id_previous, nv, minus1.data()))
        return 1;
    if (alloc_copy(s, &dp.cell, cells.size(), cells.data()))
        return 1;

    // MemoryCopy::copyConstant
    void *sym = nullptr;
    size_t bytes = 0;
    RCHECK(cudaLibraryGetGlobal(&sym, &bytes, s->lib, "dev_par"));
    if (bytes != sizeof(RParameter))
        return fail("dev_par is " + std::to_string(bytes) + " bytes, the mirror " + std::to_string(sizeof(RParameter)));
    RCHECK(cudaMemcpy(sym, &par, sizeof(par), cudaMemcpyHostToDevice));
    RCHECK(cudaLibraryGetGlobal(&sym, &bytes, s->lib, "dev_data"));
    if (bytes != sizeof(RDataPointer))
        return fail("dev_data is " + std::to_string(bytes) + " bytes, the mirror " +
                    std::to_string(sizeof(RDataPointer)));
    RCHECK(cudaMemcpy(sym, &dp, sizeof(dp), cudaMemcpyHostToDevice));
    RCHECK(cudaDeviceSynchronize());
    return 0;
}

int ref_destroy(ref_sim *s)
{
    if (!s)
        return 0;
    cudaDeviceSynchronize();
    for (void *p : s->allocations)
        cudaFree(p);
    for (int e = 0; e < 2; ++e)
        if (s->ev[e])
            cudaEventDestroy(s->ev[e]);
    if (s->lib)
        cudaLibraryUnload(s->lib);
    delete s;
    return 0;
}

int ref_phase(ref_sim *s, int phase) { return run_phase(s, phase); }

int ref_step(ref_sim *s, int nsteps) { return run_steps(s, nsteps); }

// nsteps steps bracketed by CUDA events on the default stream; *ms = elapsed.
int ref_time_steps(ref_sim *s, int nsteps, float *ms)
{
    RCHECK(cudaDeviceSynchronize());
    RCHECK(cudaEventRecord(s->ev[0], 0));
    if (run_steps(s, nsteps))
        return 1;
    RCHECK(cudaEventRecord(s->ev[1], 0));
    RCHECK(cudaEventSynchronize(s->ev[1]));
    RCHECK(cudaEventElapsedTime(ms, s->ev[0], s->ev[1]));
    return 0;
}

// Field ids follow FSIM_* fields.  Floats for float fields (vec3 as 3 floats,
// mat3 as 9 floats ROW-major like the library's API), int32 for ids and
// types; input order (the reference never reorders particles).
int ref_get(ref_sim *s, int field, void *dst)
{
    struct F { int id; const void *src; int width; bool mat; };
    const RDataPointer &d = s->data;
    const F table[] = {
        {0, d.fluid.position, 3, false}, {1, d.fluid.velocity, 3, false}, {2, d.fluid.density, 1, false},
        {3, d.fluid.pressure, 1, false}, {4, d.fluid.drho_dt, 1, false}, {5, d.fluid.du_dt, 3, false},
        {6, d.fluid.cell_id, 1, false},
        {10, d.solid.position, 3, false}, {11, d.solid.velocity, 3, false}, {12, d.solid.reference_position, 3, false},
        {13, d.solid.solid_type, 1, false}, {14, d.solid.normal, 3, false}, {15, d.solid.pressure, 1, false},
        {16, d.solid.du_dt, 3, false}, {17, d.solid.couple_dudt, 3, false}, {18, d.solid.deformation, 9, true},
        {19, d.solid.stress_1st_piola, 9, true}, {20, d.solid.correction, 9, true}, {21, d.solid.cell_id, 1, false},
        {30, d.virt.position, 3, false}, {31, d.virt.normal, 3, false}, {32, d.virt.velocity, 3, false},
        {33, d.virt.pressure, 1, false}, {34, d.virt.density, 1, false}, {35, d.virt.cell_id, 1, false},
        {40, d.fluid.color, 1, false}};
    for (const F &f : table) {
        if (f.id != field)
            continue;
        size_t n = field < 10 || field == 40 ? s->nf : field < 30 ? s->ns : s->nv;
        size_t bytes = n * f.width * 4;
        if (n == 0)
            return 0;
        RCHECK(cudaDeviceSynchronize());
        if (!f.mat) {
            RCHECK(cudaMemcpy(dst, f.src, bytes, cudaMemcpyDeviceToHost));
            return 0;
        }
        std::vector<float> colmajor(n * 9);
        RCHECK(cudaMemcpy(colmajor.data(), f.src, bytes, cudaMemcpyDeviceToHost));
        float *o = static_cast<float *>(dst);
        for (size_t i = 0; i < n; ++i)
            for (int r = 0; r < 3; ++r)
                for (int c = 0; c < 3; ++c)
                    o[9 * i + 3 * r + c] = colmajor[9 * i + 3 * c + r];
        return 0;
    }
    return fail("unknown field");
}

// For every particle of a species (0 fluid, 1 solid, 2 virtual): the cell
// whose current linked list holds it, -1 if none, -2 if more than one or if a
// list is malformed.
int ref_list_cells(ref_sim *s, int species, int *out)
{
    int n = species == 0 ? s->nf : species == 1 ? s->ns : s->nv;
    if (n == 0)
        return 0;
    std::vector<RCell> cells(s->ncell);
    std::vector<int> next(n);
    const int *next_dev = species == 0 ? s->data.fluid.next_id : species == 1 ? s->data.solid.next_id
                                                                             : s->data.virt.next_id;
    RCHECK(cudaDeviceSynchronize());
    RCHECK(cudaMemcpy(cells.data(), s->data.cell, cells.size() * sizeof(RCell), cudaMemcpyDeviceToHost));
    RCHECK(cudaMemcpy(next.data(), next_dev, n * sizeof(int), cudaMemcpyDeviceToHost));
    for (int i = 0; i < n; ++i)
        out[i] = -1;
    for (int c = 0; c < s->ncell; ++c) {
        int id = species == 0 ? cells[c].fluid_start_id : species == 1 ? cells[c].solid_start_id
                                                                        : cells[c].virt_start_id;
        for (int guard = 0; id != -1 && guard <= n; ++guard) {
            if (id < 0 || id >= n)
                return fail("malformed list");
            out[id] = out[id] == -1 ? c : -2;
            id = next[id];
        }
    }
    return 0;
}

}  // extern "C"
