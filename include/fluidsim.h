/*
 * fluidsim.h — C ABI of the GB300-native FluidSim particle hot path.
 *
 * The reference (niji127/FluidSim) is one Windows executable with no library
 * API.  Its hot path sits behind two seams, and every entry point below names
 * the reference piece it replaces:
 *   - the process contract: config/input.ini + data/{fluid,solid,virt}_particle.dat
 *     in, out/{fluid,solid,virtual}/ *-k.vtk out
 *     (src/parameter.cpp:36-63, src/sim.cu:40-151, src/output.cu:299-335);
 *   - the static phase functions DeviceCalculation::{particleCellUpdate, fillCell,
 *     coupleCalculation, virtUpdate, fluidCalculation, solidCalculation}
 *     (include/calculation.cuh:9-21) driven by DeviceCalculation::calculation
 *     (src/calculation.cu:20-35).
 *
 * Conventions
 *   - Plain C types only: pointers, sizes, ints, floats.  No CUDA or torch types.
 *   - Every call returns an fsim_status; nothing calls exit(), abort() or __trap().
 *   - A handle owns its device state and one CUDA stream.  Handles are independent
 *     (no globals); one handle is not thread-safe, different handles may run on
 *     different host threads at once.
 *   - Vectors are 3 consecutive floats (x, y, z).  3x3 matrices are 9 floats in
 *     row-major order: element (r, c) at index 3*r + c.
 *   - Per-particle fields are read and written in the ORIGINAL input order (the
 *     order of the rows of the .dat files), although the device keeps particles
 *     sorted by cell.
 *   - The vertical axis is y and gravity points along -y (src/physics.cpp:12-15).
 */
#ifndef FLUIDSIM_H
#define FLUIDSIM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ status */
typedef int fsim_status;
enum {
    FSIM_OK = 0,
    FSIM_EINVAL = 1,    /* bad argument, bad config, malformed input file      */
    FSIM_ENOMEM = 2,    /* device or host allocation failed                    */
    FSIM_ECUDA = 3,     /* a CUDA runtime call failed                          */
    FSIM_ETIMEOUT = 4,  /* a bounded device-side wait gave up                  */
    FSIM_ENUMERIC = 5,  /* the device raised a numeric/out-of-grid flag        */
    FSIM_EIO = 6        /* file could not be opened, read or written           */
};

/* Human-readable name of a status code (static string, never NULL). */
const char *fsim_status_string(fsim_status s);
/* Last error message recorded on this host thread (static per thread). */
const char *fsim_last_error(void);

/* ------------------------------------------------------------------ config */
/* Precision forms (an extension; the reference is FP32 only).
 * FP32: the reference's arithmetic and storage (absolute FP32 positions,
 *   density and pressure), cell ids and pair sets bit-exact with it.
 * MIXED: FP32 arithmetic with fluid positions stored as an integer cell plus
 *   an FP32 offset inside it, density stored as delta = rho/rho0 - 1 with the
 *   pressure its Tait EOS, neighbour-gathered density/pressure packed as FP16
 *   deviations from per-cell FP32 references, a Kahan-compensated density
 *   rate, and the solid's kernel-correction inverse L^-1 in FP64.  Fields are
 *   read and written in the same units as the FP32 form; FSIM_FLUID_P is
 *   read-only (it follows from the density). */
enum { FSIM_PRECISION_FP32 = 0, FSIM_PRECISION_MIXED = 1 };

/* Every key the reference reads from input.ini, with the same meaning.
 * Replaces Physics/FluidProperties/SolidProperties/Domain/SimTime/Kernel::
 * readParameter (src/physics.cpp:9-19, src/properties.cpp:34-43,95-104,
 * src/domain.cpp:9-26, src/sim_time.cpp:8-24, src/kernel.cpp:9-23). */
typedef struct fsim_config {
    /* [physics] */
    float gravity;                  /* magnitude, applied along -y          */
    /* [fluid] */
    int   is_viscid;
    float min_pressure, fluid_sound_speed, fluid_density, gamma, viscosity;
    /* [solid] */
    float solid_density, youngs_modulus, poisson_ratio, arti_vis_alpha, arti_vis_beta;
    /* [domain] */
    float xmin, ymin, zmin, xmax, ymax, zmax;
    /* [time] */
    float dt;
    int   istart, iend, solid_sub_step, result_interval, sort_every_step;
    /* [kernel] */
    float smoothing_length, particle_diameter, impact_length_hsml_ratio;
    int   thread_num;
    /* extension keys (a [gb300] section the reference ignores) */
    int   precision;                /* FSIM_PRECISION_*                       */
    int   keep_derivatives;         /* 1: keep drho_dt/du_dt readable         */
    int   solid_fused;              /* 1: all solid sub-steps of a step in one
                                       persistent cooperative launch (else one
                                       launch per phase per sub-step)         */
    int   solid_full_walk;          /* 1: every solid sub-step walks the fluid
                                       of its 27 cells (else sub-steps after
                                       the first walk a per-lane list recorded
                                       by the first; same results bit for bit) */
    int   barrier_wait_polls;       /* grid barrier of the solid_fused kernel:
                                       give up (FSIM_ETIMEOUT) after this many
                                       polls of about 64 ns; 0 = the default
                                       2^22 (a quarter of a second and more).
                                       Small values exist to exercise the
                                       timeout path.                         */
    float neighbor_skin;            /* > 0: both forms advance the fluid
                                       with per-particle neighbour lists of
                                       radius R (1 + skin), R the impact
                                       distance, rebuilt when a particle has
                                       moved half the skin (default 0.15);
                                       0: a cell walk every step.  Same pair
                                       set either way.                       */
} fsim_config;

/* Derived constants, as Parameter::initiateParameter computes them in FP32
 * (src/parameter.cpp:25-34 -> src/kernel.cpp:43-60, src/properties.cpp:47-66,
 * src/domain.cpp:28-47). */
typedef struct fsim_derived {
    float smoothing_length_square, smoothing_length_inverse, smoothing_length_inverse_square;
    float impact_distance_square, particle_volume;
    float kernel_coefficient_1, kernel_coefficient_2, kernel_differential;
    float coefficient_p2rho, coefficient_rho2p, gamma_inv, reference_density_inverse;
    float min_density, max_density;
    float lambda, shear_modulus, bulk_modulus, solid_sound_speed;
    float gravity_vec[3];
    float cell_min[3], cell_max[3], interval[3], interval_inv[3];
    int   cell_number[3];
    int   cell_number_total;
} fsim_derived;

/* Fill *cfg with the reference defaults (keys absent from an INI file). */
fsim_status fsim_config_defaults(fsim_config *cfg);
/* Parse an input.ini file / text with the reference's Config semantics
 * (src/config.cpp:59-129: '#' comments, '[section]' lines ignored, values
 * continued on following key-less lines, the last duplicate key wins) and
 * apply the reference defaults.  Replaces Parameter::readFieldParameter
 * (src/parameter.cpp:36-52), including its validity checks. */
fsim_status fsim_config_from_ini(const char *path, fsim_config *cfg);
fsim_status fsim_config_from_ini_text(const char *text, fsim_config *cfg);
/* Replaces Parameter::initiateParameter (src/parameter.cpp:25-34). */
fsim_status fsim_derive(const fsim_config *cfg, fsim_derived *out);

/* -------------------------------------------------------------- particles */
/* Host particle arrays in input order.  Replaces the .dat row layouts of
 * Fluid/Solid/Virt_Host_List::addList (include/host_data.cuh:20-38,79-101,147-163). */
typedef struct fsim_particles {
    int n_fluid;
    const float *fluid_pos, *fluid_vel;     /* 3*n_fluid each                  */
    const float *fluid_rho, *fluid_p;       /* n_fluid each                    */
    int n_solid;
    const float *solid_pos, *solid_vel, *solid_ref_pos;  /* 3*n_solid each    */
    const int *solid_type;                  /* 0 UNCONSTRAINED, 1 FIXED        */
    int n_virt;
    const float *virt_pos;                  /* 3*n_virt                        */
    const int *virt_type;                   /* 0 FIXED, 1 MOVING (unused)      */
} fsim_particles;

/* Host-owned particle set read from .dat files. */
typedef struct fsim_particle_set *fsim_particle_set_t;
/* Read data_dir/{fluid,solid,virt}_particle.dat.  Replaces
 * {Fluid,Solid,Virtual}Properties::readNumber (src/properties.cpp:7-32,68-93,
 * 107-132: first line is N, then exactly N rows) and Sim::readParticleData
 * (src/sim.cu:40-151).  All three files must exist (a count of 0 is allowed);
 * a missing file, a count line that disagrees with the number of rows, or a
 * row that does not parse returns FSIM_EIO / FSIM_EINVAL. */
fsim_status fsim_particles_read(const char *data_dir, fsim_particle_set_t *out);
fsim_status fsim_particles_view(fsim_particle_set_t set, fsim_particles *view);
fsim_status fsim_particles_free(fsim_particle_set_t set);
/* Write the three .dat files (same row layouts; 9 significant digits). */
fsim_status fsim_particles_write(const char *data_dir, const fsim_particles *p);

/* Project case generator for the benchmark configurations: a closed tank on
 * the lattice (i + 0.5) * dx, a fluid block at the origin, an elastic block
 * (plate or cube) and virtual wall layers outside the domain; y vertical.
 * Follows the classification of cases/dam_break/particle_generate.cpp:50-91
 * (solid first, then wall, then fluid).  Hydrostatic start: p = rho0 g (H - y)
 * with H the block height, rho from the inverse Tait EOS (src/fluid.cu:7-14).
 * The config supplies rho0, c0, gamma and g. */
typedef struct fsim_case {
    float dx;                       /* lattice spacing                          */
    int   tank_n[3];                /* tank extents in lattice cells (x, y, z)  */
    int   fluid_n[3];               /* fluid block cells, lower corner at 0     */
    int   solid_lo[3];              /* solid block lower corner (lattice index) */
    int   solid_n[3];               /* solid block cells (0 = no solid)         */
    int   solid_fixed_layers;       /* solid continued below the floor, FIXED   */
    int   virt_layers;              /* wall layers of virtual particles         */
    int   hydrostatic;              /* 1: hydrostatic initial density/pressure  */
    float jitter;                   /* uniform +-jitter*dx on fluid/solid pos   */
    uint64_t seed;
} fsim_case;
fsim_status fsim_case_generate(const fsim_case *c, const fsim_config *cfg,
                               fsim_particle_set_t *out);
/* Particle counts of a case, without generating it. */
fsim_status fsim_case_counts(const fsim_case *c, int *n_fluid, int *n_solid, int *n_virt);

/* -------------------------------------------------------------- simulation */
typedef struct fsim_sim *fsim_handle;

/* Copy a particle set to the device and build the initial cell structure.
 * Replaces Sim::initiate (include/sim.cuh:33-43: createCell, fillCell,
 * copyData) + MemoryCopy::copyConstant (src/memory_copy.cu:8-12).
 * device < 0 keeps the current device.  Creation frees no device memory
 * (which would wait for the whole GPU): its temporaries go at the instance's
 * first step, phase or batch entry, or with the instance. */
fsim_status fsim_create(const fsim_config *cfg, const fsim_particles *p,
                        int device, fsim_handle *out);
/* The same case generated on the device straight into a new handle (no host
 * particle arrays): identical particles in identical order, bit for bit, as
 * fsim_case_generate + fsim_create.  For admitting many scenarios quickly
 * (host generation and copies would dominate their start-up).  No
 * counterpart in the reference (its generator is a separate host program). */
fsim_status fsim_create_case(const fsim_config *cfg, const fsim_case *c, int device, fsim_handle *out);
fsim_status fsim_destroy(fsim_handle h);

/* Advance nsteps fluid steps (each with solid_sub_step solid sub-steps);
 * enqueued on the handle's stream, returns without waiting.  Equals the loop
 * body of DeviceCalculation::calculation (src/calculation.cu:23-33) without
 * output, repeated nsteps times. */
fsim_status fsim_step(fsim_handle h, int nsteps);
/* Wait for the handle's stream; reports device-side error flags. */
fsim_status fsim_sync(fsim_handle h);

/* Phases, for parity tests.  One call runs one reference phase function. */
enum {
    FSIM_PHASE_CELL = 0,    /* particleCellUpdate + fillCell   src/pair.cu:53-70,195-207 */
    FSIM_PHASE_COUPLE = 1,  /* coupleCalculation               src/solid.cu:346-359      */
    FSIM_PHASE_VIRT = 2,    /* virtUpdate                      src/virt.cu:77-87         */
    FSIM_PHASE_FLUID = 3,   /* fluidCalculation                src/fluid.cu:271-284      */
    FSIM_PHASE_SOLID = 4    /* solidCalculation (all sub-steps) src/solid.cu:241-260     */
};
fsim_status fsim_run_phase(fsim_handle h, int phase);

/* Per-particle fields (input order). */
enum {
    FSIM_FLUID_POS = 0, FSIM_FLUID_VEL = 1, FSIM_FLUID_RHO = 2, FSIM_FLUID_P = 3,
    FSIM_FLUID_DRHO_DT = 4, FSIM_FLUID_DU_DT = 5, FSIM_FLUID_CELL_ID = 6,
    FSIM_SOLID_POS = 10, FSIM_SOLID_VEL = 11, FSIM_SOLID_REF_POS = 12,
    FSIM_SOLID_TYPE = 13, FSIM_SOLID_NORMAL = 14, FSIM_SOLID_P = 15,
    FSIM_SOLID_DU_DT = 16, FSIM_SOLID_COUPLE_DUDT = 17, FSIM_SOLID_F = 18,
    FSIM_SOLID_PK1 = 19, FSIM_SOLID_LINV = 20, FSIM_SOLID_CELL_ID = 21,
    FSIM_VIRT_POS = 30, FSIM_VIRT_NORMAL = 31, FSIM_VIRT_VEL = 32,
    FSIM_VIRT_P = 33, FSIM_VIRT_RHO = 34, FSIM_VIRT_CELL_ID = 35
};
/* Number of float/int components per particle of a field (1, 3 or 9); 0 if unknown. */
int fsim_field_width(int field);
/* Copy a field to host memory in input order; bytes must be exactly
 * count*width*4.  Cell ids are int32, everything else float32.  Replaces the
 * thrust device->host copies of Output::write* (src/output.cu:9-10 etc.). */
fsim_status fsim_get_field(fsim_handle h, int field, void *host_dst, size_t bytes);
/* Overwrite a state field from host memory (input order).  Settable:
 * FLUID_POS/VEL/RHO/P, SOLID_POS/VEL.  Used by the end-to-end benchmark
 * (host->device inputs per step) and by tests. */
fsim_status fsim_set_field(fsim_handle h, int field, const void *host_src, size_t bytes);
/* Several fields in one call (field ids, host pointers, byte counts; same
 * checks as fsim_get_field / fsim_set_field): the device-side (un)permutes
 * run on the handle's stream while the host copies run on a copy stream, with
 * one host synchronisation for all of them.  fsim_set_fields returns once the
 * host buffers have been read.  An extension for callers that move the whole
 * state every step. */
fsim_status fsim_get_fields(fsim_handle h, int n, const int *fields, void *const *dst, const size_t *bytes);
fsim_status fsim_set_fields(fsim_handle h, int n, const int *fields, const void *const *src, const size_t *bytes);

/* Neighbour search products.
 * counts: for every fluid particle (input order) the number of fluid, solid
 * and virtual particles within the impact distance among its 27 cells
 * (3*n_fluid ints), using the same FP32 distance test as the sweep (in the
 * mixed form, offsets shifted by whole cells, as its sweep tests them). */
fsim_status fsim_neighbor_counts(fsim_handle h, int *host_counts, size_t bytes);
/* Fluid neighbour lists (no counterpart in the reference, which walks its
 * cells every step; cfg.neighbor_skin): *enabled = 1 when the instance
 * advances its fluid with lists, *builds = list builds so far, *capacity =
 * entries a particle's list holds, *check = 1 when pairs also need
 * neighbouring cells (cell sides within FP32 rounding of the impact
 * distance, and always in the mixed form, whose pair vectors come from cell
 * differences).  Any pointer may be NULL. */
fsim_status fsim_list_stats(fsim_handle h, int *enabled, int *builds, int *capacity, int *check);
/* For every fluid particle (input order, 3 ints): the fluid, solid and
 * virtual entries of its neighbour list within the impact distance of the
 * current positions; equal to fsim_neighbor_counts while no list rebuild is
 * due (after FSIM_PHASE_CELL).  FSIM_EINVAL without lists. */
fsim_status fsim_list_counts(fsim_handle h, int *host_counts, size_t bytes);
/* Cell structure of one species (0 fluid, 1 solid, 2 virtual): cell_start
 * (cell_number_total+1 ints) and the input ids in cell order (n ints). */
fsim_status fsim_get_cells(fsim_handle h, int species, int *cell_start, size_t start_bytes,
                           int *ids_in_cell_order, size_t ids_bytes);

/* Write the reference's VTK files for the current state into out_dir
 * (out_dir/fluid, out_dir/solid, out_dir/virtual, created if absent), with
 * file index file_step.  Reproduces Output::outputData (src/output.cu:299-335)
 * byte for byte, including fluid_pressure-k.vtk carrying the always-zero
 * color field (src/output.cu:75); real fluid pressure goes to the extra file
 * fluid/fluid_true_pressure-k.vtk. */
fsim_status fsim_write_vtk(fsim_handle h, const char *out_dir, int file_step);
/* The same files with BINARY legacy-VTK encoding (big-endian FP32): exact
 * values and no text formatting, for fast snapshots of large instances.  No
 * counterpart in the reference (its writer is ASCII only). */
fsim_status fsim_write_vtk_binary(fsim_handle h, const char *out_dir, int file_step);

/* Device timing: run nsteps (CUDA-graph replays) on the handle's stream
 * bracketed by CUDA events recorded on that stream; *ms = elapsed device time. */
fsim_status fsim_time_steps(fsim_handle h, int nsteps, float *ms);
/* Instrumented timing: run nsteps as CUDA-graph replays of the step graph
 * with event nodes around the fluid sweep launch (launch by launch while the
 * sweep's launch shape is still being tuned); *total_ms = elapsed device time
 * of the nsteps, *sweep_ms = summed device time of the nsteps sweep launches. */
fsim_status fsim_time_sweep(fsim_handle h, int nsteps, float *total_ms, float *sweep_ms);
/* Per-phase device time: run nsteps launch by launch with CUDA events around
 * every launch; ms[p] = summed time of phase p (FSIM_PHASE_CELL .. SOLID) for
 * p < n (at most 5).  The reference prints only wall-clock times of its I/O. */
fsim_status fsim_time_phases(fsim_handle h, int nsteps, float *ms, int n);
/* Kernel launches one fsim_step(h, 1) issues (for launch accounting). */
fsim_status fsim_launches_per_step(fsim_handle h, int *n);

/* Launch-shape autotuner of the fluid sweep (no counterpart in the reference).
 * The sweep has FSIM_SWEEP_SHAPES launch shapes (warps per block / per-lane
 * neighbour-list capacity in shared memory: 0 = 4/48, 1 = 4/32, 2 = 8/32), all
 * giving bit-identical results.  The first FSIM_SWEEP_SHAPES steps of a handle
 * (or of a batch) run one shape each, launch by launch, with CUDA events around
 * the sweep; the fastest is then used for the CUDA graph of every later step.
 * *chosen = the chosen shape (-1 while tuning), ms[k] = the timed sweep of
 * shape k (0 if not yet timed), for k < n. */
#define FSIM_SWEEP_SHAPES 3
fsim_status fsim_sweep_tuning(fsim_handle h, int *chosen, float *ms, int n);

/* Conservation totals of the current state, accumulated in FP64 on the device
 * (per-particle terms in FP64, fixed-order block sums; deterministic).  No
 * counterpart in the reference.  Particle mass m = density * particle_volume
 * (rho0 for fluid, solid_density for solid); g = gravity vector.
 *   out[0] fluid mass            out[1] solid mass
 *   out[2..4] momentum sum m u (fluid + solid)
 *   out[5] kinetic energy sum m |u|^2 / 2 (fluid + solid)
 *   out[6] potential energy sum -m g.x (fluid + solid)
 *   out[7] fluid elastic energy: sum m * integral_rho0^rho p/rho'^2 drho' of
 *          the Tait EOS (pressure floor ignored)
 *   out[8] fluid density excess sum (rho - rho0) * particle_volume
 *   out[9] solid strain energy sum V (mu E:E + lambda/2 tr(E)^2), E the Green
 *          strain of the last solid phase's F (0 before the first one) */
#define FSIM_CONSERVATION_N 10
fsim_status fsim_conservation(fsim_handle h, double *out, int n_out);

/* Measurement utility (no counterpart in the reference): FP32 FMA throughput
 * of `device` in TFLOP/s (an FMA counts 2), from a kernel of independent FMA
 * chains at full residency timed with CUDA events (best of 3 launches). */
fsim_status fsim_measure_fp32_peak(int device, double *tflops);

/* -------------------------------------------------------------- batching */
/* A batch advances several independent instances (handles created with
 * fsim_create on the same device, of any sizes and parameters) in lockstep:
 * every kernel of a step is launched once for the whole batch, and a batched
 * step is one CUDA graph.  The reference runs one instance per process
 * (src/main.cu:17-30); this has no reference counterpart and exists for
 * ensembles of small and medium instances, whose one-by-one steps would
 * leave most of the GPU idle.  While a handle belongs to a batch it is stepped
 * only through the batch; its field getters and setters wait for the batch.
 * Each member's results equal its standalone results bit for bit. */
typedef struct fsim_batch *fsim_batch_t;
fsim_status fsim_batch_create(fsim_handle *members, int n, fsim_batch_t *out);
/* Enqueue nsteps batched steps on the batch's stream. */
fsim_status fsim_batch_step(fsim_batch_t b, int nsteps);
fsim_status fsim_batch_sync(fsim_batch_t b);
/* Wait for the batch and report every member's own status (FSIM_ENUMERIC for
 * a member whose particles left the cell grid, FSIM_OK otherwise), so that a
 * caller can evict only the failing instances; n = number of members. */
fsim_status fsim_batch_sync_members(fsim_batch_t b, int *status, int n);
/* Device time of nsteps batched steps (CUDA events on the batch's stream). */
fsim_status fsim_batch_time_steps(fsim_batch_t b, int nsteps, float *ms);
/* Kernel launches of one batched step. */
fsim_status fsim_batch_launches_per_step(fsim_batch_t b, int *n);
/* The batch's own sweep autotuner (see fsim_sweep_tuning). */
fsim_status fsim_batch_sweep_tuning(fsim_batch_t b, int *chosen, float *ms, int n);
/* Change the membership of a live batch: a standalone handle joins (same
 * device, precision form and solid launch form), or a member leaves and
 * continues standalone.  The batch's step plans are rebuilt at its next step;
 * its tuned sweep shape is kept.  A batch may become empty. */
fsim_status fsim_batch_add(fsim_batch_t b, fsim_handle h);
fsim_status fsim_batch_remove(fsim_batch_t b, fsim_handle h);
/* Dissolve the batch; the members continue as standalone handles. */
fsim_status fsim_batch_destroy(fsim_batch_t b);

/* Pinned (page-locked) host memory for fast host<->device field copies. */
fsim_status fsim_host_alloc(size_t bytes, void **out);
fsim_status fsim_host_free(void *p);

/* Allocation-free cell sort.  No counterpart in the reference.
 * For callers that cannot allocate device memory while they run (hosts that
 * reserve all GPU memory up front under their own allocator or budget, and
 * real-time loops that cannot take the device synchronisation of
 * cudaMalloc/cudaFree).  Sorts n positions (device memory, 3 floats each) into
 * the cell grid of *grid (from fsim_derive): d_cell_start receives
 * cell_number_total + 1 exclusive-scan offsets, d_ids the input indices in cell
 * order, ordered by input index inside a cell — the same result as the cell
 * phase of a handle.  Both outputs are caller-owned device memory; work is
 * enqueued on `stream` (a cudaStream_t, NULL for the default stream).
 * Scratch is one fixed device array inside the library (4 MiB, held by every
 * GPU that loads the library until the process exits): at most
 * FSIM_NOALLOC_MAX_PARTICLES positions and FSIM_NOALLOC_MAX_CELLS cells, else
 * FSIM_EINVAL.  Positions outside the grid are clamped into its boundary cells
 * (NaN coordinates into the first cell of their axis).  Inside a cell of more
 * than FSIM_NOALLOC_RANK_MAX particles (only such clamped positions, or a
 * smoothing length of several particle spacings, produce one) the order is
 * unspecified: ordering by input index costs the cell's count per particle,
 * and the sort keeps its work bounded instead.  Every call looks up the
 * array's device address on the current device; the first call on a device
 * loads it there, so make that call before any stream capture.  All calls
 * share the array: calls that overlap on the GPU race, so order them. */
#define FSIM_NOALLOC_MAX_PARTICLES 262144
#define FSIM_NOALLOC_MAX_CELLS 262144
#define FSIM_NOALLOC_RANK_MAX 1024
fsim_status fsim_cell_sort_noalloc(const fsim_derived *grid, const float *d_pos, int n,
                                   int *d_cell_start, int *d_ids, void *stream);

/* Device memory an instance of this configuration and these particle
 * counts allocates (an upper estimate, for admission control). */
fsim_status fsim_estimate_bytes(const fsim_config *cfg, int n_fluid, int n_solid, int n_virt, size_t *out);
/* Device memory the instance's own arrays hold now (state, cell structures,
 * neighbour lists, solid lists, staging); step plans, their graphs and the
 * buffers of fsim_get_fields / fsim_set_fields are not counted.  The measure
 * fsim_estimate_bytes bounds.  No counterpart in the reference. */
fsim_status fsim_device_bytes(fsim_handle h, size_t *bytes);

/* Point probes.  Replaces Probe::getData (src/probe.cu and include/probe.h:8-35
 * of the reference, a 2D helper left commented out there), in 3D: at each of
 * n points (3 floats each, host memory) the Shepard average, with the weight
 * (exp(-r^2/h^2) - c1) c2 of solidPressureCalculate, of fluid velocity,
 * pressure and density and of solid velocity and pressure (solid density 0)
 * over the particles within the impact distance in the 27 cells of the point's
 * cell (cell lists of the last cell phase, current positions).  out receives 5
 * floats per point: u, v, w, p, rho; (0, 0, 0, 0, rho0) where no particle is
 * in range or the point is outside the grid. */
fsim_status fsim_probe(fsim_handle h, const float *points, int n, float *out);

/* Binary snapshots (checkpoint / resume; no counterpart in the reference,
 * whose only restartable state is its .dat input).  A snapshot holds the
 * configuration, a caller-chosen step number and the particle state in its
 * current cell-sorted order, so that an instance restored from it continues
 * bit for bit like the original.  Per-step products (cell starts, solid
 * stress, derivatives) are recomputed by the next step.  The format is this
 * library's own: fixed header ("FSIMSNP1", version 1, counts, fsim_config),
 * then raw device arrays, native byte order. */
fsim_status fsim_snapshot_bytes(fsim_handle h, size_t *bytes);
fsim_status fsim_snapshot_save(fsim_handle h, long long step, void *buf, size_t bytes);
fsim_status fsim_snapshot_load(const void *buf, size_t bytes, int device, fsim_handle *out, long long *step);
fsim_status fsim_snapshot_write(fsim_handle h, long long step, const char *path);
fsim_status fsim_snapshot_read(const char *path, int device, fsim_handle *out, long long *step);

/* Sizes of the instance. */
fsim_status fsim_counts(fsim_handle h, int *n_fluid, int *n_solid, int *n_virt);
fsim_status fsim_get_derived(fsim_handle h, fsim_derived *out);

#ifdef __cplusplus
}
#endif
#endif /* FLUIDSIM_H */
