/*
 * oracle.h — CPU restatement of the FluidSim particle hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker the parity tests, smoke() and
 * the CPU-baseline leg of bench.py compare the CUDA path against; the product
 * never links, loads or calls it.
 *
 * Built twice from oracle.c: liboracle_f64.so (REAL = double, the FP64 oracle)
 * and liboracle_f32.so (REAL = float, the same formulas in single precision,
 * used for tight per-phase comparisons).  Both parallelise over particles with
 * OpenMP; each particle's sums run in a fixed order, so results are
 * deterministic for any thread count.
 *
 * Parity status: the parameter derivation (kernel constants, EOS and material
 * coefficients, cell grid) is pinned against the reference's own host sources
 * compiled here (oracle/_ref, see build_ref.sh).  The pair physics lives in
 * CUDA sources that need the unvendored glm library, so it is restated from
 * the reference formulas and is not pinned by any reference output.
 */
#ifndef FSIM_ORACLE_H
#define FSIM_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Same field as fsim_config in include/fluidsim.h (kept layout-identical so
 * tests can pass one ctypes structure to both). */
typedef struct orc_config {
    float gravity;
    int   is_viscid;
    float min_pressure, fluid_sound_speed, fluid_density, gamma, viscosity;
    float solid_density, youngs_modulus, poisson_ratio, arti_vis_alpha, arti_vis_beta;
    float xmin, ymin, zmin, xmax, ymax, zmax;
    float dt;
    int   istart, iend, solid_sub_step, result_interval, sort_every_step;
    float smoothing_length, particle_diameter, impact_length_hsml_ratio;
    int   thread_num;
    int   precision;
    int   keep_derivatives;
    int   solid_fused; /* device launch choice; no effect on the oracle */
    int   solid_full_walk; /* device launch choice; no effect on the oracle */
    int   barrier_wait_polls; /* device launch choice; no effect on the oracle */
    float neighbor_skin; /* device search choice; no effect on the oracle */
} orc_config;

typedef struct orc_derived {
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
} orc_derived;

typedef struct orc_sim orc_sim;

/* FP32 derivation of the constants (restates src/kernel.cpp:25-60,
 * src/properties.cpp:107-126, src/domain.cpp:28-47, src/physics.cpp:12-15). */
void orc_derive(const orc_config *cfg, orc_derived *out);

/* FP32 cell index of a position (src/pair.cu:8-24). */
int orc_cell_of(const orc_derived *d, float x, float y, float z);
void orc_cell_ids(const orc_derived *d, int n, const float *pos, int *out);

orc_sim *orc_create(const orc_config *cfg,
                    int nf, const float *fpos, const float *fvel, const float *frho, const float *fp,
                    int ns, const float *spos, const float *svel, const float *sref, const int *stype,
                    int nv, const float *vpos);
void orc_destroy(orc_sim *s);
/* phase ids match FSIM_PHASE_* */
void orc_phase(orc_sim *s, int phase);
void orc_step(orc_sim *s, int nsteps);
/* field ids match FSIM_* fields; out receives count*width doubles (ids as doubles) */
int  orc_get(orc_sim *s, int field, double *out);
/* field ids FLUID_POS/VEL/RHO/P and SOLID_POS/VEL; in holds count*width doubles */
int  orc_set(orc_sim *s, int field, const double *in);
/* 3 ints per fluid particle: in-range fluid, solid, virtual neighbours (FP32 distance test) */
void orc_neighbor_counts(orc_sim *s, int *out);
/* probe sampling: n points (3 doubles each) -> 5 doubles each (u, v, w, p, rho) */
void orc_probe(orc_sim *s, int n, const double *pts, double *out);
void orc_set_threads(int n);
int  orc_real_bytes(void);

#ifdef __cplusplus
}
#endif
#endif
