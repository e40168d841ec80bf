/*
 * oracle.c — CPU restatement of the FluidSim particle hot path.
 *
 * TEST INFRASTRUCTURE ONLY (see oracle.h).  Compiled with REAL = double (the
 * FP64 oracle) or, with -DORACLE_F32, REAL = float.  Always compiled with
 * -ffp-contract=off so that the FP32 helpers below round exactly as written.
 *
 * Parity: partially pinned.  The configuration parsing, derived constants and
 * cell grid are pinned against the reference's own host sources compiled here
 * (oracle/build.py -> oracle/_ref, fixtures in tests/golden).  The pair
 * physics of src/fluid.cu, src/virt.cu and src/solid.cu needs the glm library,
 * which the reference neither vendors nor pins, so that part is restated from
 * the formulas and is unpinned.
 *
 * Every function cites the reference code it restates (paths within
 * niji127/FluidSim).  Differences from the reference that are deliberate:
 *   - Cell lists are rebuilt from scratch every step (counting sort, ascending
 *     input id inside a cell).  The reference rebuilds its linked lists
 *     incrementally from the 27 neighbour cells' previous lists
 *     (src/pair.cu:72-193), which loses a particle that moves more than one
 *     cell in one step; with a CFL-stable dt no particle does, and then both
 *     give the same membership sets.
 *   - The virtual particle's nearest fluid particle is the one with the
 *     smallest distance, ties broken by the smaller input id.  The reference
 *     keeps the first one met in its list order (src/virt.cu:42), which is not
 *     a fixed order; on the benchmark lattices the nearest one is unique.
 *   - det(F) * inverse(F)^T in the artificial viscosity (src/solid.cu:155-156)
 *     is computed as the cofactor matrix of F: the same value where F is
 *     invertible, and finite where it is not.
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifdef ORACLE_F32
typedef float real;
#define R_EXP expf
#define R_SQRT sqrtf
#define R_POW powf
#define R_FMAX fmaxf
#define R_FMIN fminf
#else
typedef double real;
#define R_EXP exp
#define R_SQRT sqrt
#define R_POW pow
#define R_FMAX fmax
#define R_FMIN fmin
#endif

#define PI_F 3.141593f          /* include/global.h:4   */
#define EPS_FOR_SUM_F 0.1f      /* include/global.h:6   */
#define EPS_FLOAT_F 1.0e-6f     /* include/global.h:7   */
#define LARGE_FLOAT_F 1.0e6f    /* include/global.h:8   */
#define VIRT_LAYER_N 8          /* include/global.h:10  */

/* field ids (same numbering as include/fluidsim.h) */
enum {
    F_POS = 0, F_VEL = 1, F_RHO = 2, F_P = 3, F_DRHO = 4, F_DUDT = 5, F_CELL = 6,
    S_POS = 10, S_VEL = 11, S_REF = 12, S_TYPE = 13, S_NORMAL = 14, S_P = 15,
    S_DUDT = 16, S_COUPLE = 17, S_F = 18, S_PK1 = 19, S_LINV = 20, S_CELL = 21,
    V_POS = 30, V_NORMAL = 31, V_VEL = 32, V_P = 33, V_RHO = 34, V_CELL = 35
};
enum { PH_CELL = 0, PH_COUPLE = 1, PH_VIRT = 2, PH_FLUID = 3, PH_SOLID = 4 };

typedef struct { real x, y, z; } v3;
typedef struct { real m[3][3]; } m3; /* row-major m[r][c] */

static inline v3 v3make(real x, real y, real z) { v3 r = {x, y, z}; return r; }
static inline v3 vadd(v3 a, v3 b) { return v3make(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 vsub(v3 a, v3 b) { return v3make(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 vscale(v3 a, real s) { return v3make(a.x * s, a.y * s, a.z * s); }
static inline real vdot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline v3 vnormalize(v3 a) { return vscale(a, (real)1 / R_SQRT(vdot(a, a))); }

static inline m3 mzero(void) { m3 r; memset(&r, 0, sizeof r); return r; }
static inline m3 meye(void) { m3 r = mzero(); r.m[0][0] = r.m[1][1] = r.m[2][2] = 1; return r; }
static inline m3 mmul(m3 a, m3 b)
{
    m3 r;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            r.m[i][j] = a.m[i][0] * b.m[0][j] + a.m[i][1] * b.m[1][j] + a.m[i][2] * b.m[2][j];
    return r;
}
static inline v3 mvec(m3 a, v3 v)
{
    return v3make(a.m[0][0] * v.x + a.m[0][1] * v.y + a.m[0][2] * v.z,
                  a.m[1][0] * v.x + a.m[1][1] * v.y + a.m[1][2] * v.z,
                  a.m[2][0] * v.x + a.m[2][1] * v.y + a.m[2][2] * v.z);
}
static inline real mdet(m3 a)
{
    return a.m[0][0] * (a.m[1][1] * a.m[2][2] - a.m[1][2] * a.m[2][1])
         - a.m[0][1] * (a.m[1][0] * a.m[2][2] - a.m[1][2] * a.m[2][0])
         + a.m[0][2] * (a.m[1][0] * a.m[2][1] - a.m[1][1] * a.m[2][0]);
}
/* cofactor matrix: cof(A) = det(A) * A^{-T} */
static inline m3 mcof(m3 a)
{
    m3 c;
    c.m[0][0] = a.m[1][1] * a.m[2][2] - a.m[1][2] * a.m[2][1];
    c.m[0][1] = a.m[1][2] * a.m[2][0] - a.m[1][0] * a.m[2][2];
    c.m[0][2] = a.m[1][0] * a.m[2][1] - a.m[1][1] * a.m[2][0];
    c.m[1][0] = a.m[0][2] * a.m[2][1] - a.m[0][1] * a.m[2][2];
    c.m[1][1] = a.m[0][0] * a.m[2][2] - a.m[0][2] * a.m[2][0];
    c.m[1][2] = a.m[0][1] * a.m[2][0] - a.m[0][0] * a.m[2][1];
    c.m[2][0] = a.m[0][1] * a.m[1][2] - a.m[0][2] * a.m[1][1];
    c.m[2][1] = a.m[0][2] * a.m[1][0] - a.m[0][0] * a.m[1][2];
    c.m[2][2] = a.m[0][0] * a.m[1][1] - a.m[0][1] * a.m[1][0];
    return c;
}
static inline m3 minverse(m3 a, real det)
{
    m3 c = mcof(a), r;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) r.m[i][j] = c.m[j][i] / det;
    return r;
}

/* ------------------------------------------------------------ derivation */

/* Kernel::calculateCoeff (src/kernel.cpp:25-41): FP32 left Riemann sum of
 * 4*pi*int_0^K x^2 exp(-x^2) dx, minus the shift term, inverted. */
static float kernel_coeff(float K, float kc1)
{
    const int n = 10000;
    const float step = K / (float)n;
    float acc = 0.0f;
    for (int i = 0; i < n; i++) {
        const float x = (float)i * step;
        const float x2 = x * x;
        acc += x2 * expf(-x2) * step;
    }
    acc = acc * (4.0f * PI_F);
    acc -= kc1 * 4.0f / 3.0f * PI_F * powf(K, 3.0f);
    return 1.0f / acc;
}

void orc_derive(const orc_config *c, orc_derived *d)
{
    memset(d, 0, sizeof *d);
    const float h = c->smoothing_length, dp = c->particle_diameter, K = c->impact_length_hsml_ratio;
    /* Kernel::initiate, src/kernel.cpp:43-60 */
    d->particle_volume = powf(dp, 3.0f);
    d->smoothing_length_square = powf(h, 2.0f);
    d->smoothing_length_inverse = 1.0f / h;
    d->smoothing_length_inverse_square = powf(d->smoothing_length_inverse, 2.0f);
    d->impact_distance_square = powf(K, 2.0f) * powf(h, 2.0f);
    const float ratio = h / dp;
    d->kernel_coefficient_1 = expf(-powf(K, 2.0f));
    const float coef = kernel_coeff(K, d->kernel_coefficient_1);
    d->kernel_coefficient_2 = coef * powf(ratio, -3.0f);
    d->kernel_differential = 2.0f * coef * powf(ratio, -3.0f) * powf(h, -2.0f);
    /* FluidProperties::initiate, src/properties.cpp:47-57 */
    d->coefficient_p2rho = c->gamma * powf(c->fluid_sound_speed, -2.0f) / c->fluid_density;
    d->coefficient_rho2p = 1.0f / d->coefficient_p2rho;
    d->gamma_inv = 1.0f / c->gamma;
    d->reference_density_inverse = 1.0f / c->fluid_density;
    d->min_density = (1.0f - 0.1f) * c->fluid_density;
    d->max_density = (1.0f + 0.1f) * c->fluid_density;
    /* SolidProperties::initiate, src/properties.cpp:59-66 */
    const float E = c->youngs_modulus, nu = c->poisson_ratio;
    d->lambda = E * nu / (1.0f - 2.0f * nu) / (1.0f + nu);
    d->shear_modulus = E / (1.0f + nu) / 2.0f;
    d->bulk_modulus = E / (3.0f * (1.0f - 2.0f * nu));
    d->solid_sound_speed = sqrtf(d->bulk_modulus / c->solid_density);
    /* Physics::readParameter, src/physics.cpp:12-15 */
    d->gravity_vec[0] = 0.0f;
    d->gravity_vec[1] = -c->gravity;
    d->gravity_vec[2] = 0.0f;
    /* Domain::initiate, src/domain.cpp:28-47 */
    const float lo[3] = {c->xmin, c->ymin, c->zmin}, hi[3] = {c->xmax, c->ymax, c->zmax};
    const float thick = (float)VIRT_LAYER_N * dp;
    const float cell_size = K * h;
    for (int i = 0; i < 3; i++) {
        d->cell_min[i] = lo[i] - thick;
        d->cell_max[i] = hi[i] + thick;
        d->cell_number[i] = (int)((d->cell_max[i] - d->cell_min[i]) / cell_size);
        d->interval[i] = (d->cell_max[i] - d->cell_min[i]) / (float)d->cell_number[i];
        d->interval_inv[i] = 1.0f / d->interval[i];
    }
    d->cell_number_total = d->cell_number[0] * d->cell_number[1] * d->cell_number[2];
}

/* findPositionCell, src/pair.cu:8-24: per-axis truncation of the FP32
 * (x - min) * inv, linearised x-major. */
int orc_cell_of(const orc_derived *d, float x, float y, float z)
{
    const int nx = (int)((x - d->cell_min[0]) * d->interval_inv[0]);
    const int ny = (int)((y - d->cell_min[1]) * d->interval_inv[1]);
    const int nz = (int)((z - d->cell_min[2]) * d->interval_inv[2]);
    return nx * d->cell_number[1] * d->cell_number[2] + ny * d->cell_number[2] + nz;
}

/* Bulk form of orc_cell_of for n positions (3 floats each). */
void orc_cell_ids(const orc_derived *d, int n, const float *pos, int *out)
{
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; i++) out[i] = orc_cell_of(d, pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
}

/* FP32 squared distance exactly as the CUDA sweep evaluates it. */
static inline float dist2_f32(float xi, float yi, float zi, float xj, float yj, float zj)
{
    const float dx = xj - xi, dy = yj - yi, dz = zj - zi;
    return fmaf(dz, dz, fmaf(dy, dy, dx * dx));
}

/* ----------------------------------------------------------------- state */
typedef struct {
    int n;
    int *cell;      /* per particle */
    int *start;     /* ncell + 1 */
    int *list;      /* ids in cell order */
} cells_t;

struct orc_sim {
    orc_config cfg;
    orc_derived d;
    int nf, ns, nv;
    /* fluid */
    v3 *fpos, *fvel, *fdudt;
    real *frho, *fp, *fdrho;
    /* solid */
    v3 *spos, *svel, *sref, *snormal, *sdudt, *scouple;
    int *stype;
    real *sp;
    m3 *sF, *sP, *sL;
    /* virtual */
    v3 *vpos, *vnormal, *vvel;
    real *vp, *vrho;
    cells_t cf, cs, cv;
    /* constants promoted to REAL */
    real R2, h_inv2, kdiff, kc1, kc2, h, eps_h2, c0, mu_f, rho0, min_p, min_rho, max_rho;
    real coef_rho2p, rho0_inv, gam, rho_s, lam, mu_s, cs_s, alpha, beta, dt;
    v3 g;
    real dmin[3], dmax[3];
};

static void *xcalloc(size_t n, size_t sz) { return calloc(n ? n : 1, sz); }

void orc_set_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

int orc_real_bytes(void) { return (int)sizeof(real); }

static int cell_of_v3(const orc_derived *d, v3 p)
{
    return orc_cell_of(d, (float)p.x, (float)p.y, (float)p.z);
}

/* particleCellUpdate + fillCell (src/pair.cu:26-70, 72-207): full rebuild. */
static void build_cells(const orc_derived *d, cells_t *c, int n, const v3 *pos)
{
    const int nc = d->cell_number_total;
    c->n = n;
    for (int i = 0; i < n; i++) {
        int id = cell_of_v3(d, pos[i]);
        if (id < 0 || id >= nc) id = id < 0 ? 0 : nc - 1; /* out of grid: clamp (never on the benchmark cases) */
        c->cell[i] = id;
    }
    memset(c->start, 0, sizeof(int) * (size_t)(nc + 1));
    for (int i = 0; i < n; i++) c->start[c->cell[i] + 1]++;
    for (int k = 0; k < nc; k++) c->start[k + 1] += c->start[k];
    int *fill = (int *)xcalloc((size_t)nc, sizeof(int));
    for (int i = 0; i < n; i++) {
        const int k = c->cell[i];
        c->list[c->start[k] + fill[k]++] = i;
    }
    free(fill);
}

/* The 27 neighbour cells (src/sim.cu:153-236 builds the same set, -1 at grid
 * edges); here enumerated x-major. Returns count. */
static int neighbor_cells(const orc_derived *d, int cell, int out[27])
{
    const int Ny = d->cell_number[1], Nz = d->cell_number[2], Nx = d->cell_number[0];
    const int cx = cell / (Ny * Nz), cy = (cell / Nz) % Ny, cz = cell % Nz;
    int k = 0;
    for (int ox = -1; ox <= 1; ox++) {
        const int x = cx + ox;
        if (x < 0 || x >= Nx) continue;
        for (int oy = -1; oy <= 1; oy++) {
            const int y = cy + oy;
            if (y < 0 || y >= Ny) continue;
            for (int oz = -1; oz <= 1; oz++) {
                const int z = cz + oz;
                if (z < 0 || z >= Nz) continue;
                out[k++] = (x * Ny + y) * Nz + z;
            }
        }
    }
    return k;
}

static real dist2(v3 a, v3 b)
{
#ifdef ORACLE_F32
    return dist2_f32(a.x, a.y, a.z, b.x, b.y, b.z);
#else
    v3 t = vsub(b, a);
    return vdot(t, t);
#endif
}

orc_sim *orc_create(const orc_config *cfg,
                    int nf, const float *fpos, const float *fvel, const float *frho, const float *fp,
                    int ns, const float *spos, const float *svel, const float *sref, const int *stype,
                    int nv, const float *vpos)
{
    orc_sim *s = (orc_sim *)calloc(1, sizeof(orc_sim));
    s->cfg = *cfg;
    orc_derive(cfg, &s->d);
    s->nf = nf; s->ns = ns; s->nv = nv;
    const int nc = s->d.cell_number_total;
    s->fpos = xcalloc(nf, sizeof(v3)); s->fvel = xcalloc(nf, sizeof(v3)); s->fdudt = xcalloc(nf, sizeof(v3));
    s->frho = xcalloc(nf, sizeof(real)); s->fp = xcalloc(nf, sizeof(real)); s->fdrho = xcalloc(nf, sizeof(real));
    for (int i = 0; i < nf; i++) {
        s->fpos[i] = v3make(fpos[3 * i], fpos[3 * i + 1], fpos[3 * i + 2]);
        s->fvel[i] = v3make(fvel[3 * i], fvel[3 * i + 1], fvel[3 * i + 2]);
        s->frho[i] = frho[i];
        s->fp[i] = fp[i];
    }
    s->spos = xcalloc(ns, sizeof(v3)); s->svel = xcalloc(ns, sizeof(v3)); s->sref = xcalloc(ns, sizeof(v3));
    s->snormal = xcalloc(ns, sizeof(v3)); s->sdudt = xcalloc(ns, sizeof(v3)); s->scouple = xcalloc(ns, sizeof(v3));
    s->stype = xcalloc(ns, sizeof(int)); s->sp = xcalloc(ns, sizeof(real));
    s->sF = xcalloc(ns, sizeof(m3)); s->sP = xcalloc(ns, sizeof(m3)); s->sL = xcalloc(ns, sizeof(m3));
    for (int i = 0; i < ns; i++) {
        s->spos[i] = v3make(spos[3 * i], spos[3 * i + 1], spos[3 * i + 2]);
        s->svel[i] = v3make(svel[3 * i], svel[3 * i + 1], svel[3 * i + 2]);
        s->sref[i] = v3make(sref[3 * i], sref[3 * i + 1], sref[3 * i + 2]);
        s->stype[i] = stype[i];
        /* initial values of Solid_Host_List::addList (include/host_data.cuh:95-100) */
        s->sF[i] = meye(); s->sP[i] = mzero(); s->sL[i] = meye();
    }
    s->vpos = xcalloc(nv, sizeof(v3)); s->vnormal = xcalloc(nv, sizeof(v3)); s->vvel = xcalloc(nv, sizeof(v3));
    s->vp = xcalloc(nv, sizeof(real)); s->vrho = xcalloc(nv, sizeof(real));
    for (int i = 0; i < nv; i++) {
        s->vpos[i] = v3make(vpos[3 * i], vpos[3 * i + 1], vpos[3 * i + 2]);
        s->vrho[i] = cfg->fluid_density; /* include/host_data.cuh:158 */
    }
    cells_t *cl[3] = {&s->cf, &s->cs, &s->cv};
    int cn[3] = {nf, ns, nv};
    for (int k = 0; k < 3; k++) {
        cl[k]->cell = xcalloc(cn[k], sizeof(int));
        cl[k]->list = xcalloc(cn[k], sizeof(int));
        cl[k]->start = xcalloc((size_t)nc + 1, sizeof(int));
    }
    /* constants: FP32 products of the formula first, then promoted */
    const orc_derived *d = &s->d;
    s->R2 = d->impact_distance_square;
    s->h_inv2 = d->smoothing_length_inverse_square;
    s->kdiff = d->kernel_differential;
    s->kc1 = d->kernel_coefficient_1;
    s->kc2 = d->kernel_coefficient_2;
    s->h = cfg->smoothing_length;
    s->eps_h2 = 0.01f * d->smoothing_length_square;
    s->c0 = cfg->fluid_sound_speed;
    s->mu_f = cfg->viscosity;
    s->rho0 = cfg->fluid_density;
    s->min_p = cfg->min_pressure;
    s->min_rho = d->min_density;
    s->max_rho = d->max_density;
    s->coef_rho2p = d->coefficient_rho2p;
    s->rho0_inv = d->reference_density_inverse;
    s->gam = cfg->gamma;
    s->rho_s = cfg->solid_density;
    s->lam = d->lambda;
    s->mu_s = d->shear_modulus;
    s->cs_s = d->solid_sound_speed;
    s->alpha = cfg->arti_vis_alpha;
    s->beta = cfg->arti_vis_beta;
    s->dt = cfg->dt;
    s->g = v3make(d->gravity_vec[0], d->gravity_vec[1], d->gravity_vec[2]);
    s->dmin[0] = cfg->xmin; s->dmin[1] = cfg->ymin; s->dmin[2] = cfg->zmin;
    s->dmax[0] = cfg->xmax; s->dmax[1] = cfg->ymax; s->dmax[2] = cfg->zmax;
    return s;
}

void orc_destroy(orc_sim *s)
{
    if (!s) return;
    void *p[] = {s->fpos, s->fvel, s->fdudt, s->frho, s->fp, s->fdrho, s->spos, s->svel, s->sref,
                 s->snormal, s->sdudt, s->scouple, s->stype, s->sp, s->sF, s->sP, s->sL, s->vpos,
                 s->vnormal, s->vvel, s->vp, s->vrho, s->cf.cell, s->cf.list, s->cf.start,
                 s->cs.cell, s->cs.list, s->cs.start, s->cv.cell, s->cv.list, s->cv.start};
    for (size_t i = 0; i < sizeof p / sizeof p[0]; i++) free(p[i]);
    free(s);
}

/* ---------------------------------------------------------------- phases */

static void phase_cell(orc_sim *s)
{
    build_cells(&s->d, &s->cf, s->nf, s->fpos);
    build_cells(&s->d, &s->cs, s->ns, s->spos);
    build_cells(&s->d, &s->cv, s->nv, s->vpos);
}

/* densityToPressure, src/fluid.cu:16-24 (Tait EOS, floored) */
static inline real eos(const orc_sim *s, real rho)
{
    real p = (R_POW(rho * s->rho0_inv, s->gam) - 1) * s->coef_rho2p;
    return R_FMAX(p, s->min_p);
}

/* solidCoupleUpdate + solidNormalCalculate + solidPressureCalculate,
 * src/solid.cu:262-344 */
static void phase_couple(orc_sim *s)
{
    if (s->nf == 0 || s->ns == 0) return;
    const real eps_sum = EPS_FOR_SUM_F, eps_f = EPS_FLOAT_F;
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < s->ns; i++) {
        int nb[27];
        const int nn = neighbor_cells(&s->d, s->cs.cell[i], nb);
        v3 normal = v3make(0, 0, 0);
        real pres = 0, wsum = 0;
        const v3 xi = s->spos[i];
        for (int c = 0; c < nn; c++) {
            for (int k = s->cf.start[nb[c]]; k < s->cf.start[nb[c] + 1]; k++) {
                const int j = s->cf.list[k];
                if (dist2(xi, s->fpos[j]) < s->R2) {
                    const v3 dx = vsub(s->fpos[j], xi);
                    const real q2 = vdot(dx, dx) * s->h_inv2;
                    const real w = (R_EXP(-q2) - s->kc1) * s->kc2;
                    wsum += w;
                    pres += s->fp[j] * w;
                }
            }
            for (int k = s->cs.start[nb[c]]; k < s->cs.start[nb[c] + 1]; k++) {
                const int j = s->cs.list[k];
                if (dist2(xi, s->spos[j]) < s->R2) {
                    const v3 dx = vsub(s->spos[j], xi);
                    const real q2 = vdot(dx, dx) * s->h_inv2;
                    const real kc = R_EXP(-q2) * s->kdiff;
                    normal = vsub(normal, vscale(dx, kc));
                }
            }
        }
        s->snormal[i] = vdot(normal, normal) < eps_sum ? v3make(0, 0, 0) : vnormalize(normal);
        s->sp[i] = wsum > eps_f ? R_FMAX(pres / wsum, s->min_p) : 0;
    }
}

/* getVirtData, src/virt.cu:9-75 */
static void phase_virt(orc_sim *s)
{
    if (s->nv == 0) return;
    const real eps_sum = EPS_FOR_SUM_F;
#pragma omp parallel for schedule(dynamic, 256)
    for (int i = 0; i < s->nv; i++) {
        int nb[27];
        const int nn = neighbor_cells(&s->d, s->cv.cell[i], nb);
        v3 vel = v3make(0, 0, 0), normal = v3make(0, 0, 0);
        real pres = 0, rho = s->rho0, best = LARGE_FLOAT_F;
        int best_id = -1;
        const v3 xi = s->vpos[i];
        for (int c = 0; c < nn; c++) {
            for (int k = s->cf.start[nb[c]]; k < s->cf.start[nb[c] + 1]; k++) {
                const int j = s->cf.list[k];
                const real d2 = dist2(xi, s->fpos[j]);
                if (d2 < best || (d2 == best && best_id >= 0 && j < best_id)) {
                    const v3 dx = vsub(s->fpos[j], xi);
                    rho = s->frho[j];
                    pres = s->fp[j] - rho * vdot(s->g, dx);
                    vel = s->fvel[j];
                    best = d2;
                    best_id = j;
                }
            }
            for (int k = s->cv.start[nb[c]]; k < s->cv.start[nb[c] + 1]; k++) {
                const int j = s->cv.list[k];
                if (j == i) continue;
                const real d2 = dist2(xi, s->vpos[j]);
                if (d2 < s->R2) {
                    const v3 dx = vsub(s->vpos[j], xi);
                    const real kc = R_EXP(-vdot(dx, dx) * s->h_inv2) * s->kdiff;
                    normal = vsub(normal, vscale(dx, kc));
                }
            }
        }
        normal = vdot(normal, normal) < eps_sum ? v3make(0, 0, 0) : vnormalize(normal);
        s->vnormal[i] = normal;
        s->vp[i] = pres;
        s->vvel[i] = vsub(vel, vscale(normal, 2 * vdot(vel, normal)));
        s->vrho[i] = rho;
    }
}

/* Riemann pair term shared by fluid-fluid / fluid-solid / fluid-virtual:
 * fluidFluidCalculate, fluidSolidCalculate, fluidVirtCalculate
 * (src/fluid.cu:26-167).  limiter: use min(3du, c) (fluid, virtual) or c (solid).
 * clamp_ps: P* >= 0 (virtual). */
static inline void riemann_pair(const orc_sim *s, v3 xi, v3 xj, v3 ui, v3 uj, real rhoi, real rhoj,
                                real pi, real pj, int limiter, int clamp_ps, real *drho, v3 *dudt)
{
    const v3 dx = vsub(xj, xi);
    const real r2 = vdot(dx, dx);
    const real q2 = r2 * s->h_inv2;
    const real kc = R_EXP(-q2) * s->kdiff;
    const v3 e = q2 != 0 ? vnormalize(dx) : v3make(0, 0, 0);
    const real rs = rhoi + rhoj;
    real ps = (rhoi * pj + rhoj * pi) / rs;
    const real du = vdot(vsub(ui, uj), e);
    if (du >= 0) ps += rhoi * rhoj * du / rs * (limiter ? R_FMIN(3 * du, s->c0) : s->c0);
    if (clamp_ps) ps = R_FMAX(ps, 0);
    v3 vs = vscale(vadd(vscale(ui, rhoi), vscale(uj, rhoj)), 1 / rs);
    vs = vadd(vs, vscale(e, (pi - pj) / rs / s->c0));
    *dudt = vadd(*dudt, vscale(dx, -2 * ps / rhoi * kc));
    *drho += 2 * rhoi * vdot(vsub(ui, vs), dx) * kc;
    if (!s->cfg.is_viscid) return;
    real vis = vdot(vsub(uj, ui), dx);
    vis /= r2 + s->eps_h2;
    *dudt = vadd(*dudt, vscale(dx, 10 * s->mu_f * vis / rhoi * kc));
}

/* findFluidPair + fluidUpdate (src/fluid.cu:169-269) */
static void phase_fluid(orc_sim *s)
{
    if (s->nf == 0) return;
#pragma omp parallel for schedule(dynamic, 256)
    for (int i = 0; i < s->nf; i++) {
        int nb[27];
        const int nn = neighbor_cells(&s->d, s->cf.cell[i], nb);
        const v3 xi = s->fpos[i], ui = s->fvel[i];
        const real rhoi = s->frho[i], pi = s->fp[i];
        real drho = 0;
        v3 dudt = v3make(0, 0, 0);
        for (int c = 0; c < nn; c++) {
            for (int k = s->cf.start[nb[c]]; k < s->cf.start[nb[c] + 1]; k++) {
                const int j = s->cf.list[k];
                if (dist2(xi, s->fpos[j]) < s->R2)
                    riemann_pair(s, xi, s->fpos[j], ui, s->fvel[j], rhoi, s->frho[j], pi, s->fp[j],
                                 1, 0, &drho, &dudt);
            }
            for (int k = s->cs.start[nb[c]]; k < s->cs.start[nb[c] + 1]; k++) {
                const int j = s->cs.list[k];
                if (dist2(xi, s->spos[j]) < s->R2) {
                    const v3 n = s->snormal[j];
                    const v3 uj = vsub(ui, vscale(n, 2 * vdot(vsub(ui, s->svel[j]), n)));
                    riemann_pair(s, xi, s->spos[j], ui, uj, rhoi, rhoi, pi, s->sp[j], 0, 0, &drho, &dudt);
                }
            }
            for (int k = s->cv.start[nb[c]]; k < s->cv.start[nb[c] + 1]; k++) {
                const int j = s->cv.list[k];
                if (dist2(xi, s->vpos[j]) < s->R2)
                    riemann_pair(s, xi, s->vpos[j], ui, s->vvel[j], rhoi, s->vrho[j], pi, s->vp[j],
                                 1, 1, &drho, &dudt);
            }
        }
        s->fdrho[i] = drho;
        s->fdudt[i] = dudt;
    }
    /* fluidUpdate, src/fluid.cu:234-269 */
#pragma omp parallel for schedule(static)
    for (int i = 0; i < s->nf; i++) {
        if (!(s->fdrho[i] == s->fdrho[i])) s->fdrho[i] = 0;
        v3 a = s->fdudt[i];
        if (!(a.x == a.x && a.y == a.y && a.z == a.z)) s->fdudt[i] = a = v3make(0, 0, 0);
        v3 x = vadd(s->fpos[i], vscale(s->fvel[i], s->dt));
        v3 u = vadd(s->fvel[i], vscale(vadd(a, s->g), s->dt));
        real rho = s->frho[i] + s->fdrho[i] * s->dt;
        rho = R_FMIN(R_FMAX(rho, s->min_rho), s->max_rho);
        s->frho[i] = rho;
        s->fp[i] = eos(s, rho);
        x.x = R_FMIN(R_FMAX(x.x, s->dmin[0]), s->dmax[0]);
        x.y = R_FMIN(R_FMAX(x.y, s->dmin[1]), s->dmax[1]);
        x.z = R_FMIN(R_FMAX(x.z, s->dmin[2]), s->dmax[2]);
        const real speed = R_SQRT(vdot(u, u));
        const real vmax = (real)0.3f * s->c0;
        if (speed > vmax) u = vscale(u, vmax / speed);
        s->fpos[i] = x;
        s->fvel[i] = u;
    }
}

/* solidDeformationCalculate + solidSolidDeformation + solidStressCalculation
 * (src/solid.cu:10-79) */
static void solid_deformation(orc_sim *s)
{
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < s->ns; i++) {
        int nb[27];
        const int nn = neighbor_cells(&s->d, s->cs.cell[i], nb);
        m3 F = mzero(), L = mzero();
        const v3 Xi = s->sref[i], xi = s->spos[i];
        for (int c = 0; c < nn; c++) {
            for (int k = s->cs.start[nb[c]]; k < s->cs.start[nb[c] + 1]; k++) {
                const int j = s->cs.list[k];
                if (dist2(Xi, s->sref[j]) < s->R2) {
                    const v3 dX = vsub(s->sref[j], Xi);
                    const v3 dx = vsub(s->spos[j], xi);
                    const real kc = R_EXP(-vdot(dX, dX) * s->h_inv2) * s->kdiff;
                    const real a[3] = {dx.x, dx.y, dx.z}, b[3] = {dX.x, dX.y, dX.z};
                    for (int r = 0; r < 3; r++)
                        for (int q = 0; q < 3; q++) {
                            F.m[r][q] += a[r] * b[q] * kc;
                            L.m[r][q] += b[r] * b[q] * kc;
                        }
                }
            }
        }
        const real det = mdet(L);
        L = det != 0 ? minverse(L, det) : meye();
        F = mmul(F, L);
        /* Green strain, St-Venant-Kirchhoff 2nd Piola, 1st Piola P = F S */
        m3 Ft = F;
        for (int r = 0; r < 3; r++)
            for (int q = 0; q < 3; q++) Ft.m[r][q] = F.m[q][r];
        m3 E = mmul(Ft, F);
        for (int r = 0; r < 3; r++) {
            E.m[r][r] -= 1;
            for (int q = 0; q < 3; q++) E.m[r][q] *= (real)0.5;
        }
        const real tr = E.m[0][0] + E.m[1][1] + E.m[2][2];
        m3 S;
        for (int r = 0; r < 3; r++)
            for (int q = 0; q < 3; q++) S.m[r][q] = 2 * s->mu_s * E.m[r][q] + (r == q ? s->lam * tr : 0);
        s->sF[i] = F;
        s->sP[i] = mmul(F, S);
        s->sL[i] = L;
    }
}

/* solidForceCalculate + solidSolidForce + solidFluidCouple (src/solid.cu:81-207) */
static void solid_force(orc_sim *s)
{
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < s->ns; i++) {
        int nb[27];
        const int nn = neighbor_cells(&s->d, s->cs.cell[i], nb);
        v3 couple = v3make(0, 0, 0), dudt = v3make(0, 0, 0);
        const v3 xi = s->spos[i], Xi = s->sref[i], vi = s->svel[i], ni = s->snormal[i];
        const m3 PLi = mmul(s->sP[i], s->sL[i]);
        const m3 AVi = mmul(mcof(s->sF[i]), s->sL[i]);
        for (int c = 0; c < nn; c++) {
            for (int k = s->cf.start[nb[c]]; k < s->cf.start[nb[c] + 1]; k++) {
                const int j = s->cf.list[k];
                if (dist2(xi, s->fpos[j]) < s->R2) {
                    const v3 uj = s->fvel[j];
                    const v3 ui = vsub(uj, vscale(ni, 2 * vdot(vsub(uj, vi), ni)));
                    const v3 dx = vsub(s->fpos[j], xi);
                    const real kc = R_EXP(-vdot(dx, dx) * s->h_inv2) * s->kdiff;
                    const real pi = s->sp[i], pj = s->fp[j], rho = s->frho[j];
                    const real len = R_SQRT(vdot(dx, dx));
                    const v3 e = len != 0 ? vnormalize(dx) : v3make(0, 0, 0);
                    real ps = (rho * pj + rho * pi) / (rho + rho);
                    const real du = vdot(vsub(ui, uj), e);
                    if (du >= 0) ps += rho * rho * du / (rho + rho) * s->c0;
                    couple = vadd(couple, vscale(dx, -2 * ps / s->rho_s * kc));
                }
            }
            for (int k = s->cs.start[nb[c]]; k < s->cs.start[nb[c] + 1]; k++) {
                const int j = s->cs.list[k];
                if (dist2(Xi, s->sref[j]) < s->R2) {
                    const v3 dX = vsub(s->sref[j], Xi);
                    const real kc = R_EXP(-vdot(dX, dX) * s->h_inv2) * s->kdiff;
                    const m3 PLj = mmul(s->sP[j], s->sL[j]);
                    m3 sum;
                    for (int r = 0; r < 3; r++)
                        for (int q = 0; q < 3; q++) sum.m[r][q] = PLj.m[r][q] + PLi.m[r][q];
                    dudt = vadd(dudt, vscale(mvec(sum, dX), kc / s->rho_s));
                    const v3 dx = vsub(s->spos[j], xi);
                    const v3 dv = vsub(s->svel[j], vi);
                    const real nu = s->h * vdot(dv, dx) / (vdot(dx, dx) + s->eps_h2);
                    const real visc = s->alpha * nu * s->cs_s - s->beta * nu * nu;
                    dudt = vadd(dudt, vscale(mvec(AVi, dX), visc * kc));
                }
            }
        }
        s->scouple[i] = couple;
        s->sdudt[i] = vadd(dudt, couple);
    }
}

/* solidUpdate (src/solid.cu:209-239) */
static void solid_update(orc_sim *s)
{
    const real dts = (real)(s->cfg.dt / (float)s->cfg.solid_sub_step);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < s->ns; i++) {
        if (s->stype[i] == 1) {
            s->svel[i] = v3make(0, 0, 0);
            s->sdudt[i] = v3make(0, 0, 0);
        } else if (s->stype[i] == 0) {
            v3 x = vadd(s->spos[i], vscale(s->svel[i], dts));
            s->svel[i] = vadd(s->svel[i], vscale(vadd(s->sdudt[i], s->g), dts));
            x.x = R_FMIN(R_FMAX(x.x, s->dmin[0]), s->dmax[0]);
            x.y = R_FMIN(R_FMAX(x.y, s->dmin[1]), s->dmax[1]);
            x.z = R_FMIN(R_FMAX(x.z, s->dmin[2]), s->dmax[2]);
            s->spos[i] = x;
        }
    }
}

/* solidCalculation (src/solid.cu:241-260) */
static void phase_solid(orc_sim *s)
{
    if (s->ns == 0) return;
    for (int k = 0; k < s->cfg.solid_sub_step; k++) {
        solid_deformation(s);
        solid_force(s);
        solid_update(s);
    }
}

void orc_phase(orc_sim *s, int phase)
{
    switch (phase) {
    case PH_CELL: phase_cell(s); break;
    case PH_COUPLE: phase_couple(s); break;
    case PH_VIRT: phase_virt(s); break;
    case PH_FLUID: phase_fluid(s); break;
    case PH_SOLID: phase_solid(s); break;
    default: break;
    }
}

/* DeviceCalculation::calculation loop body (src/calculation.cu:23-33) */
void orc_step(orc_sim *s, int nsteps)
{
    for (int k = 0; k < nsteps; k++) {
        phase_cell(s);
        phase_couple(s);
        phase_virt(s);
        phase_fluid(s);
        phase_solid(s);
    }
}

static void put_v3(double *o, const v3 *a, int n)
{
    for (int i = 0; i < n; i++) { o[3 * i] = a[i].x; o[3 * i + 1] = a[i].y; o[3 * i + 2] = a[i].z; }
}
static void put_r(double *o, const real *a, int n) { for (int i = 0; i < n; i++) o[i] = a[i]; }
static void put_i(double *o, const int *a, int n) { for (int i = 0; i < n; i++) o[i] = a[i]; }
static void put_m(double *o, const m3 *a, int n)
{
    for (int i = 0; i < n; i++)
        for (int r = 0; r < 3; r++)
            for (int q = 0; q < 3; q++) o[9 * i + 3 * r + q] = a[i].m[r][q];
}

int orc_get(orc_sim *s, int field, double *o)
{
    switch (field) {
    case F_POS: put_v3(o, s->fpos, s->nf); break;
    case F_VEL: put_v3(o, s->fvel, s->nf); break;
    case F_RHO: put_r(o, s->frho, s->nf); break;
    case F_P: put_r(o, s->fp, s->nf); break;
    case F_DRHO: put_r(o, s->fdrho, s->nf); break;
    case F_DUDT: put_v3(o, s->fdudt, s->nf); break;
    case F_CELL: put_i(o, s->cf.cell, s->nf); break;
    case S_POS: put_v3(o, s->spos, s->ns); break;
    case S_VEL: put_v3(o, s->svel, s->ns); break;
    case S_REF: put_v3(o, s->sref, s->ns); break;
    case S_TYPE: put_i(o, s->stype, s->ns); break;
    case S_NORMAL: put_v3(o, s->snormal, s->ns); break;
    case S_P: put_r(o, s->sp, s->ns); break;
    case S_DUDT: put_v3(o, s->sdudt, s->ns); break;
    case S_COUPLE: put_v3(o, s->scouple, s->ns); break;
    case S_F: put_m(o, s->sF, s->ns); break;
    case S_PK1: put_m(o, s->sP, s->ns); break;
    case S_LINV: put_m(o, s->sL, s->ns); break;
    case S_CELL: put_i(o, s->cs.cell, s->ns); break;
    case V_POS: put_v3(o, s->vpos, s->nv); break;
    case V_NORMAL: put_v3(o, s->vnormal, s->nv); break;
    case V_VEL: put_v3(o, s->vvel, s->nv); break;
    case V_P: put_r(o, s->vp, s->nv); break;
    case V_RHO: put_r(o, s->vrho, s->nv); break;
    case V_CELL: put_i(o, s->cv.cell, s->nv); break;
    default: return 1;
    }
    return 0;
}

int orc_set(orc_sim *s, int field, const double *in)
{
    switch (field) {
    case F_POS: for (int i = 0; i < s->nf; i++) s->fpos[i] = v3make(in[3 * i], in[3 * i + 1], in[3 * i + 2]); break;
    case F_VEL: for (int i = 0; i < s->nf; i++) s->fvel[i] = v3make(in[3 * i], in[3 * i + 1], in[3 * i + 2]); break;
    case F_RHO: for (int i = 0; i < s->nf; i++) s->frho[i] = in[i]; break;
    case F_P: for (int i = 0; i < s->nf; i++) s->fp[i] = in[i]; break;
    case S_POS: for (int i = 0; i < s->ns; i++) s->spos[i] = v3make(in[3 * i], in[3 * i + 1], in[3 * i + 2]); break;
    case S_VEL: for (int i = 0; i < s->ns; i++) s->svel[i] = v3make(in[3 * i], in[3 * i + 1], in[3 * i + 2]); break;
    default: return 1;
    }
    return 0;
}

/* In-range neighbour counts per fluid particle, FP32 distance test on the
 * FP32-rounded positions, over the 27 cells of the particle's current cell. */
void orc_neighbor_counts(orc_sim *s, int *out)
{
    const float R2 = s->d.impact_distance_square;
#pragma omp parallel for schedule(dynamic, 256)
    for (int i = 0; i < s->nf; i++) {
        int nb[27];
        const int nn = neighbor_cells(&s->d, s->cf.cell[i], nb);
        const float xi = (float)s->fpos[i].x, yi = (float)s->fpos[i].y, zi = (float)s->fpos[i].z;
        int cnt[3] = {0, 0, 0};
        const cells_t *cl[3] = {&s->cf, &s->cs, &s->cv};
        const v3 *ps[3] = {s->fpos, s->spos, s->vpos};
        for (int c = 0; c < nn; c++)
            for (int t = 0; t < 3; t++)
                for (int k = cl[t]->start[nb[c]]; k < cl[t]->start[nb[c] + 1]; k++) {
                    const v3 pj = ps[t][cl[t]->list[k]];
                    if (dist2_f32(xi, yi, zi, (float)pj.x, (float)pj.y, (float)pj.z) < R2) cnt[t]++;
                }
        out[3 * i] = cnt[0];
        out[3 * i + 1] = cnt[1];
        out[3 * i + 2] = cnt[2];
    }
}

/* Probe::getData (src/probe.cu, commented out in the reference, 2D), restated
 * in 3D: the Shepard average, with the weight (exp(-r^2/h^2) - c1) c2 of
 * solidPressureCalculate, of fluid velocity, pressure and density and of
 * solid velocity and pressure (solid density counts 0) over the particles
 * within the impact distance in the 27 cells of the probe's cell (cell lists
 * of the last cell phase, current positions); velocity 0, pressure 0 and
 * density rho0 when no particle is in range or the probe is outside the
 * grid.  out: 5 doubles per probe (u, v, w, p, rho). */
void orc_probe(orc_sim *s, int n, const double *pts, double *out)
{
#pragma omp parallel for schedule(dynamic, 16)
    for (int k = 0; k < n; k++) {
        const v3 xi = v3make((real)pts[3 * k], (real)pts[3 * k + 1], (real)pts[3 * k + 2]);
        real wsum = 0, p = 0, rho = 0;
        v3 u = v3make(0, 0, 0);
        int c[3], inside = 1;
        const float xf[3] = {(float)pts[3 * k], (float)pts[3 * k + 1], (float)pts[3 * k + 2]};
        for (int a = 0; a < 3; a++) {
            c[a] = (int)((xf[a] - s->d.cell_min[a]) * s->d.interval_inv[a]);
            if (c[a] < 0 || c[a] >= s->d.cell_number[a]) inside = 0;
        }
        if (inside) {
            int nb[27];
            const int cell = (c[0] * s->d.cell_number[1] + c[1]) * s->d.cell_number[2] + c[2];
            const int nn = neighbor_cells(&s->d, cell, nb);
            for (int q = 0; q < nn; q++) {
                for (int m = s->cf.start[nb[q]]; m < s->cf.start[nb[q] + 1]; m++) {
                    const int j = s->cf.list[m];
                    const real r2 = dist2(xi, s->fpos[j]);
                    if (r2 < s->R2) {
                        const real w = (R_EXP(-r2 * s->h_inv2) - s->kc1) * s->kc2;
                        wsum += w;
                        u = vadd(u, vscale(s->fvel[j], w));
                        p += s->fp[j] * w;
                        rho += s->frho[j] * w;
                    }
                }
                for (int m = s->cs.start[nb[q]]; m < s->cs.start[nb[q] + 1]; m++) {
                    const int j = s->cs.list[m];
                    const real r2 = dist2(xi, s->spos[j]);
                    if (r2 < s->R2) {
                        const real w = (R_EXP(-r2 * s->h_inv2) - s->kc1) * s->kc2;
                        wsum += w;
                        u = vadd(u, vscale(s->svel[j], w));
                        p += s->sp[j] * w;
                    }
                }
            }
        }
        double *o = out + 5 * (size_t)k;
        if (wsum != 0) {
            o[0] = u.x / wsum;
            o[1] = u.y / wsum;
            o[2] = u.z / wsum;
            o[3] = p / wsum;
            o[4] = rho / wsum;
        } else {
            o[0] = o[1] = o[2] = o[3] = 0;
            o[4] = s->rho0;
        }
    }
}
