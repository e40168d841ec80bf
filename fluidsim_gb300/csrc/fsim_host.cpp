// fsim_host.cpp — host side of the C ABI: status strings, input.ini parsing
// with the reference's semantics, FP32 parameter derivation, .dat particle
// files, the case generator and the ASCII VTK writer.
//
// Compiled with -ffp-contract=off so that the FP32 derivation rounds exactly
// like the reference's host code (pinned by tests/golden/params_*.json).
#include "fsim_internal.h"

#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <sys/stat.h>
#include <vector>

// ------------------------------------------------------------------ errors
static thread_local char g_last_error[512] = "";

void fsim_set_error(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(g_last_error, sizeof g_last_error, fmt, ap);
    va_end(ap);
}

extern "C" const char *fsim_last_error(void) { return g_last_error; }

extern "C" const char *fsim_status_string(fsim_status s)
{
    switch (s) {
    case FSIM_OK: return "FSIM_OK";
    case FSIM_EINVAL: return "FSIM_EINVAL";
    case FSIM_ENOMEM: return "FSIM_ENOMEM";
    case FSIM_ECUDA: return "FSIM_ECUDA";
    case FSIM_ETIMEOUT: return "FSIM_ETIMEOUT";
    case FSIM_ENUMERIC: return "FSIM_ENUMERIC";
    case FSIM_EIO: return "FSIM_EIO";
    default: return "FSIM_UNKNOWN";
    }
}

// ------------------------------------------------------------------ config
// Key/value store with the semantics of the reference's Config reader
// (src/config.cpp:59-129): text after '#' is dropped; a line with '=' starts a
// key; following lines without '=' that are not blank continue the value
// (joined with '\n'); a blank line ends it; lines without '=' are otherwise
// ignored, which is how '[section]' headers are skipped; keys and values are
// trimmed; a repeated key keeps the last value.
namespace {

const char *kWhitespace = " \n\t\v\r\f";

void trim(std::string &s)
{
    s.erase(0, s.find_first_not_of(kWhitespace));
    size_t last = s.find_last_not_of(kWhitespace);
    s.erase(last == std::string::npos ? 0 : last + 1);
}

std::string strip_comment(const std::string &line)
{
    size_t c = line.find('#');
    return c == std::string::npos ? line : line.substr(0, c);
}

struct IniValues {
    std::map<std::string, std::string> kv;

    void parse(std::istream &in)
    {
        std::string pending;
        bool have_pending = false;
        for (;;) {
            std::string line;
            if (have_pending) {
                line = pending;
                have_pending = false;
            } else if (!std::getline(in, line)) {
                break;
            }
            line = strip_comment(line);
            size_t eq = line.find('=');
            if (eq == std::string::npos) continue;
            std::string key = line.substr(0, eq);
            std::string value = line.substr(eq + 1);
            // continuation lines
            while (in) {
                std::string next;
                if (!std::getline(in, next)) break;
                std::string probe = next;
                trim(probe);
                if (probe.empty()) {
                    // a blank line ends the value; the reference re-reads it as a line
                    pending = next;
                    have_pending = !next.empty();
                    break;
                }
                next = strip_comment(next);
                if (next.find('=') != std::string::npos) {
                    pending = next;
                    have_pending = true;
                    break;
                }
                probe = next;
                trim(probe);
                if (!probe.empty()) value += "\n";
                value += next;
            }
            trim(key);
            trim(value);
            kv[key] = value;
        }
    }

    const std::string *find(const char *key) const
    {
        auto it = kv.find(key);
        return it == kv.end() ? nullptr : &it->second;
    }
    // string -> T through an istringstream, as the reference's string_as_T does
    float get(const char *key, float dflt) const
    {
        const std::string *v = find(key);
        if (!v) return dflt;
        float t;
        std::istringstream is(*v);
        is >> t;
        return t;
    }
    int get(const char *key, int dflt) const
    {
        const std::string *v = find(key);
        if (!v) return dflt;
        int t;
        std::istringstream is(*v);
        is >> t;
        return t;
    }
    // "false", "f", "no", "n", "0", "none" (any case, whole value) are false;
    // anything else is true (include/config.h: string_as_T<bool>)
    bool get_bool(const char *key, bool dflt) const
    {
        const std::string *v = find(key);
        if (!v) return dflt;
        std::string up = *v;
        for (char &c : up) c = (char)std::toupper((unsigned char)c);
        return !(up == "FALSE" || up == "F" || up == "NO" || up == "N" || up == "0" || up == "NONE");
    }
};

fsim_status config_from_values(const IniValues &ini, fsim_config *c)
{
    fsim_config_defaults(c);
    // [physics] src/physics.cpp:12
    c->gravity = ini.get("gravity", 9.81f);
    // [fluid] src/properties.cpp:36-42
    c->is_viscid = ini.get_bool("is_viscid", false) ? 1 : 0;
    c->min_pressure = ini.get("min_pressure", -1.013e5f);
    c->fluid_sound_speed = ini.get("fluid_sound_speed", 1500.0f);
    c->fluid_density = ini.get("fluid_density", 1000.0f);
    c->gamma = ini.get("gamma", 7.0f);
    c->viscosity = ini.get("viscosity", 1.01e-3f);
    // [solid] src/properties.cpp:97-101
    c->solid_density = ini.get("solid_density", 2700.0f);
    c->youngs_modulus = ini.get("youngs_modulus", 67.5e9f);
    c->poisson_ratio = ini.get("poisson_ratio", 0.34f);
    c->arti_vis_alpha = ini.get("arti_vis_alpha", 2.5f);
    c->arti_vis_beta = ini.get("arti_vis_beta", 2.5f);
    // [domain] src/domain.cpp:11-17
    c->xmin = ini.get("xmin", 0.0f);
    c->ymin = ini.get("ymin", 0.0f);
    c->zmin = ini.get("zmin", 0.0f);
    c->xmax = ini.get("xmax", 0.0f);
    c->ymax = ini.get("ymax", 0.0f);
    c->zmax = ini.get("zmax", 0.0f);
    // [time] src/sim_time.cpp:10-15
    c->dt = ini.get("dt", 0.0f);
    c->istart = ini.get("istart", 0);
    c->iend = ini.get("iend", 0);
    c->solid_sub_step = ini.get("solid_sub_step", 1);
    c->result_interval = ini.get("result_interval", 1);
    c->sort_every_step = ini.get("sort_every_step", 1);
    // [kernel] src/kernel.cpp:11-14
    c->smoothing_length = ini.get("smoothing_length", 0.0f);
    c->particle_diameter = ini.get("particle_diameter", 0.0f);
    c->impact_length_hsml_ratio = ini.get("impact_length_hsml_ratio", 3.0f);
    c->thread_num = ini.get("thread_num", 32);
    // extension keys, ignored by the reference
    if (const std::string *p = ini.find("gb300_precision")) {
        std::string v = *p;
        for (char &ch : v) ch = (char)std::tolower((unsigned char)ch);
        c->precision = (v == "mixed") ? FSIM_PRECISION_MIXED : FSIM_PRECISION_FP32;
    }
    c->keep_derivatives = ini.get_bool("gb300_keep_derivatives", false) ? 1 : 0;
    c->solid_fused = ini.get_bool("gb300_solid_fused", false) ? 1 : 0;
    c->solid_full_walk = ini.get_bool("gb300_solid_full_walk", false) ? 1 : 0;
    c->barrier_wait_polls = ini.get("gb300_barrier_wait_polls", 0);
    if (c->barrier_wait_polls < 0) c->barrier_wait_polls = 0;
    c->neighbor_skin = ini.get("gb300_neighbor_skin", c->neighbor_skin);
    if (!(c->neighbor_skin >= 0.0f && c->neighbor_skin <= 1.0f)) {
        fsim_set_error("gb300_neighbor_skin must lie in [0, 1]");
        return FSIM_EINVAL;
    }

    // validity checks of the readers (src/kernel.cpp:16-20, src/domain.cpp:19-23,
    // src/sim_time.cpp:17-21); the reference throws, we return EINVAL
    const char *bad = nullptr;
    if (c->smoothing_length == 0.0f || c->particle_diameter == 0.0f) bad = "failed to read kernel information";
    else if (c->xmax - c->xmin == 0.0f || c->ymax - c->ymin == 0.0f || c->zmax - c->zmin == 0.0f)
        bad = "failed to read domain information";
    else if (c->dt == 0.0f || c->istart - c->iend == 0) bad = "failed to read time information";
    if (bad) {
        fsim_set_error("FAILED TO READ INPUT.INI: %s", bad);
        return FSIM_EINVAL;
    }
    return FSIM_OK;
}

} // namespace

extern "C" fsim_status fsim_config_defaults(fsim_config *c)
{
    if (!c) return FSIM_EINVAL;
    std::memset(c, 0, sizeof *c);
    c->gravity = 9.81f;
    c->min_pressure = -1.013e5f;
    c->fluid_sound_speed = 1500.0f;
    c->fluid_density = 1000.0f;
    c->gamma = 7.0f;
    c->viscosity = 1.01e-3f;
    c->solid_density = 2700.0f;
    c->youngs_modulus = 67.5e9f;
    c->poisson_ratio = 0.34f;
    c->arti_vis_alpha = 2.5f;
    c->arti_vis_beta = 2.5f;
    c->solid_sub_step = 1;
    c->result_interval = 1;
    c->sort_every_step = 1;
    c->impact_length_hsml_ratio = 3.0f;
    c->thread_num = 32;
    c->precision = FSIM_PRECISION_FP32;
    c->neighbor_skin = 0.15f;
    return FSIM_OK;
}

extern "C" fsim_status fsim_config_from_ini_text(const char *text, fsim_config *c)
{
    if (!text || !c) return FSIM_EINVAL;
    IniValues ini;
    std::istringstream in(text);
    ini.parse(in);
    return config_from_values(ini, c);
}

extern "C" fsim_status fsim_config_from_ini(const char *path, fsim_config *c)
{
    if (!path || !c) return FSIM_EINVAL;
    std::ifstream in(path);
    if (!in) {
        fsim_set_error("cannot open %s", path);
        return FSIM_EIO;
    }
    IniValues ini;
    ini.parse(in);
    return config_from_values(ini, c);
}

// FP32 Riemann sum for the Gaussian's normalisation (src/kernel.cpp:25-41).
static float gaussian_normalisation(float K, float shift)
{
    const int n = 10000;
    const float step = K / (float)n;
    float acc = 0.0f;
    for (int i = 0; i < n; ++i) {
        const float x = (float)i * step;
        const float x2 = x * x;
        acc += x2 * expf(-x2) * step;
    }
    acc = acc * (4.0f * FSIM_PI_F);
    acc -= shift * 4.0f / 3.0f * FSIM_PI_F * powf(K, 3.0f);
    return 1.0f / acc;
}

extern "C" fsim_status fsim_derive(const fsim_config *c, fsim_derived *d)
{
    if (!c || !d) return FSIM_EINVAL;
    std::memset(d, 0, sizeof *d);
    const float h = c->smoothing_length, dp = c->particle_diameter, K = c->impact_length_hsml_ratio;
    if (!(h > 0.0f) || !(dp > 0.0f) || !(K > 0.0f)) {
        fsim_set_error("smoothing_length, particle_diameter and impact_length_hsml_ratio must be > 0");
        return FSIM_EINVAL;
    }
    // Kernel::initiate (src/kernel.cpp:43-60)
    d->particle_volume = powf(dp, 3.0f);
    d->smoothing_length_square = powf(h, 2.0f);
    d->smoothing_length_inverse = 1.0f / h;
    d->smoothing_length_inverse_square = powf(d->smoothing_length_inverse, 2.0f);
    d->impact_distance_square = powf(K, 2.0f) * powf(h, 2.0f);
    const float ratio = h / dp;
    d->kernel_coefficient_1 = expf(-powf(K, 2.0f));
    const float norm = gaussian_normalisation(K, d->kernel_coefficient_1);
    d->kernel_coefficient_2 = norm * powf(ratio, -3.0f);
    d->kernel_differential = 2.0f * norm * powf(ratio, -3.0f) * powf(h, -2.0f);
    // FluidProperties::initiate (src/properties.cpp:47-57)
    d->coefficient_p2rho = c->gamma * powf(c->fluid_sound_speed, -2.0f) / c->fluid_density;
    d->coefficient_rho2p = 1.0f / d->coefficient_p2rho;
    d->gamma_inv = 1.0f / c->gamma;
    d->reference_density_inverse = 1.0f / c->fluid_density;
    d->min_density = (1.0f - 0.1f) * c->fluid_density;
    d->max_density = (1.0f + 0.1f) * c->fluid_density;
    // SolidProperties::initiate (src/properties.cpp:59-66); "nu" there is the shear modulus
    const float E = c->youngs_modulus, pr = c->poisson_ratio;
    d->lambda = E * pr / (1.0f - 2.0f * pr) / (1.0f + pr);
    d->shear_modulus = E / (1.0f + pr) / 2.0f;
    d->bulk_modulus = E / (3.0f * (1.0f - 2.0f * pr));
    d->solid_sound_speed = sqrtf(d->bulk_modulus / c->solid_density);
    // Physics (src/physics.cpp:12-15)
    d->gravity_vec[0] = 0.0f;
    d->gravity_vec[1] = -c->gravity;
    d->gravity_vec[2] = 0.0f;
    // Domain::initiate (src/domain.cpp:28-47): grid padded by VIRT_LAYER diameters
    const float lo[3] = {c->xmin, c->ymin, c->zmin}, hi[3] = {c->xmax, c->ymax, c->zmax};
    const float pad = (float)FSIM_VIRT_LAYER * dp;
    const float cell = K * h;
    long long total = 1;
    for (int i = 0; i < 3; ++i) {
        d->cell_min[i] = lo[i] - pad;
        d->cell_max[i] = hi[i] + pad;
        d->cell_number[i] = (int)((d->cell_max[i] - d->cell_min[i]) / cell);
        if (d->cell_number[i] < 1) {
            fsim_set_error("degenerate cell grid on axis %d", i);
            return FSIM_EINVAL;
        }
        d->interval[i] = (d->cell_max[i] - d->cell_min[i]) / (float)d->cell_number[i];
        d->interval_inv[i] = 1.0f / d->interval[i];
        total *= d->cell_number[i];
    }
    if (total > (1ll << 30)) {
        fsim_set_error("cell grid too large (%lld cells)", total);
        return FSIM_EINVAL;
    }
    d->cell_number_total = (int)total;
    return FSIM_OK;
}

// --------------------------------------------------------------- particles
struct fsim_particle_set {
    std::vector<float> fpos, fvel, frho, fp;
    std::vector<float> spos, svel, sref;
    std::vector<int> stype;
    std::vector<float> vpos;
    std::vector<int> vtype;
};

namespace {

// Reads "<dir>/<name>": first line N, then exactly N rows of `width` numbers.
// The last `nint` columns are integers.  Mirrors *Properties::readNumber +
// the addList row readers (src/properties.cpp:7-32, include/host_data.cuh).
fsim_status read_dat(const std::string &path, int width, int nint, std::vector<float> &f, std::vector<int> &iv,
                     int &count)
{
    std::ifstream in(path);
    if (!in) {
        fsim_set_error("failed to read %s", path.c_str());
        return FSIM_EIO;
    }
    std::string line;
    if (!std::getline(in, line)) {
        fsim_set_error("%s: empty file", path.c_str());
        return FSIM_EINVAL;
    }
    long long n = -1;
    {
        std::istringstream is(line);
        is >> n;
    }
    if (n < 0 || n > (1ll << 31) - 1) {
        fsim_set_error("%s: particle number should >= 0", path.c_str());
        return FSIM_EINVAL;
    }
    count = (int)n;
    f.reserve((size_t)n * (width - nint));
    iv.reserve((size_t)n * nint);
    long long rows = 0;
    while (std::getline(in, line)) {
        ++rows;
        if (rows > n) continue; // counted for the mismatch error below
        const char *s = line.c_str();
        char *end = nullptr;
        for (int k = 0; k < width; ++k) {
            if (k < width - nint) {
                errno = 0;
                float v = std::strtof(s, &end);
                if (end == s) {
                    fsim_set_error("%s: row %lld does not parse", path.c_str(), rows);
                    return FSIM_EINVAL;
                }
                f.push_back(v);
            } else {
                long v = std::strtol(s, &end, 10);
                if (end == s) {
                    fsim_set_error("%s: row %lld does not parse", path.c_str(), rows);
                    return FSIM_EINVAL;
                }
                iv.push_back((int)v);
            }
            s = end;
        }
    }
    if (rows != n) {
        fsim_set_error("%s: mismatch particle numbers (%lld declared, %lld rows)", path.c_str(), n, rows);
        return FSIM_EINVAL;
    }
    return FSIM_OK;
}

void split_cols(const std::vector<float> &rows, int width, int col0, int ncol, std::vector<float> &out)
{
    size_t n = rows.size() / width;
    out.resize(n * ncol);
    for (size_t i = 0; i < n; ++i)
        for (int k = 0; k < ncol; ++k) out[i * ncol + k] = rows[i * width + col0 + k];
}

} // namespace

extern "C" fsim_status fsim_particles_read(const char *dir, fsim_particle_set_t *out)
{
    if (!dir || !out) return FSIM_EINVAL;
    *out = nullptr;
    auto *set = new (std::nothrow) fsim_particle_set;
    if (!set) return FSIM_ENOMEM;
    std::string base(dir);
    std::vector<float> rows;
    std::vector<int> ints;
    int n = 0;
    // fluid rows: x y z u v w rho p
    fsim_status st = read_dat(base + "/fluid_particle.dat", 8, 0, rows, ints, n);
    if (st) { delete set; return st; }
    split_cols(rows, 8, 0, 3, set->fpos);
    split_cols(rows, 8, 3, 3, set->fvel);
    split_cols(rows, 8, 6, 1, set->frho);
    split_cols(rows, 8, 7, 1, set->fp);
    // solid rows: x y z u v w X Y Z type
    rows.clear(); ints.clear();
    st = read_dat(base + "/solid_particle.dat", 10, 1, rows, ints, n);
    if (st) { delete set; return st; }
    split_cols(rows, 9, 0, 3, set->spos);
    split_cols(rows, 9, 3, 3, set->svel);
    split_cols(rows, 9, 6, 3, set->sref);
    set->stype = ints;
    // virtual rows: x y z type
    rows.clear(); ints.clear();
    st = read_dat(base + "/virt_particle.dat", 4, 1, rows, ints, n);
    if (st) { delete set; return st; }
    set->vpos = rows;
    set->vtype = ints;
    *out = set;
    return FSIM_OK;
}

extern "C" fsim_status fsim_particles_view(fsim_particle_set_t s, fsim_particles *v)
{
    if (!s || !v) return FSIM_EINVAL;
    std::memset(v, 0, sizeof *v);
    v->n_fluid = (int)s->frho.size();
    v->fluid_pos = s->fpos.data();
    v->fluid_vel = s->fvel.data();
    v->fluid_rho = s->frho.data();
    v->fluid_p = s->fp.data();
    v->n_solid = (int)s->stype.size();
    v->solid_pos = s->spos.data();
    v->solid_vel = s->svel.data();
    v->solid_ref_pos = s->sref.data();
    v->solid_type = s->stype.data();
    v->n_virt = (int)s->vtype.size();
    v->virt_pos = s->vpos.data();
    v->virt_type = s->vtype.data();
    return FSIM_OK;
}

extern "C" fsim_status fsim_particles_free(fsim_particle_set_t s)
{
    delete s;
    return FSIM_OK;
}

static bool make_dir(const std::string &p)
{
    if (mkdir(p.c_str(), 0755) == 0) return true;
    return errno == EEXIST;
}

extern "C" fsim_status fsim_particles_write(const char *dir, const fsim_particles *p)
{
    if (!dir || !p) return FSIM_EINVAL;
    make_dir(dir);
    std::string base(dir);
    char buf[256];
    {
        FILE *f = std::fopen((base + "/fluid_particle.dat").c_str(), "w");
        if (!f) { fsim_set_error("cannot write %s/fluid_particle.dat", dir); return FSIM_EIO; }
        std::fprintf(f, "%d\n", p->n_fluid);
        for (int i = 0; i < p->n_fluid; ++i) {
            const float *x = p->fluid_pos + 3 * i, *u = p->fluid_vel + 3 * i;
            std::snprintf(buf, sizeof buf, "%.9g %.9g %.9g %.9g %.9g %.9g %.9g %.9g\n", x[0], x[1], x[2], u[0], u[1],
                          u[2], p->fluid_rho[i], p->fluid_p[i]);
            std::fputs(buf, f);
        }
        if (std::fclose(f)) return FSIM_EIO;
    }
    {
        FILE *f = std::fopen((base + "/solid_particle.dat").c_str(), "w");
        if (!f) { fsim_set_error("cannot write %s/solid_particle.dat", dir); return FSIM_EIO; }
        std::fprintf(f, "%d\n", p->n_solid);
        for (int i = 0; i < p->n_solid; ++i) {
            const float *x = p->solid_pos + 3 * i, *u = p->solid_vel + 3 * i, *r = p->solid_ref_pos + 3 * i;
            std::snprintf(buf, sizeof buf, "%.9g %.9g %.9g %.9g %.9g %.9g %.9g %.9g %.9g %d\n", x[0], x[1], x[2], u[0],
                          u[1], u[2], r[0], r[1], r[2], p->solid_type[i]);
            std::fputs(buf, f);
        }
        if (std::fclose(f)) return FSIM_EIO;
    }
    {
        FILE *f = std::fopen((base + "/virt_particle.dat").c_str(), "w");
        if (!f) { fsim_set_error("cannot write %s/virt_particle.dat", dir); return FSIM_EIO; }
        std::fprintf(f, "%d\n", p->n_virt);
        for (int i = 0; i < p->n_virt; ++i) {
            const float *x = p->virt_pos + 3 * i;
            std::snprintf(buf, sizeof buf, "%.9g %.9g %.9g %d\n", x[0], x[1], x[2], p->virt_type ? p->virt_type[i] : 0);
            std::fputs(buf, f);
        }
        if (std::fclose(f)) return FSIM_EIO;
    }
    return FSIM_OK;
}

// --------------------------------------------------------------- generator
namespace {
// splitmix64: a small, portable, seedable generator (same stream on every host)
struct SplitMix {
    uint64_t s;
    uint64_t next()
    {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); } // [0,1)
};
} // namespace

extern "C" fsim_status fsim_case_generate(const fsim_case *cs, const fsim_config *cfg, fsim_particle_set_t *out)
{
    if (!cs || !cfg || !out) return FSIM_EINVAL;
    *out = nullptr;
    if (!(cs->dx > 0.0f) || cs->tank_n[0] <= 0 || cs->tank_n[1] <= 0 || cs->tank_n[2] <= 0 || cs->virt_layers < 0 ||
        cs->solid_fixed_layers < 0) {
        fsim_set_error("invalid case description");
        return FSIM_EINVAL;
    }
    auto *set = new (std::nothrow) fsim_particle_set;
    if (!set) return FSIM_ENOMEM;
    const double dx = cs->dx;
    const int L = cs->virt_layers;
    const int *T = cs->tank_n, *FN = cs->fluid_n, *SL = cs->solid_lo, *SN = cs->solid_n;
    const bool has_solid = SN[0] > 0 && SN[1] > 0 && SN[2] > 0;
    // hydrostatic state: p = rho0 g (H - y), rho = rho0 (p * gamma / (rho0 c0^2) + 1)^(1/gamma)
    const double rho0 = cfg->fluid_density, c0 = cfg->fluid_sound_speed, gam = cfg->gamma, g = cfg->gravity;
    const double H = FN[1] * dx;
    const double p2rho = gam / (rho0 * c0 * c0);
    SplitMix rng{cs->seed};
    const double jit = (double)cs->jitter * dx;
    auto jitter = [&](double v) { return jit > 0 ? v + (2.0 * rng.uniform() - 1.0) * jit : v; };

    for (int i = -L; i < T[0] + L; ++i) {
        for (int j = -L; j < T[1] + L; ++j) {
            for (int k = -L; k < T[2] + L; ++k) {
                const double x = (i + 0.5) * dx, y = (j + 0.5) * dx, z = (k + 0.5) * dx;
                const bool outside = i < 0 || i >= T[0] || j < 0 || j >= T[1] || k < 0 || k >= T[2];
                const bool in_solid = has_solid && i >= SL[0] && i < SL[0] + SN[0] && k >= SL[2] &&
                                      k < SL[2] + SN[2] && j >= SL[1] - cs->solid_fixed_layers && j < SL[1] + SN[1] &&
                                      (!outside || j < 0);
                if (in_solid) {
                    const bool fixed = j < 0;
                    const double sx = fixed ? x : jitter(x), sy = fixed ? y : jitter(y), sz = fixed ? z : jitter(z);
                    const float p3[3] = {(float)sx, (float)sy, (float)sz};
                    for (int a = 0; a < 3; ++a) {
                        set->spos.push_back(p3[a]);
                        set->sref.push_back(p3[a]);
                        set->svel.push_back(0.0f);
                    }
                    set->stype.push_back(fixed ? 1 : 0);
                } else if (outside) {
                    if (i >= -L && i < T[0] + L) {
                        set->vpos.push_back((float)x);
                        set->vpos.push_back((float)y);
                        set->vpos.push_back((float)z);
                        set->vtype.push_back(0);
                    }
                } else if (i < FN[0] && j < FN[1] && k < FN[2]) {
                    set->fpos.push_back((float)jitter(x));
                    set->fpos.push_back((float)jitter(y));
                    set->fpos.push_back((float)jitter(z));
                    for (int a = 0; a < 3; ++a) set->fvel.push_back(0.0f);
                    double p = 0.0, rho = rho0;
                    if (cs->hydrostatic) {
                        p = rho0 * g * (H - y);
                        rho = rho0 * std::pow(p * p2rho + 1.0, 1.0 / gam);
                    }
                    set->frho.push_back((float)rho);
                    set->fp.push_back((float)p);
                }
            }
        }
    }
    *out = set;
    return FSIM_OK;
}

// --------------------------------------------------------------------- VTK
// ASCII legacy VTK exactly as Output::write* produce it (src/output.cu:6-297):
// numbers through std::to_string(float) ("%f").
namespace {

// Legacy VTK polydata.  ASCII: the reference's text (std::to_string, 6
// decimals).  BINARY: the same sections with the numbers as big-endian FP32,
// as the legacy format defines them (exact values, ~10x smaller, no formatting).
struct VtkFile {
    std::string s;
    bool binary = false;
    void header(const char *title, int n)
    {
        s = "# vtk DataFile Version 2.0\n";
        s += title;
        s += binary ? "\nBINARY\n" : "\nASCII\n";
        s += "DATASET POLYDATA\nPOINTS " + std::to_string(n) + " float\n";
    }
    void put_be(float v)
    {
        uint32_t u;
        std::memcpy(&u, &v, 4);
        const char b[4] = {(char)(u >> 24), (char)(u >> 16), (char)(u >> 8), (char)u};
        s.append(b, 4);
    }
    void points(const float *p, int n)
    {
        if (binary) {
            s.reserve(s.size() + 12 * (size_t)n + 1);
            for (size_t i = 0; i < 3 * (size_t)n; ++i) put_be(p[i]);
            s += "\n";
            return;
        }
        for (int i = 0; i < n; ++i)
            s += std::to_string(p[3 * i]) + " " + std::to_string(p[3 * i + 1]) + " " + std::to_string(p[3 * i + 2]) +
                 "\n";
    }
    void vectors(const char *name, const float *v, int n)
    {
        s += "POINT_DATA " + std::to_string(n) + "\n";
        s += std::string("VECTORS ") + name + " float\n";
        points(v, n);
    }
    void scalars(const char *name, const float *v, int n, const float *constant = nullptr)
    {
        s += "POINT_DATA " + std::to_string(n) + "\n";
        s += std::string("SCALARS ") + name + " float 1\nLOOKUP_TABLE default\n";
        if (binary) {
            s.reserve(s.size() + 4 * (size_t)n + 1);
            for (int i = 0; i < n; ++i) put_be(constant ? *constant : v[i]);
            s += "\n";
            return;
        }
        for (int i = 0; i < n; ++i) s += std::to_string(constant ? *constant : v[i]) + "\n";
    }
    bool write(const std::string &path) const
    {
        FILE *f = std::fopen(path.c_str(), "wb");
        if (!f) return false;
        size_t w = std::fwrite(s.data(), 1, s.size(), f);
        return std::fclose(f) == 0 && w == s.size();
    }
};

} // namespace

fsim_status fsim_write_vtk_host(const char *out_dir, int file_step, const VtkHostState &st, bool binary)
{
    std::string base(out_dir);
    make_dir(base);
    const std::string k = std::to_string(file_step);
    VtkFile f;
    f.binary = binary;
    if (st.n_fluid) {
        std::string d = base + "/fluid";
        make_dir(d);
        f.header("Velocity vector file", st.n_fluid);
        f.points(st.fpos, st.n_fluid);
        f.vectors("velocity", st.fvel, st.n_fluid);
        if (!f.write(d + "/fluid_velocity-" + k + ".vtk")) return FSIM_EIO;
        f.header("scalar vector file", st.n_fluid);
        f.points(st.fpos, st.n_fluid);
        f.scalars("density", st.frho, st.n_fluid);
        if (!f.write(d + "/fluid_density-" + k + ".vtk")) return FSIM_EIO;
        // the reference writes the always-zero color array under the name pressure (src/output.cu:75)
        f.header("scalar vector file", st.n_fluid);
        f.points(st.fpos, st.n_fluid);
        const float zero = 0.0f;
        f.scalars("pressure", nullptr, st.n_fluid, &zero);
        if (!f.write(d + "/fluid_pressure-" + k + ".vtk")) return FSIM_EIO;
        // real pressure, an addition
        f.header("scalar vector file", st.n_fluid);
        f.points(st.fpos, st.n_fluid);
        f.scalars("pressure", st.fp, st.n_fluid);
        if (!f.write(d + "/fluid_true_pressure-" + k + ".vtk")) return FSIM_EIO;
    }
    if (st.n_solid) {
        std::string d = base + "/solid";
        make_dir(d);
        f.header("Velocity vector file", st.n_solid);
        f.points(st.spos, st.n_solid);
        f.vectors("velocity", st.svel, st.n_solid);
        if (!f.write(d + "/solid_velocity-" + k + ".vtk")) return FSIM_EIO;
        f.header("scalar vector file", st.n_solid);
        f.points(st.spos, st.n_solid);
        f.scalars("pressure", st.sp, st.n_solid);
        if (!f.write(d + "/solid_pressure-" + k + ".vtk")) return FSIM_EIO;
        f.header("scalar vector file", st.n_solid);
        f.points(st.spos, st.n_solid);
        f.scalars("density", nullptr, st.n_solid, &st.solid_density);
        if (!f.write(d + "/solid_density-" + k + ".vtk")) return FSIM_EIO;
        f.header("Velocity vector file", st.n_solid);
        f.points(st.spos, st.n_solid);
        f.vectors("normal", st.snormal, st.n_solid);
        if (!f.write(d + "/solid_normal-" + k + ".vtk")) return FSIM_EIO;
    }
    if (st.n_virt) {
        std::string d = base + "/virtual";
        make_dir(d);
        f.header("Velocity vector file", st.n_virt);
        f.points(st.vpos, st.n_virt);
        f.vectors("normal", st.vnormal, st.n_virt);
        if (!f.write(d + "/virt_normal-" + k + ".vtk")) return FSIM_EIO;
        f.header("scalar vector file", st.n_virt);
        f.points(st.vpos, st.n_virt);
        f.scalars("pressure", st.vp, st.n_virt);
        if (!f.write(d + "/virt_pressure-" + k + ".vtk")) return FSIM_EIO;
    }
    return FSIM_OK;
}
