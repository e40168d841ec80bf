// ref_params_main.cpp — driver around the reference's own host sources.
//
// TEST INFRASTRUCTURE ONLY.  build_ref.sh compiles this file together with the
// unmodified reference sources src/config.cpp, src/kernel.cpp,
// src/properties.cpp, src/domain.cpp, src/physics.cpp and src/sim_time.cpp
// (paths within niji127/FluidSim) into oracle/_ref/ref_params.  It mirrors the
// order of Parameter::initiate (src/parameter.cpp:25-63) — count files, read
// the INI, derive constants — and prints every value as JSON, so the golden
// fixtures in tests/golden/ record what the reference itself computes.
//
// usage: ref_params <input.ini> [<data_prefix>]
//   <data_prefix>: the reference opens <data_prefix>\fluid_particle.dat etc.
//   (a literal backslash on Linux); when given, the particle-count readers run
//   too and their numbers and error flags are printed.
#include "config.h"
#include "domain.h"
#include "kernel.h"
#include "physics.h"
#include "properties.h"
#include "sim_time.h"

#include <cstdio>
#include <string>

static void pf(const char *k, float v, bool comma = true)
{
    if (v != v || v - v != 0.0f) // NaN or infinity: JSON has no literal for them
        std::printf("  \"%s\": \"%.9g\"%s\n", k, (double)v, comma ? "," : "");
    else
        std::printf("  \"%s\": %.9g%s\n", k, (double)v, comma ? "," : "");
}
static void pi(const char *k, long v, bool comma = true)
{
    std::printf("  \"%s\": %ld%s\n", k, v, comma ? "," : "");
}

int main(int argc, char **argv)
{
    if (argc < 2) {
        std::fprintf(stderr, "usage: %s input.ini [data_prefix]\n", argv[0]);
        return 2;
    }
    Physics physics;
    FluidProperties fluid;
    SolidProperties solid;
    VirtualProperties virt;
    Domain domain;
    SimTime time;
    Kernel kernel;
    fluid.number = solid.number = virt.number = 0;

    bool count_error = false;
    if (argc > 2) {
        std::string prefix = argv[2];
        count_error = fluid.readNumber(prefix);
        count_error = solid.readNumber(prefix) || count_error;
        count_error = virt.readNumber(prefix) || count_error;
    }

    bool read_error = false;
    try {
        Config config(argv[1]);
        read_error = physics.readParameter(config);
        read_error = fluid.readParameter(config) || read_error;
        read_error = solid.readParameter(config) || read_error;
        read_error = virt.readParameter(config) || read_error;
        read_error = domain.readParameter(config) || read_error;
        read_error = time.readParameter(config) || read_error;
        read_error = kernel.readParameter(config) || read_error;
    } catch (...) {
        std::printf("{\n  \"file_not_found\": 1\n}\n");
        return 0;
    }

    physics.initiate();
    fluid.initiate();
    solid.initiate();
    virt.initiate();
    time.initiate();
    kernel.initiate();
    domain.initiate(kernel);

    std::printf("{\n");
    pi("read_error", read_error ? 1 : 0);
    pi("count_error", count_error ? 1 : 0);
    pi("n_fluid", fluid.number);
    pi("n_solid", solid.number);
    pi("n_virt", virt.number);
    // raw config values
    pf("gravity", -physics.gravity[1]);
    pi("is_viscid", fluid.is_fluid_viscid ? 1 : 0);
    pf("min_pressure", fluid.min_pressure);
    pf("fluid_sound_speed", fluid.sound_speed);
    pf("fluid_density", fluid.reference_density);
    pf("gamma", fluid.gamma);
    pf("viscosity", fluid.viscosity);
    pf("solid_density", solid.reference_density);
    pf("youngs_modulus", solid.youngs_modulus);
    pf("poisson_ratio", solid.poisson_ratio);
    pf("arti_vis_alpha", solid.artificial_viscocity[0]);
    pf("arti_vis_beta", solid.artificial_viscocity[1]);
    pf("xmin", domain.domain_min[0]);
    pf("ymin", domain.domain_min[1]);
    pf("zmin", domain.domain_min[2]);
    pf("xmax", domain.domain_max[0]);
    pf("ymax", domain.domain_max[1]);
    pf("zmax", domain.domain_max[2]);
    pf("dt", time.dt);
    pi("istart", time.istart);
    pi("iend", time.iend);
    pi("solid_sub_step", time.solid_sub_step);
    pi("result_interval", time.result_interval);
    pi("sort_every_step", time.sort_every_step);
    pf("smoothing_length", kernel.smoothing_length);
    pf("particle_diameter", kernel.particle_diameter);
    pf("impact_length_hsml_ratio", kernel.impact_length_hsml_ratio);
    pi("thread_num", kernel.thread_num);
    // derived values
    pf("smoothing_length_square", kernel.smoothing_length_square);
    pf("smoothing_length_inverse", kernel.smoothing_length_inverse);
    pf("smoothing_length_inverse_square", kernel.smoothing_length_inverse_square);
    pf("impact_distance_square", kernel.impact_distance_square);
    pf("particle_volume", kernel.particle_volume);
    pf("kernel_coefficient_1", kernel.kernel_coefficient_1);
    pf("kernel_coefficient_2", kernel.kernel_coefficient_2);
    pf("kernel_differential", kernel.kernel_differential);
    pf("coefficient_p2rho", fluid.coefficient_p2rho);
    pf("coefficient_rho2p", fluid.coefficient_rho2p);
    pf("gamma_inv", fluid.gamma_inv);
    pf("reference_density_inverse", fluid.reference_density_inverse);
    pf("min_density", fluid.min_density);
    pf("max_density", fluid.max_density);
    pf("lambda", solid.lambda);
    pf("shear_modulus", solid.nu);
    pf("bulk_modulus", solid.bulk_modulus);
    pf("solid_sound_speed", solid.sound_speed);
    pf("gravity_vec_y", physics.gravity[1]);
    for (int i = 0; i < 3; i++) {
        char k[32];
        std::snprintf(k, sizeof k, "cell_min_%d", i);
        pf(k, domain.cell_min[i]);
        std::snprintf(k, sizeof k, "cell_max_%d", i);
        pf(k, domain.cell_max[i]);
        std::snprintf(k, sizeof k, "interval_%d", i);
        pf(k, domain.interval[i]);
        std::snprintf(k, sizeof k, "interval_inv_%d", i);
        pf(k, domain.interval_inv[i]);
        std::snprintf(k, sizeof k, "cell_number_%d", i);
        pi(k, domain.cell_number[i]);
    }
    pi("cell_number_total", domain.cell_number_total, false);
    std::printf("}\n");
    return 0;
}
