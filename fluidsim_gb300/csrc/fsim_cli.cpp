// fluidsim — command-line driver with the reference's process contract.
//
// Reads input.ini and the three .dat files, advances the simulation and writes
// the VTK files on the reference's cadence: SimTime::addStep increments the
// step counter i and stops once i > iend (src/sim_time.cpp:33-39);
// Output::outputData writes before a step when (i-1) % result_interval == 0,
// with file index i / result_interval (src/sim_time.cpp:46-49,
// src/output.cu:299-335), and once more after the loop (src/calculation.cu:34).
#include "fluidsim.h"

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>

static int fail(const char *what, fsim_status st)
{
    std::fprintf(stderr, "fluidsim: %s failed: %s: %s\n", what, fsim_status_string(st), fsim_last_error());
    return 1;
}

int main(int argc, char **argv)
{
    const char *config = "../../config/input.ini", *data = "../../data", *out = "../../out";
    int device = 0;
    for (int a = 1; a < argc; ++a) {
        if (!std::strcmp(argv[a], "--config") && a + 1 < argc) config = argv[++a];
        else if (!std::strcmp(argv[a], "--data") && a + 1 < argc) data = argv[++a];
        else if (!std::strcmp(argv[a], "--out") && a + 1 < argc) out = argv[++a];
        else if (!std::strcmp(argv[a], "--device") && a + 1 < argc) device = std::atoi(argv[++a]);
        else {
            std::fprintf(stderr, "usage: fluidsim [--config PATH] [--data DIR] [--out DIR] [--device N]\n");
            return 2;
        }
    }
    fsim_config cfg;
    fsim_status st = fsim_config_from_ini(config, &cfg);
    if (st) return fail("reading the configuration", st);
    if (cfg.result_interval <= 0) {
        std::fprintf(stderr, "fluidsim: result_interval must be >= 1\n");
        return 1;
    }
    fsim_particle_set_t set = nullptr;
    if ((st = fsim_particles_read(data, &set))) return fail("reading the particles", st);
    fsim_particles p;
    fsim_particles_view(set, &p);
    std::printf("fluid %d, solid %d, virtual %d particles\n", p.n_fluid, p.n_solid, p.n_virt);
    fsim_handle h = nullptr;
    st = fsim_create(&cfg, &p, device, &h);
    fsim_particles_free(set);
    if (st) return fail("creating the simulation", st);

    const auto t0 = std::chrono::steady_clock::now();
    int i = cfg.istart;
    for (;;) {
        ++i;
        if (i > cfg.iend) break;
        if ((i - 1) % cfg.result_interval == 0) {
            if ((st = fsim_sync(h))) return fail("stepping", st);
            std::printf("output: step=%d time=%gs\n", i - 1, (double)(i - 1) * cfg.dt);
            if ((st = fsim_write_vtk(h, out, i / cfg.result_interval))) return fail("writing VTK", st);
        }
        if ((st = fsim_step(h, 1))) return fail("stepping", st);
    }
    if ((st = fsim_sync(h))) return fail("stepping", st);
    const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if ((i - 1) % cfg.result_interval == 0)
        if ((st = fsim_write_vtk(h, out, i / cfg.result_interval))) return fail("writing VTK", st);
    int nf = 0, ns = 0, nv = 0;
    fsim_counts(h, &nf, &ns, &nv);
    const long steps = (long)cfg.iend - cfg.istart;
    std::printf("%ld steps in %.3f s: %.3g particle-updates/s\n", steps, secs,
                steps > 0 ? (double)(nf + ns) * steps / secs : 0.0);
    fsim_destroy(h);
    return 0;
}
