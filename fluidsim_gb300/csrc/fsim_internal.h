// fsim_internal.h — declarations shared by the host (fsim_host.cpp) and the
// device side (fsim_sim.cu, fsim_kernels.cu) of the library.  Not part of the public ABI.
#pragma once

#include "../../include/fluidsim.h"

#include <cctype>
#include <cstdarg>

#define FSIM_PI_F 3.141593f      // PI of the reference (include/global.h:4)
#define FSIM_EPS_FOR_SUM 0.1f    // include/global.h:6
#define FSIM_EPS_FLOAT 1.0e-6f   // include/global.h:7
#define FSIM_LARGE_FLOAT 1.0e6f  // include/global.h:8
#define FSIM_VIRT_LAYER 8        // grid padding in particle diameters (include/global.h:10)

void fsim_set_error(const char *fmt, ...);

// Host copies of the state, in input order, for the VTK writer.
struct VtkHostState {
    int n_fluid, n_solid, n_virt;
    const float *fpos, *fvel, *frho, *fp;
    const float *spos, *svel, *sp, *snormal;
    float solid_density;
    const float *vpos, *vnormal, *vp;
};
fsim_status fsim_write_vtk_host(const char *out_dir, int file_step, const VtkHostState &st, bool binary = false);
