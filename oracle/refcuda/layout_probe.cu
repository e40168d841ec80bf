// Prints, from the reference's own headers, the byte offsets that
// ref_harness.cpp's ref_layout() reports for its mirror of Parameter,
// Data_Pointer and Cell, in the same order (one per line).  Built by
// oracle/build.py where the reference checkout exists; test infrastructure.
#include <stddef.h>
#include <stdio.h>

#include "sim.cuh"

int main()
{
    const long long v[] = {
        (long long)offsetof(Parameter, physics), (long long)offsetof(Parameter, fluid),
        (long long)offsetof(Parameter, solid), (long long)offsetof(Parameter, virt),
        (long long)offsetof(Parameter, domain), (long long)offsetof(Parameter, time),
        (long long)offsetof(Parameter, kernel),
        (long long)offsetof(FluidProperties, is_fluid_viscid), (long long)offsetof(SolidProperties, sound_speed),
        (long long)offsetof(Domain, cell_number_total), (long long)offsetof(SimTime, sort_every_step),
        (long long)offsetof(Kernel, thread_num), (long long)offsetof(Kernel, kernel_differential),
        (long long)offsetof(Data_Pointer, solid), (long long)offsetof(Data_Pointer, virt),
        (long long)offsetof(Data_Pointer, cell), (long long)offsetof(Solid_Data, normal),
        (long long)offsetof(Virt_Data, next_id_previous), (long long)offsetof(Cell, virt_start_id_previous),
        (long long)sizeof(Parameter), (long long)sizeof(Data_Pointer), (long long)sizeof(Cell)};
    for (size_t i = 0; i < sizeof(v) / sizeof(v[0]); ++i)
        printf("%lld\n", v[i]);
    printf("vec3 %zu mat3 %zu SolidType %zu VirtType %zu\n", sizeof(glm::vec3), sizeof(glm::mat3), sizeof(SolidType),
           sizeof(VirtType));
    return 0;
}
