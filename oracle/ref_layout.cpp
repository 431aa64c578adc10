/* Prints the host-side layout of the reference's kernel parameter classes (Parameter,
 * SimulationParam, ArchitectureParam; cpp/parameter.h:14-20, cpp/SimulationParam.h:12-60,
 * cpp/ArchitectureParam.h:8-15) and of curandState_t, as JSON. Compiled against the reference
 * headers by oracle/ref_build.py; the harness builds its by-value kernel arguments from it. */
#include <cstddef>
#include <cstdio>
#include <curand_kernel.h>
#include "parameter.h"

int main()
{
    std::printf("{\"sizeof_Parameter\": %zu, \"alignof_Parameter\": %zu, \"off_arch\": %zu, \"off_io\": %zu, "
                "\"off_simulation\": %zu, \"sizeof_SimulationParam\": %zu, \"sizeof_ArchitectureParam\": %zu, "
                "\"sizeof_IOParam\": %zu, \"sizeof_curandState\": %zu, \"off_sim_scaleHumidity\": %zu}\n",
                sizeof(Parameter), alignof(Parameter), offsetof(Parameter, arch), offsetof(Parameter, io),
                offsetof(Parameter, simulation), sizeof(SimulationParam), sizeof(ArchitectureParam),
                sizeof(IOParam), sizeof(curandState_t), offsetof(SimulationParam, scaleHumidity));
    return 0;
}
