// Drives ll::GpuZNE (include/ll_gpu_backend.h) the way the reference's ZNE checks drive ll::ZNE
// (src/Mitigation.h:618-650): a Bell circuit written against ll::Backend, <Z0 Z1> extrapolated
// from scales {1, 3}.  Prints, one per line: value std_error, then per scale "scale value se".
// Exit codes: 0 ok, 3 invalid_argument, 4 runtime_error.
#include <cstdio>
#include <cstdlib>

#include "ll_gpu_backend.h"

int main(int argc, char** argv) {
    const double p = argc > 1 ? std::atof(argv[1]) : 0.03;
    const int trajectories = argc > 2 ? std::atoi(argv[2]) : 40000;
    try {
        const ll::GpuZNE zne(trajectories);
        auto bell = [](ll::Backend& b) {
            b.h(0);
            b.cnot(0, 1);
        };
        const ll::GpuZNEResult r = zne.extrapolate(2, p, 99, bell, {{0, 1, 1.0}}, {1.0, 3.0});
        std::printf("%.17g %.17g\n", r.value, r.std_error);
        for (std::size_t k = 0; k < r.scales.size(); ++k)
            std::printf("%.0f %.17g %.17g\n", r.scales[k], r.values[k], r.std_errors[k]);
    } catch (const std::invalid_argument& e) {
        std::fprintf(stderr, "invalid_argument: %s\n", e.what());
        return 3;
    } catch (const std::runtime_error& e) {
        std::fprintf(stderr, "runtime_error: %s\n", e.what());
        return 4;
    }
    return 0;
}
