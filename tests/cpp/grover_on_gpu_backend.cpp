// Drives ll::GpuBackend through the ll::Backend interface with the Grover gate sequence of the
// reference's ll::Grover::run (src/Algorithms.h:85-90 and :111-124): H on every qubit, then per
// iteration a phase flip of each marked state (X where the state has a 0 bit, multi-controlled Z
// on all qubits, X again) and the diffusion (H, X, MCZ, X, H).  Prints the probabilities, one
// per line, with 17 significant digits.  Usage: grover_on_gpu_backend n iterations marked...
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "ll_gpu_backend.h"

static void phase_flip(ll::Backend& b, int n, int m, const std::vector<int>& all) {
    for (int q = 0; q < n; ++q)
        if (!((m >> q) & 1)) b.x(q);
    b.mcz(all);
    for (int q = 0; q < n; ++q)
        if (!((m >> q) & 1)) b.x(q);
}

int main(int argc, char** argv) {
    if (argc < 4) return 2;
    const int n = std::atoi(argv[1]);
    const int iters = std::atoi(argv[2]);
    std::vector<int> marked;
    for (int i = 3; i < argc; ++i) marked.push_back(std::atoi(argv[i]));
    std::vector<int> all(n);
    for (int q = 0; q < n; ++q) all[q] = q;
    try {
        ll::GpuBackend be(1);
        ll::Backend& b = be;
        b.reset(n);
        for (int q = 0; q < n; ++q) b.h(q);
        for (int it = 0; it < iters; ++it) {
            for (int m : marked) phase_flip(b, n, m, all);
            for (int q = 0; q < n; ++q) {
                b.h(q);
                b.x(q);
            }
            b.mcz(all);
            for (int q = 0; q < n; ++q) {
                b.x(q);
                b.h(q);
            }
        }
        for (double p : b.probabilities()) std::printf("%.17g\n", p);
        // the error contract travels through the interface
        try {
            b.cnot(0, 0);
            return 3;
        } catch (const std::invalid_argument&) {
        }
    } catch (const std::runtime_error& e) {
        std::fprintf(stderr, "runtime_error: %s\n", e.what());
        return 4;
    }
    return 0;
}
