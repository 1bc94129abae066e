// Compiles the reference's own Algorithms.h (Grover, QAOA, VQE) against ll::GpuBackend to show
// the shim is a drop-in for ll::StateVectorBackend.  Built only where the reference tree is on the
// include path.  Prints Grover's iteration count and peak probability for n = 8, marked 85
// (README.md:509: 12 iterations, P = 0.99994704), then a QAOA and a VQE energy.
#include <cstdio>

#include "Algorithms.h"
#include "ll_gpu_backend.h"

int main() {
    try {
        ll::GpuBackend be(1);
        const ll::GroverResult g = ll::Grover::run(be, 8, {85});
        std::printf("grover %d %d %.12f\n", g.iterations, g.marked_index, g.probabilities[85]);
        ll::Graph graph;
        graph.n_nodes = 4;
        graph.edges = {{0, 1, 1.0}, {1, 2, 1.0}, {2, 3, 1.0}, {3, 0, 1.0}};
        const ll::QAOAResult qa = ll::QAOA::run(be, graph, {0.4}, {0.3});
        std::printf("qaoa %.12f\n", qa.best_cut);
        ll::VQE vqe(4, 2);
        vqe.prepare(be, std::vector<double>(8, 0.3));
        const auto p = be.probabilities();
        std::printf("vqe_p0 %.12f\n", p[0]);
    } catch (const std::runtime_error& e) {
        std::fprintf(stderr, "runtime_error: %s\n", e.what());
        return 4;
    }
    return 0;
}
