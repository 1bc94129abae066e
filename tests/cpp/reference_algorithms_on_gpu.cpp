// Compiles the reference's own Algorithms.h (Grover, QAOA, VQE) against ll::GpuBackend to show
// the shim is a drop-in for ll::StateVectorBackend.  Built only where the reference tree is on the
// include path.  Prints, one line each:
//   grover <iterations> <marked index> <P(85)>           n = 8, marked 85 (README.md:509)
//   qaoa <best_cut> <p_0> ... <p_15>                     4-node ring, gamma 0.4, beta 0.3
//   vqe <p_0> ... <p_15>                                 VQE::prepare, 4 qubits, 2 layers, params argv
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "Algorithms.h"
#include "ll_gpu_backend.h"

int main(int argc, char** argv) {
    try {
        ll::GpuBackend be(1);
        const ll::GroverResult g = ll::Grover::run(be, 8, {85});
        std::printf("grover %d %d %.17g\n", g.iterations, g.marked_index, g.probabilities[85]);
        ll::Graph graph;
        graph.n_nodes = 4;
        graph.edges = {{0, 1, 1.0}, {1, 2, 1.0}, {2, 3, 1.0}, {3, 0, 1.0}};
        const ll::QAOAResult qa = ll::QAOA::run(be, graph, {0.4}, {0.3});
        std::printf("qaoa %.17g", qa.best_cut);
        for (double p : qa.probabilities) std::printf(" %.17g", p);
        std::printf("\n");
        ll::VQE vqe(4, 2);
        std::vector<double> params(8, 0.3);
        for (int k = 0; k < 8 && k + 1 < argc; ++k) params[k] = std::atof(argv[k + 1]);
        vqe.prepare(be, params);
        std::printf("vqe");
        for (double p : be.probabilities()) std::printf(" %.17g", p);
        std::printf("\n");
    } catch (const std::runtime_error& e) {
        std::fprintf(stderr, "runtime_error: %s\n", e.what());
        return 4;
    }
    return 0;
}
