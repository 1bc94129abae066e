// ref_capi.cpp -- C entry points over the REFERENCE's own header-only C++ backends, used only to
// pin the oracle and to write golden fixtures (test infrastructure; never part of the product).
//
// Built by oracle/build_oracle.py with -I<reference>/src into oracle/_ref/libref.so, directly
// from the reference's headers where they lie: src/Backend.h (ReferenceBackend),
// src/StateVectorBackend.h (StateVectorBackend), src/Algorithms.h (Grover, QAOA, VQE) and
// src/Mitigation.h (NoisyBackend, ZNE).
// Nothing from the reference is copied here; this file only drives its classes.

#include <complex>
#include <cstdint>
#include <cstring>
#include <random>
#include <stdexcept>
#include <vector>

#include "Algorithms.h"
#include "Backend.h"
#include "Mitigation.h"
#include "StateVectorBackend.h"

#include "sv_oracle.h"

namespace {

int run_on(ll::Backend& be, int n, const orc_op* ops, int nops) {
    be.reset(n);
    for (int i = 0; i < nops; ++i) {
        const orc_op& op = ops[i];
        switch (op.kind) {
            case ORC_OP_H: be.h(op.q0); break;
            case ORC_OP_X: be.x(op.q0); break;
            case ORC_OP_RX: be.rx(op.q0, op.theta); break;
            case ORC_OP_RY: be.ry(op.q0, op.theta); break;
            case ORC_OP_RZ: be.rz(op.q0, op.theta); break;
            case ORC_OP_CNOT: be.cnot(op.q0, op.q1); break;
            case ORC_OP_CZ: be.mcz({op.q0, op.q1}); break;
            case ORC_OP_MCZ: {
                std::vector<int> qs;
                for (int q = 0; q < 64; ++q)
                    if (op.mask >> q & 1) qs.push_back(q);
                be.mcz(qs);
                break;
            }
            default: throw std::invalid_argument("ref_capi: op kind has no ll::Backend call");
        }
    }
    return 0;
}

}  // namespace

extern "C" {

// backend: 0 = ll::ReferenceBackend, 1 = ll::StateVectorBackend.  out: 2*2^n doubles.
// Returns 0, 1 for std::invalid_argument, 2 for any other exception.
int ref_run_ops(int backend, int n, const orc_op* ops, int nops, double* out) {
    try {
        std::vector<std::complex<double>> s;
        if (backend == 0) {
            ll::ReferenceBackend be(1);
            run_on(be, n, ops, nops);
            s = be.state();
        } else {
            ll::StateVectorBackend be(1);
            run_on(be, n, ops, nops);
            s = be.state();
        }
        std::memcpy(out, s.data(), s.size() * sizeof(std::complex<double>));
        return 0;
    } catch (const std::invalid_argument&) {
        return 1;
    } catch (...) {
        return 2;
    }
}

// Probabilities through the backend's own probabilities() (StateVectorBackend.h:153-161).
int ref_probabilities(int backend, int n, const orc_op* ops, int nops, double* out) {
    try {
        std::vector<double> p;
        if (backend == 0) {
            ll::ReferenceBackend be(1);
            run_on(be, n, ops, nops);
            p = be.probabilities();
        } else {
            ll::StateVectorBackend be(1);
            run_on(be, n, ops, nops);
            p = be.probabilities();
        }
        std::memcpy(out, p.data(), p.size() * sizeof(double));
        return 0;
    } catch (const std::invalid_argument&) {
        return 1;
    } catch (...) {
        return 2;
    }
}

// The reference's random-circuit recipe (tests/test_backends.cpp:85-103) driven from one
// mt19937_64 stream: draws happen in the order kind, qubit a, angle, then b (cnot) or the coin
// flips (mcz).  Writes up to cap ops; returns the count.  rng_state carries the engine across
// calls so successive circuits continue the same stream, as the reference's test loop does.
struct RefRng {
    std::mt19937_64 rng;
};

void* ref_rng_new(uint64_t seed) { return new RefRng{std::mt19937_64(seed)}; }
void ref_rng_free(void* r) { delete static_cast<RefRng*>(r); }

int ref_random_circuit(void* r, int n, int depth, orc_op* out) {
    std::mt19937_64& rng = static_cast<RefRng*>(r)->rng;
    std::uniform_int_distribution<int> qd(0, n - 1);
    std::uniform_int_distribution<int> kd(0, n >= 2 ? 6 : 4);
    std::uniform_real_distribution<double> ang(-3.2, 3.2);
    std::bernoulli_distribution coin(0.5);
    for (int d = 0; d < depth; ++d) {
        orc_op op;
        std::memset(&op, 0, sizeof(op));
        op.param = -1;
        op.kind = kd(rng);
        op.q0 = qd(rng);
        op.theta = ang(rng);
        if (op.kind == 5) {
            do op.q1 = qd(rng);
            while (op.q1 == op.q0);
        } else if (op.kind == 6) {
            for (int q = 0; q < n; ++q)
                if (coin(rng)) op.mask |= 1ULL << q;
            if (op.mask == 0) op.mask = 1ULL << op.q0;
        }
        out[d] = op;
    }
    return depth;
}

// ll::Grover::run on StateVectorBackend (Algorithms.h:62-101).
int ref_grover(int n, const int* marked, int nmarked, int iterations, double* probs, int* marked_index, int* iters) {
    try {
        ll::StateVectorBackend be(1);
        std::vector<int> m(marked, marked + nmarked);
        ll::GroverResult res = ll::Grover::run(be, n, m, iterations);
        std::memcpy(probs, res.probabilities.data(), res.probabilities.size() * sizeof(double));
        *marked_index = res.marked_index;
        *iters = res.iterations;
        return 0;
    } catch (const std::invalid_argument&) {
        return 1;
    } catch (...) {
        return 2;
    }
}

// ll::VQE::prepare (Algorithms.h:240-252) on StateVectorBackend: RY layer + CNOT ring per layer.
int ref_vqe_prepare(int n, int layers, const double* params, double* out_state) {
    try {
        ll::VQE vqe(n, layers);
        ll::StateVectorBackend be(1);
        std::vector<double> p(params, params + vqe.n_params());
        vqe.prepare(be, p);
        const auto s = be.state();
        std::memcpy(out_state, s.data(), s.size() * sizeof(std::complex<double>));
        return 0;
    } catch (const std::invalid_argument&) {
        return 1;
    } catch (...) {
        return 2;
    }
}

// Diagonal observable sum_k c[k] Z_a[k] Z_b[k] (b < 0: Z_a) from the backend's probabilities().
static double zz_observable(const ll::Backend& b, int nterms, const int* za, const int* zb, const double* zc) {
    const std::vector<double> p = b.probabilities();
    double e = 0.0;
    for (std::size_t i = 0; i < p.size(); ++i) {
        double d = 0.0;
        for (int k = 0; k < nterms; ++k) {
            int par = (int)((i >> za[k]) & 1);
            if (zb[k] >= 0) par ^= (int)((i >> zb[k]) & 1);
            d += par ? -zc[k] : zc[k];
        }
        e += p[i] * d;
    }
    return e;
}

// ll::NoisyBackend over ll::ReferenceBackend (Mitigation.h:110-240): `ntraj` trajectories in order
// on one noisy backend (one mt19937_64 stream), the observable of each.
int ref_noisy_obs(int n, const orc_op* ops, int nops, double p, int scale, uint64_t seed, int ntraj, int nterms,
                  const int* za, const int* zb, const double* zc, double* out) {
    try {
        ll::ReferenceBackend inner(n);
        ll::NoisyBackend nb(inner, p, seed);
        nb.set_scale(scale);
        for (int t = 0; t < ntraj; ++t) {
            run_on(nb, n, ops, nops);
            out[t] = zz_observable(nb, nterms, za, zb, zc);
        }
        return 0;
    } catch (const std::invalid_argument&) {
        return 1;
    } catch (...) {
        return 2;
    }
}

// ll::ZNE::extrapolate (Mitigation.h:313-377).  out: value, std_error, trajectories, then
// values[ns], std_errors[ns], weights[ns].  Returns 1 for std::invalid_argument, 3 for
// std::runtime_error, 2 otherwise.
int ref_zne(int n, const orc_op* ops, int nops, double p, uint64_t seed, const double* scales, int ns, int trajectories,
            int nterms, const int* za, const int* zb, const double* zc, double* out) {
    try {
        ll::ReferenceBackend inner(n);
        ll::NoisyBackend nb(inner, p, seed);
        nb.reset(n);
        const ll::ZNE zne(trajectories);
        const ll::ZNEResult r = zne.extrapolate(
            nb, [&](ll::Backend& b) { run_on(b, n, ops, nops); },
            [&](const ll::Backend& b) { return zz_observable(b, nterms, za, zb, zc); },
            std::vector<double>(scales, scales + ns));
        out[0] = r.value;
        out[1] = r.std_error;
        out[2] = r.trajectories;
        for (int k = 0; k < ns; ++k) {
            out[3 + k] = r.values[k];
            out[3 + ns + k] = r.std_errors[k];
            out[3 + 2 * ns + k] = r.weights[k];
        }
        return 0;
    } catch (const std::invalid_argument&) {
        return 1;
    } catch (const std::runtime_error&) {
        return 3;
    } catch (...) {
        return 2;
    }
}

// ll::QAOA::run on StateVectorBackend (Algorithms.h:156-191): edges (ei[k], ej[k], w[k]), p layers.
// probs: 2^n_nodes doubles.
int ref_qaoa(int n_nodes, int nedges, const int* ei, const int* ej, const double* w, int p, const double* gammas,
             const double* betas, double* probs, double* best_cut) {
    try {
        ll::Graph g;
        g.n_nodes = n_nodes;
        for (int k = 0; k < nedges; ++k) g.edges.emplace_back(ei[k], ej[k], w[k]);
        ll::StateVectorBackend be(1);
        const ll::QAOAResult r = ll::QAOA::run(be, g, std::vector<double>(gammas, gammas + p),
                                               std::vector<double>(betas, betas + p));
        std::memcpy(probs, r.probabilities.data(), r.probabilities.size() * sizeof(double));
        *best_cut = r.best_cut;
        return 0;
    } catch (const std::invalid_argument&) {
        return 1;
    } catch (...) {
        return 2;
    }
}

// ll::VQE::optimize on StateVectorBackend (Algorithms.h:255-307) with the energy function the
// reference's run_vqe builds from a diagonal (python/algorithms.py:172-181): prepare, then
// probabilities() . diag, here with diag = sum_k c_k Z_a Z_b.  params: n * layers doubles out;
// probs: the best state's probabilities (2^n doubles).
int ref_vqe_optimize(int n, int layers, uint64_t seed, int max_iter, double lr, int nterms, const int* za, const int* zb,
                     const double* zc, double* energy, double* params, int* iterations, double* probs) {
    try {
        ll::VQE vqe(n, layers, seed);
        ll::StateVectorBackend be(1);
        auto fn = [&](const std::vector<double>& th) {
            vqe.prepare(be, th);
            return zz_observable(be, nterms, za, zb, zc);
        };
        const ll::VQEResult r = vqe.optimize(be, fn, max_iter, lr);
        *energy = r.energy;
        std::memcpy(params, r.params.data(), r.params.size() * sizeof(double));
        *iterations = r.iterations;
        const auto p = be.probabilities();
        std::memcpy(probs, p.data(), p.size() * sizeof(double));
        return 0;
    } catch (const std::invalid_argument&) {
        return 1;
    } catch (...) {
        return 2;
    }
}

}  // extern "C"
