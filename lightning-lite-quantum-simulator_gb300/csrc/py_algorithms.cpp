// py_algorithms.cpp -- quantum_sim_algorithms on the GPU: the reference module of the same name
// (src/bindings_algorithms.cpp:31-125) with a GPU backend behind its factories.
//
// make_gpu_backend(n, precision) -- and make_statevector_backend(n), the reference's factory
// name (src/bindings_algorithms.cpp:52-54) -- return a Backend whose state lives in HBM and whose
// gates go through libllgpu.so's queue (fused into shared-memory tile passes at the next
// readout).  Grover.run, QAOA.run and VQE.prepare / VQE.optimize issue the same gate sequences as
// the reference's Algorithms.h (Grover::run :62-101, QAOA::run :156-191, VQE::prepare :240-252,
// VQE::optimize :255-307), so their probabilities agree with ll::StateVectorBackend's to rounding.
// Beyond the reference, Backend.expect_diagonal / expect_zz evaluate a diagonal energy on the
// device, so an energy function need not copy 2^n probabilities to the host per evaluation.
//
// The reference module cannot be built without Eigen (pybind11/eigen.h, EigenBackend.h); this one
// needs neither.  make_reference_backend / make_eigen_backend (CPU engines) are not provided.
#include <pybind11/complex.h>
#include <pybind11/functional.h>
#include <pybind11/numpy.h>
#include <pybind11/pybind11.h>
#include <pybind11/stl.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <functional>
#include <memory>
#include <random>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

#include "llgpu.h"

namespace py = pybind11;

namespace {

void check(int rc) {
    if (rc == LLG_OK) return;
    const std::string msg = llg_last_error();
    if (rc == LLG_EINVAL) throw std::invalid_argument(msg);
    if (rc == LLG_ENOMEM) throw std::bad_alloc();
    throw std::runtime_error(msg);
}

int parse_precision(const std::string& p) {
    if (p == "df64") return LLG_DF64;
    if (p == "complex128" || p == "c128" || p == "fp64" || p == "f64") return LLG_F64;
    if (p == "complex64" || p == "c64" || p == "f32") return LLG_F32;
    throw std::invalid_argument("precision must be 'complex128' (IEEE FP64), 'df64' or 'complex64'");
}

[[noreturn]] void fail(const char* who, const char* msg) { throw std::invalid_argument(std::string(who) + ": " + msg); }

constexpr double kPi = 3.14159265358979323846;

// The ll::Backend calls (src/Backend.h:25-45) over one engine state.
class GpuBackend {
public:
    GpuBackend(int n_qubits, int precision) { check(llg_create(n_qubits, precision, &st_)); }
    ~GpuBackend() {
        if (st_) llg_destroy(st_);
    }
    GpuBackend(const GpuBackend&) = delete;
    GpuBackend& operator=(const GpuBackend&) = delete;

    void reset(int n) { check(llg_reset(st_, n)); }
    int n_qubits() const {
        int n = 0;
        check(llg_num_qubits(st_, &n));
        return n;
    }
    void h(int q) { check(llg_h(st_, q)); }
    void x(int q) { check(llg_x(st_, q)); }
    void rx(int q, double t) { check(llg_rx(st_, q, t)); }
    void ry(int q, double t) { check(llg_ry(st_, q, t)); }
    void rz(int q, double t) { check(llg_rz(st_, q, t)); }
    void cnot(int c, int t) { check(llg_cnot(st_, c, t)); }
    void mcz(const std::vector<int>& qs) { check(llg_mcz(st_, qs.data(), (int)qs.size())); }
    std::vector<double> probabilities() const {
        std::vector<double> p(size());
        check(llg_probabilities(st_, p.data()));
        return p;
    }
    std::vector<std::complex<double>> state() const {
        std::vector<std::complex<double>> s(size());
        check(llg_copy_to_host(st_, reinterpret_cast<double*>(s.data())));
        return s;
    }
    double expect_diagonal(const double* d, int on_device) const {
        double v = 0.0;
        check(llg_expect_diagonal(st_, d, on_device, &v));
        return v;
    }
    double expect_zz(const std::vector<int>& a, const std::vector<int>& b, const std::vector<double>& c) const {
        if (a.size() != b.size() || a.size() != c.size()) fail("expect_zz", "term lists differ in length");
        double v = 0.0;
        check(llg_expect_zz(st_, (int)a.size(), a.data(), b.data(), c.data(), &v));
        return v;
    }
    size_t size() const {
        uint64_t n = 0;
        check(llg_size(st_, &n));
        return (size_t)n;
    }

private:
    llg_state* st_ = nullptr;
};

// ---- Grover (src/Algorithms.h:62-119) --------------------------------------------------------
struct GroverResult {
    std::vector<double> probabilities;
    int marked_index = -1;
    int iterations = 0;
};

GroverResult grover_run(GpuBackend& be, int n, const std::vector<int>& marked_states, int iterations) {
    const char* who = "Grover::run";
    if (n < 1 || n > 30) fail(who, "n_qubits must be in [1, 30]");
    if (iterations < -1) fail(who, "iterations must be >= 0, or -1 for automatic");
    const long long states = 1LL << n;
    std::vector<int> marked = marked_states;
    for (int m : marked)
        if (m < 0 || m >= states) fail(who, "marked state outside [0, 2^n)");
    std::sort(marked.begin(), marked.end());
    marked.erase(std::unique(marked.begin(), marked.end()), marked.end());
    if (marked.empty()) fail(who, "no marked states");
    if ((long long)marked.size() >= states) fail(who, "marked states must be a proper subset of the search space");
    int k = iterations;
    if (k < 0) {  // the rotation angle per iteration: sin(theta) = sqrt(M / N)
        const double theta = std::asin(std::sqrt((double)marked.size() / (double)states));
        k = std::max(0, (int)std::lround(kPi / (4.0 * theta) - 0.5));
    }
    std::vector<int> all(n);
    for (int q = 0; q < n; ++q) all[q] = q;
    be.reset(n);
    for (int q = 0; q < n; ++q) be.h(q);
    for (int it = 0; it < k; ++it) {
        for (int m : marked) {  // oracle: -1 on |m>, by an X frame around the all-qubit CZ
            for (int q = 0; q < n; ++q)
                if (!((m >> q) & 1)) be.x(q);
            be.mcz(all);
            for (int q = 0; q < n; ++q)
                if (!((m >> q) & 1)) be.x(q);
        }
        for (int q = 0; q < n; ++q) {  // diffusion, up to a global sign
            be.h(q);
            be.x(q);
        }
        be.mcz(all);
        for (int q = 0; q < n; ++q) {
            be.x(q);
            be.h(q);
        }
    }
    GroverResult r;
    r.probabilities = be.probabilities();
    r.marked_index = (int)(std::max_element(r.probabilities.begin(), r.probabilities.end()) - r.probabilities.begin());
    r.iterations = k;
    return r;
}

// ---- QAOA for MaxCut (src/Algorithms.h:121-200) ----------------------------------------------
struct Graph {
    int n_nodes = 0;
    std::vector<std::tuple<int, int, double>> edges;
};

struct QAOAResult {
    std::vector<double> probabilities;
    double best_cut = 0.0;
};

double cut_value(const Graph& g, uint64_t z) {
    double c = 0.0;
    for (const auto& e : g.edges)
        if (((z >> std::get<0>(e)) & 1u) != ((z >> std::get<1>(e)) & 1u)) c += std::get<2>(e);
    return c;
}

QAOAResult qaoa_run(GpuBackend& be, const Graph& g, const std::vector<double>& gammas, const std::vector<double>& betas) {
    const char* who = "QAOA::run";
    if (g.n_nodes < 1 || g.n_nodes > 30) fail(who, "n_nodes must be in [1, 30]");
    if (gammas.empty() || gammas.size() != betas.size()) fail(who, "gammas and betas must be non-empty and of equal length");
    for (const auto& e : g.edges) {
        const int i = std::get<0>(e), j = std::get<1>(e);
        if (i < 0 || j < 0 || i >= g.n_nodes || j >= g.n_nodes) fail(who, "edge endpoint outside [0, n_nodes)");
        if (i == j) fail(who, "self-loop edge");
        if (!std::isfinite(std::get<2>(e))) fail(who, "non-finite edge weight");
    }
    for (double a : gammas)
        if (!std::isfinite(a)) fail(who, "non-finite gamma");
    for (double a : betas)
        if (!std::isfinite(a)) fail(who, "non-finite beta");
    be.reset(g.n_nodes);
    for (int q = 0; q < g.n_nodes; ++q) be.h(q);
    for (size_t l = 0; l < gammas.size(); ++l) {
        for (const auto& e : g.edges) {  // exp(+i gamma w Z_i Z_j / 2) as CNOT, RZ(-gamma w), CNOT
            const int i = std::get<0>(e), j = std::get<1>(e);
            be.cnot(i, j);
            be.rz(j, -gammas[l] * std::get<2>(e));
            be.cnot(i, j);
        }
        for (int q = 0; q < g.n_nodes; ++q) be.rx(q, 2.0 * betas[l]);
    }
    QAOAResult r;
    r.probabilities = be.probabilities();
    const auto best = std::max_element(r.probabilities.begin(), r.probabilities.end());
    r.best_cut = cut_value(g, (uint64_t)(best - r.probabilities.begin()));
    return r;
}

// ---- VQE (src/Algorithms.h:202-309) ----------------------------------------------------------
struct VQEResult {
    double energy = 0.0;
    std::vector<double> params;
    int iterations = 0;
};

class VQE {
public:
    VQE(int n_qubits, int n_layers, uint64_t seed) : n_(n_qubits), layers_(n_layers), seed_(seed) {
        if (n_qubits < 1 || n_qubits > 30) fail("VQE", "n_qubits must be in [1, 30]");
        if (n_layers < 1) fail("VQE", "n_layers must be >= 1");
    }
    int n_qubits() const { return n_; }
    int n_layers() const { return layers_; }
    int n_params() const { return n_ * layers_; }

    // RY(theta[l n + q]) on every qubit, then the CNOT ring, per layer
    void prepare(GpuBackend& be, const std::vector<double>& params) const {
        if ((int)params.size() != n_params()) fail("VQE::prepare", "wrong number of parameters");
        be.reset(n_);
        for (int l = 0; l < layers_; ++l) {
            for (int q = 0; q < n_; ++q) be.ry(q, params[(size_t)(l * n_ + q)]);
            if (n_ == 2) be.cnot(0, 1);
            else if (n_ > 2)
                for (int q = 0; q < n_; ++q) be.cnot(q, (q + 1) % n_);
        }
    }

    // Gradient descent with parameter-shift gradients dE/dt_k = (E(t + pi/2 e_k) - E(t - pi/2 e_k)) / 2,
    // initial parameters uniform in [-0.1, 0.1) from std::mt19937_64(seed); the lowest energy seen
    // is returned and left prepared on the backend.
    VQEResult optimize(GpuBackend& be, const std::function<double(const std::vector<double>&)>& energy_fn, int max_iter,
                       double lr) const {
        const char* who = "VQE::optimize";
        if (max_iter < 0) fail(who, "max_iter must be >= 0");
        if (!(std::isfinite(lr) && lr > 0.0)) fail(who, "lr must be finite and > 0");
        if (!energy_fn) fail(who, "energy_fn is empty");
        auto eval = [&](const std::vector<double>& t) {
            const double e = energy_fn(t);
            if (!std::isfinite(e)) throw std::runtime_error(std::string(who) + ": non-finite energy");
            return e;
        };
        std::mt19937_64 rng(seed_);
        std::uniform_real_distribution<double> init(-0.1, 0.1);
        std::vector<double> theta((size_t)n_params());
        for (double& t : theta) t = init(rng);
        VQEResult out;
        out.energy = eval(theta);
        out.params = theta;
        std::vector<double> grad(theta.size());
        for (int it = 0; it < max_iter; ++it) {
            double norm2 = 0.0;
            for (size_t k = 0; k < theta.size(); ++k) {
                const double t0 = theta[k];
                theta[k] = t0 + kPi / 2.0;
                const double ep = eval(theta);
                theta[k] = t0 - kPi / 2.0;
                const double em = eval(theta);
                theta[k] = t0;
                grad[k] = 0.5 * (ep - em);
                norm2 += grad[k] * grad[k];
            }
            if (std::sqrt(norm2) < 1e-6) break;
            for (size_t k = 0; k < theta.size(); ++k) theta[k] -= lr * grad[k];
            ++out.iterations;
            const double e = eval(theta);
            if (e < out.energy) {
                out.energy = e;
                out.params = theta;
            }
        }
        prepare(be, out.params);
        return out;
    }

private:
    int n_, layers_;
    uint64_t seed_;
};

py::array_t<double> to_array(const std::vector<double>& v) { return py::array_t<double>((py::ssize_t)v.size(), v.data()); }

}  // namespace

PYBIND11_MODULE(quantum_sim_algorithms, m) {
    m.doc() = "Grover, QAOA and VQE on the GB300 state-vector engine (the reference module's API)";
    py::register_exception_translator([](std::exception_ptr p) {
        try {
            if (p) std::rethrow_exception(p);
        } catch (const std::invalid_argument& e) {
            PyErr_SetString(PyExc_ValueError, e.what());
        }
    });

    py::class_<GpuBackend>(m, "Backend")
        .def("n_qubits", &GpuBackend::n_qubits)
        .def("probabilities", [](const GpuBackend& b) {
            std::vector<double> p;
            {
                py::gil_scoped_release rel;
                p = b.probabilities();
            }
            return to_array(p);
        }, "|amplitude|^2 of every basis state, qubit q = bit q of the index.")
        .def("state", [](const GpuBackend& b) {
            std::vector<std::complex<double>> s;
            {
                py::gil_scoped_release rel;
                s = b.state();
            }
            return py::array_t<std::complex<double>>((py::ssize_t)s.size(), s.data());
        }, "Complex amplitudes, size 2^n.")
        .def("reset", &GpuBackend::reset)
        .def("h", &GpuBackend::h)
        .def("x", &GpuBackend::x)
        .def("rx", &GpuBackend::rx)
        .def("ry", &GpuBackend::ry)
        .def("rz", &GpuBackend::rz)
        .def("cnot", &GpuBackend::cnot)
        .def("mcz", &GpuBackend::mcz)
        .def("expect_diagonal", [](const GpuBackend& b, py::object diag) {
            // a CUDA array (__cuda_array_interface__, e.g. a torch tensor) is read in place; anything
            // else is copied from host memory
            if (py::hasattr(diag, "__cuda_array_interface__")) {
                py::dict cai = diag.attr("__cuda_array_interface__");
                const auto shape = cai["shape"].cast<std::vector<py::ssize_t>>();
                if (cai["typestr"].cast<std::string>() != "<f8" || shape.size() != 1 ||
                    (size_t)shape[0] != b.size() || (!cai["strides"].is_none()))
                    throw std::invalid_argument("expect_diagonal: a contiguous float64 vector of 2^n entries");
                const auto ptr = (uintptr_t)py::tuple(cai["data"])[0].cast<uint64_t>();
                py::gil_scoped_release rel;
                return b.expect_diagonal(reinterpret_cast<const double*>(ptr), 1);
            }
            auto a = py::array_t<double, py::array::c_style | py::array::forcecast>::ensure(diag);
            if (!a || a.ndim() != 1 || (size_t)a.size() != b.size())
                throw std::invalid_argument("expect_diagonal: a vector of 2^n entries");
            py::gil_scoped_release rel;
            return b.expect_diagonal(a.data(), 0);
        }, py::arg("diag"), "sum_z P(z) diag[z] on the device (no host copy of the probabilities).")
        .def("expect_zz", &GpuBackend::expect_zz, py::arg("a"), py::arg("b"), py::arg("coeff"),
             py::call_guard<py::gil_scoped_release>(),
             "sum_k coeff_k <Z_a Z_b> (b_k < 0: <Z_a>), any number of terms, on the device.");

    m.def("make_gpu_backend",
          [](int n_qubits, const std::string& precision) {
              return std::unique_ptr<GpuBackend>(new GpuBackend(n_qubits, parse_precision(precision)));
          },
          py::arg("n_qubits"), py::arg("precision") = "complex128",
          "GB300 state vector in HBM (IEEE complex128 by default; 'df64' or 'complex64'), up to 34 qubits.");
    m.def("make_statevector_backend",
          [](int n_qubits) { return std::unique_ptr<GpuBackend>(new GpuBackend(n_qubits, LLG_F64)); },
          py::arg("n_qubits"), "The reference's factory name, backed by the GPU engine (complex128).");

    py::class_<GroverResult>(m, "GroverResult")
        .def_property_readonly("probabilities", [](const GroverResult& r) { return to_array(r.probabilities); })
        .def_readonly("marked_index", &GroverResult::marked_index)
        .def_readonly("iterations", &GroverResult::iterations);
    struct GroverNS {};
    py::class_<GroverNS>(m, "Grover")
        .def_static("run", &grover_run, py::arg("backend"), py::arg("n_qubits"), py::arg("marked_states"),
                    py::arg("iterations") = -1, py::call_guard<py::gil_scoped_release>(),
                    "iterations = -1 picks round(pi/(4 theta) - 1/2), theta = asin sqrt(M/N).");

    py::class_<Graph>(m, "Graph")
        .def(py::init<>())
        .def(py::init([](int n_nodes, std::vector<std::tuple<int, int, double>> edges) {
                 Graph g;
                 g.n_nodes = n_nodes;
                 g.edges = std::move(edges);
                 return g;
             }),
             py::arg("n_nodes"), py::arg("edges"))
        .def_readwrite("n_nodes", &Graph::n_nodes)
        .def_readwrite("edges", &Graph::edges)
        .def("add_edge", [](Graph& g, int i, int j, double w) { g.edges.emplace_back(i, j, w); }, py::arg("i"),
             py::arg("j"), py::arg("weight") = 1.0);
    py::class_<QAOAResult>(m, "QAOAResult")
        .def_property_readonly("probabilities", [](const QAOAResult& r) { return to_array(r.probabilities); })
        .def_readonly("best_cut", &QAOAResult::best_cut);
    struct QAOANS {};
    py::class_<QAOANS>(m, "QAOA")
        .def_static("run", &qaoa_run, py::arg("backend"), py::arg("graph"), py::arg("gammas"), py::arg("betas"),
                    py::call_guard<py::gil_scoped_release>(),
                    "p = len(gammas) = len(betas) layers of U_C(gamma) then U_B(beta) on |+>^n.")
        .def_static("cut_value", &cut_value, py::arg("graph"), py::arg("z"), "Cut weight of the bitstring with index z.");

    py::class_<VQEResult>(m, "VQEResult")
        .def_readonly("energy", &VQEResult::energy)
        .def_property_readonly("params", [](const VQEResult& r) { return to_array(r.params); })
        .def_readonly("iterations", &VQEResult::iterations);
    py::class_<VQE>(m, "VQE")
        .def(py::init<int, int, uint64_t>(), py::arg("n_qubits"), py::arg("n_layers"), py::arg("seed") = 1)
        .def_property_readonly("n_qubits", &VQE::n_qubits)
        .def_property_readonly("n_layers", &VQE::n_layers)
        .def_property_readonly("n_params", &VQE::n_params)
        .def("prepare", &VQE::prepare, py::arg("backend"), py::arg("params"), py::call_guard<py::gil_scoped_release>(),
             "Reset the backend and apply the ansatz; params ordered layer by layer, theta[l * n + q].")
        .def("optimize",
             [](const VQE& vqe, GpuBackend& be, const py::function& energy_fn, int max_iter, double lr) {
                 auto fn = [&energy_fn](const std::vector<double>& th) {
                     py::array_t<double> arr((py::ssize_t)th.size(), th.data());
                     return energy_fn(arr).cast<double>();
                 };
                 return vqe.optimize(be, fn, max_iter, lr);
             },
             py::arg("backend"), py::arg("energy_fn"), py::arg("max_iter") = 200, py::arg("lr") = 0.05,
             "energy_fn(params) -> float, typically vqe.prepare(backend, params) then an energy from the backend; "
             "gradients by the parameter-shift rule.");
}
