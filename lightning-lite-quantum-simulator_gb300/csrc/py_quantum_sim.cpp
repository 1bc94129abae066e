// py_quantum_sim.cpp -- pybind11 drop-in for the reference's quantum_sim_v3 / quantum_sim_v2
// modules (src/StateVectorOptimized.cpp:112-134, src/bindings_v2.cpp:87-102), forwarding to the
// C ABI of libllgpu.so.  Built twice: -DLLG_MODULE_V3 and -DLLG_MODULE_V2.
//
// Same class name (StateVector), constructors and method names as the reference, plus the
// ll::StateVectorBackend gate helpers (h, x, rx, ry, rz, cnot, cz, mcz; src/StateVectorBackend.h:
// 61-151) with its error contract (std::invalid_argument -> ValueError).
//
// Ownership differs from the reference in one documented way: amplitudes live in GPU memory.
//  * StateVector(ndarray) copies the array to the GPU and keeps a reference to it; the caller's
//    array is brought up to date at sync points -- get_numpy_view(), sync(), and when the object
//    is destroyed -- not after every gate.  Arrays that are not 1-D C-contiguous complex128 are
//    rejected (TypeError) instead of being force-cast into a temporary.
//  * get_numpy_view() flushes pending gates, copies the amplitudes to a host buffer owned by the
//    object (the caller's array for the ndarray constructor) and returns a view of it whose base
//    is the StateVector, as in the reference.  Writes made to that buffer reach the GPU only
//    through push().
//  * Blocking calls release the GIL.
#include <pybind11/complex.h>
#include <pybind11/numpy.h>
#include <pybind11/pybind11.h>
#include <pybind11/stl.h>

#include <complex>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "llgpu.h"

namespace py = pybind11;

namespace {

void check(int rc) {
    if (rc == LLG_OK) return;
    const std::string msg = llg_last_error();
    if (rc == LLG_EINVAL) throw py::value_error(msg);
    if (rc == LLG_ENOMEM) throw std::bad_alloc();
    throw std::runtime_error(msg);
}

int parse_precision(const std::string& p) {
    if (p == "df64") return LLG_DF64;
    if (p == "complex128" || p == "c128" || p == "fp64" || p == "f64") return LLG_F64;
    if (p == "complex64" || p == "c64" || p == "f32") return LLG_F32;
    throw py::value_error("precision must be 'complex128' (IEEE FP64, default; alias 'fp64'), 'df64' (double-float) "
                          "or 'complex64'");
}

const char* precision_name(int p) {
    return p == LLG_F64 ? "complex128" : (p == LLG_F32 ? "complex64" : "df64");
}

// A 2x2 gate given as any sequence of 4 complex-castable entries (the reference takes a list).
void gate8(const py::handle& g, double out[8]) {
    if (py::isinstance<py::array>(g)) {
        auto a = py::array_t<std::complex<double>, py::array::c_style | py::array::forcecast>::ensure(g);
        if (!a || a.size() != 4) throw py::value_error("gate must have 4 entries");
        const std::complex<double>* d = a.data();
        for (int i = 0; i < 4; ++i) {
            out[2 * i] = d[i].real();
            out[2 * i + 1] = d[i].imag();
        }
        return;
    }
    py::sequence s = py::reinterpret_borrow<py::sequence>(g);
    if (py::len(s) < 4) throw py::index_error("gate must have 4 entries");
    for (int i = 0; i < 4; ++i) {
        const std::complex<double> v = s[i].cast<std::complex<double>>();
        out[2 * i] = v.real();
        out[2 * i + 1] = v.imag();
    }
}

class StateVector {
public:
    explicit StateVector(int n, const std::string& precision) {
        const int p = parse_precision(precision);
        int rc;
        {
            py::gil_scoped_release nogil;
            rc = llg_create(n, p, &st_);
        }
        check(rc);
    }

    StateVector(py::array arr, const std::string& precision) {
        const int p = parse_precision(precision);
        if (!py::isinstance<py::array_t<std::complex<double>>>(arr) || arr.ndim() != 1 ||
            !(arr.flags() & py::array::c_style))
            throw py::type_error("StateVector(ndarray) needs a 1-D C-contiguous complex128 array");
        if (arr.ndim() != 1) throw std::runtime_error("NumPy array must be 1-dimensional");
        user_ = arr;
        has_user_ = true;
        const size_t len = (size_t)arr.shape(0);
        const double* data = static_cast<const double*>(arr.data());
        int rc;
        {
            py::gil_scoped_release nogil;
            rc = llg_create_from_host(data, len, p, &st_);
        }
        check(rc);
    }

    ~StateVector() {
        if (st_ && has_user_) {
            try {
                writeback();
            } catch (...) {
            }
        }
        if (st_) llg_destroy(st_);
        if (mirror_) llg_host_free(mirror_);
    }

    StateVector(const StateVector&) = delete;
    StateVector& operator=(const StateVector&) = delete;

    int num_qubits() const {
        int n = 0;
        check(llg_num_qubits(st_, &n));
        return n;
    }
    uint64_t size() const {
        uint64_t s = 0;
        check(llg_size(st_, &s));
        return s;
    }
    std::string precision() const {
        int p = 0;
        check(llg_get_precision(st_, &p));
        return precision_name(p);
    }

    void apply_gate(int target, py::handle gate) {
        double g[8];
        gate8(gate, g);
        check(llg_apply_gate(st_, target, g));
    }

    void h(int q) { check(llg_h(st_, q)); }
    void x(int q) { check(llg_x(st_, q)); }
    void rx(int q, double t) { check(llg_rx(st_, q, t)); }
    void ry(int q, double t) { check(llg_ry(st_, q, t)); }
    void rz(int q, double t) { check(llg_rz(st_, q, t)); }
    void cnot(int c, int t) { check(llg_cnot(st_, c, t)); }
    void cz(int a, int b) { check(llg_cz(st_, a, b)); }
    void mcz(const std::vector<int>& qs) { check(llg_mcz(st_, qs.data(), (int)qs.size())); }

    // Output of GateFuser.fuse_circuit (python/gate_fusion.py:15-37): (target, [g00, g01, g10, g11])
    void apply_fused(py::iterable fused) {
        for (py::handle item : fused) {
            py::tuple t = py::reinterpret_borrow<py::tuple>(item);
            apply_gate(t[0].cast<int>(), t[1]);
        }
    }

    // dense k-qubit block (k <= 5): `m` is a 2^k x 2^k complex128 array (or nested lists);
    // bit j of its row / column index is qubits[j]
    void apply_matrix(const std::vector<int>& qubits, py::object m) {
        py::array_t<std::complex<double>, py::array::c_style | py::array::forcecast> a(m);
        const size_t dim = (size_t)1 << qubits.size();
        if (qubits.empty() || qubits.size() > 5 || (size_t)a.size() != dim * dim)
            throw py::value_error("apply_matrix: need 1..5 qubits and a 2^k x 2^k matrix");
        check(llg_apply_matrix(st_, (int)qubits.size(), qubits.data(), reinterpret_cast<const double*>(a.data())));
    }

    void apply_ops(py::array ops) {
        if (ops.itemsize() * ops.size() % (py::ssize_t)sizeof(llg_op) != 0 || !(ops.flags() & py::array::c_style))
            throw py::type_error("apply_ops needs a C-contiguous array of llg_op records");
        const int n = (int)(ops.itemsize() * ops.size() / (py::ssize_t)sizeof(llg_op));
        check(llg_apply_ops(st_, static_cast<const llg_op*>(ops.data()), n));
    }

    void set_fusion(const std::string& mode, int tile_qubits) {
        int m;
        if (mode == "tile") m = LLG_FUSE_TILE;
        else if (mode == "reg") m = LLG_FUSE_REG;
        else if (mode == "none") m = LLG_FUSE_NONE;
        else throw py::value_error("fusion mode must be 'tile', 'reg' or 'none'");
        check(llg_set_fusion(st_, m, tile_qubits));
    }

    // picks fusion mode, tile width and CTA threads by timing ops[:sample_ops] on a scratch state
    py::dict autotune(py::array ops, int sample_ops) {
        if (ops.itemsize() * ops.size() % (py::ssize_t)sizeof(llg_op) != 0 || !(ops.flags() & py::array::c_style))
            throw py::type_error("autotune needs a C-contiguous array of llg_op records");
        const int n = (int)(ops.itemsize() * ops.size() / (py::ssize_t)sizeof(llg_op));
        llg_tune_result r;
        check(llg_autotune(st_, static_cast<const llg_op*>(ops.data()), n, sample_ops, &r));
        py::dict d;
        d["fuse_mode"] = r.fuse_mode == LLG_FUSE_TILE ? "tile" : (r.fuse_mode == LLG_FUSE_REG ? "reg" : "none");
        d["tile_qubits"] = r.tile_qubits;
        d["cta_threads"] = r.cta_threads;
        d["candidates"] = r.candidates;
        d["cached"] = r.cached;
        d["best_ms"] = r.best_ms;
        d["default_ms"] = r.default_ms;
        return d;
    }

    void flush() { check(llg_flush(st_)); }

    // Copy amplitudes into the host mirror (or the caller's array) and return a view of it.
    py::array_t<std::complex<double>> get_numpy_view(py::object self) {
        double* buf = host_buffer();
        int rc;
        {
            py::gil_scoped_release nogil;
            rc = llg_copy_to_host(st_, buf);
        }
        check(rc);
        return py::array_t<std::complex<double>>({(py::ssize_t)size()}, {(py::ssize_t)sizeof(std::complex<double>)},
                                                 reinterpret_cast<std::complex<double>*>(buf), self);
    }

    void sync() {
        int rc;
        {
            py::gil_scoped_release nogil;
            rc = llg_sync(st_);
        }
        check(rc);
        if (has_user_) writeback();
        else if (mirror_) {
            py::gil_scoped_release nogil;
            rc = llg_copy_to_host(st_, mirror_);
        }
        check(rc);
    }

    // Upload the host buffer (the caller's array, or the get_numpy_view mirror) to the GPU.
    void push() {
        const double* src = has_user_ ? static_cast<const double*>(user_.data()) : mirror_;
        if (!src) throw std::runtime_error("push: no host buffer (call get_numpy_view first)");
        int rc;
        {
            py::gil_scoped_release nogil;
            rc = llg_copy_from_host(st_, src);
        }
        check(rc);
    }

    py::array_t<double> probabilities() {
        py::array_t<double> out((py::ssize_t)size());
        double* d = out.mutable_data();
        int rc;
        {
            py::gil_scoped_release nogil;
            rc = llg_probabilities(st_, d);
        }
        check(rc);
        return out;
    }

    py::array_t<std::complex<double>> state() {
        py::array_t<std::complex<double>> out((py::ssize_t)size());
        double* d = reinterpret_cast<double*>(out.mutable_data());
        int rc;
        {
            py::gil_scoped_release nogil;
            rc = llg_copy_to_host(st_, d);
        }
        check(rc);
        return out;
    }

    double norm2() {
        double v = 0;
        int rc;
        {
            py::gil_scoped_release nogil;
            rc = llg_norm2(st_, &v);
        }
        check(rc);
        return v;
    }

    double expect_zz(const std::vector<int>& a, const std::vector<int>& b, const std::vector<double>& coeff) {
        if (a.size() != b.size() || a.size() != coeff.size()) throw py::value_error("expect_zz: length mismatch");
        double v = 0;
        int rc;
        {
            py::gil_scoped_release nogil;
            rc = llg_expect_zz(st_, (int)a.size(), a.data(), b.data(), coeff.data(), &v);
        }
        check(rc);
        return v;
    }

    void renormalize() { check(llg_renormalize(st_)); }

    void reset(int n) { check(llg_reset(st_, n)); }

private:
    double* host_buffer() {
        if (has_user_) return static_cast<double*>(user_.mutable_data());
        const size_t bytes = (size_t)size() * 16;
        if (!mirror_) {
            mirror_ = static_cast<double*>(llg_host_alloc(bytes));
            if (!mirror_) throw std::bad_alloc();
        }
        return mirror_;
    }

    void writeback() {
        double* d = static_cast<double*>(user_.mutable_data());
        int rc;
        {
            py::gil_scoped_release nogil;
            rc = llg_copy_to_host(st_, d);
        }
        check(rc);
    }

    llg_state* st_ = nullptr;
    // The caller's array for the ndarray constructor.  A default py::array is an empty array, not a
    // null handle, so `has_user_` (not the handle) says whether there is one.
    py::array user_;
    bool has_user_ = false;
    double* mirror_ = nullptr;
};

}  // namespace

#if defined(LLG_MODULE_V2)
PYBIND11_MODULE(quantum_sim_v2, m) {
    m.doc() = "GPU state vector (GB300), drop-in for quantum_sim_v2";
#else
PYBIND11_MODULE(quantum_sim_v3, m) {
    m.doc() = "GPU state vector (GB300), drop-in for quantum_sim_v3";
#endif
    py::class_<StateVector> cls(m, "StateVector");
    cls.def(py::init<int, const std::string&>(), py::arg("n"), py::arg("precision") = "complex128")
        .def(py::init<py::array, const std::string&>(), py::arg("array"), py::arg("precision") = "complex128")
#if defined(LLG_MODULE_V2)
        .def("apply_gate", &StateVector::apply_gate, py::arg("target"), py::arg("gate"))
#else
        .def("apply_gate_cache_optimized", &StateVector::apply_gate, py::arg("target"), py::arg("gate"))
        .def("apply_gate_standard", &StateVector::apply_gate, py::arg("target"), py::arg("gate"))
#endif
        .def("get_numpy_view", [](py::object self) { return self.cast<StateVector&>().get_numpy_view(self); })
        .def("get_num_qubits", &StateVector::num_qubits)
        .def("get_size", &StateVector::size)
        .def("h", &StateVector::h)
        .def("x", &StateVector::x)
        .def("rx", &StateVector::rx)
        .def("ry", &StateVector::ry)
        .def("rz", &StateVector::rz)
        .def("cnot", &StateVector::cnot)
        .def("cz", &StateVector::cz)
        .def("mcz", &StateVector::mcz)
        .def("apply_fused", &StateVector::apply_fused)
        .def("apply_ops", &StateVector::apply_ops)
        .def("apply_matrix", &StateVector::apply_matrix, py::arg("qubits"), py::arg("matrix"))
        .def("set_fusion", &StateVector::set_fusion, py::arg("mode"), py::arg("tile_qubits") = 0)
        .def("autotune", &StateVector::autotune, py::arg("ops"), py::arg("sample_ops") = 0)
        .def("flush", &StateVector::flush)
        .def("sync", &StateVector::sync)
        .def("push", &StateVector::push)
        .def("probabilities", &StateVector::probabilities)
        .def("state", &StateVector::state)
        .def("norm2", &StateVector::norm2)
        .def("expect_zz", &StateVector::expect_zz)
        .def("renormalize", &StateVector::renormalize)
        .def("reset", &StateVector::reset)
        .def_property_readonly("precision", &StateVector::precision);
    m.attr("LLG_VERSION") = llg_version();
}
