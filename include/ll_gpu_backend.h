// ll_gpu_backend.h -- ll::GpuBackend, a GPU implementation of the reference's ll::Backend
// interface (src/Backend.h:25-45) forwarding every call to the C ABI of libllgpu.so.
//
// Drop-in for ll::StateVectorBackend (src/StateVectorBackend.h:43-219): the reference's
// Algorithms.h (Grover, QAOA, VQE) and Mitigation.h (NoisyBackend, ZNE) compile against it
// unchanged.  Include it after putting the directory that holds the reference's Backend.h on the
// include path, and link with -lllgpu.
//
// Error contract as in the reference: a bad qubit, a non-finite angle, cnot(q, q), an empty or
// repeated mcz list, or reset() outside [1, 34] qubits throw std::invalid_argument; CUDA failures
// (for example, no GPU) throw std::runtime_error.  There is no CPU fallback.
//
// Gates are queued on the device and fused at the next readout (probabilities() / state()), so
// a long gate stream costs a few HBM passes instead of one per gate.
#pragma once

#include <complex>
#include <stdexcept>
#include <string>
#include <vector>

#include "Backend.h"
#include "llgpu.h"

namespace ll {

class GpuBackend final : public Backend {
public:
    // precision: LLG_DF64 (complex128 as double-float, default), LLG_F64 or LLG_F32.
    explicit GpuBackend(int n_qubits = 1, int precision = LLG_DF64) : precision_(precision) {
        check(llg_create(n_qubits, precision_, &st_));
    }
    ~GpuBackend() override {
        if (st_) llg_destroy(st_);
    }
    GpuBackend(const GpuBackend&) = delete;
    GpuBackend& operator=(const GpuBackend&) = delete;

    void reset(int n_qubits) override { check(llg_reset(st_, n_qubits)); }

    int n_qubits() const override {
        int n = 0;
        check(llg_num_qubits(st_, &n));
        return n;
    }

    void h(int q) override { check(llg_h(st_, q)); }
    void x(int q) override { check(llg_x(st_, q)); }
    void rx(int q, double theta) override { check(llg_rx(st_, q, theta)); }
    void ry(int q, double theta) override { check(llg_ry(st_, q, theta)); }
    void rz(int q, double theta) override { check(llg_rz(st_, q, theta)); }
    void cnot(int control, int target) override { check(llg_cnot(st_, control, target)); }
    void mcz(const std::vector<int>& qubits) override {
        check(llg_mcz(st_, qubits.data(), static_cast<int>(qubits.size())));
    }

    std::vector<double> probabilities() const override {
        std::vector<double> p(size());
        check(llg_probabilities(st_, p.data()));
        return p;
    }

    std::vector<std::complex<double>> state() const override {
        std::vector<std::complex<double>> s(size());
        check(llg_copy_to_host(st_, reinterpret_cast<double*>(s.data())));
        return s;
    }

    // Extensions over the interface.
    double expect_zz(const std::vector<int>& a, const std::vector<int>& b, const std::vector<double>& coeff) const {
        double v = 0.0;
        check(llg_expect_zz(st_, static_cast<int>(a.size()), a.data(), b.data(), coeff.data(), &v));
        return v;
    }
    llg_state* handle() const { return st_; }

private:
    static void check(int rc) {
        if (rc == LLG_OK) return;
        const std::string msg = llg_last_error();
        if (rc == LLG_EINVAL) throw std::invalid_argument(msg);
        throw std::runtime_error(msg);
    }
    std::size_t size() const {
        uint64_t s = 0;
        check(llg_size(st_, &s));
        return static_cast<std::size_t>(s);
    }

    llg_state* st_ = nullptr;
    int precision_;
};

}  // namespace ll
