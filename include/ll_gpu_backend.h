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

#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <functional>
#include <stdexcept>
#include <string>
#include <vector>

#include "Backend.h"
#include "llgpu.h"

namespace ll {

class GpuBackend final : public Backend {
public:
    // precision: LLG_F64 (complex128 in IEEE binary64, the reference's arithmetic; default),
    // LLG_DF64 (double-float, faster on this GPU) or LLG_F32 (complex64).
    explicit GpuBackend(int n_qubits = 1, int precision = LLG_F64) : precision_(precision) {
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

// Records the gates a circuit function applies, as llg_op records, without a state: the input of
// the batched trajectory engines.  Validates like the reference's backends (invalid_argument on
// a bad qubit, a non-finite angle, cnot(q, q) or an empty / repeated mcz list).
class RecordingBackend final : public Backend {
public:
    explicit RecordingBackend(int n_qubits = 1) { reset(n_qubits); }

    void reset(int n_qubits) override {
        if (n_qubits < 1 || n_qubits > 14) throw std::invalid_argument("RecordingBackend: n must be in [1, 14]");
        n_ = n_qubits;
        ops_.clear();
    }
    int n_qubits() const override { return n_; }

    void h(int q) override { push(LLG_OP_H, q); }
    void x(int q) override { push(LLG_OP_X, q); }
    void rx(int q, double t) override { push(LLG_OP_RX, q, 0, t); }
    void ry(int q, double t) override { push(LLG_OP_RY, q, 0, t); }
    void rz(int q, double t) override { push(LLG_OP_RZ, q, 0, t); }
    void cnot(int control, int target) override {
        if (control == target) throw std::invalid_argument("cnot: control == target");
        qubit(target);
        push(LLG_OP_CNOT, control, target);
    }
    void mcz(const std::vector<int>& qubits) override {
        if (qubits.empty()) throw std::invalid_argument("mcz: empty qubit list");
        uint64_t mask = 0;
        for (int q : qubits) {
            qubit(q);
            if ((mask >> q) & 1) throw std::invalid_argument("mcz: repeated qubit");
            mask |= 1ULL << q;
        }
        llg_op op = blank(LLG_OP_MCZ, qubits[0]);
        op.mask = mask;
        ops_.push_back(op);
    }

    std::vector<double> probabilities() const override {
        throw std::logic_error("RecordingBackend holds no state");
    }
    std::vector<std::complex<double>> state() const override {
        throw std::logic_error("RecordingBackend holds no state");
    }

    const std::vector<llg_op>& ops() const { return ops_; }

private:
    void qubit(int q) const {
        if (q < 0 || q >= n_) throw std::invalid_argument("qubit " + std::to_string(q) + " out of range");
    }
    static llg_op blank(int kind, int q0) {
        llg_op op;
        std::memset(&op, 0, sizeof(op));
        op.kind = kind;
        op.q0 = q0;
        op.param = -1;
        return op;
    }
    void push(int kind, int q0, int q1 = 0, double theta = 0.0) {
        qubit(q0);
        if (!std::isfinite(theta)) throw std::invalid_argument("non-finite angle");
        llg_op op = blank(kind, q0);
        op.q1 = q1;
        op.theta = theta;
        ops_.push_back(op);
    }

    int n_ = 1;
    std::vector<llg_op> ops_;
};

// One diagonal observable term coeff * Z_a Z_b (b < 0: coeff * Z_a).
struct GpuZTerm {
    int a;
    int b;
    double coeff;
};

// Same fields as the reference's ll::ZNEResult (src/Mitigation.h:247-255).
struct GpuZNEResult {
    double value = 0.0;
    double std_error = 0.0;
    std::vector<double> scales, values, std_errors, weights;
    int trajectories = 0;
};

// ll::ZNE (src/Mitigation.h:258-377) with ll::NoisyBackend's depolarizing model, batched: the
// circuit function is recorded once, and every scale's trajectories run in one persistent GPU
// launch (llg_zne_run).  The observable is diagonal (a sum of Z / ZZ terms, at most 16 with at
// most 3 distinct coefficients), the form the reference's own ZNE checks use.  Uniforms come
// from Philox4x32-10 per (site, trajectory), not the reference's sequential mt19937_64 stream,
// so results agree with the reference in distribution, not draw for draw.
class GpuZNE {
public:
    explicit GpuZNE(int trajectories = 1000, int precision = LLG_F64) : trajectories_(trajectories), precision_(precision) {
        if (trajectories < 1) throw std::invalid_argument("ZNE: trajectories must be >= 1");
    }

    GpuZNEResult extrapolate(int n_qubits, double p, std::uint64_t seed, const std::function<void(Backend&)>& circuit_fn,
                             const std::vector<GpuZTerm>& observable,
                             const std::vector<double>& scales = {1.0, 3.0, 5.0}) const {
        if (!circuit_fn) throw std::invalid_argument("ZNE::extrapolate: circuit_fn is empty");
        RecordingBackend rec(n_qubits);
        circuit_fn(rec);
        std::vector<int> a, b;
        std::vector<double> c;
        for (const GpuZTerm& t : observable) {
            a.push_back(t.a);
            b.push_back(t.b);
            c.push_back(t.coeff);
        }
        llg_zne_result r;
        const int rc = llg_zne_run(n_qubits, rec.ops().data(), static_cast<int>(rec.ops().size()), p, precision_,
                                   scales.data(), static_cast<int>(scales.size()), trajectories_, seed,
                                   static_cast<int>(a.size()), a.data(), b.data(), c.data(), &r);
        if (rc == LLG_EINVAL) throw std::invalid_argument(llg_last_error());
        if (rc != LLG_OK) throw std::runtime_error(llg_last_error());
        GpuZNEResult out;
        out.value = r.value;
        out.std_error = r.std_error;
        out.trajectories = static_cast<int>(r.trajectories);
        out.scales.assign(r.scales, r.scales + r.nscales);
        out.values.assign(r.values, r.values + r.nscales);
        out.std_errors.assign(r.std_errors, r.std_errors + r.nscales);
        out.weights.assign(r.weights, r.weights + r.nscales);
        return out;
    }

private:
    int trajectories_;
    int precision_;
};

}  // namespace ll
