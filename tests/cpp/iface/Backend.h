// The ll::Backend interface restated for builds where the reference tree is absent (the GPU test
// machine).  It must stay signature-identical to the reference's src/Backend.h:25-45 so
// ll::GpuBackend compiles against either; only the abstract interface is restated here.
#pragma once

#include <complex>
#include <vector>

namespace ll {

class Backend {
public:
    virtual ~Backend() = default;
    virtual void reset(int n_qubits) = 0;
    virtual int n_qubits() const = 0;
    virtual void h(int q) = 0;
    virtual void x(int q) = 0;
    virtual void rx(int q, double theta) = 0;
    virtual void ry(int q, double theta) = 0;
    virtual void rz(int q, double theta) = 0;
    virtual void cnot(int control, int target) = 0;
    virtual void mcz(const std::vector<int>& qubits) = 0;
    virtual std::vector<double> probabilities() const = 0;
    virtual std::vector<std::complex<double>> state() const = 0;
};

}  // namespace ll
