// llg_diag.h -- diagonal observables of any size: O = sum_k c_k Z_{a_k} Z_{b_k} (b_k < 0: the single
// Z_{a_k}) with any number of terms and any coefficients -- the reference's ising_diagonal(n, zz, z)
// (python/algorithms.py:139-152) -- evaluated without ever materialising the 2^n diagonal.
//
// Layout for the chunked kernels (llg_diag.cu): the register's index splits into the low L bits
// (L = min(n, 12)) and the rest.  A chunk is 2^L contiguous amplitudes with fixed high bits, and
//   d(i) = T_lo[lo] + H1[lo mod 2^L1] + H2[lo >> L1] + d_hi
// where T_lo (host-built, 2^L doubles) sums the terms inside the low bits, d_hi sums the terms
// inside the high bits at the chunk's high index, and the terms that couple a low qubit a to a
// high qubit b become a field h_a = sum c z_b(hi) on the low qubits, tabulated per chunk over the
// first L1 and the last L - L1 low qubits (H1, H2: 2^L1 and 2^(L-L1) entries).  Per amplitude that
// is three table reads and three additions, whatever the number of terms.
//
// Plain C++ (no CUDA types): the builder and its host evaluator compile and are tested without a
// GPU.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

namespace llg {

constexpr int kDiagMaxLow = 12;

// Device view of a built observable (pointers into one device buffer); diag != nullptr means a
// full 2^n diagonal read per amplitude instead of the terms.
struct DiagObs {
    int32_t n, L, L1, n_hi;
    int32_t n_cross, pad0;
    const double* t_lo;        // 2^L
    const int32_t* hi_ab;      // n_hi pairs (a, b), both >= L (b = -1: Z_a alone)
    const double* hi_c;        // n_hi coefficients
    const int32_t* cross_off;  // L + 1 offsets into cross_b / cross_c, one run per low qubit
    const int32_t* cross_b;    // the high qubit of each coupling term
    const double* cross_c;
    const double* diag;
};

// Host image of a built observable: one byte buffer (uploaded as is) and the offsets of its parts.
struct DiagObsHost {
    int n = 0, L = 0, L1 = 0, n_hi = 0, n_cross = 0, nterms = 0;
    std::vector<unsigned char> bytes;
    size_t off_tlo = 0, off_hi_ab = 0, off_hi_c = 0, off_cross_off = 0, off_cross_b = 0, off_cross_c = 0;
    // the source terms (to recognise a repeated observable)
    std::vector<int32_t> a, b;
    std::vector<double> c;
};

// Validates and lays out the terms (a[k] in [0, n), b[k] in [0, n) and != a[k], or b[k] < 0;
// finite coefficients).  Returns false with `err` set otherwise.
bool build_diag_obs(int n, int nterms, const int* a, const int* b, const double* c, DiagObsHost& out, std::string& err);

// True when `h` was built from exactly these terms on n qubits.
bool diag_obs_same(const DiagObsHost& h, int n, int nterms, const int* a, const int* b, const double* c);

// The device view of `h` once its bytes live at `dev` (16-byte aligned).
DiagObs diag_obs_view(const DiagObsHost& h, const void* dev);

// d(i) for every basis index by the chunked decomposition, on the host (tests and introspection).
void diag_obs_eval_host(const DiagObsHost& h, double* out);

}  // namespace llg
