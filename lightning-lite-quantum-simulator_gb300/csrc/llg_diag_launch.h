// llg_diag_launch.h -- host launchers of the diagonal-observable kernels (llg_diag.cu).
#pragma once

#include <cuda_runtime.h>

#include "llg_diag.h"

namespace llg {

// Largest grid of the expectation kernel: d_partials holds 2 doubles per block.
constexpr int kDiagMaxBlocks = 1024;

// Blocks the expectation kernel uses for n qubits (a chunk of 2^L amplitudes at least per block).
int diag_expect_blocks(int n);

// d_out[0] = sum_i |a_i|^2 d(i), d_out[1] = sum_i |a_i|^2 (device), via d_partials (device,
// 2 * kDiagMaxBlocks doubles).  o.diag set: d(i) read from that 2^n device array.
cudaError_t launch_expect_diag(int P, const void* psi, const DiagObs& o, double* d_partials, double* d_out,
                               cudaStream_t s);

// For `batch` states of 2^o.n amplitudes side by side: lam = O psi (lam_all may be nullptr) and
// d_energies[b] = sum_i |psi_b,i|^2 d(i); d_epart holds batch * blocks doubles.
cudaError_t launch_lambda_diag(int P, const void* psi_all, void* lam_all, const DiagObs& o, int batch, int blocks,
                               double* d_epart, double* d_energies, cudaStream_t s);

}  // namespace llg
