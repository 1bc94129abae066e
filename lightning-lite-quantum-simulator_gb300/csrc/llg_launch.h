// llg_launch.h -- host-side launchers of the state-vector kernels (llg_kernels.cu).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/llgpu.h"
#include "llg_internal.h"

namespace llg {

// Observable sum_k coef[cls[k]] * Z_{a[k]} (Z_{b[k]} if b[k] >= 0), terms grouped into at most
// kMaxZClasses coefficient classes so the kernels count parities per class in integers.
constexpr int kMaxZTerms = 64;
constexpr int kMaxZClasses = 4;
struct ZTerms {
    int32_t nterms;
    int32_t nclass;
    int32_t a[kMaxZTerms];
    int32_t b[kMaxZTerms];
    int32_t cls[kMaxZTerms];
    double coef[kMaxZClasses];
};

// Per-block partial results of a reduction: up to kRedSlots doubles per block (kCmpSlots for the
// two-state comparison); the engine's partial buffer holds kRedBlocks x kPartialSlots doubles.
constexpr int kRedSlots = 1 + kMaxZClasses;
constexpr int kCmpSlots = 6;
constexpr int kPartialSlots = 8;
constexpr int kRedBlocks = 1024;

size_t elem_bytes(int precision);

cudaError_t launch_init_basis(int P, void* psi, uint64_t size, uint64_t index, cudaStream_t s);
cudaError_t launch_exec_op(int P, void* psi, int n, const ExecOp& op, cudaStream_t s);
// threads: CTA size of the tile kernel (0: 512 for tiles of 10+ qubits, else half the tile)
// mirror: nullptr, or the device address of a host buffer that also receives the pass's output as
// FP64 (2 doubles per amplitude, full-state indexing)
// d_tables: the plan's phase tables (Plan::tables on the device), or nullptr for a plan without
// EX_PTAB ops; err_flag: a device int of the caller's that a CTA sets to 1 when its bulk tile load
// does not complete within the wait limit (the CTA then stores nothing)
cudaError_t launch_tile_pass(int P, void* psi, int n, const PassDesc& pd, const ExecOp* d_ops, const uint64_t* d_tables,
                             int threads, int* err_flag, cudaStream_t s, double* mirror = nullptr);
cudaError_t launch_from_f64(int P, const double* src, void* dst, uint64_t count, cudaStream_t s);
cudaError_t launch_to_f64(int P, const void* src, double* dst, uint64_t count, cudaStream_t s);
cudaError_t launch_probabilities(int P, const void* psi, double* out, uint64_t count, cudaStream_t s);
cudaError_t launch_scale(int P, void* psi, uint64_t count, double factor, cudaStream_t s);
// Writes [norm2, W_0 .. W_{nclass-1}] (W_c = sum_i |a_i|^2 * #odd-parity terms of class c in i)
// to d_out (device, kRedSlots doubles), via d_partials (device, kRedBlocks * kRedSlots doubles).
cudaError_t launch_reduce_z(int P, const void* psi, int n, const ZTerms& terms, double* d_partials, double* d_out,
                            cudaStream_t s);

// Two states of equal size, any precisions: per block (kCmpSlots doubles each) Re <a|b>, Im <a|b>,
// <a|a>, <b|b>, max |a_i - b_i| and max |b_i| (over re and im parts); *nblocks = blocks written
cudaError_t launch_compare(int PA, const void* a, int PB, const void* b, uint64_t size, double* partials, int* nblocks,
                           cudaStream_t s);

int tile_max_qubits(int P);

// register-tiled pass (llg_tile_reg.cu) over a register program (to_register_program): complex64
// states, pd.t in [9, 13]; 2^(t-4) threads per CTA
cudaError_t launch_tile_reg(int P, void* psi, int n, const PassDesc& pd, const ExecOp* d_ops, cudaStream_t s,
                            double* mirror = nullptr);

// FP64 FMA operations per second of the current device (one timed launch of `iters` iterations)
cudaError_t fp64_fma_rate(int iters, double* fma_per_s);

// dense k-qubit block (llg_block.cu): bit j of a row/column index is qubit q[j]; the matrix is
// 2 * 4^k coefficient slots, row-major (re, im), packed for the state's precision
constexpr int kMaxBlockQubits = 5;
constexpr int kMaxBlockDim = 1 << kMaxBlockQubits;
struct BlockDesc {
    int32_t k;
    int32_t q[kMaxBlockQubits];
    uint64_t tmask;
};
cudaError_t launch_block(int P, void* psi, int n, const BlockDesc& bd, const uint64_t* d_mat, cudaStream_t s);
// Which entries of a block of k <= 4 qubits are nonzero (bit c of rows[r]) and real (bit c of
// real[r]); the block kernel then sums row r over those columns only.
struct BlockSparsity {
    uint32_t rows[16];
    uint32_t real[16];
};
cudaError_t launch_block_sparse(int P, void* psi, int n, const BlockDesc& bd, const uint64_t* d_mat,
                                const BlockSparsity& nz, cudaStream_t s);

// 4- and 5-qubit blocks on double-float states of at least k + 7 qubits on the tensor cores
// (llg_block_tc.cu): the host slices the matrix (2 * 4^k doubles, row-major re/im) into
// block_tc_weight_bytes(k) of device input; a kernel whose products do not arrive within its
// wait limit sets *err_flag (a device int of the caller's) to 1
bool block_tc_eligible(int P, int n, int k);
size_t block_tc_weight_bytes(int P, int k);
void block_tc_prepare(int P, int k, const double* m, void* weights);
cudaError_t launch_block_tc(int P, void* psi, int n, const BlockDesc& bd, const void* d_weights, int* err_flag,
                            cudaStream_t s);

// process-wide tuning cache (llg_tune.cu), keyed by an FNV-1a hash of the workload's shape
uint64_t tune_hash(uint64_t h, uint64_t v);
uint64_t tune_hash_ops(uint64_t h, const llg_op* ops, int nops);
bool tune_cache_get(uint64_t key, llg_tune_result* out);
void tune_cache_put(uint64_t key, const llg_tune_result& r);

}  // namespace llg
