// llg_diag.cu -- diagonal observables of any size on the device (layout: llg_diag.h).
//
//  * k_expect_diag: sum_i |a_i|^2 d(i) and sum_i |a_i|^2 of one state -- the reference's
//    energy = probabilities() . diag (python/algorithms.py:177-179) with the diagonal of
//    ising_diagonal (python/algorithms.py:139-152) computed on the fly, or read from a full
//    2^n diagonal in device memory.
//  * k_lambda_diag: for a batch of states, lambda = O psi and the per-state energies (the adjoint
//    method's starting bra).
// Each CTA walks chunks of 2^L contiguous amplitudes (grid-stride): it tabulates the chunk's
// coupling field (H1, H2) and high-bit sum in shared memory, then reads every amplitude once
// (coalesced).  Accumulation is per thread in the state's accumulator (double for FP64 states,
// double-float otherwise); the sums across threads, warps and CTAs are in IEEE double, in a fixed
// order.
#include <cuda_runtime.h>

#include "llg_common.cuh"
#include "llg_diag.h"
#include "llg_diag_launch.h"

namespace llg {

namespace {

constexpr int kThreadsD = 256;

struct DiagSmem {
    double tlo[1 << kDiagMaxLow];
    double h1[1 << (kDiagMaxLow / 2)];
    double h2[1 << (kDiagMaxLow - kDiagMaxLow / 2)];
    double heff[kDiagMaxLow];
    double dhi;
};

__device__ __forceinline__ double block_sum_dbl(double v, double* sh) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    double r = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) r += sh[w];
    return r;
}

// The chunk's coupling field and high-bit sum (ends with a barrier; the caller must have
// finished reading the previous chunk's tables, i.e. passed a barrier, before calling).
__device__ void diag_chunk_prep(const DiagObs& o, uint64_t hi, DiagSmem& s) {
    const int L = o.L, L1 = o.L1, L2 = L - L1;
    const int t = threadIdx.x;
    if (t < L) {
        double v = 0.0;
        for (int k = o.cross_off[t]; k < o.cross_off[t + 1]; ++k) v += ((hi >> o.cross_b[k]) & 1) ? -o.cross_c[k] : o.cross_c[k];
        s.heff[t] = v;
    }
    const int last_warp = (int)(blockDim.x >> 5) - 1;
    if ((t >> 5) == last_warp) {  // the high-bit terms, one warp, lanes in a fixed order
        const int lane = t & 31;
        double v = 0.0;
        for (int k = lane; k < o.n_hi; k += 32) {
            int par = (int)((hi >> o.hi_ab[2 * k]) & 1);
            const int b = o.hi_ab[2 * k + 1];
            if (b >= 0) par ^= (int)((hi >> b) & 1);
            v += par ? -o.hi_c[k] : o.hi_c[k];
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
        if (lane == 0) s.dhi = v;
    }
    __syncthreads();
    const int n1 = 1 << L1, n2 = 1 << L2;
    for (int j = t; j < n1 + n2; j += blockDim.x) {
        if (j < n1) {
            double v = 0.0;
            for (int l = 0; l < L1; ++l) v += ((j >> l) & 1) ? -s.heff[l] : s.heff[l];
            s.h1[j] = v;
        } else {
            const int jj = j - n1;
            double v = 0.0;
            for (int l = 0; l < L2; ++l) v += ((jj >> l) & 1) ? -s.heff[L1 + l] : s.heff[L1 + l];
            s.h2[jj] = v;
        }
    }
    __syncthreads();
}

__device__ __forceinline__ double diag_value(const DiagSmem& s, uint32_t lo, int L1) {
    return ((s.tlo[lo] + s.h1[lo & ((1u << L1) - 1)]) + s.h2[lo >> L1]) + s.dhi;
}

template <class P>
__global__ void __launch_bounds__(kThreadsD) k_expect_diag(const typename P::S* __restrict__ psi, DiagObs o,
                                                           double* __restrict__ partials) {
    __shared__ DiagSmem s;
    __shared__ double red[kThreadsD / 32];
    typename P::Acc ae = P::acc_zero(), an = P::acc_zero();
    const uint64_t size = 1ULL << o.n;
    if (o.diag) {
        const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
        for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < size; i += step) {
            const auto a = P::load(psi[i]);
            ae = P::acc_norm_d(ae, a, o.diag[i]);
            an = P::acc_norm(an, a);
        }
    } else {
        const int L = o.L;
        const uint32_t csize = 1u << L;
        for (uint32_t l = threadIdx.x; l < csize; l += blockDim.x) s.tlo[l] = o.t_lo[l];
        const uint64_t nchunks = size >> L;
        for (uint64_t ch = blockIdx.x; ch < nchunks; ch += gridDim.x) {
            const uint64_t hi = ch << L;
            diag_chunk_prep(o, hi, s);
            for (uint32_t lo = threadIdx.x; lo < csize; lo += blockDim.x) {
                const auto a = P::load(psi[hi | lo]);
                ae = P::acc_norm_d(ae, a, diag_value(s, lo, o.L1));
                an = P::acc_norm(an, a);
            }
            __syncthreads();  // the tables are read before the next chunk rewrites them
        }
    }
    const double e = block_sum_dbl(P::acc_to_double(ae), red);
    const double nn = block_sum_dbl(P::acc_to_double(an), red);
    if (threadIdx.x == 0) {
        partials[2 * (size_t)blockIdx.x] = e;
        partials[2 * (size_t)blockIdx.x + 1] = nn;
    }
}

// out[0] = energy, out[1] = norm^2: per-block partials summed in block order
__global__ void k_finish_diag(const double* __restrict__ partials, int nblocks, double* __restrict__ out) {
    const int s = threadIdx.x;
    if (s >= 2) return;
    double r = 0.0;
    for (int b = 0; b < nblocks; ++b) r += partials[2 * (size_t)b + s];
    out[s] = r;
}

// Batch b of grid.y: lambda_b = O psi_b (if lam != nullptr) and per-block energy partials
// epart[b][blockIdx.x].
template <class P>
__global__ void __launch_bounds__(kThreadsD) k_lambda_diag(const typename P::S* __restrict__ psi_all,
                                                           typename P::S* __restrict__ lam_all, DiagObs o,
                                                           double* __restrict__ epart) {
    __shared__ DiagSmem s;
    __shared__ double red[kThreadsD / 32];
    const uint64_t size = 1ULL << o.n;
    const uint64_t b = blockIdx.y;
    const typename P::S* psi = psi_all + b * size;
    typename P::S* lam = lam_all ? lam_all + b * size : nullptr;
    typename P::Acc ae = P::acc_zero();
    const int L = o.L;
    const uint32_t csize = 1u << L;
    for (uint32_t l = threadIdx.x; l < csize; l += blockDim.x) s.tlo[l] = o.t_lo[l];
    const uint64_t nchunks = size >> L;
    for (uint64_t ch = blockIdx.x; ch < nchunks; ch += gridDim.x) {
        const uint64_t hi = ch << L;
        diag_chunk_prep(o, hi, s);
        for (uint32_t lo = threadIdx.x; lo < csize; lo += blockDim.x) {
            const auto a = P::load(psi[hi | lo]);
            const double d = diag_value(s, lo, o.L1);
            ae = P::acc_norm_d(ae, a, d);
            if (lam) {
                const auto k = P::k_from_double(d);
                typename P::C out;
                out.re = P::mulk(k, a.re);
                out.im = P::mulk(k, a.im);
                lam[hi | lo] = P::store(out);
            }
        }
        __syncthreads();
    }
    const double e = block_sum_dbl(P::acc_to_double(ae), red);
    if (threadIdx.x == 0) epart[b * gridDim.x + blockIdx.x] = e;
}

__global__ void k_finish_lambda(const double* __restrict__ epart, int blocks, int batch, double* __restrict__ energies) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= batch) return;
    double e = 0.0;
    for (int k = 0; k < blocks; ++k) e += epart[(size_t)b * blocks + k];
    energies[b] = e;
}

int sms_of_current_device() {
    int dev = 0, sms = 1;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
        cudaGetLastError();
        return 1;
    }
    return sms > 0 ? sms : 1;
}

#define LLG_DDISPATCH(P, ...)                                \
    switch (P) {                                             \
        case 0: { using Pol = PolF64; __VA_ARGS__; }         \
        case 1: { using Pol = PolDF64; __VA_ARGS__; }        \
        case 2: { using Pol = PolF32; __VA_ARGS__; }         \
        default: return cudaErrorInvalidValue;               \
    }

}  // namespace

int diag_expect_blocks(int n) {
    const uint64_t size = 1ULL << n;
    const uint64_t nchunks = size >> (n < kDiagMaxLow ? n : kDiagMaxLow);
    const uint64_t cap = (uint64_t)sms_of_current_device() * 4;
    uint64_t g = nchunks < cap ? nchunks : cap;
    if (g > (uint64_t)kDiagMaxBlocks) g = kDiagMaxBlocks;
    return (int)(g < 1 ? 1 : g);
}

cudaError_t launch_expect_diag(int P, const void* psi, const DiagObs& o, double* d_partials, double* d_out,
                               cudaStream_t s) {
    int g = diag_expect_blocks(o.n);
    if (o.diag) {  // a full diagonal: plain grid-stride, no chunks
        const uint64_t want = ((1ULL << o.n) + kThreadsD * 4 - 1) / (kThreadsD * 4);
        const uint64_t cap = (uint64_t)sms_of_current_device() * 16 < (uint64_t)kDiagMaxBlocks
                                 ? (uint64_t)sms_of_current_device() * 16
                                 : (uint64_t)kDiagMaxBlocks;
        g = (int)(want < 1 ? 1 : (want > cap ? cap : want));
    }
    LLG_DDISPATCH(P, k_expect_diag<Pol><<<g, kThreadsD, 0, s>>>(static_cast<const typename Pol::S*>(psi), o, d_partials);
                  cudaError_t e = cudaGetLastError(); if (e != cudaSuccess) return e;
                  k_finish_diag<<<1, 32, 0, s>>>(d_partials, g, d_out); return cudaGetLastError());
}

cudaError_t launch_lambda_diag(int P, const void* psi_all, void* lam_all, const DiagObs& o, int batch, int blocks,
                               double* d_epart, double* d_energies, cudaStream_t s) {
    const dim3 grid((unsigned)blocks, (unsigned)batch);
    LLG_DDISPATCH(P, k_lambda_diag<Pol><<<grid, kThreadsD, 0, s>>>(static_cast<const typename Pol::S*>(psi_all),
                                                                   static_cast<typename Pol::S*>(lam_all), o, d_epart);
                  cudaError_t e = cudaGetLastError(); if (e != cudaSuccess) return e;
                  k_finish_lambda<<<(batch + 127) / 128, 128, 0, s>>>(d_epart, blocks, batch, d_energies);
                  return cudaGetLastError());
}

}  // namespace llg
