// llg_block.cu -- dense k-qubit blocks (llg_apply_matrix, include/llgpu.h): a 2^k x 2^k complex
// matrix applied to every group of 2^k amplitudes that differ only in the k target qubits, the
// fused form of python/gate_fusion.py:7-37 widened to k qubits (k <= 5).
//
// k <= 3 (k_group): one thread per group holds its 2^k amplitudes in registers and forms the rows
// of M a one after another, storing each as it is done; the matrix and the 2^k target offsets are
// read from shared memory by broadcast.  k = 4, 5 (k_block): one warp holds 32 >> k groups, one
// lane per row: lane r of a group loads amplitude r (the group's base index with the bits of r
// deposited at the target positions, bit j -> qubits[j]), then forms row r of M a with the group's
// amplitudes broadcast by warp shuffles; the matrix sits in shared memory.  complex128 (double-float) rows are accumulated as exact products summed with
// TwoSum (the Dot2 scheme of Ogita, Rump and Oishi, SIAM J. Sci. Comput. 2005) and rounded once to
// double-float; FP64 and complex64 rows use fused multiply-adds.
#include <cuda_runtime.h>

#include "llg_common.cuh"
#include "llg_internal.h"
#include "llg_launch.h"

namespace llg {

namespace {

constexpr int kBlockThreads = 256;

__device__ __forceinline__ float shfl(float v, int src) { return __shfl_sync(0xffffffffu, v, src); }
__device__ __forceinline__ double shfl(double v, int src) { return __shfl_sync(0xffffffffu, v, src); }
__device__ __forceinline__ df shfl(df v, int src) { return {shfl(v.hi, src), shfl(v.lo, src)}; }

// Row accumulators: sum of products a * b (DotDF, the double-float Dot2, is in llg_common.cuh).
struct DotD {
    double s = 0.0;
    __device__ __forceinline__ void add(double a, double b) { s = fma(a, b, s); }
    __device__ __forceinline__ double value() const { return s; }
};
struct DotF {
    float s = 0.0f;
    __device__ __forceinline__ void add(float a, float b) { s = fmaf(a, b, s); }
    __device__ __forceinline__ float value() const { return s; }
};
template <class P> struct DotOf;
template <> struct DotOf<PolDF64> { using T = DotDF; };
template <> struct DotOf<PolF64> { using T = DotD; };
template <> struct DotOf<PolF32> { using T = DotF; };

template <class P>
__global__ void __launch_bounds__(kBlockThreads) k_block(typename P::S* __restrict__ psi, int n, BlockDesc bd,
                                                         const uint64_t* __restrict__ mat) {
    using K = typename P::K;
    using C = typename P::C;
    using D = typename DotOf<P>::T;
    // (re, im) per entry, stored transposed (column-major): at step j the lanes of a group read
    // M[r][j] for consecutive r, so a warp's reads are contiguous instead of one bank apart
    __shared__ K sm[2 * kMaxBlockDim * kMaxBlockDim];
    const int k = bd.k, dk = 1 << k;
    for (int i = threadIdx.x; i < dk * dk; i += blockDim.x) {
        const int row = i / dk, col = i % dk;
        sm[2 * (col * dk + row)] = P::k_from_bits(mat[2 * i]);
        sm[2 * (col * dk + row) + 1] = P::k_from_bits(mat[2 * i + 1]);
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int r = lane & (dk - 1);
    const int gsub = lane >> k;
    const int gpw = 32 >> k;
    uint64_t toff = 0;
    for (int j = 0; j < k; ++j)
        if ((r >> j) & 1) toff |= 1ULL << bd.q[j];
    const uint64_t ngroups = 1ULL << (n - k);
    const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    // g0 is the same on every lane of the warp, so every shuffle below has all 32 lanes
    for (uint64_t g0 = warp * gpw; g0 < ngroups; g0 += nwarps * gpw) {
        const uint64_t g = g0 + (uint64_t)gsub;
        const bool valid = g < ngroups;
        const uint64_t idx = insert0_mask(valid ? g : 0, bd.tmask) | toff;
        C a;
        if (valid) a = P::load(psi[idx]);
        else a.re = a.im = P::zero();
        D re, im;
        const int src0 = gsub << k;
        for (int j = 0; j < dk; ++j) {
            const auto xr = shfl(a.re, src0 | j), xi = shfl(a.im, src0 | j);
            const K mr = sm[2 * (j * dk + r)], mi = sm[2 * (j * dk + r) + 1];
            re.add(mr, xr);
            re.add(P::kneg(mi), xi);
            im.add(mr, xi);
            im.add(mi, xr);
        }
        C out;
        out.re = re.value();
        out.im = im.value();
        if (valid) psi[idx] = P::store(out);
    }
}

template <class P, int K>
__global__ void __launch_bounds__(kBlockThreads) k_group(typename P::S* __restrict__ psi, int n, BlockDesc bd,
                                                         const uint64_t* __restrict__ mat) {
    using Kt = typename P::K;
    using C = typename P::C;
    using D = typename DotOf<P>::T;
    constexpr int A = 1 << K;
    __shared__ Kt sm[2 * A * A];  // row-major (re, im)
    __shared__ uint64_t soff[A];  // the bits of j deposited at the target qubits
    for (int i = threadIdx.x; i < 2 * A * A; i += blockDim.x) sm[i] = P::k_from_bits(mat[i]);
    for (int j = threadIdx.x; j < A; j += blockDim.x) {
        uint64_t off = 0;
        for (int b = 0; b < K; ++b)
            if ((j >> b) & 1) off |= 1ULL << bd.q[b];
        soff[j] = off;
    }
    __syncthreads();
    const uint64_t ngroups = 1ULL << (n - K);
    const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; g < ngroups; g += step) {
        const uint64_t base = insert0_mask(g, bd.tmask);
        C a[A];
#pragma unroll
        for (int j = 0; j < A; ++j) a[j] = P::load(psi[base | soff[j]]);
        // rows rolled: the matrix is read from shared memory per row instead of being hoisted
        // into registers for the whole loop over groups
#pragma unroll 1
        for (int r = 0; r < A; ++r) {
            D re, im;
#pragma unroll
            for (int j = 0; j < A; ++j) {
                const Kt mr = sm[2 * (r * A + j)], mi = sm[2 * (r * A + j) + 1];
                re.add(mr, a[j].re);
                re.add(P::kneg(mi), a[j].im);
                im.add(mr, a[j].im);
                im.add(mi, a[j].re);
            }
            C out;
            out.re = re.value();
            out.im = im.value();
            psi[base | soff[r]] = P::store(out);
        }
    }
}

// The sparse block for double-float and complex64 states: the group's amplitudes in registers and
// row r tested against uniform masks of its nonzero (bit c of nz.rows[r]) and real (bit c of
// nz.real[r]) entries.  The compiler may issue the skipped terms as predicated-off instructions,
// which costs little on the wide FP32 pipe; measured 15-25 % faster than the list form below for
// double-float density-matrix channels.
template <class P, int K>
__global__ void __launch_bounds__(kBlockThreads) k_group_sparse_masks(typename P::S* __restrict__ psi, int n, BlockDesc bd,
                                                                const uint64_t* __restrict__ mat, BlockSparsity nz) {
    using Kt = typename P::K;
    using C = typename P::C;
    constexpr int A = 1 << K;
    __shared__ Kt sm[2 * A * A];  // row-major (re, im)
    __shared__ uint64_t soff[A];
    __shared__ uint32_t srows[A], sreal[A];
    for (int i = threadIdx.x; i < 2 * A * A; i += blockDim.x) sm[i] = P::k_from_bits(mat[i]);
    for (int j = threadIdx.x; j < A; j += blockDim.x) {
        uint64_t off = 0;
        for (int b = 0; b < K; ++b)
            if ((j >> b) & 1) off |= 1ULL << bd.q[b];
        soff[j] = off;
        srows[j] = nz.rows[j];
        sreal[j] = nz.real[j];
    }
    __syncthreads();
    const uint64_t ngroups = 1ULL << (n - K);
    const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; g < ngroups; g += step) {
        const uint64_t base = insert0_mask(g, bd.tmask);
        C a[A];
#pragma unroll
        for (int j = 0; j < A; ++j) a[j] = P::load(psi[base | soff[j]]);
        // rows rolled: the entries are read from shared memory per row, not hoisted into
        // registers for the whole loop over groups
#pragma unroll 1
        for (int r = 0; r < A; ++r) {
            const uint32_t rows = srows[r], reals = sreal[r];
            auto re = P::zero(), im = P::zero();
#pragma unroll
            for (int j = 0; j < A; ++j) {
                if (!((rows >> j) & 1)) continue;
                const Kt mr = sm[2 * (r * A + j)];
                re = P::fma1(mr, a[j].re, re);
                im = P::fma1(mr, a[j].im, im);
                if (!((reals >> j) & 1)) {
                    const Kt mi = sm[2 * (r * A + j) + 1];
                    re = P::fma1(P::kneg(mi), a[j].im, re);
                    im = P::fma1(mi, a[j].re, im);
                }
            }
            C out;
            out.re = re;
            out.im = im;
            psi[base | soff[r]] = P::store(out);
        }
    }
}

// A sparse block (k <= 4): a thread per group as in k_group, but row r sums only over its nonzero
// entries, listed once per CTA in shared memory.  Every loop runs exactly over the nonzeros with a
// trip count that is the same on every thread, and a real matrix (REAL: every nonzero entry real,
// as in the superoperators of amplitude damping, dephasing and depolarizing channels) has an
// instantiation without the imaginary-part multiply-adds: on this GPU a predicated-off FP64
// instruction still takes the FP64 pipe, and the first form of this kernel, which skipped zero and
// imaginary terms by uniform tests, issued twice the FP64 instructions it executed.  The group's
// amplitudes are staged column-major in shared memory, where the rows read them by column index.
template <class P, int K, bool REAL>
__global__ void __launch_bounds__(kBlockThreads) k_group_sparse(typename P::S* __restrict__ psi, int n, BlockDesc bd,
                                                                const uint64_t* __restrict__ mat, BlockSparsity nz) {
    using Kt = typename P::K;
    using S = typename P::S;
    using C = typename P::C;
    constexpr int A = 1 << K;
    extern __shared__ __align__(16) unsigned char smem_sparse[];
    S* buf = reinterpret_cast<S*>(smem_sparse);  // [column][thread]
    __shared__ Kt sre[A * A], sim[A * A];        // the nonzero entries of each row, in row order
    __shared__ uint8_t scol[A * A];
    __shared__ int sbeg[A + 1];
    __shared__ uint64_t soff[A];
    if (threadIdx.x == 0) {
        int cnt = 0;
        for (int r = 0; r < A; ++r) {
            sbeg[r] = cnt;
            for (int c = 0; c < A; ++c)
                if ((nz.rows[r] >> c) & 1) {
                    scol[cnt] = (uint8_t)c;
                    sre[cnt] = P::k_from_bits(mat[2 * (r * A + c)]);
                    sim[cnt] = P::k_from_bits(mat[2 * (r * A + c) + 1]);
                    ++cnt;
                }
        }
        sbeg[A] = cnt;
    }
    for (int j = threadIdx.x; j < A; j += blockDim.x) {
        uint64_t off = 0;
        for (int b = 0; b < K; ++b)
            if ((j >> b) & 1) off |= 1ULL << bd.q[b];
        soff[j] = off;
    }
    __syncthreads();
    const uint64_t ngroups = 1ULL << (n - K);
    const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
    const int tid = threadIdx.x;
    for (uint64_t g = (uint64_t)blockIdx.x * blockDim.x + tid; g < ngroups; g += step) {
        const uint64_t base = insert0_mask(g, bd.tmask);
        // the group into this thread's column of the staging buffer (only this thread reads it)
#pragma unroll
        for (int j = 0; j < A; ++j) buf[j * kBlockThreads + tid] = psi[base | soff[j]];
#pragma unroll 1
        for (int r = 0; r < A; ++r) {
            auto re = P::zero(), im = P::zero();
            const int e1 = sbeg[r + 1];
            for (int e = sbeg[r]; e < e1; ++e) {
                const C x = P::load(buf[scol[e] * kBlockThreads + tid]);
                const Kt mr = sre[e];
                re = P::fma1(mr, x.re, re);
                im = P::fma1(mr, x.im, im);
                if (!REAL) {
                    const Kt mi = sim[e];
                    re = P::fma1(P::kneg(mi), x.im, re);
                    im = P::fma1(mi, x.re, im);
                }
            }
            C out;
            out.re = re;
            out.im = im;
            psi[base | soff[r]] = P::store(out);
        }
    }
}

template <class P, int K, bool REAL>
cudaError_t group_sparse_t(void* psi, int n, const BlockDesc& bd, const uint64_t* d_mat, const BlockSparsity& nz,
                           cudaStream_t s) {
    const uint64_t ngroups = 1ULL << (n - K);
    const uint64_t blocks = (ngroups + kBlockThreads - 1) / kBlockThreads;
    const unsigned grid = (unsigned)(blocks < 152ULL * 8 ? blocks : 152ULL * 8);
    const size_t smem = (size_t)(1 << K) * kBlockThreads * sizeof(typename P::S);
    static const cudaError_t attr =
        cudaFuncSetAttribute(k_group_sparse<P, K, REAL>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (attr != cudaSuccess) return attr;
    k_group_sparse<P, K, REAL><<<grid, kBlockThreads, smem, s>>>(static_cast<typename P::S*>(psi), n, bd, d_mat, nz);
    return cudaGetLastError();
}

template <class P, int K>
cudaError_t group_sparse_k(void* psi, int n, const BlockDesc& bd, const uint64_t* d_mat, const BlockSparsity& nz,
                           cudaStream_t s) {
    if constexpr (P::kPrecision != LLG_F64) {  // the mask form on the FP32 pipe
        const uint64_t ngroups = 1ULL << (n - K);
        const uint64_t blocks = (ngroups + kBlockThreads - 1) / kBlockThreads;
        const unsigned grid = (unsigned)(blocks < 152ULL * 8 ? blocks : 152ULL * 8);
        k_group_sparse_masks<P, K><<<grid, kBlockThreads, 0, s>>>(static_cast<typename P::S*>(psi), n, bd, d_mat, nz);
        return cudaGetLastError();
    } else {
        bool real = true;
        for (int r = 0; r < (1 << K); ++r) real = real && nz.real[r] == nz.rows[r];
        return real ? group_sparse_t<P, K, true>(psi, n, bd, d_mat, nz, s)
                    : group_sparse_t<P, K, false>(psi, n, bd, d_mat, nz, s);
    }
}

template <class P>
cudaError_t block_sparse_t(void* psi, int n, const BlockDesc& bd, const uint64_t* d_mat, const BlockSparsity& nz,
                           cudaStream_t s) {
    switch (bd.k) {
        case 1: return group_sparse_k<P, 1>(psi, n, bd, d_mat, nz, s);
        case 2: return group_sparse_k<P, 2>(psi, n, bd, d_mat, nz, s);
        case 3: return group_sparse_k<P, 3>(psi, n, bd, d_mat, nz, s);
        case 4: return group_sparse_k<P, 4>(psi, n, bd, d_mat, nz, s);
        default: return cudaErrorInvalidValue;
    }
}

template <class P, int K>
cudaError_t group_t(void* psi, int n, const BlockDesc& bd, const uint64_t* d_mat, cudaStream_t s) {
    const uint64_t ngroups = 1ULL << (n - K);
    const uint64_t blocks = (ngroups + kBlockThreads - 1) / kBlockThreads;
    const unsigned grid = (unsigned)(blocks < 152ULL * 8 ? blocks : 152ULL * 8);
    k_group<P, K><<<grid, kBlockThreads, 0, s>>>(static_cast<typename P::S*>(psi), n, bd, d_mat);
    return cudaGetLastError();
}

template <class P>
cudaError_t block_t(void* psi, int n, const BlockDesc& bd, const uint64_t* d_mat, cudaStream_t s) {
    switch (bd.k) {
        case 1: return group_t<P, 1>(psi, n, bd, d_mat, s);
        case 2: return group_t<P, 2>(psi, n, bd, d_mat, s);
        case 3: return group_t<P, 3>(psi, n, bd, d_mat, s);
        default: break;
    }
    const uint64_t ngroups = 1ULL << (n - bd.k);
    const uint64_t warps = (ngroups + (uint64_t)(32 >> bd.k) - 1) / (uint64_t)(32 >> bd.k);
    const uint64_t blocks = (warps + kBlockThreads / 32 - 1) / (kBlockThreads / 32);
    const unsigned grid = (unsigned)(blocks < 152ULL * 8 ? blocks : 152ULL * 8);
    k_block<P><<<grid, kBlockThreads, 0, s>>>(static_cast<typename P::S*>(psi), n, bd, d_mat);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_block_sparse(int P, void* psi, int n, const BlockDesc& bd, const uint64_t* d_mat,
                                const BlockSparsity& nz, cudaStream_t s) {
    switch (P) {
        case LLG_F64: return block_sparse_t<PolF64>(psi, n, bd, d_mat, nz, s);
        case LLG_F32: return block_sparse_t<PolF32>(psi, n, bd, d_mat, nz, s);
        default: return block_sparse_t<PolDF64>(psi, n, bd, d_mat, nz, s);
    }
}

cudaError_t launch_block(int P, void* psi, int n, const BlockDesc& bd, const uint64_t* d_mat, cudaStream_t s) {
    switch (P) {
        case LLG_F64: return block_t<PolF64>(psi, n, bd, d_mat, s);
        case LLG_F32: return block_t<PolF32>(psi, n, bd, d_mat, s);
        default: return block_t<PolDF64>(psi, n, bd, d_mat, s);
    }
}

}  // namespace llg
