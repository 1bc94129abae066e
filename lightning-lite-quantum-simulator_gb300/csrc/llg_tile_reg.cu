// llg_tile_reg.cu -- register-tiled pass: the tile of a pass lives in registers, 16 amplitudes per
// thread, and moves through shared memory only when the register layout changes (the register
// programs of to_register_program, llg_plan.cpp).
//
// In the shared-memory tile pass every op reads and writes each amplitude pair in shared memory
// and ends in a barrier; for complex64 (8 FMA per rotation pair) that traffic, the index arithmetic
// and the barriers bound the pass.  Here a thread holds the amplitudes whose tile-local indices
// vary over 4 register positions; an op on a register position is pure register arithmetic with
// the pair pattern fixed at compile time, diagonal ops and CNOT controls on any position read the
// thread's index bits, and a layout change is one shared-memory round trip (write, barrier, read)
// for a run of ops.  The tile is read from and written to HBM directly from registers in the base
// layout (thread-index bits on the low positions: 16 lanes cover one 128-byte run).
//
// Shared memory is swizzled: local index l lives at slot l ^ fold(l >> 4), fold XOR-ing the 4-bit
// groups together.  A lane bit on position p toggles slot bit (p mod 4); the planner puts the first
// four lane bits on positions of distinct residues, so a half-warp's 16 accesses hit 16 distinct
// 8-byte bank pairs.
#include <cuda_runtime.h>

#include "llg_common.cuh"
#include "llg_internal.h"
#include "llg_launch.h"
#include "llg_tile.cuh"

namespace llg {

namespace {

constexpr int kRA = 16;         // amplitudes per thread
constexpr int kROpChunk = 32;   // op records staged per shared-memory chunk

__device__ __forceinline__ uint32_t swz(uint32_t l) {
    const uint32_t x = l >> 4;
    return l ^ ((x ^ (x >> 4) ^ (x >> 8)) & 15u);
}

// local-index offset of register amplitude e: bit j of e at register position j
__device__ __forceinline__ uint32_t reg_off(const uint32_t rb[4], int e) {
    return ((e & 1) ? rb[0] : 0u) | ((e & 2) ? rb[1] : 0u) | ((e & 4) ? rb[2] : 0u) | ((e & 8) ? rb[3] : 0u);
}

template <class P, int J, int KIND>
__device__ __forceinline__ void reg_pairs_j(typename P::C (&a)[kRA], const ExecOp& o) {
    const PairMath<P, KIND> m(o);
#pragma unroll
    for (int e = 0; e < kRA; ++e)
        if (!(e & (1 << J))) m.apply(a[e], a[e | (1 << J)]);
}

template <class P, int KIND>
__device__ __forceinline__ void reg_pairs(typename P::C (&a)[kRA], const ExecOp& o) {
    switch (o.q0) {
        case 0: reg_pairs_j<P, 0, KIND>(a, o); break;
        case 1: reg_pairs_j<P, 1, KIND>(a, o); break;
        case 2: reg_pairs_j<P, 2, KIND>(a, o); break;
        default: reg_pairs_j<P, 3, KIND>(a, o); break;
    }
}

// CNOT with target slot J and control slot K, both in registers: the swaps are register renames
// fixed at compile time; with OPF_PHASE the amplitudes that end at control = target = 1 are
// multiplied by c[0] + i c[1]
template <class P, int J, int K>
__device__ __forceinline__ void reg_cnot_jk(typename P::C (&a)[kRA], const ExecOp& o) {
    using Kt = typename P::K;
    using C = typename P::C;
    const bool phased = (o.flags & OPF_PHASE) != 0;
    const Kt pr = P::k_from_bits(o.c[0]), pi = P::k_from_bits(o.c[1]), mpi = P::kneg(pi);
#pragma unroll
    for (int e = 0; e < kRA; ++e)
        if (!(e & (1 << J)) && (e & (1 << K))) {
            const C x = a[e];
            a[e] = a[e | (1 << J)];
            a[e | (1 << J)] = x;
            if (phased) cmul_const<P>(a[e | (1 << J)], pr, pi, mpi);
        }
}

// CNOT with target slot J whose control is uniform for this thread (a thread-index position) or
// for the tile (a global qubit): all of the thread's pairs on J, or none
template <class P, int J>
__device__ __forceinline__ void reg_cnot_uniform(typename P::C (&a)[kRA], const ExecOp& o) {
    using Kt = typename P::K;
    using C = typename P::C;
    const bool phased = (o.flags & OPF_PHASE) != 0;
    const Kt pr = P::k_from_bits(o.c[0]), pi = P::k_from_bits(o.c[1]), mpi = P::kneg(pi);
#pragma unroll
    for (int e = 0; e < kRA; ++e)
        if (!(e & (1 << J))) {
            const C x = a[e];
            a[e] = a[e | (1 << J)];
            a[e | (1 << J)] = x;
            if (phased) cmul_const<P>(a[e | (1 << J)], pr, pi, mpi);
        }
}

template <class P, int J>
__device__ __forceinline__ void reg_cnot_j(typename P::C (&a)[kRA], const ExecOp& o, uint32_t tb, uint64_t base) {
    if (o.flags & OPF_SLOT_Q0) {
        switch (o.q0) {
            case 0: if (J != 0) reg_cnot_jk<P, J, (J == 0 ? 1 : 0)>(a, o); break;
            case 1: if (J != 1) reg_cnot_jk<P, J, (J == 1 ? 0 : 1)>(a, o); break;
            case 2: if (J != 2) reg_cnot_jk<P, J, (J == 2 ? 0 : 2)>(a, o); break;
            default: if (J != 3) reg_cnot_jk<P, J, (J == 3 ? 0 : 3)>(a, o); break;
        }
        return;
    }
    const bool on = (o.flags & OPF_NONLOCAL_Q0) ? ((base >> o.q0) & 1) : ((tb >> o.q0) & 1);
    if (on) reg_cnot_uniform<P, J>(a, o);
}

template <class P>
__device__ __forceinline__ void reg_cnot(typename P::C (&a)[kRA], const ExecOp& o, uint32_t tb, uint64_t base) {
    switch (o.q1) {
        case 0: reg_cnot_j<P, 0>(a, o, tb, base); break;
        case 1: reg_cnot_j<P, 1>(a, o, tb, base); break;
        case 2: reg_cnot_j<P, 2>(a, o, tb, base); break;
        default: reg_cnot_j<P, 3>(a, o, tb, base); break;
    }
}

// diag(d0, d1) (EX_DIAG) or diag(1, ph) (EX_PHASE1) on register slot J
template <class P, int J>
__device__ __forceinline__ void reg_diag_j(typename P::C (&a)[kRA], const ExecOp& o) {
    using K = typename P::K;
    const bool ph1 = o.kind == EX_PHASE1;
    const K d1r = P::k_from_bits(ph1 ? o.c[0] : o.c[2]), d1i = P::k_from_bits(ph1 ? o.c[1] : o.c[3]), md1i = P::kneg(d1i);
#pragma unroll
    for (int e = 0; e < kRA; ++e)
        if (e & (1 << J)) cmul_const<P>(a[e], d1r, d1i, md1i);
    if (!ph1) {
        const K d0r = P::k_from_bits(o.c[0]), d0i = P::k_from_bits(o.c[1]), md0i = P::kneg(d0i);
#pragma unroll
        for (int e = 0; e < kRA; ++e)
            if (!(e & (1 << J))) cmul_const<P>(a[e], d0r, d0i, md0i);
    }
}

// the same on a register slot, a thread-index position or a global qubit (the last two: one
// factor for all the thread's amplitudes)
template <class P>
__device__ __forceinline__ void reg_diag(typename P::C (&a)[kRA], const ExecOp& o, uint32_t tb, uint64_t base) {
    using K = typename P::K;
    if (o.flags & OPF_SLOT_Q0) {
        switch (o.q0) {
            case 0: reg_diag_j<P, 0>(a, o); break;
            case 1: reg_diag_j<P, 1>(a, o); break;
            case 2: reg_diag_j<P, 2>(a, o); break;
            default: reg_diag_j<P, 3>(a, o); break;
        }
        return;
    }
    const bool ph1 = o.kind == EX_PHASE1;
    const bool one = (o.flags & OPF_NONLOCAL_Q0) ? ((base >> o.q0) & 1) : ((tb >> o.q0) & 1);
    if (ph1 && !one) return;
    const int s = (one && !ph1) ? 2 : 0;  // EX_DIAG: d1 in c[2..3]; EX_PHASE1: the phase in c[0..1]
    const K dr = P::k_from_bits(o.c[s]), di = P::k_from_bits(o.c[s + 1]), mdi = P::kneg(di);
#pragma unroll
    for (int e = 0; e < kRA; ++e) cmul_const<P>(a[e], dr, di, mdi);
}

// negate the amplitudes with every bit of the local mask set (and every global bit of nl_mask)
template <class P>
__device__ __forceinline__ void reg_mcz(typename P::C (&a)[kRA], const ExecOp& o, uint32_t tb, const uint32_t rb[4],
                                        uint64_t base) {
    if ((base & o.nl_mask) != o.nl_mask) return;
    const uint32_t lm = (uint32_t)o.mask;
#pragma unroll
    for (int e = 0; e < kRA; ++e)
        if (((tb | reg_off(rb, e)) & lm) == lm) {
            a[e].re = P::neg(a[e].re);
            a[e].im = P::neg(a[e].im);
        }
}

// thread-index bits of this thread in a layout: bit k of threadIdx.x at position (tm >> 4k) & 15
__device__ __forceinline__ uint32_t thread_bits(uint64_t tm, int nthr) {
    uint32_t tb = 0;
    for (int k = 0; k < nthr; ++k)
        if ((threadIdx.x >> k) & 1) tb |= 1u << ((tm >> (4 * k)) & 15);
    return tb;
}

template <class P>
__global__ void __launch_bounds__(512, 1) k_tile_reg(typename P::S* __restrict__ psi, PassDesc pd,
                                                    const ExecOp* __restrict__ ops, double2* __restrict__ mirror) {
    using S = typename P::S;
    using C = typename P::C;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int t = pd.t, low = pd.low;
    const uint32_t tsize = 1u << t, nhi = 1u << (t - low);
    S* sm = reinterpret_cast<S*>(smem_raw);
    uint64_t* hi_off = reinterpret_cast<uint64_t*>(smem_raw + (size_t)tsize * sizeof(S));
    __shared__ __align__(16) ExecOp sops[kROpChunk];

    const uint64_t base = insert0_mask((uint64_t)blockIdx.x, pd.local_mask);
    for (uint32_t h = threadIdx.x; h < nhi; h += blockDim.x) {
        uint64_t off = 0;
        for (int j = 0; j < t - low; ++j)
            if ((h >> j) & 1) off |= 1ULL << pd.hi_pos[j];
        hi_off[h] = off;
    }
    __syncthreads();
    const uint32_t lowmask = (1u << low) - 1;
    // base layout: register positions t-4 .. t-1, thread-index bits on positions 0 .. t-5 in order
    uint32_t rb[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) rb[j] = 1u << (t - 4 + j);
    uint32_t tb = threadIdx.x;
    C a[kRA];
#pragma unroll
    for (int e = 0; e < kRA; ++e) {
        const uint32_t l = tb | reg_off(rb, e);
        a[e] = P::load(psi[base | hi_off[l >> low] | (l & lowmask)]);
    }

    constexpr int kWords = (int)(sizeof(ExecOp) / 16);
    for (int k = 0; k < pd.nops; ++k) {
        if (k % kROpChunk == 0) {
            const int cnt = min(kROpChunk, pd.nops - k);
            __syncthreads();  // every thread is done with the previous chunk
            const uint4* src = reinterpret_cast<const uint4*>(ops + pd.op_begin + k);
            for (int w = threadIdx.x; w < cnt * kWords; w += blockDim.x) reinterpret_cast<uint4*>(sops)[w] = src[w];
            __syncthreads();
        }
        const ExecOp& o = sops[k % kROpChunk];
        // one jump table over (kind, register slots): the planner's dense dispatch code
#define LLG_RP(KI, KIND)                                                          \
    case RC_PAIR + 4 * KI + 0: reg_pairs_j<P, 0, KIND>(a, o); break;              \
    case RC_PAIR + 4 * KI + 1: reg_pairs_j<P, 1, KIND>(a, o); break;              \
    case RC_PAIR + 4 * KI + 2: reg_pairs_j<P, 2, KIND>(a, o); break;              \
    case RC_PAIR + 4 * KI + 3: reg_pairs_j<P, 3, KIND>(a, o); break;
#define LLG_RCN(J, K) \
    case RC_CNOT_SLOT + 4 * J + K: reg_cnot_jk<P, J, K>(a, o); break;
        switch (o.flags >> kRegCodeShift) {
            LLG_RP(0, EX_U2)
            LLG_RP(1, EX_ZYZ)
            LLG_RP(2, EX_ZY)
            LLG_RP(3, EX_ZT)
            LLG_RP(4, EX_ZC)
            LLG_RP(5, EX_RT)
            LLG_RP(6, EX_RC)
            LLG_RP(7, EX_RX)
            LLG_RP(8, EX_RY)
            LLG_RP(9, EX_H)
            LLG_RP(10, EX_X)
            LLG_RCN(0, 1) LLG_RCN(0, 2) LLG_RCN(0, 3)
            LLG_RCN(1, 0) LLG_RCN(1, 2) LLG_RCN(1, 3)
            LLG_RCN(2, 0) LLG_RCN(2, 1) LLG_RCN(2, 3)
            LLG_RCN(3, 0) LLG_RCN(3, 1) LLG_RCN(3, 2)
            case RC_CNOT_UNIFORM + 0:
            case RC_CNOT_UNIFORM + 1:
            case RC_CNOT_UNIFORM + 2:
            case RC_CNOT_UNIFORM + 3: reg_cnot<P>(a, o, tb, base); break;
            case RC_DIAG_SLOT + 0:
            case RC_PHASE_SLOT + 0: reg_diag_j<P, 0>(a, o); break;
            case RC_DIAG_SLOT + 1:
            case RC_PHASE_SLOT + 1: reg_diag_j<P, 1>(a, o); break;
            case RC_DIAG_SLOT + 2:
            case RC_PHASE_SLOT + 2: reg_diag_j<P, 2>(a, o); break;
            case RC_DIAG_SLOT + 3:
            case RC_PHASE_SLOT + 3: reg_diag_j<P, 3>(a, o); break;
            case RC_DIAG_UNIFORM: reg_diag<P>(a, o, tb, base); break;
            case RC_MCZ: reg_mcz<P>(a, o, tb, rb, base); break;
#undef LLG_RP
#undef LLG_RCN
            case RC_LAYOUT: {
                // the swizzle is linear over the index bits (XOR), and tb and the register offsets
                // occupy disjoint bits: slot(tb | off) = slot(tb) ^ slot(off), with slot(off) the XOR
                // of the register positions' slots selected by e
                __syncthreads();  // the previous layout's reads of sm are done
                {
                    const uint32_t st = swz(tb), s0 = swz(rb[0]), s1 = swz(rb[1]), s2 = swz(rb[2]), s3 = swz(rb[3]);
#pragma unroll
                    for (int e = 0; e < kRA; ++e)
                        sm[st ^ ((e & 1) ? s0 : 0u) ^ ((e & 2) ? s1 : 0u) ^ ((e & 4) ? s2 : 0u) ^ ((e & 8) ? s3 : 0u)] =
                            P::store(a[e]);
                }
#pragma unroll
                for (int j = 0; j < 4; ++j) rb[j] = 1u << ((o.mask >> (4 * j)) & 15);
                tb = thread_bits(o.nl_mask, o.q0);
                __syncthreads();
                {
                    const uint32_t st = swz(tb), s0 = swz(rb[0]), s1 = swz(rb[1]), s2 = swz(rb[2]), s3 = swz(rb[3]);
#pragma unroll
                    for (int e = 0; e < kRA; ++e)
                        a[e] = P::load(sm[st ^ ((e & 1) ? s0 : 0u) ^ ((e & 2) ? s1 : 0u) ^ ((e & 4) ? s2 : 0u) ^
                                          ((e & 8) ? s3 : 0u)]);
                }
                break;
            }
            default: break;
        }
    }
    // the program ends in the base layout: store from registers (and, for the last pass before a
    // readback, the FP64 copy into the mapped host buffer)
#pragma unroll
    for (int e = 0; e < kRA; ++e) {
        const uint32_t l = tb | reg_off(rb, e);
        const uint64_t g = base | hi_off[l >> low] | (l & lowmask);
        psi[g] = P::store(a[e]);
        if (mirror) mirror[g] = P::to_f64(a[e]);
    }
}

template <class P>
cudaError_t tile_reg_t(void* vpsi, int n, const PassDesc& pd, const ExecOp* d_ops, double* mirror, cudaStream_t s) {
    using S = typename P::S;
    static const cudaError_t attr =
        cudaFuncSetAttribute(k_tile_reg<P>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)(((size_t)1 << 13) * sizeof(S) + ((size_t)1 << 9) * sizeof(uint64_t)));
    if (attr != cudaSuccess) return attr;
    if (pd.t < 9 || pd.t > 13) return cudaErrorInvalidValue;
    const size_t smem = ((size_t)1 << pd.t) * sizeof(S) + ((size_t)1 << (pd.t - pd.low)) * sizeof(uint64_t);
    const unsigned threads = 1u << (pd.t - 4);
    const uint64_t ntiles = 1ULL << (n - pd.t);
    k_tile_reg<P><<<(unsigned)ntiles, threads, smem, s>>>(static_cast<S*>(vpsi), pd, d_ops, reinterpret_cast<double2*>(mirror));
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_tile_reg(int P, void* psi, int n, const PassDesc& pd, const ExecOp* d_ops, cudaStream_t s,
                            double* mirror) {
    switch (P) {
        case LLG_F32: return tile_reg_t<PolF32>(psi, n, pd, d_ops, mirror, s);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace llg
