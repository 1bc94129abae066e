// llg_kernels.cu -- state-vector kernels for sm_103a (GB300).
//
//  * streaming passes (one kernel per gate, the reference's own per-gate algorithm,
//    src/StateVectorBackend.h:109-218 and src/StateVectorOptimized.cpp:56-78): every thread
//    owns amplitude pairs p -> (i0 = insert0(p, q), i0 | 2^q); consecutive threads take
//    consecutive p, so both halves of a pair stream coalesced for every q (for q = 0 one thread
//    reads the 32 contiguous bytes of its pair).  CNOT walks the N/4 quads with control = 1 and
//    swaps target halves; MCZ touches only the 2^(n-m) amplitudes with every mask bit set.
//  * tile passes (llg_plan.cpp): one CTA loads 2^t amplitudes spread over a chosen qubit set into
//    shared memory in 2^low-amplitude contiguous runs, applies a list of ops there, writes back.
//  * conversions to/from complex128, |a|^2, scaling, and deterministic two-stage reductions
//    (fixed grid, per-block partials, one FP64 pass over the partials).
#include <atomic>
#include <cstdio>

#include "llg_common.cuh"
#include "llg_launch.h"
#include "llg_tile.cuh"

namespace llg {

namespace {

constexpr int kThreads = 256;

// SM count of each device, read once per device (the current device at launch time)
constexpr int kMaxDevices = 64;
std::atomic<int> g_sms[kMaxDevices];
int sm_count() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        cudaGetLastError();
        return 1;
    }
    int v = g_sms[dev].load(std::memory_order_relaxed);
    if (v <= 0) {
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) {
            cudaGetLastError();
            v = 1;
        }
        g_sms[dev].store(v, std::memory_order_relaxed);
    }
    return v;
}

unsigned grid_for(uint64_t items, int per_thread) {
    const uint64_t want = (items + (uint64_t)kThreads * per_thread - 1) / ((uint64_t)kThreads * per_thread);
    const uint64_t cap = (uint64_t)sm_count() * 16;
    return (unsigned)(want < 1 ? 1 : (want > cap ? cap : want));
}

// ------------------------------------------------------------------------------------------
// streaming kernels (global qubit indices)
// ------------------------------------------------------------------------------------------
template <class P, int KIND>
__global__ void __launch_bounds__(kThreads) k_pairs(typename P::S* __restrict__ psi, uint64_t npairs, int q, ExecOp op) {
    using S = typename P::S;
    using C = typename P::C;
    const PairMath<P, KIND> m(op);
    const uint64_t bit = 1ULL << q;
    const uint64_t step = (uint64_t)gridDim.x * kThreads * 2;
    for (uint64_t base = (uint64_t)blockIdx.x * kThreads * 2 + threadIdx.x; base < npairs; base += step) {
        const uint64_t pA = base, pB = base + kThreads;
        const bool hasB = pB < npairs;
        const uint64_t iA = insert0(pA, q), iB = insert0(hasB ? pB : pA, q);
        S sA0 = psi[iA], sA1 = psi[iA | bit];
        S sB0, sB1;
        if (hasB) {
            sB0 = psi[iB];
            sB1 = psi[iB | bit];
        }
        C a0 = P::load(sA0), a1 = P::load(sA1);
        m.apply(a0, a1);
        psi[iA] = P::store(a0);
        psi[iA | bit] = P::store(a1);
        if (hasB) {
            C b0 = P::load(sB0), b1 = P::load(sB1);
            m.apply(b0, b1);
            psi[iB] = P::store(b0);
            psi[iB | bit] = P::store(b1);
        }
    }
}

// diag(d0, d1) on qubit q
template <class P>
__global__ void __launch_bounds__(kThreads) k_diag(typename P::S* __restrict__ psi, uint64_t size, int q, ExecOp op) {
    using K = typename P::K;
    const K d0r = P::k_from_bits(op.c[0]), d0i = P::k_from_bits(op.c[1]);
    const K d1r = P::k_from_bits(op.c[2]), d1i = P::k_from_bits(op.c[3]);
    const K md0i = P::kneg(d0i), md1i = P::kneg(d1i);
    const uint64_t step = (uint64_t)gridDim.x * kThreads;
    for (uint64_t i = (uint64_t)blockIdx.x * kThreads + threadIdx.x; i < size; i += step) {
        auto a = P::load(psi[i]);
        if ((i >> q) & 1) cmul_const<P>(a, d1r, d1i, md1i);
        else cmul_const<P>(a, d0r, d0i, md0i);
        psi[i] = P::store(a);
    }
}

// diag(1, p) on qubit q: only the amplitudes with bit q set are read and written (p = c[0] + i c[1])
template <class P>
__global__ void __launch_bounds__(kThreads) k_phase1(typename P::S* __restrict__ psi, uint64_t half, int q, ExecOp op) {
    using K = typename P::K;
    const K pr = P::k_from_bits(op.c[0]), pi = P::k_from_bits(op.c[1]), mpi = P::kneg(pi);
    const uint64_t bit = 1ULL << q;
    const uint64_t step = (uint64_t)gridDim.x * kThreads * 2;
    for (uint64_t base = (uint64_t)blockIdx.x * kThreads * 2 + threadIdx.x; base < half; base += step) {
        const uint64_t pB = base + kThreads;
        const bool hasB = pB < half;
        const uint64_t iA = insert0(base, q) | bit, iB = insert0(hasB ? pB : base, q) | bit;
        auto a = P::load(psi[iA]);
        typename P::C b;
        if (hasB) b = P::load(psi[iB]);
        cmul_const<P>(a, pr, pi, mpi);
        psi[iA] = P::store(a);
        if (hasB) {
            cmul_const<P>(b, pr, pi, mpi);
            psi[iB] = P::store(b);
        }
    }
}

// CNOT: swap (c=1, t=0) <-> (c=1, t=1) over the N/4 quads (src/StateVectorBackend.h:109-135).
// kStreamItems quads per thread per step, all loads issued before the stores (memory-level
// parallelism for a kernel that does no arithmetic).
constexpr int kStreamItems = 4;

template <class P>
__global__ void __launch_bounds__(kThreads) k_cnot(typename P::S* __restrict__ psi, uint64_t nquads, int c, int t) {
    using S = typename P::S;
    const int lo = c < t ? c : t, hi = c < t ? t : c;
    const uint64_t cbit = 1ULL << c, tbit = 1ULL << t;
    const uint64_t step = (uint64_t)gridDim.x * kThreads * kStreamItems;
    for (uint64_t base = (uint64_t)blockIdx.x * kThreads * kStreamItems + threadIdx.x; base < nquads; base += step) {
        uint64_t idx[kStreamItems];
        S x[kStreamItems], y[kStreamItems];
#pragma unroll
        for (int u = 0; u < kStreamItems; ++u) {
            const uint64_t r = base + (uint64_t)u * kThreads;
            idx[u] = r < nquads ? (insert0(insert0(r, lo), hi) | cbit) : ~0ULL;
            if (idx[u] != ~0ULL) {
                x[u] = psi[idx[u]];
                y[u] = psi[idx[u] | tbit];
            }
        }
#pragma unroll
        for (int u = 0; u < kStreamItems; ++u)
            if (idx[u] != ~0ULL) {
                psi[idx[u]] = y[u];
                psi[idx[u] | tbit] = x[u];
            }
    }
}

// MCZ: negate the amplitudes with every mask bit set (src/StateVectorBackend.h:137-151)
template <class P>
__global__ void __launch_bounds__(kThreads) k_mcz(typename P::S* __restrict__ psi, uint64_t count, uint64_t mask) {
    using S = typename P::S;
    const uint64_t step = (uint64_t)gridDim.x * kThreads * kStreamItems;
    for (uint64_t base = (uint64_t)blockIdx.x * kThreads * kStreamItems + threadIdx.x; base < count; base += step) {
        uint64_t idx[kStreamItems];
        S v[kStreamItems];
#pragma unroll
        for (int u = 0; u < kStreamItems; ++u) {
            const uint64_t r = base + (uint64_t)u * kThreads;
            idx[u] = r < count ? (insert0_mask(r, mask) | mask) : ~0ULL;
            if (idx[u] != ~0ULL) v[u] = psi[idx[u]];
        }
#pragma unroll
        for (int u = 0; u < kStreamItems; ++u)
            if (idx[u] != ~0ULL) {
                auto a = P::load(v[u]);
                a.re = P::neg(a.re);
                a.im = P::neg(a.im);
                psi[idx[u]] = P::store(a);
            }
    }
}

// ------------------------------------------------------------------------------------------
// tile pass
// ------------------------------------------------------------------------------------------
constexpr int kOpChunk = 32;  // op records staged per shared-memory chunk in k_tile
constexpr long kTileCopyWaitLimit = 1L << 24;  // mbarrier polls before a tile load is reported as timed out

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// bounded wait for phase `parity` of an mbarrier; false if it did not complete
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
    uint32_t done = 0;
    for (long it = 0; it < kTileCopyWaitLimit && !done; ++it)
        asm volatile("{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}"
                     : "=r"(done)
                     : "r"(smem_addr(bar)), "r"(parity));
    return done != 0;
}

// EX_U4 (fuse_two_qubit) on a complex64 tile: the 4x4 block on local qubits q0 (index bit 0) and
// q1 (index bit 1), one quad of amplitudes per thread and iteration; the 16 complex entries are
// read once per thread (the table is L2/L1-resident: 128 bytes per block)
template <class P>
__device__ __forceinline__ void tile_u4_f32(typename P::S* tile, uint32_t tsize, const ExecOp& o,
                                            const uint64_t* __restrict__ tables) {
    static_assert(sizeof(typename P::S) == 8, "complex64 tiles only");
    const uint64_t* mt = tables + 2 * o.mask;
    float mr[16], mi[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        mr[i] = P::k_from_bits(__ldg(mt + 2 * i));
        mi[i] = P::k_from_bits(__ldg(mt + 2 * i + 1));
    }
    const uint32_t bx = 1u << o.q0, by = 1u << o.q1;
    const uint32_t lo = bx < by ? bx : by, hi = bx < by ? by : bx;
    float2* t2 = reinterpret_cast<float2*>(tile);
    for (uint32_t r = threadIdx.x; r < (tsize >> 2); r += blockDim.x) {
        const uint32_t j0 = ins0(ins0(r, lo), hi);
        const uint32_t idx[4] = {j0, j0 | bx, j0 | by, j0 | bx | by};
        float2 v[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) v[k] = t2[idx[k]];
#pragma unroll
        for (int row = 0; row < 4; ++row) {
            float re = 0.0f, im = 0.0f;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                re = fmaf(mr[row * 4 + k], v[k].x, re);
                re = fmaf(-mi[row * 4 + k], v[k].y, re);
                im = fmaf(mr[row * 4 + k], v[k].y, im);
                im = fmaf(mi[row * 4 + k], v[k].x, im);
            }
            t2[idx[row]] = make_float2(re, im);
        }
    }
}

// MAXT: the largest CTA the instantiation runs.  1024 caps a thread at 64 registers; the 256-thread
// form keeps three CTAs per SM (the shared-memory limit of 12- and 13-qubit tiles) and may use 85,
// enough for a two-qubit block's 16 complex coefficients to stay in registers across its quads.
template <class P, int MAXT>
__global__ void __launch_bounds__(MAXT, MAXT == 256 ? 3 : 1) k_tile(typename P::S* __restrict__ psi, PassDesc pd, const ExecOp* __restrict__ ops,
                                               const uint64_t* __restrict__ tables, double2* __restrict__ mirror,
                                               int* __restrict__ err_flag) {
    using S = typename P::S;
    using K = typename P::K;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int t = pd.t, low = pd.low;
    const uint32_t tsize = 1u << t;
    const uint32_t nhi = 1u << (t - low);
    S* tile = reinterpret_cast<S*>(smem_raw);
    uint64_t* hi_off = reinterpret_cast<uint64_t*>(smem_raw + (size_t)tsize * sizeof(S));

    const uint64_t base = insert0_mask((uint64_t)blockIdx.x, pd.local_mask);
    for (uint32_t h = threadIdx.x; h < nhi; h += blockDim.x) {
        uint64_t off = 0;
        for (int j = 0; j < t - low; ++j)
            if ((h >> j) & 1) off |= 1ULL << pd.hi_pos[j];
        hi_off[h] = off;
    }
    // The tile is nhi contiguous runs of 2^low amplitudes, each starting at a multiple of its own
    // size (base and hi_off are zero in the low bits).  Runs of 128 bytes or more move with the
    // bulk-copy engine (cp.async.bulk into shared memory, completing on an mbarrier that expects
    // the tile's bytes; stores back the same way); shorter ones with plain loads and stores.
    __shared__ __align__(8) uint64_t tile_bar;
    const uint32_t run_bytes = (uint32_t)sizeof(S) << low;
    const bool bulk = run_bytes >= 128;
    if (bulk && threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&tile_bar)));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(&tile_bar)),
                     "r"((uint32_t)(tsize * sizeof(S)))
                     : "memory");
    }
    __syncthreads();
    const uint32_t lowmask = (1u << low) - 1;
    bool loaded = true;
    if (bulk) {
        for (uint32_t h = threadIdx.x; h < nhi; h += blockDim.x)
            asm volatile(
                "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                    smem_addr(tile + ((size_t)h << low))),
                "l"(psi + (base | hi_off[h])), "r"(run_bytes), "r"(smem_addr(&tile_bar))
                : "memory");
        loaded = mbar_wait(&tile_bar, 0);
        if (!loaded && threadIdx.x == 0) atomicExch(err_flag, 1);
    } else {
        for (uint32_t l = threadIdx.x; l < tsize; l += blockDim.x) tile[l] = psi[base | hi_off[l >> low] | (l & lowmask)];
    }
    __syncthreads();
    if (!__syncthreads_and(loaded)) {
        (void)mbar_wait(&tile_bar, 0);  // give copies still in flight a second bounded wait, store nothing
        return;
    }

    // op records are staged through shared memory in chunks (one coalesced copy per chunk
    // instead of a dependent global load before every op's barrier)
    __shared__ __align__(16) ExecOp sops[kOpChunk];
    static_assert(sizeof(ExecOp) % 16 == 0, "ExecOp copies as 16-byte words");
    constexpr int kWords = (int)(sizeof(ExecOp) / 16);
    for (int k = 0; k < pd.nops; ++k) {
        if (k % kOpChunk == 0) {
            const int cnt = min(kOpChunk, pd.nops - k);
            const uint4* src = reinterpret_cast<const uint4*>(ops + pd.op_begin + k);
            for (int w = threadIdx.x; w < cnt * kWords; w += blockDim.x) reinterpret_cast<uint4*>(sops)[w] = src[w];
            __syncthreads();
        }
        const ExecOp& o = sops[k % kOpChunk];
        const int kind = o.kind;
        switch (kind) {
            case EX_U2: tile_pairs<P, EX_U2>(tile, tsize >> 1, o.q0, o); break;
            case EX_ZYZ: tile_pairs<P, EX_ZYZ>(tile, tsize >> 1, o.q0, o); break;
            case EX_ZY: tile_pairs<P, EX_ZY>(tile, tsize >> 1, o.q0, o); break;
            case EX_ZT: tile_pairs<P, EX_ZT>(tile, tsize >> 1, o.q0, o); break;
            case EX_ZC: tile_pairs<P, EX_ZC>(tile, tsize >> 1, o.q0, o); break;
            case EX_RT: tile_pairs<P, EX_RT>(tile, tsize >> 1, o.q0, o); break;
            case EX_RC: tile_pairs<P, EX_RC>(tile, tsize >> 1, o.q0, o); break;
            case EX_PTAB: tile_ptab<P>(tile, tsize, o, tables); break;
            case EX_PHASE1: tile_phase1<P>(tile, tsize, base, o); break;
            case EX_RX: tile_pairs<P, EX_RX>(tile, tsize >> 1, o.q0, o); break;
            case EX_RY: tile_pairs<P, EX_RY>(tile, tsize >> 1, o.q0, o); break;
            case EX_H: tile_pairs<P, EX_H>(tile, tsize >> 1, o.q0, o); break;
            case EX_X: tile_pairs<P, EX_X>(tile, tsize >> 1, o.q0, o); break;
            case EX_DIAG: {
                const K d0r = P::k_from_bits(o.c[0]), d0i = P::k_from_bits(o.c[1]);
                const K d1r = P::k_from_bits(o.c[2]), d1i = P::k_from_bits(o.c[3]);
                if (o.flags & OPF_NONLOCAL_Q0) {
                    const bool one = (base >> o.q0) & 1;
                    const K dr = one ? d1r : d0r, di = one ? d1i : d0i;
                    const K mdi = P::kneg(di);
                    for (uint32_t l = threadIdx.x; l < tsize; l += blockDim.x) {
                        auto a = P::load(tile[l]);
                        cmul_const<P>(a, dr, di, mdi);
                        tile[l] = P::store(a);
                    }
                } else {
                    const K md0i = P::kneg(d0i), md1i = P::kneg(d1i);
                    const int q = o.q0;
                    for (uint32_t l = threadIdx.x; l < tsize; l += blockDim.x) {
                        auto a = P::load(tile[l]);
                        if ((l >> q) & 1) cmul_const<P>(a, d1r, d1i, md1i);
                        else cmul_const<P>(a, d0r, d0i, md0i);
                        tile[l] = P::store(a);
                    }
                }
                break;
            }
            case EX_CNOT: tile_cnot<P>(tile, tsize, base, o); break;
            case EX_U4:  // emitted for complex64 plans only
                if constexpr (sizeof(S) == 8) tile_u4_f32<P>(tile, tsize, o, tables);
                break;
            case EX_U2C: {  // the 2x2 for this tile's control bit, applied as a generic pair op
                ExecOp u = o;
                const uint64_t* mt = tables + 2 * (o.mask + 4 * ((base >> o.q0) & 1));
#pragma unroll
                for (int i = 0; i < 8; ++i) u.c[i] = __ldg(mt + i);
                tile_pairs<P, EX_U2>(tile, tsize >> 1, o.q1, u);
                break;
            }
            case EX_MCZ: {
                if ((base & o.nl_mask) == o.nl_mask) {
                    const uint32_t lm = (uint32_t)o.mask;
                    const uint32_t cnt = tsize >> __popc(lm);
                    for (uint32_t r = threadIdx.x; r < cnt; r += blockDim.x) {
                        const uint32_t j = (uint32_t)insert0_mask(r, lm) | lm;
                        auto a = P::load(tile[j]);
                        a.re = P::neg(a.re);
                        a.im = P::neg(a.im);
                        tile[j] = P::store(a);
                    }
                }
                break;
            }
            default: break;
        }
        __syncthreads();
    }

    if (bulk) {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // this thread's tile writes, to the copy engine
        __syncthreads();
        for (uint32_t h = threadIdx.x; h < nhi; h += blockDim.x)
            asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(psi + (base | hi_off[h])),
                         "r"(smem_addr(tile + ((size_t)h << low))), "r"(run_bytes)
                         : "memory");
        asm volatile("cp.async.bulk.commit_group;" ::: "memory");
    } else {
        for (uint32_t l = threadIdx.x; l < tsize; l += blockDim.x) psi[base | hi_off[l >> low] | (l & lowmask)] = tile[l];
    }
    // the last pass before a host readback also writes the amplitudes, as FP64, into the mapped
    // host buffer (while the copy engine of the bulk stores still reads the tile)
    if (mirror)
        for (uint32_t l = threadIdx.x; l < tsize; l += blockDim.x)
            mirror[base | hi_off[l >> low] | (l & lowmask)] = P::to_f64(P::load(tile[l]));
    if (bulk) asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");  // the tile is read before the CTA exits
}

// ------------------------------------------------------------------------------------------
// conversions, probabilities, scaling
// ------------------------------------------------------------------------------------------
template <class P>
__global__ void k_from_f64(const double2* __restrict__ src, typename P::S* __restrict__ dst, uint64_t count) {
    const uint64_t step = (uint64_t)gridDim.x * kThreads;
    for (uint64_t i = (uint64_t)blockIdx.x * kThreads + threadIdx.x; i < count; i += step) dst[i] = P::store(P::from_f64(src[i]));
}

template <class P>
__global__ void k_to_f64(const typename P::S* __restrict__ src, double2* __restrict__ dst, uint64_t count) {
    const uint64_t step = (uint64_t)gridDim.x * kThreads;
    for (uint64_t i = (uint64_t)blockIdx.x * kThreads + threadIdx.x; i < count; i += step) dst[i] = P::to_f64(P::load(src[i]));
}

template <class P>
__global__ void k_probs(const typename P::S* __restrict__ src, double* __restrict__ out, uint64_t count) {
    const uint64_t step = (uint64_t)gridDim.x * kThreads;
    for (uint64_t i = (uint64_t)blockIdx.x * kThreads + threadIdx.x; i < count; i += step)
        out[i] = P::acc_to_double(P::acc_norm(P::acc_zero(), P::load(src[i])));
}

template <class P>
__global__ void k_scale(typename P::S* __restrict__ psi, uint64_t count, uint64_t fbits) {
    const typename P::K f = P::k_from_bits(fbits);
    const uint64_t step = (uint64_t)gridDim.x * kThreads;
    for (uint64_t i = (uint64_t)blockIdx.x * kThreads + threadIdx.x; i < count; i += step) {
        auto a = P::load(psi[i]);
        a.re = P::mulk(f, a.re);
        a.im = P::mulk(f, a.im);
        psi[i] = P::store(a);
    }
}

template <class S>
__global__ void k_set_one(S* psi, uint64_t index, S one) { psi[index] = one; }

// ------------------------------------------------------------------------------------------
// reductions: slot 0 = sum |a|^2, slot 1+c = sum |a_i|^2 * (#odd-parity terms of class c in i)
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ double block_sum(double v, double* sh) {
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

template <class P>
__global__ void __launch_bounds__(kThreads) k_reduce_z(const typename P::S* __restrict__ psi, uint64_t size, ZTerms z,
                                                      double* __restrict__ partials) {
    __shared__ double sh[kThreads / 32];
    typename P::Acc acc[kRedSlots];
#pragma unroll
    for (int s = 0; s < kRedSlots; ++s) acc[s] = P::acc_zero();
    const uint64_t step = (uint64_t)gridDim.x * kThreads;
    for (uint64_t i = (uint64_t)blockIdx.x * kThreads + threadIdx.x; i < size; i += step) {
        const auto a = P::load(psi[i]);
        acc[0] = P::acc_norm(acc[0], a);
        if (z.nterms > 0) {
            int cnt[kMaxZClasses] = {0, 0, 0, 0};
            for (int k = 0; k < z.nterms; ++k) {
                int par = (int)((i >> z.a[k]) & 1);
                if (z.b[k] >= 0) par ^= (int)((i >> z.b[k]) & 1);
                cnt[z.cls[k]] += par;
            }
#pragma unroll
            for (int c = 0; c < kMaxZClasses; ++c)
                if (c < z.nclass && cnt[c]) acc[1 + c] = P::acc_norm_w(acc[1 + c], a, (float)cnt[c]);
        }
    }
#pragma unroll
    for (int s = 0; s < kRedSlots; ++s) {
        const double v = block_sum(P::acc_to_double(acc[s]), sh);
        if (threadIdx.x == 0) partials[(size_t)blockIdx.x * kRedSlots + s] = v;
    }
}

__device__ __forceinline__ double block_max(double v, double* sh) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, off));
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    double r = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) r = fmax(r, sh[w]);
    return r;
}

// Two states of any precisions, in double: per block [Re <a|b>, Im <a|b>, <a|a>, <b|b>, max |a_i - b_i|]
template <class PA, class PB>
__global__ void __launch_bounds__(kThreads) k_compare(const typename PA::S* __restrict__ a, const typename PB::S* __restrict__ b,
                                                      uint64_t size, double* __restrict__ partials) {
    __shared__ double sh[kThreads / 32];
    double re = 0.0, im = 0.0, na = 0.0, nb = 0.0, mx = 0.0, mb = 0.0;
    const uint64_t step = (uint64_t)gridDim.x * kThreads;
    for (uint64_t i = (uint64_t)blockIdx.x * kThreads + threadIdx.x; i < size; i += step) {
        const double2 x = PA::to_f64(PA::load(a[i])), y = PB::to_f64(PB::load(b[i]));
        re = fma(x.x, y.x, fma(x.y, y.y, re));
        im = fma(x.x, y.y, fma(-x.y, y.x, im));
        na = fma(x.x, x.x, fma(x.y, x.y, na));
        nb = fma(y.x, y.x, fma(y.y, y.y, nb));
        mx = fmax(mx, fmax(fabs(x.x - y.x), fabs(x.y - y.y)));
        mb = fmax(mb, fmax(fabs(y.x), fabs(y.y)));
    }
    const double v[4] = {re, im, na, nb};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const double t = block_sum(v[k], sh);
        if (threadIdx.x == 0) partials[(size_t)blockIdx.x * kCmpSlots + k] = t;
    }
    const double m = block_max(mx, sh);
    if (threadIdx.x == 0) partials[(size_t)blockIdx.x * kCmpSlots + 4] = m;
    const double m2 = block_max(mb, sh);
    if (threadIdx.x == 0) partials[(size_t)blockIdx.x * kCmpSlots + 5] = m2;
}

__global__ void k_finish(const double* __restrict__ partials, int nblocks, double* __restrict__ out) {
    // one thread per slot, fixed order: deterministic
    const int s = threadIdx.x;
    if (s >= kRedSlots) return;
    double r = 0.0;
    for (int b = 0; b < nblocks; ++b) r += partials[(size_t)b * kRedSlots + s];
    out[s] = r;
}

// FP64 FMA throughput probe: eight independent dependency chains per thread keep the FP64
// pipe's latency covered; the sum is stored only if it takes an impossible value, so the compiler
// keeps every FMA and nothing is written.
__global__ void __launch_bounds__(256) k_dfma_rate(double* out, int iters, double m, double c) {
    double a[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = 1.0 + 1e-3 * (threadIdx.x + k);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 8; ++k) a[k] = fma(a[k], m, c);
    }
    const double s = ((a[0] + a[1]) + (a[2] + a[3])) + ((a[4] + a[5]) + (a[6] + a[7]));
    if (s == -1.0) out[0] = s;
}

template <class P>
cudaError_t exec_op_t(void* vpsi, int n, const ExecOp& op, cudaStream_t s) {
    using S = typename P::S;
    S* psi = static_cast<S*>(vpsi);
    const uint64_t size = 1ULL << n;
    switch (op.kind) {
        case EX_U2: k_pairs<P, EX_U2><<<grid_for(size / 2, 2), kThreads, 0, s>>>(psi, size / 2, op.q0, op); break;
        case EX_RX: k_pairs<P, EX_RX><<<grid_for(size / 2, 2), kThreads, 0, s>>>(psi, size / 2, op.q0, op); break;
        case EX_RY: k_pairs<P, EX_RY><<<grid_for(size / 2, 2), kThreads, 0, s>>>(psi, size / 2, op.q0, op); break;
        case EX_H: k_pairs<P, EX_H><<<grid_for(size / 2, 2), kThreads, 0, s>>>(psi, size / 2, op.q0, op); break;
        case EX_X: k_pairs<P, EX_X><<<grid_for(size / 2, 2), kThreads, 0, s>>>(psi, size / 2, op.q0, op); break;
        case EX_RT: k_pairs<P, EX_RT><<<grid_for(size / 2, 2), kThreads, 0, s>>>(psi, size / 2, op.q0, op); break;
        case EX_RC: k_pairs<P, EX_RC><<<grid_for(size / 2, 2), kThreads, 0, s>>>(psi, size / 2, op.q0, op); break;
        case EX_RXT: k_pairs<P, EX_RXT><<<grid_for(size / 2, 2), kThreads, 0, s>>>(psi, size / 2, op.q0, op); break;
        case EX_RXC: k_pairs<P, EX_RXC><<<grid_for(size / 2, 2), kThreads, 0, s>>>(psi, size / 2, op.q0, op); break;
        case EX_HS: k_pairs<P, EX_HS><<<grid_for(size / 2, 2), kThreads, 0, s>>>(psi, size / 2, op.q0, op); break;
        case EX_ZTZ: k_pairs<P, EX_ZTZ><<<grid_for(size / 2, 2), kThreads, 0, s>>>(psi, size / 2, op.q0, op); break;
        case EX_ZCZ: k_pairs<P, EX_ZCZ><<<grid_for(size / 2, 2), kThreads, 0, s>>>(psi, size / 2, op.q0, op); break;
        case EX_ZYZ: k_pairs<P, EX_ZYZ><<<grid_for(size / 2, 2), kThreads, 0, s>>>(psi, size / 2, op.q0, op); break;
        case EX_PHASE1: k_phase1<P><<<grid_for(size / 2, 2), kThreads, 0, s>>>(psi, size / 2, op.q0, op); break;
        case EX_DIAG: k_diag<P><<<grid_for(size, 1), kThreads, 0, s>>>(psi, size, op.q0, op); break;
        case EX_CNOT: k_cnot<P><<<grid_for(size / 4, kStreamItems), kThreads, 0, s>>>(psi, size / 4, op.q0, op.q1); break;
        case EX_MCZ: {
            const uint64_t cnt = size >> __builtin_popcountll(op.mask);
            k_mcz<P><<<grid_for(cnt, kStreamItems), kThreads, 0, s>>>(psi, cnt, op.mask);
            break;
        }
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

template <class P>
size_t tile_smem_bytes(int t, int low) {
    return ((size_t)1 << t) * sizeof(typename P::S) + ((size_t)1 << (t - low)) * sizeof(uint64_t);
}

template <class P>
cudaError_t tile_pass_t(void* vpsi, int n, const PassDesc& pd, const ExecOp* d_ops, const uint64_t* d_tables, int threads,
                        double* mirror, int* err_flag, cudaStream_t s) {
    // the largest dynamic shared memory of any tile, set once per instantiation (thread-safe static
    // initialisation)
    const int max_smem = (int)tile_smem_bytes<P>(tile_max_qubits(P::kPrecision), 4);
    static const cudaError_t attr =
        cudaFuncSetAttribute(k_tile<P, 1024>, cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem);
    static const cudaError_t attr256 =
        cudaFuncSetAttribute(k_tile<P, 256>, cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem);
    if (attr != cudaSuccess) return attr;
    if (attr256 != cudaSuccess) return attr256;
    const size_t smem = tile_smem_bytes<P>(pd.t, pd.low);
    const uint64_t ntiles = 1ULL << (n - pd.t);
    if (threads <= 0) threads = pd.t >= 10 ? 512 : (pd.t >= 6 ? (1 << (pd.t - 1)) : 32);
    if (threads <= 256)
        k_tile<P, 256><<<(unsigned)ntiles, threads, smem, s>>>(static_cast<typename P::S*>(vpsi), pd, d_ops, d_tables,
                                                               reinterpret_cast<double2*>(mirror), err_flag);
    else
        k_tile<P, 1024><<<(unsigned)ntiles, threads, smem, s>>>(static_cast<typename P::S*>(vpsi), pd, d_ops, d_tables,
                                                                reinterpret_cast<double2*>(mirror), err_flag);
    return cudaGetLastError();
}

template <class P>
cudaError_t init_basis_t(void* vpsi, uint64_t size, uint64_t index, cudaStream_t s) {
    using S = typename P::S;
    cudaError_t e = cudaMemsetAsync(vpsi, 0, size * sizeof(S), s);
    if (e != cudaSuccess) return e;
    S one;
    if (sizeof(S) == 16 && P::kPrecision == 0) {
        double2 d = make_double2(1.0, 0.0);
        memcpy(&one, &d, sizeof(S));
    } else if (P::kPrecision == 1) {
        float4 f = make_float4(1.0f, 0.0f, 0.0f, 0.0f);
        memcpy(&one, &f, sizeof(S));
    } else {
        float2 f = make_float2(1.0f, 0.0f);
        memcpy(&one, &f, sizeof(S));
    }
    k_set_one<S><<<1, 1, 0, s>>>(static_cast<S*>(vpsi), index, one);
    return cudaGetLastError();
}

}  // namespace

size_t elem_bytes(int P) { return P == LLG_F32 ? 8 : 16; }

int tile_max_qubits(int P) { return P == LLG_F32 ? 14 : 13; }

#define LLG_DISPATCH(P, ...)                                 \
    switch (P) {                                             \
        case LLG_F64: { using Pol = PolF64; __VA_ARGS__; }   \
        case LLG_DF64: { using Pol = PolDF64; __VA_ARGS__; } \
        case LLG_F32: { using Pol = PolF32; __VA_ARGS__; }   \
        default: return cudaErrorInvalidValue;               \
    }

cudaError_t launch_init_basis(int P, void* psi, uint64_t size, uint64_t index, cudaStream_t s) {
    LLG_DISPATCH(P, return init_basis_t<Pol>(psi, size, index, s));
}

cudaError_t launch_exec_op(int P, void* psi, int n, const ExecOp& op, cudaStream_t s) {
    LLG_DISPATCH(P, return exec_op_t<Pol>(psi, n, op, s));
}

cudaError_t fp64_fma_rate(int iters, double* fma_per_s) {
    const unsigned grid = (unsigned)sm_count() * 8;
    cudaStream_t s = nullptr;
    cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (e != cudaSuccess) return e;
    cudaEvent_t a = nullptr, b = nullptr;
    if ((e = cudaEventCreate(&a)) == cudaSuccess && (e = cudaEventCreate(&b)) == cudaSuccess) {
        k_dfma_rate<<<grid, 256, 0, s>>>(nullptr, iters / 8 + 1, 0.9999999, 1e-9);
        cudaEventRecord(a, s);
        k_dfma_rate<<<grid, 256, 0, s>>>(nullptr, iters, 0.9999999, 1e-9);
        cudaEventRecord(b, s);
        e = cudaEventSynchronize(b);
        float ms = 0.0f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
        if (e == cudaSuccess) *fma_per_s = (double)grid * 256.0 * 8.0 * (double)iters / (ms * 1e-3);
    }
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
    cudaStreamDestroy(s);
    return e;
}

cudaError_t launch_tile_pass(int P, void* psi, int n, const PassDesc& pd, const ExecOp* d_ops, const uint64_t* d_tables,
                             int threads, int* err_flag, cudaStream_t s, double* mirror) {
    LLG_DISPATCH(P, return tile_pass_t<Pol>(psi, n, pd, d_ops, d_tables, threads, mirror, err_flag, s));
}

template <class PA>
cudaError_t compare_a(int PB, const void* a, const void* b, uint64_t size, double* partials, cudaStream_t s) {
    const unsigned grid = (unsigned)std::min<uint64_t>(kRedBlocks, (size + kThreads - 1) / kThreads);
    LLG_DISPATCH(PB, k_compare<PA, Pol><<<grid, kThreads, 0, s>>>(static_cast<const typename PA::S*>(a),
                                                                    static_cast<const typename Pol::S*>(b), size, partials);
                 return cudaGetLastError());
}

cudaError_t launch_compare(int PA, const void* a, int PB, const void* b, uint64_t size, double* partials, int* nblocks,
                           cudaStream_t s) {
    *nblocks = (int)std::min<uint64_t>(kRedBlocks, (size + kThreads - 1) / kThreads);
    LLG_DISPATCH(PA, return compare_a<Pol>(PB, a, b, size, partials, s));
}

cudaError_t launch_from_f64(int P, const double* src, void* dst, uint64_t count, cudaStream_t s) {
    LLG_DISPATCH(P, k_from_f64<Pol><<<grid_for(count, 1), kThreads, 0, s>>>(reinterpret_cast<const double2*>(src),
                                                                            static_cast<typename Pol::S*>(dst), count);
                 return cudaGetLastError());
}

cudaError_t launch_to_f64(int P, const void* src, double* dst, uint64_t count, cudaStream_t s) {
    LLG_DISPATCH(P, k_to_f64<Pol><<<grid_for(count, 1), kThreads, 0, s>>>(static_cast<const typename Pol::S*>(src),
                                                                          reinterpret_cast<double2*>(dst), count);
                 return cudaGetLastError());
}

cudaError_t launch_probabilities(int P, const void* psi, double* out, uint64_t count, cudaStream_t s) {
    LLG_DISPATCH(P, k_probs<Pol><<<grid_for(count, 1), kThreads, 0, s>>>(static_cast<const typename Pol::S*>(psi), out,
                                                                         count);
                 return cudaGetLastError());
}

cudaError_t launch_scale(int P, void* psi, uint64_t count, double factor, cudaStream_t s) {
    const uint64_t bits = pack_coef(P, factor);
    LLG_DISPATCH(P, k_scale<Pol><<<grid_for(count, 1), kThreads, 0, s>>>(static_cast<typename Pol::S*>(psi), count, bits);
                 return cudaGetLastError());
}

cudaError_t launch_reduce_z(int P, const void* psi, int n, const ZTerms& terms, double* d_partials, double* d_out,
                            cudaStream_t s) {
    const uint64_t size = 1ULL << n;
    unsigned g = grid_for(size, 4);
    if (g > (unsigned)kRedBlocks) g = kRedBlocks;
    LLG_DISPATCH(P, k_reduce_z<Pol><<<g, kThreads, 0, s>>>(static_cast<const typename Pol::S*>(psi), size, terms, d_partials);
                 cudaError_t e = cudaGetLastError(); if (e != cudaSuccess) return e;
                 k_finish<<<1, 32, 0, s>>>(d_partials, (int)g, d_out); return cudaGetLastError());
}

}  // namespace llg
