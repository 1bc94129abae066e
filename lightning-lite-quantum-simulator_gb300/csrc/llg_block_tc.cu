// llg_block_tc.cu -- dense 4- and 5-qubit blocks on complex128 (double-float) states with the
// fifth-generation tensor cores (tcgen05.mma, accumulators in tensor memory).
//
// A k-qubit block maps every group of A = 2^k amplitudes that differ only in the target qubits
// through an A x A complex matrix.  Written over reals it is one product per tile of 128 groups:
//     D[g][r] = sum_c X[g][c] W[r][c],   X[g] = (re a_0 .. re a_(A-1), im a_0 .. im a_(A-1)),
// with W the 2A x 2A real form of the matrix (K = N = 64 for k = 5, 32 for k = 4).  Double-float operands (~48-bit significands) are
// split exactly into six signed 8-bit slices against a power-of-two scale per row (the Ozaki
// scheme: Ozaki, Ogita, Oishi and Rump, Numer. Algorithms 2012):
//     X[g][k] = 2^(e_g - 8) sum_i x_i[g][k] 2^(-8 i),   W[r][k] = 2^(e_r - 8) sum_j w_j[r][k] 2^(-8 j),
// where every slice is an integer of magnitude <= 256, exact in bf16.  The 21 slice products
// with i + j <= 5 are accumulated by diagonal d = i + j into six fp32 accumulators in tensor
// memory.  A product of two slices is below 2^16 and 64 of them below 2^22, so each diagonal sum
// is an integer below 2^24 and the fp32 accumulation is exact (K = 32 leaves a factor 2 spare).
// Diagonals 0, 1 and 2 get an accumulator each; 3, 4 and 5 share one, filled by Horner's rule with
// the MMA's input scale (D = A B + 2^-8 D on the first product of a diagonal): it holds
// D_3 + 2^-8 D_4 + 2^-16 D_5, rounded at fp32 precision of D_3's scale.  The epilogue recombines
//     D = 2^(e_g + e_r - 16) (D_0 + 2^-8 D_1 + 2^-16 D_2 + 2^-24 D_345)
// into double-float, the first three terms exactly.  Dropped terms (i + j >= 6) and the
// rounding stay near 2^-46 of each group's largest amplitude.
//
// Persistent CTAs (k = 5: one of 512 threads per SM; k = 4: two of 256), pipelined by one tile:
// tensor memory holds two accumulator sets, and while the tensor cores compute tile i into one,
// the threads recombine tile i - 1 from the other and store it.  Per tile: every thread takes its
// 8 amplitudes from shared memory (copied asynchronously during the previous tile), the group
// scales come from the largest high part, the next tile's copies start, the threads wait
// (bounded) until the tensor cores have finished tile i - 1 (they read the slice buffer), write
// the slices in the no-swizzle K-major core-matrix layout, and one thread issues the 21 x K/16
// MMAs (M = 128 groups, N = 2A, K = 16 per instruction) and commits them to an mbarrier.  Then
// the epilogue of tile i - 1: tcgen05.ld of its accumulators, recombination, and stores straight
// from registers (a warp's lanes hold 32 consecutive groups).  The gate's slices are prepared on
// the host in double (exact) and copied to shared memory once per CTA.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include <cuda_runtime.h>

#include "llg_common.cuh"
#include "llg_internal.h"
#include "llg_launch.h"

namespace llg {

namespace {

constexpr int kTcGroups = 128;            // groups per tile (the MMA's M)
constexpr int kTcSlices = 6;              // 8-bit slices per operand
constexpr int kTcAcc = 4;                 // accumulators per set: diagonals 0, 1, 2 and 3..5
constexpr long kTcWaitLimit = 1L << 26;   // mbarrier polls before the kernel reports a timeout

// shapes of the k = 4 and k = 5 kernels
template <int KQ>
struct TcShape {
    static constexpr int kAmps = 1 << KQ;                          // amplitudes per group
    static constexpr int kReals = 2 * kAmps;                       // the MMA's K and N
    static constexpr int kThreads = KQ == 5 ? 512 : 256;
    static constexpr int kMinBlocks = KQ == 5 ? 1 : 2;             // CTAs per SM
    static constexpr int kPer = kTcGroups * kAmps / kThreads;      // amplitudes per thread (8)
    static constexpr int kSliceBytes = kTcGroups * kReals * 2;     // one state slice, bf16
    static constexpr int kWSliceBytes = kReals * kReals * 2;       // one gate slice, bf16
    static constexpr int kSetCols = kTcAcc * kReals;               // one accumulator set
    static constexpr int kTmemCols = 2 * kSetCols;                 // two sets (512 / 256: powers of two)
    static constexpr size_t kSmem =
        (size_t)kTcSlices * (kSliceBytes + kWSliceBytes) + (size_t)kTcGroups * kAmps * sizeof(float4);
    static_assert(kPer == 8, "one 8-wide core of real and one of imaginary parts per thread");
    static_assert(kTmemCols == 512 || kTmemCols == 256, "a power-of-two allocation of at most 512 columns");
    static_assert(kTmemCols * kMinBlocks <= 512, "the CTAs of an SM fit its tensor memory");
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// tcgen05 shared-memory descriptor, no swizzle: start, leading (K-direction core) byte offset,
// stride (8-row group) byte offset, descriptor version 1
__device__ __forceinline__ uint64_t tc_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((addr >> 4) & 0x3FFF);
    d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// byte offset of element (row, c) of a rows x kreals bf16 operand in the core-matrix layout:
// 8x8 cores of 128 bytes, K-direction cores adjacent, 8-row groups kreals / 8 cores apart
__host__ __device__ __forceinline__ uint32_t core_off(int row, int c, int kreals) {
    return (uint32_t)((row >> 3) * (kreals / 8) * 128 + (c >> 3) * 128 + (row & 7) * 16 + (c & 7) * 2);
}

// 2^e as a float for e in [-126, 127]
__device__ __forceinline__ float pow2f(int e) { return __uint_as_float((uint32_t)(e + 127) << 23); }

// double-float plus float (error-free up to the final renormalisation)
__device__ __forceinline__ df df_add_f(df a, float b) {
    const df s = two_sum(a.hi, b);
    return fast_two_sum(s.hi, __fadd_rn(s.lo, a.lo));
}

template <int KQ>
__global__ void __launch_bounds__(TcShape<KQ>::kThreads, TcShape<KQ>::kMinBlocks)
    k_block_tc(float4* __restrict__ psi, int n, BlockDesc bd, const uint16_t* __restrict__ wslices,
               const int32_t* __restrict__ wexp, int* __restrict__ err_flag) {
    using T = TcShape<KQ>;
    constexpr int kAmps = T::kAmps, kReals = T::kReals, kPer = T::kPer;
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char* sA = smem;                                  // kTcSlices state slices
    unsigned char* sW = smem + kTcSlices * T::kSliceBytes;     // kTcSlices gate slices
    // the next tile's amplitudes, [amplitude][group] so that a warp's 32 groups are 32 consecutive
    // float4s (a [group][amplitude] layout puts them kAmps * 16 bytes apart: 32-way bank conflicts)
    float4* sIn = reinterpret_cast<float4*>(sW + kTcSlices * T::kWSliceBytes);
    __shared__ uint64_t toff[kAmps];
    // group exponents, three tiles in turn: a tile's row is zeroed two tiles after its epilogue read it
    __shared__ int32_t eg_s[3][kTcGroups];
    __shared__ int32_t er_s[kReals];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_s;
    __shared__ int abort_s;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    for (int j = tid; j < kAmps; j += blockDim.x) {
        uint64_t o = 0;
        for (int b = 0; b < KQ; ++b)
            if ((j >> b) & 1) o |= 1ULL << bd.q[b];
        toff[j] = o;
    }
    for (int r = tid; r < kReals; r += blockDim.x) er_s[r] = wexp[r];
    {
        const uint4* src = reinterpret_cast<const uint4*>(wslices);
        uint4* dst = reinterpret_cast<uint4*>(sW);
        for (int i = tid; i < kTcSlices * T::kWSliceBytes / 16; i += blockDim.x) dst[i] = src[i];
    }
    if (tid == 0) {
        abort_s = 0;
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar)));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_s)),
                     "r"(T::kTmemCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_s;

    const uint64_t ngroups = 1ULL << (n - KQ);
    const uint64_t ntiles = ngroups / kTcGroups;
    // instruction descriptor: fp32 accumulate, bf16 A and B, both K-major, N = kReals, M = 128
    const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kReals >> 3) << 17) |
                           ((uint32_t)(kTcGroups >> 4) << 24);
    const uint32_t lbo = 128, sbo = (kReals / 8) * 128;
    // a group's kAmps / kPer threads sit in one warp: G consecutive lanes take G groups, the next G
    // lanes the same groups' next kPer amplitudes, and so on, so the group's scale is a shuffle
    // reduction (the slice stores of a warp still fill whole core-matrix rows)
    constexpr int kH = kAmps / kPer, kG = 32 / kH;
    const int gl = (tid % kG) + kG * (tid >> 5);  // the group this thread loads, slices and stores
    const int h = (tid / kG) % kH;                 // which kPer of its kAmps amplitudes
    uint32_t phase = 0;
    // a thread's amplitudes of a tile go to sIn[(kPer h + i) * 128 + gl] by asynchronous copies,
    // issued one tile ahead so that their latency hides behind the products and the epilogue
    auto prefetch = [&](uint64_t tile) {
        const uint64_t b = insert0_mask(tile * kTcGroups + (uint64_t)gl, bd.tmask);
#pragma unroll
        for (int i = 0; i < kPer; ++i)
            asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(&sIn[(kPer * h + i) * kTcGroups + gl])),
                         "l"(psi + (b | toff[kPer * h + i]))
                         : "memory");
        asm volatile("cp.async.commit_group;" ::: "memory");
    };
    __syncthreads();  // toff
    if ((uint64_t)blockIdx.x < ntiles) prefetch(blockIdx.x);

    // bounded wait for the products committed with parity `ph`; false: the limit ran out
    auto wait_mma = [&](uint32_t ph) {
        uint32_t done = 0;
        for (long it = 0; it < kTcWaitLimit && !done; ++it)
            asm volatile("{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}"
                         : "=r"(done)
                         : "r"(smem_u32(&mbar)), "r"(ph));
        return done != 0;
    };
    // recombine the tile in accumulator set `set` and store it: warp w reads lanes 32 (w & 3) ..
    // +31 (its groups) and the real and imaginary columns of amplitudes 8 (w >> 2) .. +7, so that
    // each thread writes whole amplitudes, a warp 32 consecutive groups per amplitude
    auto epilogue = [&](uint64_t tile, int set, int egb, int a0) {
        const int row = 32 * (warp & 3) + lane;
        const int eg = eg_s[egb][row] - 1000;  // stored with an offset of 1000
        df out[2][8];
#pragma unroll
        for (int part = 0; part < 2; ++part) {
            uint32_t v[kTcAcc][8];
#pragma unroll
            for (int d = 0; d < kTcAcc; ++d) {
                const uint32_t taddr = tmem + ((uint32_t)(32 * (warp & 3)) << 16) +
                                       (uint32_t)(set * T::kSetCols + d * kReals + kAmps * part + a0);
                asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                             : "=r"(v[d][0]), "=r"(v[d][1]), "=r"(v[d][2]), "=r"(v[d][3]), "=r"(v[d][4]), "=r"(v[d][5]),
                               "=r"(v[d][6]), "=r"(v[d][7])
                             : "r"(taddr));
            }
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
            for (int c = 0; c < 8; ++c) {
                // D_0 + 2^-8 D_1 + 2^-16 D_2 exactly, 2^-24 D_345 rounded once (below 2^-46)
                const float d0 = __uint_as_float(v[0][c]), d1 = __uint_as_float(v[1][c]) * 0x1p-8f;
                const float d2 = __uint_as_float(v[2][c]) * 0x1p-16f;
                const float t = __uint_as_float(v[3][c]) * 0x1p-24f;
                df acc = two_sum(d0, d1);
                acc = df_add_f(acc, d2);
                acc = fast_two_sum(acc.hi, __fadd_rn(acc.lo, t));
                // 2^(e_g + e_r - 16), split in two factors so that each stays a normal float
                const int et = eg + er_s[kAmps * part + a0 + c] - 16;
                const int e1 = max(min(et, 100), -100), e2 = max(min(et - e1, 100), -126);
                const float f1 = pow2f(e1), f2 = pow2f(e2);
                out[part][c] = {acc.hi * f1 * f2, acc.lo * f1 * f2};
            }
        }
        const uint64_t base = insert0_mask(tile * kTcGroups + (uint64_t)row, bd.tmask);
#pragma unroll
        for (int c = 0; c < 8; ++c)
            psi[base | toff[a0 + c]] = make_float4(out[0][c].hi, out[1][c].hi, out[0][c].lo, out[1][c].lo);
        // the accumulator set is read: the next MMAs into it may follow the next barrier
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    };
    // one MMA: D (+)= A B, with D first scaled by 2^-8 when `scale` is set
    auto mma = [&](uint32_t dcol, uint64_t da, uint64_t dw, uint32_t acc, bool scale) {
        if (scale)
            asm volatile("{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\ntcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p, 8;\n}" ::"r"(
                             dcol),
                         "l"(da), "l"(dw), "r"(idesc), "r"(acc));
        else
            asm volatile("{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\ntcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(
                             dcol),
                         "l"(da), "l"(dw), "r"(idesc), "r"(acc));
    };

    uint64_t prev_tile = 0;
    bool have_prev = false;
    int set = 0, egb = 0;
    for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x, set ^= 1, egb = egb == 2 ? 0 : egb + 1) {
        // ---- this thread's amplitudes of group gl (its own copies), the group's scale ----
        asm volatile("cp.async.wait_group 0;" ::: "memory");
        float4 a[kPer];
        float mx = 0.0f;
#pragma unroll
        for (int i = 0; i < kPer; ++i) {
            // stored pairs may be unnormalised (|lo| above half an ulp of hi): TwoSum makes hi the
            // leading part, which the scale and the split into slices below rely on
            const float4 v = sIn[(kPer * h + i) * kTcGroups + gl];
            const df re = two_sum(v.x, v.z), im = two_sum(v.y, v.w);
            a[i] = make_float4(re.hi, im.hi, re.lo, im.lo);
            mx = fmaxf(mx, fmaxf(fabsf(a[i].x), fabsf(a[i].y)));
        }
        // the group's threads agree on the largest high part (lanes kG, 2 kG, ... apart)
#pragma unroll
        for (int off = kG; off < 32; off <<= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, off));
        // all |x| < 2^e with e from the high parts' largest exponent; clamped so that the scale
        // factors 2^(8 - e) and 2^(32 - e) below stay normal floats (groups under 2^-94 keep their
        // absolute error below 2^-134 instead of a relative one)
        int e = (int)((__float_as_uint(mx) >> 23) & 0xFF) - 126;
        e = max(e, -94);
        // for the epilogue of this tile (during the next one, after this tile's slicing barrier);
        // eg_s[egb] was last read by the epilogue of tile i - 3, during tile i - 1
        if (h == 0) eg_s[egb][gl] = e + 1000;
        // ---- the previous tile's products must be done before its slices are overwritten; the
        // barrier also ends every thread's reads of sIn before the next tile's copies start ----
        if (have_prev && !wait_mma(phase)) abort_s = 1;
        __syncthreads();
        if (abort_s) {
            // report, then give the products in flight a second bounded wait before the
            // accumulators are freed
            if (tid == 0) atomicExch(err_flag, 1);
            wait_mma(phase);
            have_prev = false;
            break;
        }
        if (have_prev) {
            phase ^= 1;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        }
        if (tile + gridDim.x < ntiles) prefetch(tile + gridDim.x);
        // ---- six 8-bit slices per real, into the core-matrix layout ----
        {
            const float sc = pow2f(8 - e), sclo = pow2f(32 - e);
#pragma unroll
            for (int part = 0; part < 2; ++part) {  // 0: real parts (c = j), 1: imaginary (c = kAmps + j)
                uint32_t packed[kTcSlices][4];
#pragma unroll
                for (int i2 = 0; i2 < 4; ++i2) {
                    float sl[2][kTcSlices];
#pragma unroll
                    for (int w = 0; w < 2; ++w) {
                        const float4 v = a[2 * i2 + w];
                        const float hi = part ? v.y : v.x, lo = part ? v.w : v.z;
                        float r = hi * sc;
#pragma unroll
                        for (int s = 0; s < 3; ++s) {
                            sl[w][s] = rintf(r);
                            r = (r - sl[w][s]) * 256.0f;
                        }
                        r = fmaf(lo, sclo, r);
#pragma unroll
                        for (int s = 3; s < kTcSlices; ++s) {
                            sl[w][s] = rintf(r);
                            r = (r - sl[w][s]) * 256.0f;
                        }
                    }
                    // integers of magnitude <= 256: the bf16 value is the float's high half
#pragma unroll
                    for (int s = 0; s < kTcSlices; ++s)
                        packed[s][i2] = (__float_as_uint(sl[0][s]) >> 16) | (__float_as_uint(sl[1][s]) & 0xFFFF0000u);
                }
                const int c0 = kAmps * part + kPer * h;
#pragma unroll
                for (int s = 0; s < kTcSlices; ++s)
                    *reinterpret_cast<uint4*>(sA + s * T::kSliceBytes + core_off(gl, c0, kReals)) =
                        make_uint4(packed[s][0], packed[s][1], packed[s][2], packed[s][3]);
            }
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();  // the slices are written; the epilogue two tiles back has read this set
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        // ---- 21 slice products (i + j <= 5) into four accumulators of this set, K / 16 steps each ----
        if (tid == 0) {
            const uint32_t tset = tmem + (uint32_t)(set * T::kSetCols);
            const uint64_t da0 = tc_desc(smem_u32(sA), lbo, sbo), dw0 = tc_desc(smem_u32(sW), lbo, sbo);
            auto diagonal = [&](int d, uint32_t dcol, bool first_fresh) {
                bool first = true;
                for (int i = 0; i <= d; ++i) {
                    const int j = d - i;
                    for (int ks = 0; ks < kReals / 16; ++ks) {
                        // the start address is the descriptor's low field (bytes / 16, below 2^14 for
                        // any shared-memory address): offsets add to it directly
                        const uint64_t da = da0 + (uint64_t)((i * T::kSliceBytes + ks * 256) >> 4);
                        const uint64_t dw = dw0 + (uint64_t)((j * T::kWSliceBytes + ks * 256) >> 4);
                        // a diagonal's first product starts the accumulator (first_fresh) or scales
                        // the diagonals above it by 2^-8 (Horner)
                        mma(dcol, da, dw, (first && first_fresh) ? 0u : 1u, first && !first_fresh);
                        first = false;
                    }
                }
            };
            for (int d = 0; d < 3; ++d) diagonal(d, tset + (uint32_t)(d * kReals), true);
            diagonal(5, tset + (uint32_t)(3 * kReals), true);
            diagonal(4, tset + (uint32_t)(3 * kReals), false);
            diagonal(3, tset + (uint32_t)(3 * kReals), false);
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(&mbar)));
        }
        // ---- the previous tile's epilogue, under this tile's products.  Warp 0 issued the
        // products; its share of the epilogue (lanes 0-31, amplitudes 0-7) goes to warp 4, which
        // reads the same tensor-memory lanes, so that the issue does not delay the next barrier ----
        if (have_prev) {
            const int egp = egb == 0 ? 2 : egb - 1;
            if (warp != 0) epilogue(prev_tile, set ^ 1, egp, 8 * (warp >> 2));
            if (warp == 4) epilogue(prev_tile, set ^ 1, egp, 0);
            if (warp == 0) asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        }
        prev_tile = tile;
        have_prev = true;
    }
    // the last tile
    if (have_prev) {
        if (!wait_mma(phase)) abort_s = 1;
        __syncthreads();
        if (abort_s) {
            if (tid == 0) atomicExch(err_flag, 1);
            wait_mma(phase);
        } else {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            epilogue(prev_tile, set ^ 1, egb == 0 ? 2 : egb - 1, 8 * (warp >> 2));
        }
    }
    asm volatile("cp.async.wait_group 0;" ::: "memory");  // no copy left in flight on any exit
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(T::kTmemCols));
}

template <int KQ>
cudaError_t launch_tc(void* psi, int n, const BlockDesc& bd, const void* d_weights, int* err_flag, cudaStream_t s) {
    using T = TcShape<KQ>;
    // once per block size (thread-safe static initialisation)
    static const cudaError_t attr = cudaFuncSetAttribute(k_block_tc<KQ>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)T::kSmem);
    if (attr != cudaSuccess) return attr;
    const uint64_t ntiles = (1ULL << (n - KQ)) / kTcGroups;
    int sms = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const uint64_t cap = (uint64_t)sms * T::kMinBlocks;
    const unsigned grid = (unsigned)(ntiles < cap ? ntiles : cap);
    const uint16_t* w = static_cast<const uint16_t*>(d_weights);
    const int32_t* ex = reinterpret_cast<const int32_t*>(static_cast<const unsigned char*>(d_weights) +
                                                          (size_t)kTcSlices * T::kWSliceBytes);
    k_block_tc<KQ><<<grid, T::kThreads, T::kSmem, s>>>(static_cast<float4*>(psi), n, bd, w, ex, err_flag);
    return cudaGetLastError();
}

// ------------------------------------------------------------------------------------------
// IEEE complex128 (FP64) states, k = 4: the same pipeline with eight slices per operand and an
// exact recombination, so the products leave the FP64 pipe altogether.
//   * A real x of a group whose largest biased exponent is e_g is the 62-bit fixed-point integer
//     X = m 2^(9 - e_g + e) (m the 53-bit significand, e its exponent; truncated below 2^-61 of the
//     group's scale), split into its signed top byte and seven unsigned bytes:
//     x = 2^(e_g - 1028) sum_s d_s 2^(-8 s), d_0 in [-64, 64], d_1..7 in [0, 255], all exact in
//     bf16.  The gate's rows are split on the host into balanced digits of magnitude <= 128 (eight
//     slices capture a double exactly).
//   * The 36 slice products with i + j <= 7 go by diagonal into six accumulators: d = 0..4 one each
//     (a diagonal has at most eight products of 32 terms, each below 2^15: below 2^23, exact in
//     fp32), d = 5, 6, 7 shared by Horner's rule through the MMA's input scale.
//   * Epilogue: every exact diagonal becomes an integer (round-to-nearest conversion), the Horner
//     accumulator is rounded to an integer at 2^-40 of D_0's unit, the six combine exactly in a
//     64-bit integer (below 2^61), which is converted to double once (the only rounding of the
//     product, apart from the slicing's 2^-61 truncation and the dropped diagonals near 2^-64) and
//     scaled by 2^(e_g + e_r - 1075) through its exponent field.
// One CTA of 512 threads per SM, four amplitudes per thread: two accumulator sets of 6 x 32
// columns take 384 of the 512 columns of tensor memory.
// ------------------------------------------------------------------------------------------
constexpr int kTcSlicesF64 = 8;
constexpr int kTcAccF64 = 6;

template <int KQ>
struct TcShapeF64 {
    static constexpr int kAmps = 1 << KQ;
    static constexpr int kReals = 2 * kAmps;                   // the MMA's K and N (32 / 16)
    static constexpr int kThreads = KQ == 4 ? 512 : 256;
    static constexpr int kCtas = KQ == 4 ? 1 : 2;              // CTAs per SM
    static constexpr int kPer = kTcGroups * kAmps / kThreads;  // amplitudes per thread (4)
    static constexpr int kEpi = kAmps / (kThreads / 128);      // amplitudes per warp in the epilogue (4)
    static constexpr int kSliceBytes = kTcGroups * kReals * 2;
    static constexpr int kWSliceBytes = kReals * kReals * 2;
    static constexpr int kSetCols = kTcAccF64 * kReals;
    static constexpr int kTmemCols = 512 / kCtas;
    static constexpr size_t kSmemUsed =
        (size_t)kTcSlicesF64 * (kSliceBytes + kWSliceBytes) + (size_t)kTcGroups * kAmps * sizeof(double2);
    // padded so that no more than kCtas CTAs share an SM: one more would wait for the others'
    // tensor-memory columns for its whole run
    static constexpr size_t kSmemFloor = (size_t)(228 * 1024) / (kCtas + 1) + 1024;
    static constexpr size_t kSmem = kSmemUsed > kSmemFloor ? kSmemUsed : kSmemFloor;
    static_assert(KQ == 3 || KQ == 4, "the eight-slice FP64 form fits shared memory for 3- and 4-qubit blocks");
    static_assert(kPer == 4 && kEpi == 4, "half an 8-wide core row of real and of imaginary parts per thread");
    static_assert(2 * kSetCols <= kTmemCols, "two accumulator sets in the allocation");
    static_assert(kSmem * kCtas <= 227 * 1024, "kCtas CTAs fit an SM's shared memory");
};

// bf16 bits of a small integer d (|d| <= 256): the float d built by the magic addition, whose value
// has at most 8 significant bits, keeps its high half exactly
__device__ __forceinline__ uint32_t bf16_of_int(int d) {
    const float f = __int_as_float(0x4B400000 + d) - 12582912.0f;
    return __float_as_uint(f) >> 16;
}

// the eight digits of x against the group exponent eg (see above), most significant first: the
// signed top byte of the 62-bit integer X and its seven low bytes unsigned (X = t 2^56 +
// sum_s u_s 2^(8 (7 - s)), u_s in [0, 255], |t| <= 64), read straight from X's two 32-bit words
__device__ __forceinline__ void slice_f64(double x, int eg, uint32_t (&bits)[kTcSlicesF64]) {
    const long long b = __double_as_longlong(x);
    const int ex = (int)((b >> 52) & 0x7FF);
    const long long m = (b & 0xFFFFFFFFFFFFFLL) | (ex ? (1LL << 52) : 0LL);
    const int sh = 9 - (eg - (ex ? ex : 1));
    long long X = sh >= 0 ? (m << sh) : (sh > -63 ? (m >> -sh) : 0LL);
    if (b < 0) X = -X;
    const uint32_t lo = (uint32_t)X, hi = (uint32_t)((unsigned long long)X >> 32);
    bits[0] = bf16_of_int((int)hi >> 24);
#pragma unroll
    for (int s = 1; s < 4; ++s) bits[s] = bf16_of_int((int)((hi >> (24 - 8 * s)) & 0xFF));
#pragma unroll
    for (int s = 4; s < kTcSlicesF64; ++s) bits[s] = bf16_of_int((int)((lo >> (56 - 8 * s)) & 0xFF));
}

// an fp32 integer value v (|v| < 2^24: every diagonal sum), or v rounded to the nearest integer
__device__ __forceinline__ int int_of_f32(float v) { return __float2int_rn(v); }

template <int KQ>
__global__ void __launch_bounds__(TcShapeF64<KQ>::kThreads, TcShapeF64<KQ>::kCtas)
    k_block_tc_f64(double2* __restrict__ psi, int n, BlockDesc bd, const uint16_t* __restrict__ wslices,
                   const int32_t* __restrict__ wexp, int* __restrict__ err_flag) {
    using T = TcShapeF64<KQ>;
    constexpr int kAmps = T::kAmps, kReals = T::kReals, kPer = T::kPer;
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char* sA = smem;                                   // kTcSlicesF64 state slices
    unsigned char* sW = smem + kTcSlicesF64 * T::kSliceBytes;   // kTcSlicesF64 gate slices
    double2* sIn = reinterpret_cast<double2*>(sW + kTcSlicesF64 * T::kWSliceBytes);  // [amplitude][group]
    __shared__ uint64_t toff[kAmps];
    __shared__ int32_t eg_s[3][kTcGroups];
    __shared__ int32_t er_s[kReals];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_s;
    __shared__ int abort_s;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    for (int j = tid; j < kAmps; j += blockDim.x) {
        uint64_t o = 0;
        for (int b = 0; b < KQ; ++b)
            if ((j >> b) & 1) o |= 1ULL << bd.q[b];
        toff[j] = o;
    }
    for (int r = tid; r < kReals; r += blockDim.x) er_s[r] = wexp[r];
    {
        const uint4* src = reinterpret_cast<const uint4*>(wslices);
        uint4* dst = reinterpret_cast<uint4*>(sW);
        for (int i = tid; i < kTcSlicesF64 * T::kWSliceBytes / 16; i += blockDim.x) dst[i] = src[i];
    }
    if (tid == 0) {
        abort_s = 0;
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar)));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_s)),
                     "r"(T::kTmemCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_s;

    const uint64_t ngroups = 1ULL << (n - KQ);
    const uint64_t ntiles = ngroups / kTcGroups;
    const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kReals >> 3) << 17) |
                           ((uint32_t)(kTcGroups >> 4) << 24);
    const uint32_t lbo = 128, sbo = (kReals / 8) * 128;
    constexpr int kH = kAmps / kPer, kG = 32 / kH;
    const int gl = (tid % kG) + kG * (tid >> 5);
    const int h = (tid / kG) % kH;
    uint32_t phase = 0;
    auto prefetch = [&](uint64_t tile) {
        const uint64_t b = insert0_mask(tile * kTcGroups + (uint64_t)gl, bd.tmask);
#pragma unroll
        for (int i = 0; i < kPer; ++i)
            asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(&sIn[(kPer * h + i) * kTcGroups + gl])),
                         "l"(psi + (b | toff[kPer * h + i]))
                         : "memory");
        asm volatile("cp.async.commit_group;" ::: "memory");
    };
    __syncthreads();  // toff
    if ((uint64_t)blockIdx.x < ntiles) prefetch(blockIdx.x);

    auto wait_mma = [&](uint32_t ph) {
        uint32_t done = 0;
        for (long it = 0; it < kTcWaitLimit && !done; ++it)
            asm volatile("{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}"
                         : "=r"(done)
                         : "r"(smem_u32(&mbar)), "r"(ph));
        return done != 0;
    };
    // warp w reads tensor-memory lanes 32 (w & 3) .. +31 (its groups) and amplitudes
    // kEpi (w >> 2) .. + kEpi - 1
    constexpr int kEpi = T::kEpi;
    auto epilogue = [&](uint64_t tile, int set, int egb, int a0) {
        const int row = 32 * (warp & 3) + lane;
        const int eg = eg_s[egb][row];
        double out[2][kEpi];
#pragma unroll
        for (int part = 0; part < 2; ++part) {
            uint32_t v[kTcAccF64][kEpi];
#pragma unroll
            for (int d = 0; d < kTcAccF64; ++d) {
                const uint32_t taddr = tmem + ((uint32_t)(32 * (warp & 3)) << 16) +
                                       (uint32_t)(set * T::kSetCols + d * kReals + kAmps * part + a0);
                asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
                             : "=r"(v[d][0]), "=r"(v[d][1]), "=r"(v[d][2]), "=r"(v[d][3])
                             : "r"(taddr));
            }
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
            for (int c = 0; c < kEpi; ++c) {
                // 2^40 sum_d 2^(-8 d) D_d as one integer: D_0..D_4 exact, D_567 rounded at 2^-40
                long long acc = (long long)int_of_f32(__uint_as_float(v[5][c]));
#pragma unroll
                for (int d = 0; d < 5; ++d) acc += (long long)int_of_f32(__uint_as_float(v[d][c])) << (40 - 8 * d);
                double r = __ll2double_rn(acc);
                // times 2^(e_g - 1028) 2^(e_r - 7) 2^-40 through the exponent field
                const int et = eg + er_s[kAmps * part + a0 + c] - 1075;
                const long long rb = __double_as_longlong(r);
                const int ef = (int)((rb >> 52) & 0x7FF), ne = ef + et;
                if (ef != 0 && ne >= 1 && ne <= 2046) r = __longlong_as_double(rb + ((long long)et << 52));
                else if (r != 0.0) r = ldexp(r, et);
                out[part][c] = r;
            }
        }
        const uint64_t base = insert0_mask(tile * kTcGroups + (uint64_t)row, bd.tmask);
#pragma unroll
        for (int c = 0; c < kEpi; ++c) psi[base | toff[a0 + c]] = make_double2(out[0][c], out[1][c]);
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    };
    auto mma = [&](uint32_t dcol, uint64_t da, uint64_t dw, uint32_t acc, bool scale) {
        if (scale)
            asm volatile("{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\ntcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p, 8;\n}" ::"r"(
                             dcol),
                         "l"(da), "l"(dw), "r"(idesc), "r"(acc));
        else
            asm volatile("{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\ntcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(
                             dcol),
                         "l"(da), "l"(dw), "r"(idesc), "r"(acc));
    };

    uint64_t prev_tile = 0;
    bool have_prev = false;
    int set = 0, egb = 0;
    for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x, set ^= 1, egb = egb == 2 ? 0 : egb + 1) {
        asm volatile("cp.async.wait_group 0;" ::: "memory");
        double2 a[kPer];
        int mx = 0;
#pragma unroll
        for (int i = 0; i < kPer; ++i) {
            a[i] = sIn[(kPer * h + i) * kTcGroups + gl];
            mx = max(mx, (int)((__double_as_longlong(a[i].x) >> 52) & 0x7FF));
            mx = max(mx, (int)((__double_as_longlong(a[i].y) >> 52) & 0x7FF));
        }
#pragma unroll
        for (int off = kG; off < 32; off <<= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, off));
        const int eg = max(mx, 1);  // subnormal and zero groups take the smallest normal scale
        if (h == 0) eg_s[egb][gl] = eg;
        if (have_prev && !wait_mma(phase)) abort_s = 1;
        __syncthreads();
        if (abort_s) {
            if (tid == 0) atomicExch(err_flag, 1);
            wait_mma(phase);
            have_prev = false;
            break;
        }
        if (have_prev) {
            phase ^= 1;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        }
        if (tile + gridDim.x < ntiles) prefetch(tile + gridDim.x);
        // ---- eight balanced 8-bit slices per real, into the core-matrix layout (half a core row
        // of 8 bytes per thread and slice) ----
#pragma unroll
        for (int part = 0; part < 2; ++part) {
            uint32_t packed[kTcSlicesF64][kPer / 2];
#pragma unroll
            for (int i2 = 0; i2 < kPer / 2; ++i2) {
                uint32_t b0[kTcSlicesF64], b1[kTcSlicesF64];
                slice_f64(part ? a[2 * i2].y : a[2 * i2].x, eg, b0);
                slice_f64(part ? a[2 * i2 + 1].y : a[2 * i2 + 1].x, eg, b1);
#pragma unroll
                for (int s = 0; s < kTcSlicesF64; ++s) packed[s][i2] = b0[s] | (b1[s] << 16);
            }
            const int c0 = kAmps * part + kPer * h;
#pragma unroll
            for (int s = 0; s < kTcSlicesF64; ++s)
                *reinterpret_cast<uint2*>(sA + s * T::kSliceBytes + core_off(gl, c0, kReals)) =
                    make_uint2(packed[s][0], packed[s][1]);
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        // ---- 36 slice products (i + j <= 7): diagonals 0..4 one accumulator each, 5..7 one by Horner ----
        if (tid == 0) {
            const uint32_t tset = tmem + (uint32_t)(set * T::kSetCols);
            const uint64_t da0 = tc_desc(smem_u32(sA), lbo, sbo), dw0 = tc_desc(smem_u32(sW), lbo, sbo);
            auto diagonal = [&](int d, uint32_t dcol, bool first_fresh) {
                bool first = true;
                for (int i = 0; i <= d; ++i) {
                    const int j = d - i;
                    if (i >= kTcSlicesF64 || j >= kTcSlicesF64) continue;
                    for (int ks = 0; ks < kReals / 16; ++ks) {
                        const uint64_t da = da0 + (uint64_t)((i * T::kSliceBytes + ks * 256) >> 4);
                        const uint64_t dw = dw0 + (uint64_t)((j * T::kWSliceBytes + ks * 256) >> 4);
                        mma(dcol, da, dw, (first && first_fresh) ? 0u : 1u, first && !first_fresh);
                        first = false;
                    }
                }
            };
            for (int d = 0; d < 5; ++d) diagonal(d, tset + (uint32_t)(d * kReals), true);
            diagonal(7, tset + (uint32_t)(5 * kReals), true);
            diagonal(6, tset + (uint32_t)(5 * kReals), false);
            diagonal(5, tset + (uint32_t)(5 * kReals), false);
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(&mbar)));
        }
        if (have_prev) {
            const int egp = egb == 0 ? 2 : egb - 1;
            if (warp != 0) epilogue(prev_tile, set ^ 1, egp, kEpi * (warp >> 2));
            if (warp == 4) epilogue(prev_tile, set ^ 1, egp, 0);
            if (warp == 0) asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        }
        prev_tile = tile;
        have_prev = true;
    }
    if (have_prev) {
        if (!wait_mma(phase)) abort_s = 1;
        __syncthreads();
        if (abort_s) {
            if (tid == 0) atomicExch(err_flag, 1);
            wait_mma(phase);
        } else {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            epilogue(prev_tile, set ^ 1, egb == 0 ? 2 : egb - 1, kEpi * (warp >> 2));
        }
    }
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(T::kTmemCols));
}

// IEEE complex128, k = 5: the same arithmetic as k_block_tc_f64 on 32-amplitude groups (K = N = 64).
// Six accumulators of 64 columns take 384 of the 512 columns, so there is one set and a tile's
// products and epilogue run one after the other; eight 16 KB state slices and eight 8 KB gate
// slices take 192 KB, so the next tile is prefetched into registers (eight 16-byte loads per
// thread, issued before the products) instead of a shared-memory buffer.
struct TcShapeF64x5 {
    static constexpr int kAmps = 32, kReals = 64, kThreads = 512;
    static constexpr int kPer = kTcGroups * kAmps / kThreads;  // 8
    static constexpr int kEpi = kAmps / (kThreads / 128);      // 8
    static constexpr int kSliceBytes = kTcGroups * kReals * 2;
    static constexpr int kWSliceBytes = kReals * kReals * 2;
    static constexpr int kTmemCols = 512;
    static constexpr size_t kSmem = (size_t)kTcSlicesF64 * (kSliceBytes + kWSliceBytes);
    static_assert(kTcAccF64 * kReals <= kTmemCols, "one accumulator set");
    static_assert(kSmem <= 200 * 1024, "slices fit shared memory");
};

__global__ void __launch_bounds__(TcShapeF64x5::kThreads, 1)
    k_block_tc_f64x5(double2* __restrict__ psi, int n, BlockDesc bd, const uint16_t* __restrict__ wslices,
                     const int32_t* __restrict__ wexp, int* __restrict__ err_flag) {
    using T = TcShapeF64x5;
    constexpr int KQ = 5, kAmps = T::kAmps, kReals = T::kReals, kPer = T::kPer, kEpi = T::kEpi;
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char* sA = smem;
    unsigned char* sW = smem + kTcSlicesF64 * T::kSliceBytes;
    __shared__ uint64_t toff[kAmps];
    __shared__ int32_t eg_s[2][kTcGroups];  // by tile parity: a row is rewritten two tiles later
    __shared__ int32_t er_s[kReals];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_s;
    __shared__ int abort_s;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    for (int j = tid; j < kAmps; j += blockDim.x) {
        uint64_t o = 0;
        for (int b = 0; b < KQ; ++b)
            if ((j >> b) & 1) o |= 1ULL << bd.q[b];
        toff[j] = o;
    }
    for (int r = tid; r < kReals; r += blockDim.x) er_s[r] = wexp[r];
    {
        const uint4* src = reinterpret_cast<const uint4*>(wslices);
        uint4* dst = reinterpret_cast<uint4*>(sW);
        for (int i = tid; i < kTcSlicesF64 * T::kWSliceBytes / 16; i += blockDim.x) dst[i] = src[i];
    }
    if (tid == 0) {
        abort_s = 0;
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar)));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_s)),
                     "r"(T::kTmemCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_s;

    const uint64_t ngroups = 1ULL << (n - KQ);
    const uint64_t ntiles = ngroups / kTcGroups;
    const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kReals >> 3) << 17) |
                           ((uint32_t)(kTcGroups >> 4) << 24);
    const uint32_t lbo = 128, sbo = (kReals / 8) * 128;
    constexpr int kH = kAmps / kPer, kG = 32 / kH;
    const int gl = (tid % kG) + kG * (tid >> 5);
    const int h = (tid / kG) % kH;
    uint32_t phase = 0;
    double2 nxt[kPer];
    auto prefetch = [&](uint64_t tile) {
        const uint64_t b = insert0_mask(tile * kTcGroups + (uint64_t)gl, bd.tmask);
#pragma unroll
        for (int i = 0; i < kPer; ++i) nxt[i] = __ldcg(psi + (b | toff[kPer * h + i]));
    };
    __syncthreads();  // toff
    if ((uint64_t)blockIdx.x < ntiles) prefetch(blockIdx.x);

    auto wait_mma = [&](uint32_t ph) {
        uint32_t done = 0;
        for (long it = 0; it < kTcWaitLimit && !done; ++it)
            asm volatile("{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}"
                         : "=r"(done)
                         : "r"(smem_u32(&mbar)), "r"(ph));
        return done != 0;
    };
    auto mma = [&](uint32_t dcol, uint64_t da, uint64_t dw, uint32_t acc, bool scale) {
        if (scale)
            asm volatile("{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\ntcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p, 8;\n}" ::"r"(
                             dcol),
                         "l"(da), "l"(dw), "r"(idesc), "r"(acc));
        else
            asm volatile("{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\ntcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(
                             dcol),
                         "l"(da), "l"(dw), "r"(idesc), "r"(acc));
    };

    int par = 0;
    for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x, par ^= 1) {
        double2 a[kPer];
        int mx = 0;
#pragma unroll
        for (int i = 0; i < kPer; ++i) {
            a[i] = nxt[i];
            mx = max(mx, (int)((__double_as_longlong(a[i].x) >> 52) & 0x7FF));
            mx = max(mx, (int)((__double_as_longlong(a[i].y) >> 52) & 0x7FF));
        }
#pragma unroll
        for (int off = kG; off < 32; off <<= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, off));
        const int eg = max(mx, 1);
        if (h == 0) eg_s[par][gl] = eg;  // read by this tile's epilogue, after the barrier below
        if (tile + gridDim.x < ntiles) prefetch(tile + gridDim.x);
        // ---- eight balanced 8-bit slices per real (the previous tile's products are done) ----
#pragma unroll
        for (int part = 0; part < 2; ++part) {
            uint32_t packed[kTcSlicesF64][kPer / 2];
#pragma unroll
            for (int i2 = 0; i2 < kPer / 2; ++i2) {
                uint32_t b0[kTcSlicesF64], b1[kTcSlicesF64];
                slice_f64(part ? a[2 * i2].y : a[2 * i2].x, eg, b0);
                slice_f64(part ? a[2 * i2 + 1].y : a[2 * i2 + 1].x, eg, b1);
#pragma unroll
                for (int s = 0; s < kTcSlicesF64; ++s) packed[s][i2] = b0[s] | (b1[s] << 16);
            }
            const int c0 = kAmps * part + kPer * h;
#pragma unroll
            for (int s = 0; s < kTcSlicesF64; ++s)
                *reinterpret_cast<uint4*>(sA + s * T::kSliceBytes + core_off(gl, c0, kReals)) =
                    make_uint4(packed[s][0], packed[s][1], packed[s][2], packed[s][3]);
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();  // slices and exponents written; the previous epilogue has read the accumulators
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        if (abort_s) break;  // written before the barrier: the same on every thread
        if (tid == 0) {
            const uint64_t da0 = tc_desc(smem_u32(sA), lbo, sbo), dw0 = tc_desc(smem_u32(sW), lbo, sbo);
            auto diagonal = [&](int d, uint32_t dcol, bool first_fresh) {
                bool first = true;
                for (int i = 0; i <= d; ++i) {
                    const int j = d - i;
                    if (i >= kTcSlicesF64 || j >= kTcSlicesF64) continue;
                    for (int ks = 0; ks < kReals / 16; ++ks) {
                        const uint64_t da = da0 + (uint64_t)((i * T::kSliceBytes + ks * 256) >> 4);
                        const uint64_t dw = dw0 + (uint64_t)((j * T::kWSliceBytes + ks * 256) >> 4);
                        mma(dcol, da, dw, (first && first_fresh) ? 0u : 1u, first && !first_fresh);
                        first = false;
                    }
                }
            };
            for (int d = 0; d < 5; ++d) diagonal(d, tmem + (uint32_t)(d * kReals), true);
            diagonal(7, tmem + (uint32_t)(5 * kReals), true);
            diagonal(6, tmem + (uint32_t)(5 * kReals), false);
            diagonal(5, tmem + (uint32_t)(5 * kReals), false);
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(&mbar)));
        }
        if (!wait_mma(phase)) abort_s = 1;
        phase ^= 1;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        // ---- epilogue: warp w, tensor-memory lanes 32 (w & 3) .. +31, amplitudes kEpi (w >> 2) .. ----
        {
            const int row = 32 * (warp & 3) + lane;
            const int a0 = kEpi * (warp >> 2);
            const int egr = eg_s[par][row];
            double out[2][kEpi];
#pragma unroll
            for (int part = 0; part < 2; ++part) {
                uint32_t v[kTcAccF64][kEpi];
#pragma unroll
                for (int d = 0; d < kTcAccF64; ++d) {
                    const uint32_t taddr = tmem + ((uint32_t)(32 * (warp & 3)) << 16) + (uint32_t)(d * kReals + kAmps * part + a0);
                    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                                 : "=r"(v[d][0]), "=r"(v[d][1]), "=r"(v[d][2]), "=r"(v[d][3]), "=r"(v[d][4]), "=r"(v[d][5]),
                                   "=r"(v[d][6]), "=r"(v[d][7])
                                 : "r"(taddr));
                }
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
                for (int c = 0; c < kEpi; ++c) {
                    long long acc = (long long)int_of_f32(__uint_as_float(v[5][c]));
#pragma unroll
                    for (int d = 0; d < 5; ++d) acc += (long long)int_of_f32(__uint_as_float(v[d][c])) << (40 - 8 * d);
                    double r = __ll2double_rn(acc);
                    const int et = egr + er_s[kAmps * part + a0 + c] - 1075;
                    const long long rb = __double_as_longlong(r);
                    const int ef = (int)((rb >> 52) & 0x7FF), ne = ef + et;
                    if (ef != 0 && ne >= 1 && ne <= 2046) r = __longlong_as_double(rb + ((long long)et << 52));
                    else if (r != 0.0) r = ldexp(r, et);
                    out[part][c] = r;
                }
            }
            if (!abort_s) {
                const uint64_t base = insert0_mask(tile * kTcGroups + (uint64_t)row, bd.tmask);
#pragma unroll
                for (int c = 0; c < kEpi; ++c) psi[base | toff[a0 + c]] = make_double2(out[0][c], out[1][c]);
            }
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (abort_s) {
        // report, then give products still in flight a second bounded wait before the columns are freed
        if (tid == 0) atomicExch(err_flag, 1);
        wait_mma(phase ^ 1);
    }
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(T::kTmemCols));
}

cudaError_t launch_tc_f64x5(void* psi, int n, const BlockDesc& bd, const void* d_weights, int* err_flag, cudaStream_t s) {
    using T = TcShapeF64x5;
    static const cudaError_t attr =
        cudaFuncSetAttribute(k_block_tc_f64x5, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)T::kSmem);
    if (attr != cudaSuccess) return attr;
    const uint64_t ntiles = (1ULL << (n - 5)) / kTcGroups;
    int sms = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const unsigned grid = (unsigned)(ntiles < (uint64_t)sms ? ntiles : (uint64_t)sms);
    const uint16_t* w = static_cast<const uint16_t*>(d_weights);
    const int32_t* ex = reinterpret_cast<const int32_t*>(static_cast<const unsigned char*>(d_weights) +
                                                          (size_t)kTcSlicesF64 * T::kWSliceBytes);
    k_block_tc_f64x5<<<grid, T::kThreads, T::kSmem, s>>>(static_cast<double2*>(psi), n, bd, w, ex, err_flag);
    return cudaGetLastError();
}

template <int KQ>
cudaError_t launch_tc_f64(void* psi, int n, const BlockDesc& bd, const void* d_weights, int* err_flag, cudaStream_t s) {
    using T = TcShapeF64<KQ>;
    static const cudaError_t attr =
        cudaFuncSetAttribute(k_block_tc_f64<KQ>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)T::kSmem);
    if (attr != cudaSuccess) return attr;
    const uint64_t ntiles = (1ULL << (n - KQ)) / kTcGroups;
    int sms = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const uint64_t cap = (uint64_t)sms * T::kCtas;
    const unsigned grid = (unsigned)(ntiles < cap ? ntiles : cap);
    const uint16_t* w = static_cast<const uint16_t*>(d_weights);
    const int32_t* ex = reinterpret_cast<const int32_t*>(static_cast<const unsigned char*>(d_weights) +
                                                          (size_t)kTcSlicesF64 * T::kWSliceBytes);
    k_block_tc_f64<KQ><<<grid, T::kThreads, T::kSmem, s>>>(static_cast<double2*>(psi), n, bd, w, ex, err_flag);
    return cudaGetLastError();
}

}  // namespace

// Host side: the gate's real form in slices (exact in double), in the kernel's layout:
// kTcSlices slices of 2A x 2A bf16, then 2A row exponents.
namespace {
// The gate's real form, row r split as W[r][c] = 2^(e_r - top) sum_j w_j[r][c] 2^(-8 j) into
// `slices` slices (|w_0| < 2^top; later slices are balanced remainders of magnitude <= 128, so
// eight slices hold a double exactly), in the kernel's core-matrix layout, then the 2A row
// exponents.
void prepare_slices(int k, const double* m, void* weights, int slices, int top) {
    const int amps = 1 << k, reals = 2 * amps;
    const size_t wslice = (size_t)reals * reals * 2;
    unsigned char* out = static_cast<unsigned char*>(weights);
    int32_t* wexp = reinterpret_cast<int32_t*>(out + slices * wslice);
    std::memset(out, 0, slices * wslice);
    std::vector<double> w(reals);
    for (int r = 0; r < reals; ++r) {
        const int orow = r & (amps - 1), oim = r >> k;
        for (int c = 0; c < reals; ++c) {
            const int col = c & (amps - 1), iim = c >> k;
            const double re = m[2 * (orow * amps + col)], im = m[2 * (orow * amps + col) + 1];
            // re out: Re M x_re - Im M x_im; im out: Im M x_re + Re M x_im
            w[c] = oim == 0 ? (iim == 0 ? re : -im) : (iim == 0 ? im : re);
        }
        int e = -1000;
        for (int c = 0; c < reals; ++c)
            if (w[c] != 0.0) {
                int ex;
                std::frexp(w[c], &ex);  // |w| < 2^ex
                e = std::max(e, ex);
            }
        if (e == -1000) e = 0;
        wexp[r] = e;
        for (int c = 0; c < reals; ++c) {
            double v = std::ldexp(w[c], top - e);
            for (int s = 0; s < slices; ++s) {
                const double q = std::nearbyint(v);
                v = (v - q) * 256.0;
                const float f = (float)q;  // an integer of magnitude <= 256: exact in bf16
                uint32_t bits;
                std::memcpy(&bits, &f, 4);
                std::memcpy(out + s * wslice + core_off(r, c, reals), reinterpret_cast<const unsigned char*>(&bits) + 2, 2);
            }
        }
    }
}
}  // namespace

void block_tc_prepare(int P, int k, const double* m, void* weights) {
    if (P == LLG_F64) prepare_slices(k, m, weights, kTcSlicesF64, 7);
    else prepare_slices(k, m, weights, kTcSlices, 8);
}

size_t block_tc_weight_bytes(int P, int k) {
    const size_t reals = (size_t)2 << k;
    return (P == LLG_F64 ? kTcSlicesF64 : kTcSlices) * reals * reals * 2 + reals * sizeof(int32_t);
}

bool block_tc_eligible(int P, int n, int k) {
    return (P == LLG_DF64 && (k == 4 || k == 5) && n >= k + 7) || (P == LLG_F64 && k >= 3 && k <= 5 && n >= k + 7);
}

cudaError_t launch_block_tc(int P, void* psi, int n, const BlockDesc& bd, const void* d_weights, int* err_flag,
                            cudaStream_t s) {
    if (P == LLG_F64) {
        if (bd.k == 5) return launch_tc_f64x5(psi, n, bd, d_weights, err_flag, s);
        return bd.k == 3 ? launch_tc_f64<3>(psi, n, bd, d_weights, err_flag, s) : launch_tc_f64<4>(psi, n, bd, d_weights, err_flag, s);
    }
    return bd.k == 5 ? launch_tc<5>(psi, n, bd, d_weights, err_flag, s) : launch_tc<4>(psi, n, bd, d_weights, err_flag, s);
}

}  // namespace llg
