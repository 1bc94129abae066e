// llg_adjoint.cu -- batched circuits with parameters: forward passes, adjoint-method gradients
// and the parameter-shift comparison (include/llgpu.h, "adjoint" section).
//
// The reference differentiates with the parameter-shift rule, 2 circuit evaluations per
// parameter (src/Algorithms.h:277-292).  Here one forward sweep and one reverse sweep give every
// gradient (adjoint method; Jones & Gacon, arXiv:2009.02823):
//   forward   psi = U_N .. U_1 |0>, then lambda = O psi and E = <psi|lambda> in one pass
//             (O = sum_k c_k Z_a Z_b is diagonal);
//   backward  for g = N .. 1: if U_g = exp(-i theta P / 2), dE/dtheta += Im <lambda|P|psi>;
//             then psi <- U_g^+ psi, lambda <- U_g^+ lambda.
// Both sweeps run as shared-memory tile passes (the forward plan's passes mirrored for the
// backward), over a batch of parameter sets laid out [batch][2^n]; a tile's batch index picks its
// row of the (cos, sin) coefficient table.  Inner products are reduced per tile into a partial
// array and summed in a fixed order, so gradients are deterministic.  Forward states can be
// checkpointed every C passes; the backward sweep then restarts psi from each checkpoint instead
// of relying on uncomputation alone (deep circuits).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/llgpu.h"
#include "llg_common.cuh"
#include "llg_internal.h"
#include "llg_diag_launch.h"
#include "llg_launch.h"
#include "llg_tile.cuh"

namespace llg {
int set_error(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);
}  // namespace llg

using namespace llg;

#define ADJ_CUDA(call, what)                               \
    do {                                                   \
        cudaError_t e_ = (call);                           \
        if (e_ != cudaSuccess) return cuda_fail(e_, what); \
    } while (0)

namespace {

constexpr int kAdjTile = 11;  // two 2^11 tiles (psi, lambda) per CTA in the backward pass
constexpr int kAdjOpChunk = 32;  // op records staged per shared-memory chunk

// Stages ops[first, first + cnt) into shared memory (ExecOp is a whole number of 16-byte words);
// the caller synchronises before and after.
__device__ __forceinline__ void stage_ops(ExecOp* sops, const ExecOp* __restrict__ ops, int first, int cnt) {
    constexpr int kWords = (int)(sizeof(ExecOp) / 16);
    const uint4* src = reinterpret_cast<const uint4*>(ops + first);
    for (int w = threadIdx.x; w < cnt * kWords; w += blockDim.x) reinterpret_cast<uint4*>(sops)[w] = src[w];
}
constexpr int kEBlocksPerState = 64;

// ------------------------------------------------------------------------------------------
// Parametrised RX / RY in scale-free form (IEEE complex128 and double-float).  The FP64 passes
// are bound by this GPU's FP64 pipe (2 multiply-adds per clock per SM), the double-float ones by
// instruction issue.  The table row of an RX / RY occurrence holds (v, f) and a form byte: form 0
// (|sin| <= |cos|) v = tan(theta/2), f = cos(theta/2), and the rotation is f [1, -v; v, 1] (RY)
// or f [1, -iv; -iv, 1] (RX); form 1 v = cot(theta/2), f = sin(theta/2), and it is
// f [v, -1; 1, v] or f [v, -i; -i, v].  v is packed in the state's format, f is an IEEE double.
// The tile applies the bracket, one multiply-add per real component instead of two, and the
// kernel multiplies f into the tile's running factor F (a double): the tile holds the amplitudes
// divided by F, and its store multiplies F back in, so states between passes (and checkpoints)
// are at their true scale.  The inverse negates v, and in form 1 f too
// (RY(-theta) = (-s) [-u, -1; 1, -u]).  An inner product of psi and lambda tiles, which share F,
// is F^2 times that of the stored values.  |f| >= 1/sqrt(2); when |F| falls below 2^kMinExp
// (2^-300 in FP64; 2^-40 in double-float, whose floats reach 2^-126) the tiles are rescaled in
// place.  complex64 keeps the full forms.
// ------------------------------------------------------------------------------------------
template <class P>
constexpr bool kScaleFree = P::kPrecision == LLG_F64 || P::kPrecision == LLG_DF64;

template <class P>
constexpr int kMinExp = P::kPrecision == LLG_F64 ? -300 : -40;

struct RotSF {
    uint64_t v;  // packed in the state's format
    double f;
    bool cform;
};

// (negations flip sign bits on the integer pipe)
template <class P>
__device__ __forceinline__ RotSF rot_sf(const ExecOp& o, const uint64_t* __restrict__ trow, const uint8_t* __restrict__ frow) {
    constexpr uint64_t kSign = 0x8000000000000000ULL;
    constexpr uint64_t kSignV = P::kPrecision == LLG_F64 ? kSign : 0x8000000080000000ULL;  // double-float: hi and lo
    RotSF r;
    r.cform = frow[o.q1] != 0;
    const bool inv = (o.flags & OPF_ADJOINT) != 0;
    r.v = trow[2 * o.q1] ^ (inv ? kSignV : 0);
    r.f = __longlong_as_double((long long)(trow[2 * o.q1 + 1] ^ (inv && r.cform ? kSign : 0)));
    return r;
}

// |F| < 2^kMinExp, from the exponent field (no FP64 instruction)
template <class P>
__device__ __forceinline__ bool below_min_scale(double F) {
    return ((__double_as_longlong(F) >> 52) & 0x7ff) < 1023 + kMinExp<P>;
}

// the bracket of a scale-free rotation on one tile
template <class P>
__device__ __forceinline__ void tile_rot_sf(typename P::S* tile, uint32_t tsize, const ExecOp& o, const RotSF& r) {
    ExecOp e = o;
    e.c[2] = r.v;
    if (o.kind == EX_RY_P) {
        if (r.cform) tile_pairs<P, EX_RC>(tile, tsize >> 1, o.q0, e);
        else tile_pairs<P, EX_RT>(tile, tsize >> 1, o.q0, e);
    } else {
        if (r.cform) tile_pairs<P, EX_RXC>(tile, tsize >> 1, o.q0, e);
        else tile_pairs<P, EX_RXT>(tile, tsize >> 1, o.q0, e);
    }
}

// F != 1 from its bits (no FP64 instruction)
__device__ __forceinline__ bool is_not_one(double F) { return __double_as_longlong(F) != 0x3FF0000000000000LL; }

template <class P>
__device__ __forceinline__ typename P::S scaled(typename P::S x, double F) {
    const typename P::K k = P::k_from_double(F);
    typename P::C a = P::load(x);
    a.re = P::mulk(k, a.re);
    a.im = P::mulk(k, a.im);
    return P::store(a);
}

template <class P>
__device__ __forceinline__ void tile_scale(typename P::S* tile, uint32_t tsize, double F) {
    for (uint32_t l = threadIdx.x; l < tsize; l += blockDim.x) tile[l] = scaled<P>(tile[l], F);
}

__device__ __forceinline__ bool is_rot_p(int kind) { return kind == EX_RX_P || kind == EX_RY_P; }

// RZ gradients from the q = 1 half alone (see tile_grad_apply) in the 16-byte formats; complex64
// keeps both halves, whose rounding would not cancel to its tolerance
template <class P>
constexpr bool kHalfRZ = P::kPrecision != LLG_F32;

// the weight of tile_grad_apply's sum: an RZ summed over the q = 1 half only counts -2 x
template <class P>
__device__ __forceinline__ double grad_weight(int kind) {
    return (kHalfRZ<P> && kind == EX_RZ_P) ? -2.0 : 1.0;
}

// ------------------------------------------------------------------------------------------
// coefficient table: table[row][j] = (cos(theta/2), sin(theta/2)) packed for the precision; for an
// RZ occurrence (cos theta, sin theta): RZ runs as diag(1, e^{i theta}) without its global phase
// e^{-i theta/2}.  psi and lambda pick up the same phases through both sweeps, so energies
// <psi|O|psi> and gradients Im <lambda|P|psi> are unchanged, and RZ costs one complex product on
// half of the amplitudes instead of one on every amplitude.  In IEEE complex128 and double-float
// an RX / RY entry holds the scale-free (v, f) instead, with its form byte in form[row][j].
// ------------------------------------------------------------------------------------------
template <class P>
__device__ uint64_t pack_dev(double x) {
    if (P::kPrecision == 0) return (uint64_t)__double_as_longlong(x);
    if (P::kPrecision == 2) return (uint64_t)__float_as_uint(__double2float_rn(x));
    const df d = double_to_df(x);
    return (uint64_t)__float_as_uint(d.hi) | ((uint64_t)__float_as_uint(d.lo) << 32);
}

template <class P>
__global__ void k_coef_table(const double* __restrict__ params, int nparams, const int* __restrict__ occ_param, int nocc,
                             int rows, const int* __restrict__ row_set, const int* __restrict__ shift_occ,
                             const double* __restrict__ shift_val, uint64_t* __restrict__ table,
                             uint8_t* __restrict__ form) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= rows * nocc) return;
    const int r = idx / nocc, j = idx % nocc;
    const int set = row_set ? row_set[r] : r;
    const int code = occ_param[j];  // 2 * parameter + (1 for an RZ occurrence)
    double theta = params[(size_t)set * nparams + (code >> 1)];
    if (shift_occ && shift_occ[r] == j) theta += shift_val[r];
    double s, c;
    sincos((code & 1) ? theta : 0.5 * theta, &s, &c);
    if (kScaleFree<P> && !(code & 1)) {  // RX / RY: the scale-free (v, f) and its form
        const bool cform = fabs(s) > fabs(c);
        table[2 * (size_t)idx] = pack_dev<P>(cform ? c / s : s / c);
        table[2 * (size_t)idx + 1] = (uint64_t)__double_as_longlong(cform ? s : c);  // f stays a double
        form[idx] = cform ? 1 : 0;
        return;
    }
    table[2 * (size_t)idx] = pack_dev<P>(c);
    table[2 * (size_t)idx + 1] = pack_dev<P>(s);
    if (form) form[idx] = 0;
}

// A rotation's part of the gradient and its inverse on both tiles: Y (YDOT) accumulates
// Re(conj(l1) p0) - Re(conj(l0) p1), X accumulates Im(conj(l0) p1) + Im(conj(l1) p0).  In IEEE
// complex128 the subtracted terms enter one accumulator through negated multiply-add operands
// (no separate FP64 subtraction).
template <class P, int KIND, bool YDOT>
__device__ __forceinline__ typename P::Acc grad_pairs(typename P::S* psi, typename P::S* lam, uint32_t tsize, uint32_t bit,
                                                      const PairMath<P, KIND>& m) {
    using C = typename P::C;
    constexpr bool kOne = P::kPrecision == LLG_F64;
    typename P::Acc pos = P::acc_zero(), neg = P::acc_zero();
    for (uint32_t pp = threadIdx.x; pp < (tsize >> 1); pp += blockDim.x) {
        const uint32_t j0 = ins0(pp, bit), j1 = j0 | bit;
        C p0 = P::load(psi[j0]), p1 = P::load(psi[j1]), q0 = P::load(lam[j0]), q1 = P::load(lam[j1]);
        if (YDOT) {
            pos = P::acc_dot_re(pos, q1, p0);
            if constexpr (kOne) pos = fma(-q0.re, p1.re, fma(-q0.im, p1.im, pos));
            else neg = P::acc_dot_re(neg, q0, p1);
        } else {
            pos = P::acc_dot_im(pos, q0, p1);
            pos = P::acc_dot_im(pos, q1, p0);
        }
        m.apply(p0, p1);
        m.apply(q0, q1);
        psi[j0] = P::store(p0);
        psi[j1] = P::store(p1);
        lam[j0] = P::store(q0);
        lam[j1] = P::store(q1);
    }
    if constexpr (kOne) return pos;
    else return YDOT ? acc_minus(pos, neg) : pos;
}

// One gradient op fused: this thread's part of Im <lambda | P | psi> from the amplitudes before the
// op, and the op's inverse applied to both tiles in the same loop (each pair or amplitude belongs
// to one thread, so it reads its values before it overwrites them).  The caller reduces the
// result and provides the barrier before the next op.
template <class P>
__device__ typename P::Acc tile_grad_apply(typename P::S* psi, typename P::S* lam, uint32_t tsize, uint64_t base,
                                           const ExecOp& o, const uint64_t* __restrict__ trow,
                                           const uint8_t* __restrict__ frow) {
    using K = typename P::K;
    using C = typename P::C;
    typename P::Acc pos = P::acc_zero(), neg = P::acc_zero();
    const K c0 = P::k_from_bits(trow[2 * o.q1]);
    K s0 = P::k_from_bits(trow[2 * o.q1 + 1]);
    if (o.flags & OPF_ADJOINT) s0 = P::kneg(s0);
    if (o.kind == EX_RZ_P) {  // generator Z; the op is diag(1, e^{i t}) (table row cos t, sin t)
        const K ms0 = P::kneg(s0);
        if (o.flags & OPF_NONLOCAL_Q0) {
            const bool one = (base >> o.q0) & 1;
            if constexpr (kHalfRZ<P>) {
                if (!one) return pos;  // the q = 0 half: no contribution, no change (see below)
            }
            for (uint32_t l = threadIdx.x; l < tsize; l += blockDim.x) {
                C p = P::load(psi[l]), q = P::load(lam[l]);
                pos = P::acc_dot_im(pos, q, p);
                if (one) {
                    cmul_const<P>(p, c0, s0, ms0);
                    cmul_const<P>(q, c0, s0, ms0);
                    psi[l] = P::store(p);
                    lam[l] = P::store(q);
                }
            }
            if constexpr (kHalfRZ<P>) return pos;  // weighted -2 by the caller
            else return one ? acc_minus(P::acc_zero(), pos) : pos;
        }
        const uint32_t bit = 1u << o.q0;
        if constexpr (kHalfRZ<P>) {
            // <lambda|psi> = <psi_N|O|psi_N> is real at every step of the reverse sweep (both
            // vectors go through the same unitaries, O is a real diagonal), so summed over all
            // tiles Im <lambda|Z|psi> = -2 sum_{q = 1} Im(conj(l) p): the q = 0 half is not read.
            // The sum is returned unweighted; the caller applies grad_weight's -2.
            for (uint32_t pp = threadIdx.x; pp < (tsize >> 1); pp += blockDim.x) {
                const uint32_t j1 = ins0(pp, bit) | bit;
                C p1 = P::load(psi[j1]), q1 = P::load(lam[j1]);
                pos = P::acc_dot_im(pos, q1, p1);
                cmul_const<P>(p1, c0, s0, ms0);
                cmul_const<P>(q1, c0, s0, ms0);
                psi[j1] = P::store(p1);
                lam[j1] = P::store(q1);
            }
            return pos;
        } else {
            for (uint32_t pp = threadIdx.x; pp < (tsize >> 1); pp += blockDim.x) {
                const uint32_t j0 = ins0(pp, bit), j1 = j0 | bit;
                const C p0 = P::load(psi[j0]), q0 = P::load(lam[j0]);
                C p1 = P::load(psi[j1]), q1 = P::load(lam[j1]);
                pos = P::acc_dot_im(pos, q0, p0);
                neg = P::acc_dot_im(neg, q1, p1);
                cmul_const<P>(p1, c0, s0, ms0);
                cmul_const<P>(q1, c0, s0, ms0);
                psi[j1] = P::store(p1);
                lam[j1] = P::store(q1);
            }
            return acc_minus(pos, neg);
        }
    }
    const uint32_t bit = 1u << o.q0;
    if constexpr (kScaleFree<P>) {  // the scale-free brackets (the caller carries f)
        const RotSF rs = rot_sf<P>(o, trow, frow);
        ExecOp e = o;
        e.c[2] = rs.v;
        if (o.kind == EX_RY_P)
            return rs.cform ? grad_pairs<P, EX_RC, true>(psi, lam, tsize, bit, PairMath<P, EX_RC>(e))
                            : grad_pairs<P, EX_RT, true>(psi, lam, tsize, bit, PairMath<P, EX_RT>(e));
        return rs.cform ? grad_pairs<P, EX_RXC, false>(psi, lam, tsize, bit, PairMath<P, EX_RXC>(e))
                        : grad_pairs<P, EX_RXT, false>(psi, lam, tsize, bit, PairMath<P, EX_RXT>(e));
    } else {
        ExecOp r = o;  // RX / RY with the (possibly negated) sine of the table row
        r.c[0] = trow[2 * o.q1];
        if (o.kind == EX_RY_P) {
            PairMath<P, EX_RY> m(r);
            m.k[1] = s0;
            return grad_pairs<P, EX_RY, true>(psi, lam, tsize, bit, m);
        }
        PairMath<P, EX_RX> m(r);
        m.k[1] = s0;
        return grad_pairs<P, EX_RX, false>(psi, lam, tsize, bit, m);
    }
}

// ------------------------------------------------------------------------------------------
// batched forward tile pass: grid (tiles per state, batch)
// ------------------------------------------------------------------------------------------
template <class P>
__global__ void __launch_bounds__(512) k_tile_fwd(typename P::S* __restrict__ psi_all, int n, PassDesc pd,
                                                  const ExecOp* __restrict__ ops, const uint64_t* __restrict__ table,
                                                  const uint8_t* __restrict__ form, int nocc) {
    using S = typename P::S;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int t = pd.t, low = pd.low;
    const uint32_t tsize = 1u << t, nhi = 1u << (t - low);
    S* tile = reinterpret_cast<S*>(smem_raw);
    uint64_t* hi_off = reinterpret_cast<uint64_t*>(smem_raw + (size_t)tsize * sizeof(S));
    const uint64_t b = blockIdx.y;
    S* psi = psi_all + (b << n);
    const uint64_t* trow = table + b * (uint64_t)nocc * 2;
    const uint8_t* frow = form + b * (uint64_t)nocc;
    const uint64_t base = insert0_mask((uint64_t)blockIdx.x, pd.local_mask);
    for (uint32_t h = threadIdx.x; h < nhi; h += blockDim.x) {
        uint64_t off = 0;
        for (int j = 0; j < t - low; ++j)
            if ((h >> j) & 1) off |= 1ULL << pd.hi_pos[j];
        hi_off[h] = off;
    }
    __syncthreads();
    const uint32_t lowmask = (1u << low) - 1;
    for (uint32_t l = threadIdx.x; l < tsize; l += blockDim.x) tile[l] = psi[base | hi_off[l >> low] | (l & lowmask)];
    __syncthreads();
    __shared__ __align__(16) ExecOp sops[kAdjOpChunk];
    double F = 1.0;  // scale-free formats: the tile holds the amplitudes divided by F
    for (int k = 0; k < pd.nops; ++k) {
        if (k % kAdjOpChunk == 0) {
            stage_ops(sops, ops, pd.op_begin + k, min(kAdjOpChunk, pd.nops - k));
            __syncthreads();
        }
        const ExecOp& o = sops[k % kAdjOpChunk];
        if constexpr (kScaleFree<P>) {
            if (is_rot_p(o.kind)) {
                const RotSF rs = rot_sf<P>(o, trow, frow);
                tile_rot_sf<P>(tile, tsize, o, rs);
                F *= rs.f;
                __syncthreads();
                if (below_min_scale<P>(F)) {
                    tile_scale<P>(tile, tsize, F);
                    F = 1.0;
                    __syncthreads();
                }
                continue;
            }
        }
        tile_apply<P>(tile, tsize, base, o, trow);
        __syncthreads();
    }
    const bool rescale = kScaleFree<P> && is_not_one(F);  // uniform across the CTA
    for (uint32_t l = threadIdx.x; l < tsize; l += blockDim.x) {
        S a = tile[l];
        if (rescale) a = scaled<P>(a, F);
        psi[base | hi_off[l >> low] | (l & lowmask)] = a;
    }
}

// batched backward tile pass over psi and lambda; gpart[b][occ][tile]
template <class P>
__global__ void __maxnreg__(80) k_tile_bwd(typename P::S* __restrict__ psi_all, typename P::S* __restrict__ lam_all,
                                                  int n, PassDesc pd, const ExecOp* __restrict__ ops,
                                                  const uint64_t* __restrict__ table, const uint8_t* __restrict__ form,
                                                  int nocc, double* __restrict__ gpart, int tiles) {
    using S = typename P::S;
    using A = typename P::Acc;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    // Gradient sums: each warp reduces its part of a parametrised op's inner product with
    // shuffles and parks it here, so the op ends in one CTA barrier; the sums across warps are
    // finished for up to kGradBuf ops at once, one thread per op (at most 512 threads, 16 warps).
    constexpr int kGradBuf = 32;
    __shared__ double gred[kGradBuf][16];  // per-warp parts, converted to IEEE double
    __shared__ double gscale[kGradBuf];    // each buffered sum's weight (F^2 and grad_weight)
    __shared__ int gslot[kGradBuf];
    const int t = pd.t, low = pd.low;
    const uint32_t tsize = 1u << t, nhi = 1u << (t - low);
    S* tp = reinterpret_cast<S*>(smem_raw);
    S* tl = tp + tsize;
    uint64_t* hi_off = reinterpret_cast<uint64_t*>(smem_raw + 2 * (size_t)tsize * sizeof(S));
    const uint64_t b = blockIdx.y;
    S* psi = psi_all + (b << n);
    S* lam = lam_all + (b << n);
    const uint64_t* trow = table + b * (uint64_t)nocc * 2;
    const uint8_t* frow = form + b * (uint64_t)nocc;
    const uint64_t base = insert0_mask((uint64_t)blockIdx.x, pd.local_mask);
    for (uint32_t h = threadIdx.x; h < nhi; h += blockDim.x) {
        uint64_t off = 0;
        for (int j = 0; j < t - low; ++j)
            if ((h >> j) & 1) off |= 1ULL << pd.hi_pos[j];
        hi_off[h] = off;
    }
    __syncthreads();
    const uint32_t lowmask = (1u << low) - 1;
    for (uint32_t l = threadIdx.x; l < tsize; l += blockDim.x) {
        const uint64_t g = base | hi_off[l >> low] | (l & lowmask);
        tp[l] = psi[g];
        tl[l] = lam[g];
    }
    __syncthreads();
    int ng = 0;  // buffered gradients (the same count in every thread)
    auto flush = [&]() {  // after a barrier: the warps' partials of each buffered op, in warp order
        if ((int)threadIdx.x < ng) {
            double sum = gred[threadIdx.x][0];
            for (int w = 1; w < (int)(blockDim.x >> 5); ++w) sum += gred[threadIdx.x][w];
            gpart[((size_t)b * nocc + gslot[threadIdx.x]) * tiles + blockIdx.x] = sum * gscale[threadIdx.x];
        }
    };
    __shared__ __align__(16) ExecOp sops[kAdjOpChunk];
    double F = 1.0;  // scale-free formats: both tiles hold their amplitudes divided by F
    for (int k = 0; k < pd.nops; ++k) {
        if (k % kAdjOpChunk == 0) {
            stage_ops(sops, ops, pd.op_begin + k, min(kAdjOpChunk, pd.nops - k));
            __syncthreads();
        }
        const ExecOp& o = sops[k % kAdjOpChunk];
        if (o.flags & OPF_GRAD) {
            // inner product and un-application in one loop.  The slot is read before the barrier:
            // once it is passed, the next chunk may be staged over this op's record.
            // the warp's sum in the accumulator's format, then IEEE double across warps and tiles
            const double v = acc_value(warp_sum_acc(tile_grad_apply<P>(tp, tl, tsize, base, o, trow, frow)));
            if ((threadIdx.x & 31) == 0) gred[ng][threadIdx.x >> 5] = v;
            if (threadIdx.x == 0) {
                gslot[ng] = o.q1;
                gscale[ng] = kScaleFree<P> ? grad_weight<P>(o.kind) * (F * F) : 1.0;  // F before the op
            }
            if constexpr (kScaleFree<P>) {
                if (is_rot_p(o.kind)) F *= rot_sf<P>(o, trow, frow).f;
            }
            ++ng;
            __syncthreads();  // the tile writes before the next op, the partials before a flush
            if (ng == kGradBuf) {
                flush();
                __syncthreads();  // the buffer is read before it is refilled
                ng = 0;
            }
        } else {
            tile_apply<P>(tp, tsize, base, o, trow);
            tile_apply<P>(tl, tsize, base, o, trow);
            __syncthreads();
        }
        if constexpr (kScaleFree<P>) {
            if (below_min_scale<P>(F)) {  // uniform across the CTA; the last op ended in a barrier
                tile_scale<P>(tp, tsize, F);
                tile_scale<P>(tl, tsize, F);
                F = 1.0;
                __syncthreads();
            }
        }
    }
    flush();  // every op ended in a barrier, so the last partials are visible
    const bool rescale = kScaleFree<P> && is_not_one(F);  // uniform across the CTA
    for (uint32_t l = threadIdx.x; l < tsize; l += blockDim.x) {
        const uint64_t g = base | hi_off[l >> low] | (l & lowmask);
        S a = tp[l], c = tl[l];
        if (rescale) {
            a = scaled<P>(a, F);
            c = scaled<P>(c, F);
        }
        psi[g] = a;
        lam[g] = c;
    }
}

// grads[b][k] = sum over the occurrences of parameter k (CSR list) and tiles, fixed order
__global__ void k_grad_finish(const double* __restrict__ gpart, int batch, int nocc, int tiles, int nparams,
                              const int* __restrict__ csr_ptr, const int* __restrict__ csr_occ, double* __restrict__ grads) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= batch * nparams) return;
    const int b = idx / nparams, k = idx % nparams;
    double g = 0.0;
    for (int e = csr_ptr[k]; e < csr_ptr[k + 1]; ++e) {
        const double* row = gpart + ((size_t)b * nocc + csr_occ[e]) * tiles;
        for (int t = 0; t < tiles; ++t) g += row[t];
    }
    grads[idx] = g;
}

template <class P>
size_t fwd_smem(int t, int low) {
    return ((size_t)1 << t) * sizeof(typename P::S) + ((size_t)1 << (t - low)) * sizeof(uint64_t);
}
template <class P>
size_t bwd_smem(int t, int low) {
    return 2 * ((size_t)1 << t) * sizeof(typename P::S) + ((size_t)1 << (t - low)) * sizeof(uint64_t);
}

template <class P>
cudaError_t set_smem_attrs() {
    // once per precision (thread-safe static initialisation)
    static const cudaError_t e = [] {
        cudaError_t r = cudaFuncSetAttribute(k_tile_fwd<P>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)fwd_smem<P>(kAdjTile, 4));
        if (r == cudaSuccess)
            r = cudaFuncSetAttribute(k_tile_bwd<P>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bwd_smem<P>(kAdjTile, 4));
        return r;
    }();
    return e;
}

// |0..0> in every batch element: element 0 of each row is 1 (the rows were zeroed)
template <class P>
__global__ void k_set_rows(typename P::S* psi, int n, int batch) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= batch) return;
    typename P::C one;
    one.re = P::r_from_float(1.0f);
    one.im = P::zero();
    psi[(uint64_t)b << n] = P::store(one);
}

int threads_for(int t, int fixed) {
    if (fixed > 0) return fixed;
    // 128 threads for 8+-qubit tiles.  The passes are bound by the FP64 pipe (complex128) or the
    // FP32 pipe (double-float), which a few warps per scheduler keep busy; fewer threads per tile
    // mean fewer warps per gradient reduction and per barrier (measured on the 20-qubit,
    // 400-parameter ansatz, batch 64: 65.3k against 63.3k gradients/s at 256 threads in complex128,
    // 155k against 151k in double-float; 512 threads were slower still)
    return t >= 8 ? 128 : (t >= 6 ? (1 << (t - 1)) : 32);
}

}  // namespace

// ------------------------------------------------------------------------------------------
// host object
// ------------------------------------------------------------------------------------------
struct llg_adjoint {
    int n = 0, P = LLG_DF64, nparams = 0, max_batch = 0, nocc = 0, tiles = 1;
    int threads = 0;  // CTA threads of the tile passes (0: 256 for tiles of 10+ qubits)
    DiagObsHost obs;   // the observable: any number of Z / ZZ terms with any coefficients
    void* d_obs = nullptr;
    Plan fwd;
    std::vector<PassDesc> bwd_passes;
    std::vector<ExecOp> bwd_ops;
    std::vector<int> occ_param;
    cudaStream_t stream = nullptr;
    void* d_psi = nullptr;
    void* d_lam = nullptr;
    ExecOp* d_fwd_ops = nullptr;
    ExecOp* d_bwd_ops = nullptr;
    uint64_t* d_table = nullptr;
    uint8_t* d_form = nullptr;  // the scale-free form of each RX / RY table entry (16-byte formats)
    int* d_occ_param = nullptr;
    int* d_csr_ptr = nullptr;
    int* d_csr_occ = nullptr;
    double* d_params = nullptr;
    double* d_gpart = nullptr;
    double* d_epart = nullptr;
    double* d_energy = nullptr;
    double* d_grad = nullptr;
    int* d_row_set = nullptr;
    int* d_shift_occ = nullptr;
    double* d_shift_val = nullptr;
    std::vector<void*> ckpt;
    size_t state_bytes = 0;  // one batch element
};

namespace {

template <class T>
int dmalloc(T** p, size_t count, const char* what) {
    cudaError_t e = cudaMalloc((void**)p, std::max<size_t>(count, 1) * sizeof(T));
    if (e != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        return set_error(LLG_ENOMEM, std::string("adjoint: cannot allocate ") + what + ": " + cudaGetErrorString(e));
    }
    return LLG_OK;
}

bool is_device_ptr(const void* p) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

// conjugate-transpose an executor op in place (packed coefficients: negation flips sign bits)
uint64_t neg_packed(int P, uint64_t v) {
    if (P == LLG_F64) return v ^ 0x8000000000000000ULL;
    if (P == LLG_F32) return v ^ 0x80000000ULL;
    return v ^ 0x8000000080000000ULL;
}

ExecOp adjoint_of(int P, const ExecOp& e) {
    ExecOp a = e;
    switch (e.kind) {
        case EX_U2:  // (g^+)_{rc} = conj(g_{cr})
            a.c[0] = e.c[0];
            a.c[1] = neg_packed(P, e.c[1]);
            a.c[2] = e.c[4];
            a.c[3] = neg_packed(P, e.c[5]);
            a.c[4] = e.c[2];
            a.c[5] = neg_packed(P, e.c[3]);
            a.c[6] = e.c[6];
            a.c[7] = neg_packed(P, e.c[7]);
            break;
        case EX_RX:
        case EX_RY: a.c[1] = neg_packed(P, e.c[1]); break;
        case EX_DIAG:
            a.c[1] = neg_packed(P, e.c[1]);
            a.c[3] = neg_packed(P, e.c[3]);
            break;
        case EX_RX_P:
        case EX_RY_P:
        case EX_RZ_P: a.flags |= OPF_ADJOINT | OPF_GRAD; break;
        default: break;  // H, X, CNOT, MCZ are their own inverses
    }
    return a;
}

template <class P>
int run_forward(llg_adjoint* h, int batch, bool make_lambda, const int* ckpt_every) {
    const uint64_t size = 1ULL << h->n;
    cudaStream_t s = h->stream;
    ADJ_CUDA(cudaMemsetAsync(h->d_psi, 0, (size_t)batch * h->state_bytes, s), "memset psi");
    k_set_rows<P><<<(batch + 255) / 256, 256, 0, s>>>(static_cast<typename P::S*>(h->d_psi), h->n, batch);
    ADJ_CUDA(cudaGetLastError(), "init rows");
    ADJ_CUDA(set_smem_attrs<P>(), "smem attribute");
    const int C = ckpt_every ? *ckpt_every : 0;
    for (size_t j = 0; j < h->fwd.passes.size(); ++j) {
        const PassDesc& pd = h->fwd.passes[j];
        const dim3 grid((unsigned)(1ULL << (h->n - pd.t)), (unsigned)batch);
        k_tile_fwd<P><<<grid, threads_for(pd.t, h->threads), fwd_smem<P>(pd.t, pd.low), s>>>(
            static_cast<typename P::S*>(h->d_psi), h->n, pd, h->d_fwd_ops, h->d_table, h->d_form, h->nocc);
        ADJ_CUDA(cudaGetLastError(), "forward tile pass");
        if (C > 0 && (j + 1) % C == 0 && j + 1 < h->fwd.passes.size()) {
            const size_t m = (j + 1) / C - 1;
            ADJ_CUDA(cudaMemcpyAsync(h->ckpt[m], h->d_psi, (size_t)batch * h->state_bytes, cudaMemcpyDeviceToDevice, s),
                     "checkpoint");
        }
    }
    // lambda = O psi and the energies: the observable's chunked kernel, one chunk of up to 2^12
    // amplitudes per block at a time
    const uint64_t chunks = size >> h->obs.L;
    const int eblocks = (int)std::min<uint64_t>(kEBlocksPerState, chunks);
    ADJ_CUDA(launch_lambda_diag(h->P, h->d_psi, make_lambda ? h->d_lam : nullptr, diag_obs_view(h->obs, h->d_obs), batch,
                                eblocks, h->d_epart, h->d_energy, s),
             "energy");
    return LLG_OK;
}

template <class P>
int run_backward(llg_adjoint* h, int batch, int C) {
    cudaStream_t s = h->stream;
    const int np = (int)h->bwd_passes.size();
    for (int j = 0; j < np; ++j) {
        const PassDesc& pd = h->bwd_passes[j];
        const dim3 grid((unsigned)(1ULL << (h->n - pd.t)), (unsigned)batch);
        k_tile_bwd<P><<<grid, threads_for(pd.t, h->threads), bwd_smem<P>(pd.t, pd.low), s>>>(
            static_cast<typename P::S*>(h->d_psi), static_cast<typename P::S*>(h->d_lam), h->n, pd, h->d_bwd_ops,
            h->d_table, h->d_form, h->nocc, h->d_gpart, h->tiles);
        ADJ_CUDA(cudaGetLastError(), "backward tile pass");
        // backward pass j undoes forward pass fj = np - 1 - j; psi is now the state after fj forward
        // passes; restart it from the checkpoint taken there, if any
        const int fj = np - 1 - j;
        if (C > 0 && fj > 0 && fj % C == 0) {
            const size_t m = fj / C - 1;
            ADJ_CUDA(cudaMemcpyAsync(h->d_psi, h->ckpt[m], (size_t)batch * h->state_bytes, cudaMemcpyDeviceToDevice, s),
                     "restore checkpoint");
        }
    }
    const int total = batch * h->nparams;
    k_grad_finish<<<(total + 255) / 256, 256, 0, s>>>(h->d_gpart, batch, h->nocc, h->tiles, h->nparams, h->d_csr_ptr,
                                                      h->d_csr_occ, h->d_grad);
    ADJ_CUDA(cudaGetLastError(), "gradient finish");
    return LLG_OK;
}

int build_table(llg_adjoint* h, int rows, bool shifted) {
    const int total = rows * h->nocc;
    if (total == 0) return LLG_OK;
    const int blocks = (total + 255) / 256;
    switch (h->P) {
        case LLG_F64:
            k_coef_table<PolF64><<<blocks, 256, 0, h->stream>>>(h->d_params, h->nparams, h->d_occ_param, h->nocc, rows,
                                                                shifted ? h->d_row_set : nullptr,
                                                                shifted ? h->d_shift_occ : nullptr, h->d_shift_val, h->d_table,
                                                                h->d_form);
            break;
        case LLG_F32:
            k_coef_table<PolF32><<<blocks, 256, 0, h->stream>>>(h->d_params, h->nparams, h->d_occ_param, h->nocc, rows,
                                                                shifted ? h->d_row_set : nullptr,
                                                                shifted ? h->d_shift_occ : nullptr, h->d_shift_val, h->d_table,
                                                                h->d_form);
            break;
        default:
            k_coef_table<PolDF64><<<blocks, 256, 0, h->stream>>>(h->d_params, h->nparams, h->d_occ_param, h->nocc, rows,
                                                                 shifted ? h->d_row_set : nullptr,
                                                                 shifted ? h->d_shift_occ : nullptr, h->d_shift_val, h->d_table,
                                                                 h->d_form);
    }
    ADJ_CUDA(cudaGetLastError(), "coefficient table");
    return LLG_OK;
}

int forward_dispatch(llg_adjoint* h, int batch, bool lam, const int* C) {
    switch (h->P) {
        case LLG_F64: return run_forward<PolF64>(h, batch, lam, C);
        case LLG_F32: return run_forward<PolF32>(h, batch, lam, C);
        default: return run_forward<PolDF64>(h, batch, lam, C);
    }
}

int backward_dispatch(llg_adjoint* h, int batch, int C) {
    switch (h->P) {
        case LLG_F64: return run_backward<PolF64>(h, batch, C);
        case LLG_F32: return run_backward<PolF32>(h, batch, C);
        default: return run_backward<PolDF64>(h, batch, C);
    }
}

int load_params(llg_adjoint* h, const double* params, int sets) {
    const size_t bytes = (size_t)sets * h->nparams * sizeof(double);
    if (bytes == 0) return LLG_OK;
    ADJ_CUDA(cudaMemcpyAsync(h->d_params, params, bytes, is_device_ptr(params) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                             h->stream),
             "params upload");
    return LLG_OK;
}

int store_out(llg_adjoint* h, double* dst, const double* src, size_t count) {
    if (!dst || count == 0) return LLG_OK;
    ADJ_CUDA(cudaMemcpyAsync(dst, src, count * sizeof(double), is_device_ptr(dst) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                             h->stream),
             "result copy");
    return LLG_OK;
}

int ensure_checkpoints(llg_adjoint* h, int C) {
    if (C <= 0) return LLG_OK;
    const size_t need = h->fwd.passes.size() > 1 ? (h->fwd.passes.size() - 1) / C : 0;
    while (h->ckpt.size() < need) {
        void* p = nullptr;
        cudaError_t e = cudaMalloc(&p, (size_t)h->max_batch * h->state_bytes);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return set_error(LLG_ENOMEM, "adjoint: cannot allocate checkpoint states");
        }
        h->ckpt.push_back(p);
    }
    return LLG_OK;
}

}  // namespace

extern "C" {

int llg_adjoint_create(int n, const llg_op* ops, int nops, int nparams, int max_batch, int precision, int nterms,
                       const int* za, const int* zb, const double* zcoeff, llg_adjoint** out) {
    if (!out) return set_error(LLG_EINVAL, "adjoint_create: out is NULL");
    *out = nullptr;
    if (n < 1 || n > 30) return set_error(LLG_EINVAL, "adjoint_create: n must be in [1, 30]");
    if (nops < 0 || (nops > 0 && !ops) || nparams < 0 || max_batch < 1 || max_batch > 65535)
        return set_error(LLG_EINVAL, "adjoint_create: bad sizes");
    if (precision != LLG_F64 && precision != LLG_DF64 && precision != LLG_F32)
        return set_error(LLG_EINVAL, "adjoint_create: unknown precision");
    if (nterms < 1 || !za || !zb || !zcoeff) return set_error(LLG_EINVAL, "adjoint_create: observable needs 1 or more terms");
    llg_adjoint* h = new llg_adjoint();
    h->n = n;
    h->P = precision;
    h->nparams = nparams;
    h->max_batch = max_batch;
    // observable
    {
        std::string oerr;
        if (!build_diag_obs(n, nterms, za, zb, zcoeff, h->obs, oerr)) {
            delete h;
            return set_error(LLG_EINVAL, "adjoint_create: " + oerr);
        }
    }
    // validate ops (bad qubits, angles; parameter indices)
    for (int i = 0; i < nops; ++i) {
        const llg_op& o = ops[i];
        const bool rot = o.kind == LLG_OP_RX || o.kind == LLG_OP_RY || o.kind == LLG_OP_RZ;
        bool ok = o.q0 >= 0 && o.q0 < n;
        if (o.kind == LLG_OP_CNOT || o.kind == LLG_OP_CZ) ok = ok && o.q1 >= 0 && o.q1 < n && o.q1 != o.q0;
        if (o.kind == LLG_OP_MCZ) ok = o.mask != 0 && (n >= 64 || (o.mask >> n) == 0);
        if (o.kind < 0 || o.kind > LLG_OP_U2) ok = false;
        if (rot && o.param < 0 && !std::isfinite(o.theta)) ok = false;
        if (o.param >= nparams || (o.param >= 0 && !rot)) ok = false;
        if (!ok) {
            delete h;
            return set_error(LLG_EINVAL, "adjoint_create: invalid op " + std::to_string(i));
        }
        if (o.param >= 0) h->occ_param.push_back(o.param);
    }
    h->nocc = (int)h->occ_param.size();
    std::vector<int> occ_code;  // the device copy: 2 * parameter + (1 for RZ, whose table entry is the full angle)
    for (int i = 0; i < nops; ++i)
        if (ops[i].param >= 0) occ_code.push_back(2 * ops[i].param + (ops[i].kind == LLG_OP_RZ ? 1 : 0));
    std::string err;
    const int t = std::min(n, kAdjTile);
    if (!plan_tiles(n, ops, nops, t, precision, h->fwd, err, true)) {
        delete h;
        return set_error(LLG_EINVAL, "adjoint_create: " + err);
    }
    h->tiles = 1 << (n - t);
    // backward plan: passes reversed, ops reversed and inverted, parametrised ops flagged
    for (int j = (int)h->fwd.passes.size() - 1; j >= 0; --j) {
        PassDesc pd = h->fwd.passes[j];
        const int begin = (int)h->bwd_ops.size();
        for (int k = pd.op_begin + pd.nops - 1; k >= pd.op_begin; --k) h->bwd_ops.push_back(adjoint_of(precision, h->fwd.ops[k]));
        pd.op_begin = begin;
        h->bwd_passes.push_back(pd);
    }
    h->state_bytes = ((size_t)1 << n) * elem_bytes(precision);
    // CSR: parameter -> occurrences
    std::vector<int> ptr(nparams + 1, 0), occ(h->nocc);
    for (int j = 0; j < h->nocc; ++j) ptr[h->occ_param[j] + 1]++;
    for (int k = 0; k < nparams; ++k) ptr[k + 1] += ptr[k];
    {
        std::vector<int> fill(ptr.begin(), ptr.end() - 1);
        for (int j = 0; j < h->nocc; ++j) occ[fill[h->occ_param[j]]++] = j;
    }
    int rc = LLG_OK;
    cudaError_t e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) rc = cuda_fail(e, "cudaStreamCreate");
    if (!rc) rc = dmalloc((char**)&h->d_psi, (size_t)max_batch * h->state_bytes, "psi");
    if (!rc) rc = dmalloc((char**)&h->d_lam, (size_t)max_batch * h->state_bytes, "lambda");
    if (!rc) rc = dmalloc(&h->d_fwd_ops, h->fwd.ops.size(), "ops");
    if (!rc) rc = dmalloc(&h->d_bwd_ops, h->bwd_ops.size(), "ops");
    if (!rc) rc = dmalloc(&h->d_table, (size_t)max_batch * h->nocc * 2, "coefficient table");
    if (!rc) rc = dmalloc(&h->d_form, (size_t)max_batch * h->nocc, "coefficient table");
    if (!rc) rc = dmalloc(&h->d_occ_param, h->nocc, "occurrence map");
    if (!rc) rc = dmalloc(&h->d_csr_ptr, nparams + 1, "csr");
    if (!rc) rc = dmalloc(&h->d_csr_occ, h->nocc, "csr");
    if (!rc) rc = dmalloc(&h->d_params, (size_t)max_batch * std::max(nparams, 1), "params");
    if (!rc) rc = dmalloc(&h->d_gpart, (size_t)max_batch * h->nocc * h->tiles, "gradient partials");
    if (!rc) rc = dmalloc(&h->d_epart, (size_t)max_batch * kEBlocksPerState, "energy partials");
    if (!rc) rc = dmalloc((char**)&h->d_obs, h->obs.bytes.size(), "observable");
    if (!rc)
        rc = cudaMemcpy(h->d_obs, h->obs.bytes.data(), h->obs.bytes.size(), cudaMemcpyHostToDevice)
                 ? set_error(LLG_ECUDA, "adjoint_create: observable upload") : LLG_OK;
    if (!rc) rc = dmalloc(&h->d_energy, max_batch, "energies");
    if (!rc) rc = dmalloc(&h->d_grad, (size_t)max_batch * std::max(nparams, 1), "gradients");
    if (!rc) rc = dmalloc(&h->d_row_set, max_batch, "rows");
    if (!rc) rc = dmalloc(&h->d_shift_occ, max_batch, "rows");
    if (!rc) rc = dmalloc(&h->d_shift_val, max_batch, "rows");
    if (!rc && !h->fwd.ops.empty())
        rc = cudaMemcpy(h->d_fwd_ops, h->fwd.ops.data(), h->fwd.ops.size() * sizeof(ExecOp), cudaMemcpyHostToDevice)
                 ? set_error(LLG_ECUDA, "adjoint_create: op upload") : LLG_OK;
    if (!rc && !h->bwd_ops.empty())
        rc = cudaMemcpy(h->d_bwd_ops, h->bwd_ops.data(), h->bwd_ops.size() * sizeof(ExecOp), cudaMemcpyHostToDevice)
                 ? set_error(LLG_ECUDA, "adjoint_create: op upload") : LLG_OK;
    if (!rc && h->nocc)
        rc = cudaMemcpy(h->d_occ_param, occ_code.data(), h->nocc * sizeof(int), cudaMemcpyHostToDevice) ||
                     cudaMemcpy(h->d_csr_occ, occ.data(), h->nocc * sizeof(int), cudaMemcpyHostToDevice)
                 ? set_error(LLG_ECUDA, "adjoint_create: map upload") : LLG_OK;
    if (!rc)
        rc = cudaMemcpy(h->d_csr_ptr, ptr.data(), (nparams + 1) * sizeof(int), cudaMemcpyHostToDevice)
                 ? set_error(LLG_ECUDA, "adjoint_create: map upload") : LLG_OK;
    if (rc) {
        llg_adjoint_destroy(h);
        return rc;
    }
    *out = h;
    return LLG_OK;
}

int llg_adjoint_destroy(llg_adjoint* h) {
    if (!h) return LLG_OK;
    if (h->stream) cudaStreamSynchronize(h->stream);
    void* ptrs[] = {h->d_psi, h->d_lam, h->d_fwd_ops, h->d_bwd_ops, h->d_table, h->d_form, h->d_occ_param, h->d_csr_ptr,
                    h->d_csr_occ, h->d_params, h->d_gpart, h->d_epart, h->d_energy, h->d_grad, h->d_row_set,
                    h->d_shift_occ, h->d_shift_val, h->d_obs};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    for (void* p : h->ckpt) cudaFree(p);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return LLG_OK;
}

int llg_adjoint_set_threads(llg_adjoint* h, int threads) {
    if (!h) return set_error(LLG_EINVAL, "adjoint_set_threads: NULL handle");
    if (threads != 0 && (threads < 32 || threads > 512 || (threads & 31)))
        return set_error(LLG_EINVAL, "adjoint_set_threads: threads must be 0 or a multiple of 32 in [32, 512]");
    h->threads = threads;
    return LLG_OK;
}

int llg_adjoint_info(const llg_adjoint* h, int* fwd_passes, int* bwd_passes, int* n_param_ops) {
    if (!h) return set_error(LLG_EINVAL, "adjoint_info: NULL handle");
    if (fwd_passes) *fwd_passes = (int)h->fwd.passes.size();
    if (bwd_passes) *bwd_passes = (int)h->bwd_passes.size();
    if (n_param_ops) *n_param_ops = h->nocc;
    return LLG_OK;
}

int llg_adjoint_run(llg_adjoint* h, const double* params, int batch, double* energies, double* grads, int checkpoint_every) {
    if (!h || (!params && h->nparams > 0)) return set_error(LLG_EINVAL, "adjoint_run: NULL argument");
    if (batch < 1 || batch > h->max_batch)
        return set_error(LLG_EINVAL, "adjoint_run: batch must be in [1, " + std::to_string(h->max_batch) + "]");
    if (checkpoint_every < 0) return set_error(LLG_EINVAL, "adjoint_run: checkpoint_every must be >= 0");
    int rc = load_params(h, params, batch);
    if (!rc) rc = build_table(h, batch, false);
    if (!rc && grads) rc = ensure_checkpoints(h, checkpoint_every);
    if (!rc) rc = forward_dispatch(h, batch, grads != nullptr, grads ? &checkpoint_every : nullptr);
    if (!rc && grads) rc = backward_dispatch(h, batch, checkpoint_every);
    if (!rc) rc = store_out(h, energies, h->d_energy, batch);
    if (!rc && grads) rc = store_out(h, grads, h->d_grad, (size_t)batch * h->nparams);
    if (!rc) ADJ_CUDA(cudaStreamSynchronize(h->stream), "cudaStreamSynchronize");
    return rc;
}

int llg_param_shift_run(llg_adjoint* h, const double* params, int sets, double* energies, double* grads) {
    if (!h || (!params && h->nparams > 0) || !grads) return set_error(LLG_EINVAL, "param_shift_run: NULL argument");
    if (sets < 1 || sets > h->max_batch)
        return set_error(LLG_EINVAL, "param_shift_run: sets must be in [1, " + std::to_string(h->max_batch) + "]");
    int rc = load_params(h, params, sets);
    if (rc) return rc;
    const double half_pi = 1.57079632679489661923;
    const int rows_per_set = 1 + 2 * h->nocc;
    std::vector<double> g((size_t)sets * h->nparams, 0.0), e(sets, 0.0);
    std::vector<int> row_set(h->max_batch), shift_occ(h->max_batch);
    std::vector<double> shift_val(h->max_batch), row_e(h->max_batch);
    // rows enumerate (set, r): r = 0 unshifted, r = 2j+1 occurrence j shifted +pi/2, r = 2j+2 -pi/2
    const long long total = (long long)sets * rows_per_set;
    for (long long start = 0; start < total; start += h->max_batch) {
        const int rows = (int)std::min<long long>(h->max_batch, total - start);
        for (int i = 0; i < rows; ++i) {
            const long long g_row = start + i;
            const int set = (int)(g_row / rows_per_set), r = (int)(g_row % rows_per_set);
            row_set[i] = set;
            shift_occ[i] = r == 0 ? -1 : (r - 1) / 2;
            shift_val[i] = r == 0 ? 0.0 : ((r % 2) ? half_pi : -half_pi);
        }
        ADJ_CUDA(cudaMemcpyAsync(h->d_row_set, row_set.data(), rows * sizeof(int), cudaMemcpyHostToDevice, h->stream), "rows");
        ADJ_CUDA(cudaMemcpyAsync(h->d_shift_occ, shift_occ.data(), rows * sizeof(int), cudaMemcpyHostToDevice, h->stream), "rows");
        ADJ_CUDA(cudaMemcpyAsync(h->d_shift_val, shift_val.data(), rows * sizeof(double), cudaMemcpyHostToDevice, h->stream),
                 "rows");
        if ((rc = build_table(h, rows, true))) return rc;
        if ((rc = forward_dispatch(h, rows, false, nullptr))) return rc;
        ADJ_CUDA(cudaMemcpyAsync(row_e.data(), h->d_energy, rows * sizeof(double), cudaMemcpyDeviceToHost, h->stream), "energies");
        ADJ_CUDA(cudaStreamSynchronize(h->stream), "cudaStreamSynchronize");
        for (int i = 0; i < rows; ++i) {
            const int set = row_set[i], occ = shift_occ[i];
            if (occ < 0) e[set] = row_e[i];
            else g[(size_t)set * h->nparams + h->occ_param[occ]] += (shift_val[i] > 0 ? 0.5 : -0.5) * row_e[i];
        }
    }
    const bool dev_g = is_device_ptr(grads);
    ADJ_CUDA(cudaMemcpy(grads, g.data(), g.size() * sizeof(double), dev_g ? cudaMemcpyHostToDevice : cudaMemcpyHostToHost),
             "gradients");
    if (energies)
        ADJ_CUDA(cudaMemcpy(energies, e.data(), e.size() * sizeof(double),
                            is_device_ptr(energies) ? cudaMemcpyHostToDevice : cudaMemcpyHostToHost),
                 "energies");
    return LLG_OK;
}

int llg_adjoint_stream(const llg_adjoint* h, void** out) {
    if (!h || !out) return set_error(LLG_EINVAL, "adjoint_stream: NULL argument");
    *out = (void*)h->stream;
    return LLG_OK;
}

}  // extern "C"
