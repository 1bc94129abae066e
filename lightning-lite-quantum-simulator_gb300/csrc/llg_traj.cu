// llg_traj.cu -- batched noisy trajectories in one persistent launch (include/llgpu.h,
// "trajectories" section).
//
// Each trajectory runs a circuit on an n-qubit state held entirely in shared memory.  After
// every gate, for each qubit the gate touches (the order of the reference's NoisyBackend noise
// sites, src/Mitigation.h:146-176 and :183-204), two single-qubit Kraus channels are unravelled:
// amplitude damping then phase damping (src/Noise.cpp:274-298, :366-372), each with the
// reference trajectory solver's jump rule (src/TrajectorySolver.h:421-455):
//     P1 = P(bit q = 1);  survive = 1 - g * P1;  jump if u1 >= survive (and g * P1 > 0);
//     jump:    psi <- K1 psi / sqrt(g * P1)        no jump: psi <- K0 psi / sqrt(survive)
// with P1 after amplitude damping taken from its closed form ((1 - g) P1 / survive, or 0 after
// a jump).  Uniforms are (x >> 11) * 2^-53 (src/Mitigation.h:207) from Philox4x32-10 with
// key = seed and counter = (site, trajectory): one Philox call per channel, u1 from its low
// 64 bits.  Every step renormalises the state (the periodic renormalisation of the complex64
// path happens at every noise site).
//
// Layout: a CTA holds 2^nl amplitudes.  Complex64 states up to 14 qubits fit one CTA (128 KiB);
// complex128 states (double-float or FP64, 16 B per amplitude) of 14 qubits use a cluster of two
// CTAs, rank r holding the amplitudes whose top qubit is r.  Gates and Kraus moves on the top
// qubit read the partner's half through distributed shared memory between cluster barriers; the
// P1 reduction sums the two halves in a fixed order on both CTAs, so both take the same decision.
// Every cluster barrier is executed unconditionally in the same sequence by both CTAs.  An op that
// touches only this CTA's half ends in a CTA barrier; an op that reads the partner's half starts
// with a cluster barrier (the partner has finished its earlier writes), and the exchange words of
// the reductions alternate between two slots.
#include <cooperative_groups.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/llgpu.h"
#include "llg_common.cuh"
#include "llg_internal.h"
#include "llg_launch.h"
#include "llg_tile.cuh"

namespace cg = cooperative_groups;

namespace llg {
int set_error(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);
}  // namespace llg

using namespace llg;

namespace {

constexpr int kTrajThreads = 1024;
constexpr int kPartWarps = kTrajThreads / 32;  // warp parts per reduction
constexpr int kMaxPerThread = 16;  // amplitudes per thread in a cross-CTA step (2^14 / 1024)
constexpr int kMaxGrid = 4096;     // persistent CTAs at most (per-CTA margin slots)
constexpr int kUChunk = 512;       // noise sites whose uniforms are drawn together (one Philox call per thread)

// one gate of a trajectory circuit: the executor op (global qubits) and the touched qubits
struct TrajGate {
    ExecOp op;
    int32_t nt;     // touched qubits, in noise-site order
    int32_t q[6];
    int32_t pair;   // depolarizing mode: 1 = one 2-qubit site over (q[0], q[1]), 0 = a 1-qubit site per qubit
    // Kraus mode: the real factor the op leaves out (RX / RY in their scale-free forms, EX_RXT,
    // EX_RXC, EX_RT, EX_RC; 1 otherwise).  The state is then held at 1 / f of its size until the
    // noise site that follows the gate, whose P(1) and renormalising factors take f into account.
    double f;
};

constexpr int kObsTerms = 16;
constexpr int kObsClasses = 3;

// Observable sum_k coef[cls[k]] Z_a[k] Z_b[k] (b < 0: Z_a alone) read at the end of every
// trajectory; nterms = 0 reads <Z_0>.  Terms are grouped into coefficient classes so the kernel
// counts parities in integers and weights |a|^2 once per class.
struct ObsTerms {
    int32_t nterms, nclass;
    int32_t a[kObsTerms], b[kObsTerms], cls[kObsTerms];
    double coef[kObsClasses];
};

enum : int32_t { NOISE_KRAUS = 0, NOISE_DEPOL = 1 };

struct KrausParams {
    double gamma, lambda;  // NOISE_DEPOL: gamma = p, the non-identity Pauli probability per site
    double sq1mg, sq1ml;   // sqrt(1 - gamma), sqrt(1 - lambda)
    uint64_t seed;
    int32_t mode;          // NOISE_KRAUS / NOISE_DEPOL
    int32_t pad;
};

// ------------------------------------------------------------------------------------------
// Philox4x32-10 (Salmon et al., SC'11) and the 53-bit uniform
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ double philox_u1(uint64_t seed, uint64_t traj, uint64_t site) {
    uint32_t c0 = (uint32_t)site, c1 = (uint32_t)(site >> 32), c2 = (uint32_t)traj, c3 = (uint32_t)(traj >> 32);
    uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r > 0) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        const uint32_t hi0 = __umulhi(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
        const uint32_t hi1 = __umulhi(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
        const uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0;
        c1 = lo1;
        c2 = n2;
        c3 = lo0;
    }
    const uint64_t a = ((uint64_t)c1 << 32) | c0;
    return (double)(a >> 11) * (1.0 / 9007199254740992.0);
}

// both uniforms of one Philox call: u1 from the low 64 bits, u2 from the high 64 bits
__device__ __forceinline__ void philox_u12(uint64_t seed, uint64_t traj, uint64_t site, double* u1, double* u2) {
    uint32_t c0 = (uint32_t)site, c1 = (uint32_t)(site >> 32), c2 = (uint32_t)traj, c3 = (uint32_t)(traj >> 32);
    uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r > 0) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        const uint32_t hi0 = __umulhi(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
        const uint32_t hi1 = __umulhi(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
        const uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0;
        c1 = lo1;
        c2 = n2;
        c3 = lo0;
    }
    const uint64_t a = ((uint64_t)c1 << 32) | c0, b = ((uint64_t)c3 << 32) | c2;
    *u1 = (double)(a >> 11) * (1.0 / 9007199254740992.0);
    *u2 = (double)(b >> 11) * (1.0 / 9007199254740992.0);
}

template <class P>
__device__ __forceinline__ uint64_t packk(double x) {
    if (P::kPrecision == 0) return (uint64_t)__double_as_longlong(x);
    if (P::kPrecision == 2) return (uint64_t)__float_as_uint(__double2float_rn(x));
    const df d = double_to_df(x);
    return (uint64_t)__float_as_uint(d.hi) | ((uint64_t)__float_as_uint(d.lo) << 32);
}

// shared decision record written by thread 0
struct Decision {
    // packed scale factors of the pair: g0 = f_ad0 f_pd0 for the |0> amplitudes (or the |1>
    // amplitudes moved down by an amplitude-damping jump), g1 = f_ad1 f_pd1 for the |1> ones, each
    // product formed once in double so that a site pair costs one multiply per real instead of two
    uint64_t g0, g1;
    int ad_jump, pd_jump;
    // Without a jump the |0> factor f_ad0 f_pd0 sig is carried
    // (sig_next) instead of applied, and only the |1> amplitudes are scaled, by
    // g1 = f_ad1 f_pd1 / (f_ad0 f_pd0) = sqrt(1 - gamma) sqrt(1 - lambda): one multiply per real of
    // half of the state instead of one per real of all of it
    int carry;
    double sig_next;  // the held state's factor after the pair (1 unless carry)
    double p1;
};

// |x| < 2^-L or |x| >= 2^L (x not 0; L = 300 for FP64 states, 40 for the float-based formats,
// whose floats end at 2^-126), from the exponent field: no FP64 instruction in the per-gate path
template <class P>
__device__ __forceinline__ bool outside_carry_range(double x) {
    constexpr int L = P::kPrecision == LLG_F64 ? 300 : 40;
    const int e = (int)((__double_as_longlong(x) >> 52) & 0x7ff) - 1023;
    return e < -L || e >= L;
}

// barrier for the trajectory's CTA group
template <int CL>
__device__ __forceinline__ void group_sync() {
    if (CL == 1) __syncthreads();
    else cg::this_cluster().sync();
}

template <class P, int CL>
struct Traj {
    using S = typename P::S;
    using C = typename P::C;
    using K = typename P::K;
    S* s;         // this CTA's amplitudes
    S* remote;    // partner's amplitudes (CL == 2)
    int nl;       // local qubits
    int rank;     // top-qubit value held by this CTA (0 for CL == 1)
    uint32_t NL;  // 2^nl

    __device__ bool cross(int q) const { return CL == 2 && q == nl; }

    // --- gates ---
    template <int KIND>
    __device__ void pair_gate(int q, const ExecOp& o) {
        if (!cross(q)) {
            tile_pairs<P, KIND>(s, NL >> 1, q, o);
            __syncthreads();
            return;
        }
        const PairMath<P, KIND> m(o);
        C out[kMaxPerThread];
        int cnt = 0;
        group_sync<CL>();  // the partner's earlier (CTA-local) writes are complete
        for (uint32_t l = threadIdx.x; l < NL; l += blockDim.x, ++cnt) {
            C mine = P::load(s[l]), other = P::load(remote[l]);
            C a0 = rank ? other : mine, a1 = rank ? mine : other;
            m.apply(a0, a1);
            out[cnt] = rank ? a1 : a0;
        }
        group_sync<CL>();  // the partner has read this CTA's half
        cnt = 0;
        for (uint32_t l = threadIdx.x; l < NL; l += blockDim.x, ++cnt) s[l] = P::store(out[cnt]);
        __syncthreads();
    }

    __device__ void gate(const ExecOp& o) {
        switch (o.kind) {
            case EX_U2: pair_gate<EX_U2>(o.q0, o); break;
            case EX_RX: pair_gate<EX_RX>(o.q0, o); break;
            case EX_RY: pair_gate<EX_RY>(o.q0, o); break;
            case EX_RT: pair_gate<EX_RT>(o.q0, o); break;
            case EX_RC: pair_gate<EX_RC>(o.q0, o); break;
            case EX_RXT: pair_gate<EX_RXT>(o.q0, o); break;
            case EX_RXC: pair_gate<EX_RXC>(o.q0, o); break;
            case EX_H: pair_gate<EX_H>(o.q0, o); break;
            case EX_X: pair_gate<EX_X>(o.q0, o); break;
            case EX_DIAG: {
                const K d0r = P::k_from_bits(o.c[0]), d0i = P::k_from_bits(o.c[1]);
                const K d1r = P::k_from_bits(o.c[2]), d1i = P::k_from_bits(o.c[3]);
                const K md0i = P::kneg(d0i), md1i = P::kneg(d1i);
                for (uint32_t l = threadIdx.x; l < NL; l += blockDim.x) {
                    const int bit = cross(o.q0) ? rank : (int)((l >> o.q0) & 1);
                    auto a = P::load(s[l]);
                    if (bit) cmul_const<P>(a, d1r, d1i, md1i);
                    else cmul_const<P>(a, d0r, d0i, md0i);
                    s[l] = P::store(a);
                }
                __syncthreads();
                break;
            }
            case EX_CNOT: {
                const int c = o.q0, t = o.q1;
                if (!cross(t)) {
                    if (cross(c)) {
                        if (rank) tile_pairs<P, EX_X>(s, NL >> 1, t, o);
                    } else {
                        const int lo = c < t ? c : t, hi = c < t ? t : c;
                        const uint32_t cbit = 1u << c, tbit = 1u << t;
                        for (uint32_t r = threadIdx.x; r < (NL >> 2); r += blockDim.x) {
                            const uint32_t j = ins0(ins0(r, 1u << lo), 1u << hi) | cbit;
                            const S x = s[j];
                            s[j] = s[j | tbit];
                            s[j | tbit] = x;
                        }
                    }
                    __syncthreads();
                } else {  // target is the top qubit: swap the control = 1 halves across the CTAs
                    S out[kMaxPerThread];
                    int cnt = 0;
                    group_sync<CL>();  // the partner's earlier writes are complete
                    for (uint32_t l = threadIdx.x; l < NL; l += blockDim.x, ++cnt) out[cnt] = ((l >> c) & 1) ? remote[l] : s[l];
                    group_sync<CL>();
                    cnt = 0;
                    for (uint32_t l = threadIdx.x; l < NL; l += blockDim.x, ++cnt) s[l] = out[cnt];
                    __syncthreads();
                }
                break;
            }
            case EX_MCZ: {
                uint64_t m = o.mask;
                bool active = true;
                if (CL == 2 && ((m >> nl) & 1)) {
                    active = rank == 1;
                    m &= ~(1ULL << nl);
                }
                if (active) {
                    const uint32_t lm = (uint32_t)m;
                    const uint32_t cntm = NL >> __popc(lm);
                    for (uint32_t r = threadIdx.x; r < cntm; r += blockDim.x) {
                        const uint32_t j = (uint32_t)insert0_mask(r, lm) | lm;
                        auto a = P::load(s[j]);
                        a.re = P::neg(a.re);
                        a.im = P::neg(a.im);
                        s[j] = P::store(a);
                    }
                }
                __syncthreads();
                break;
            }
            default: __syncthreads(); break;
        }
    }

    // sum over the group of |a|^2 for amplitudes with (global bit q) == 1 (q < 0: all), or of
    // (1 - 2 bit0)|a|^2 when z0 is set; identical in every CTA of the group
    __device__ double reduce(int q, bool z0, double* part2) {
        typename P::Acc pos = P::acc_zero(), neg = P::acc_zero();
        if (z0) {
            for (uint32_t l = threadIdx.x; l < NL; l += blockDim.x) {
                const auto a = P::load(s[l]);
                if (l & 1) neg = P::acc_norm(neg, a);
                else pos = P::acc_norm(pos, a);
            }
        } else if (cross(q)) {  // the partner with the top qubit set holds the whole bit-1 half
            if (rank)
                for (uint32_t l = threadIdx.x; l < NL; l += blockDim.x) pos = P::acc_norm(pos, P::load(s[l]));
        } else {  // only the amplitudes with bit q set are read
            const uint32_t bit = 1u << q;
            for (uint32_t p = threadIdx.x; p < (NL >> 1); p += blockDim.x) pos = P::acc_norm(pos, P::load(s[ins0(p, bit) | bit]));
        }
        return group_total(acc_minus(pos, neg), part2);
    }

    // group-wide sum of one accumulator per thread, returned in thread 0 (the deciding thread;
    // other threads get 0).  Each warp parks its shuffle-reduced part in `part`, one group barrier
    // later warp 0 adds both CTAs' parts warp by warp in rank order and reduces them, so both CTAs
    // of a cluster get the same bits.  `part2` is two sets of kPartWarps words used in turn: a CTA
    // writes set k % 2 at call k only after the group barrier of call k - 1, which the partner's
    // warp 0 reaches after reading call k - 2's words.
    int sbuf = 0;
    // The warp stage runs in the accumulator's format (double-float on the FP32 pipe for
    // double-float and complex64 states); the warp's sum is then converted once, and the stages
    // across warps and CTAs add IEEE doubles.
    __device__ double group_total(typename P::Acc v, double* part2) {
        const double wsum = acc_value(warp_sum_acc(v));
        double* part = part2 + kPartWarps * sbuf;
        sbuf ^= 1;
        const int lane = threadIdx.x & 31, nw = (int)(blockDim.x >> 5);
        if (lane == 0) part[threadIdx.x >> 5] = wsum;
        group_sync<CL>();
        if (threadIdx.x >= 32) return 0.0;
        double x = 0.0;
        if (lane < nw) {
            if (CL == 1) {
                x = part[lane];
            } else {
                cg::cluster_group cl = cg::this_cluster();
                x = cl.map_shared_rank(part, 0)[lane] + cl.map_shared_rank(part, 1)[lane];
            }
        }
        return warp_sum_dbl(x);
    }

    // the observable sum_c coef_c * sum_i |a_i|^2 (tot_c - 2 odd_c(i)) over the group's state
    __device__ double observable(const ObsTerms& ob, double* part2) {
        typename P::Acc acc[kObsClasses];
        int tot[kObsClasses] = {0, 0, 0};
#pragma unroll
        for (int c = 0; c < kObsClasses; ++c) acc[c] = P::acc_zero();
        for (int k = 0; k < ob.nterms; ++k) tot[ob.cls[k]] += 1;
        for (uint32_t l = threadIdx.x; l < NL; l += blockDim.x) {
            const uint32_t gi = l | ((uint32_t)rank << nl);
            int odd[kObsClasses] = {0, 0, 0};
            for (int k = 0; k < ob.nterms; ++k) {
                int par = (int)((gi >> ob.a[k]) & 1);
                if (ob.b[k] >= 0) par ^= (int)((gi >> ob.b[k]) & 1);
                odd[ob.cls[k]] += par;
            }
            const auto a = P::load(s[l]);
#pragma unroll
            for (int c = 0; c < kObsClasses; ++c)
                if (c < ob.nclass) acc[c] = P::acc_norm_w(acc[c], a, (float)(tot[c] - 2 * odd[c]));
        }
        double e = 0.0;
        for (int c = 0; c < ob.nclass; ++c) {
            e += ob.coef[c] * group_total(acc[c], part2);
        }
        return e;
    }

    // Pauli Z on global qubit q: negate the amplitudes whose bit q is 1
    __device__ void pauli_z(int q) {
        if (cross(q)) {
            if (rank == 1)
                for (uint32_t l = threadIdx.x; l < NL; l += blockDim.x) {
                    auto a = P::load(s[l]);
                    a.re = P::neg(a.re);
                    a.im = P::neg(a.im);
                    s[l] = P::store(a);
                }
        } else {
            const uint32_t bit = 1u << q;
            for (uint32_t p = threadIdx.x; p < (NL >> 1); p += blockDim.x) {
                const uint32_t j = ins0(p, bit) | bit;
                auto a = P::load(s[j]);
                a.re = P::neg(a.re);
                a.im = P::neg(a.im);
                s[j] = P::store(a);
            }
        }
        __syncthreads();
    }

    // Pauli X on global qubit q: swap the amplitude pairs along q (across the two CTAs for the
    // top qubit of a cluster: each CTA takes the partner's half)
    __device__ void pauli_x(int q) {
        if (cross(q)) {
            S out[kMaxPerThread];
            int cnt = 0;
            group_sync<CL>();  // the partner's earlier writes are complete
            for (uint32_t l = threadIdx.x; l < NL; l += blockDim.x, ++cnt) out[cnt] = remote[l];
            group_sync<CL>();  // both CTAs hold the partner's half
            cnt = 0;
            for (uint32_t l = threadIdx.x; l < NL; l += blockDim.x, ++cnt) s[l] = out[cnt];
        } else {
            const uint32_t bit = 1u << q;
            for (uint32_t p = threadIdx.x; p < (NL >> 1); p += blockDim.x) {
                const uint32_t j0 = ins0(p, bit), j1 = j0 | bit;
                const S t = s[j0];
                s[j0] = s[j1];
                s[j1] = t;
            }
        }
        __syncthreads();
    }

    // Pauli 1 = X, 2 = Y (Z then X, up to a global phase), 3 = Z
    __device__ void pauli(int q, int which) {
        if (which == 2 || which == 3) pauli_z(q);
        if (which == 1 || which == 2) pauli_x(q);
    }

    // every held amplitude times f (this CTA's slice; each CTA of a cluster scales its own)
    __device__ void rescale(double f) {
        const K fk = P::k_from_double(f);
        for (uint32_t l = threadIdx.x; l < NL; l += blockDim.x) {
            C a = P::load(s[l]);
            a.re = P::mulk(fk, a.re);
            a.im = P::mulk(fk, a.im);
            s[l] = P::store(a);
        }
        __syncthreads();
    }

    // amplitude damping then phase damping on qubit q, decisions in *d (already filled)
    __device__ void kraus_apply(int q, const Decision* d) {
        const K g0 = P::k_from_bits(d->g0), g1 = P::k_from_bits(d->g1);
        const int adj = d->ad_jump, pdj = d->pd_jump;
        auto scale = [](C a, K f) {
            C r;
            r.re = P::mulk(f, a.re);
            r.im = P::mulk(f, a.im);
            return r;
        };
        auto zero = []() {
            C r;
            r.re = P::zero();
            r.im = P::zero();
            return r;
        };
        if (d->carry) {  // no jump, the |0> factor carried: the |1> amplitudes times g1
            if (!cross(q)) {
                const uint32_t bit = 1u << q;
                for (uint32_t p = threadIdx.x; p < (NL >> 1); p += blockDim.x) {
                    const uint32_t j1 = ins0(p, bit) | bit;
                    s[j1] = P::store(scale(P::load(s[j1]), g1));
                }
            } else if (rank == 1) {  // the cluster's bit-1 half; nothing read across the cluster
                for (uint32_t l = threadIdx.x; l < NL; l += blockDim.x) s[l] = P::store(scale(P::load(s[l]), g1));
            }
            __syncthreads();
            return;
        }
        if (!cross(q)) {
            const uint32_t bit = 1u << q;
            for (uint32_t p = threadIdx.x; p < (NL >> 1); p += blockDim.x) {
                const uint32_t j0 = ins0(p, bit), j1 = j0 | bit;
                C a0 = P::load(s[j0]), a1 = P::load(s[j1]);
                C t0, t1;
                if (adj) {
                    t0 = scale(a1, g0);
                    t1 = zero();
                } else {
                    t0 = scale(a0, g0);
                    t1 = scale(a1, g1);
                }
                if (pdj) t0 = zero();
                s[j0] = P::store(t0);
                s[j1] = P::store(t1);
            }
            __syncthreads();
            return;
        }
        // top qubit across the cluster: rank 0 holds the bit-0 half, rank 1 the bit-1 half
        C out[kMaxPerThread];
        int cnt = 0;
        group_sync<CL>();  // the partner's earlier writes are complete
        for (uint32_t l = threadIdx.x; l < NL; l += blockDim.x, ++cnt) {
            C t;
            if (rank == 0) {
                t = adj ? scale(P::load(remote[l]), g0) : scale(P::load(s[l]), g0);
                if (pdj) t = zero();
            } else {
                t = adj ? zero() : scale(P::load(s[l]), g1);
            }
            out[cnt] = t;
        }
        group_sync<CL>();
        cnt = 0;
        for (uint32_t l = threadIdx.x; l < NL; l += blockDim.x, ++cnt) s[l] = P::store(out[cnt]);
        __syncthreads();
    }
};

// thread 0: decide one site pair (AD at a site, PD at the next) from its two uniforms, as the
// oracle does
template <class P>
// The comparisons and p1 (which decides the dephasing jump) are computed exactly as the oracle
// computes them, in IEEE double with correctly rounded division; the scale factors only rescale
// amplitudes and use rsqrt (within 1 ulp) instead of a square root and a division.
// sig: the factor the held state is short of its true size (scale-free rotations, and the |0>
// factors of jump-free sites, carried so far); P1_held is the held state's P(1), so the true one
// is sig^2 P1_held, and the factors that renormalise the held amplitudes carry sig.
__device__ void decide(double P1_held, double sig, const KrausParams& kp, double u1, double u2, Decision* d,
                       double* min_margin) {
    const double P1 = sig == 1.0 ? P1_held : sig * sig * P1_held;
    // amplitude damping
    double s_ad = 1.0 - kp.gamma * P1;
    const double tot_ad = kp.gamma * P1;
    double m = fabs(u1 - s_ad);
    if (m < *min_margin) *min_margin = m;
    double p1, fa0, fa1, fp0, fp1;
    if (u1 >= s_ad && tot_ad > 0.0) {
        d->ad_jump = 1;
        fa0 = rsqrt(P1);
        fa1 = 0.0;
        p1 = 0.0;
    } else {
        d->ad_jump = 0;
        const double s0 = rsqrt(s_ad);
        fa0 = s0;
        fa1 = kp.sq1mg * s0;
        p1 = (1.0 - kp.gamma) * P1 / s_ad;
    }
    // phase damping
    const double s_pd = 1.0 - kp.lambda * p1;
    const double tot_pd = kp.lambda * p1;
    m = fabs(u2 - s_pd);
    if (m < *min_margin) *min_margin = m;
    if (u2 >= s_pd && tot_pd > 0.0) {
        d->pd_jump = 1;
        fp0 = 0.0;
        fp1 = rsqrt(p1);
    } else {
        d->pd_jump = 0;
        const double s0 = rsqrt(s_pd);
        fp0 = s0;
        fp1 = kp.sq1ml * s0;
    }
    d->p1 = p1;
    if (!d->ad_jump && !d->pd_jump) {
        d->carry = 1;
        d->sig_next = fa0 * fp0 * sig;
        d->g0 = packk<P>(1.0);
        d->g1 = packk<P>(kp.sq1mg * kp.sq1ml);
        return;
    }
    d->carry = 0;
    d->sig_next = 1.0;
    d->g0 = packk<P>(fa0 * fp0 * sig);
    d->g1 = packk<P>(fa1 * fp1 * sig);
}

template <class P, int CL>
__device__ void traj_kernel_body(int n, const TrajGate* __restrict__ gates, int ngates, KrausParams kp,
                                 const ObsTerms* __restrict__ obs, uint64_t traj_begin,
                                 uint64_t n_traj, double* __restrict__ z0_out, uint32_t* __restrict__ jumps_out,
                                 uint8_t* __restrict__ jump_log, int64_t log_stride, double* __restrict__ margin_out) {
    using S = typename P::S;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ double part2[2 * kPartWarps];  // group_total's warp parts (double), two sets used in turn
    __shared__ Decision dec;
    __shared__ ObsTerms ob;  // the observable, copied once from global memory
    // uniforms of sites [u_begin, u_end): Kraus mode uni[site - u_begin] = philox_u1(site); depolarizing
    // mode (uni[2 i], uni[2 i + 1]) = philox_u12(u_begin + i).  Drawn together, one Philox call per
    // thread, instead of serially by the deciding thread.
    __shared__ double uni[2 * kUChunk];
    uint64_t u_begin = 0, u_end = 0;
    static_assert(sizeof(ObsTerms) % 4 == 0, "ObsTerms copies as 32-bit words");
    for (uint32_t w = threadIdx.x; w < sizeof(ObsTerms) / 4; w += blockDim.x)
        reinterpret_cast<int32_t*>(&ob)[w] = reinterpret_cast<const int32_t*>(obs)[w];
    __syncthreads();
    Traj<P, CL> T;
    T.nl = (CL == 2) ? n - 1 : n;
    T.NL = 1u << T.nl;
    T.s = reinterpret_cast<S*>(smem_raw);
    if (CL == 2) {
        cg::cluster_group cl = cg::this_cluster();
        T.rank = (int)cl.block_rank();
        T.remote = cl.map_shared_rank(T.s, T.rank ^ 1);
    } else {
        T.rank = 0;
        T.remote = nullptr;
    }
    const uint64_t group = blockIdx.x / CL, ngroups = gridDim.x / CL;
    double min_margin = 1.0;
    for (uint64_t tt = group; tt < n_traj; tt += ngroups) {
        const uint64_t traj = traj_begin + tt;
        // |0..0>
        for (uint32_t l = threadIdx.x; l < T.NL; l += blockDim.x) {
            typename P::C z;
            z.re = P::r_from_float((l == 0 && T.rank == 0) ? 1.0f : 0.0f);
            z.im = P::zero();
            T.s[l] = P::store(z);
        }
        group_sync<CL>();
        uint64_t site = 0;
        uint32_t jumps = 0;
        double sig = 1.0;  // the held state is 1 / sig of its true size (the same on every thread)
        u_begin = u_end = 0;
        auto draw = [&](uint64_t first) {  // every thread, at the same site
            __syncthreads();
            for (int i = threadIdx.x; i < kUChunk; i += blockDim.x) {
                if (kp.mode == NOISE_DEPOL) philox_u12(kp.seed, traj, first + i, &uni[2 * i], &uni[2 * i + 1]);
                else uni[i] = philox_u1(kp.seed, traj, first + i);
            }
            u_begin = first;
            u_end = first + kUChunk;
            __syncthreads();
        };
        for (int g = 0; g < ngates; ++g) {
            const TrajGate& G = gates[g];
            T.gate(G.op);
            sig *= G.f;
            // the held state is rescaled before it could leave its format's range (2^300 away
            // from its true size in FP64, 2^40 in the float-based formats): scale-free rotations
            // shrink sig, carried Kraus factors grow it
            if (outside_carry_range<P>(sig)) {
                T.rescale(sig);
                sig = 1.0;
            }
            if (kp.mode == NOISE_DEPOL) {
                // unitary sites: the factor is carried to the observable
                // decisions do not depend on the state: every thread draws the same uniforms, so
                // the branch is uniform and needs no broadcast
                if (!(kp.gamma > 0.0)) continue;
                const int nsites = G.pair ? 1 : G.nt;
                for (int k = 0; k < nsites; ++k) {
                    if (site >= u_end) draw(site);
                    const double u = uni[2 * (site - u_begin)], u2 = uni[2 * (site - u_begin) + 1];
                    ++site;
                    if (u >= kp.gamma) continue;
                    ++jumps;
                    if (G.pair) {
                        const int idx = 1 + (int)(u2 * 15.0);
                        T.pauli(G.q[0], idx & 3);
                        T.pauli(G.q[1], idx >> 2);
                    } else {
                        T.pauli(G.q[k], 1 + (int)(u2 * 3.0));
                    }
                }
                continue;
            }
            for (int k = 0; k < G.nt; ++k) {
                const int q = G.q[k];
                if (site + 1 >= u_end) draw(site);  // AD and PD uniforms of this pair in one chunk
                const double P1 = T.reduce(q, false, part2);
                if (threadIdx.x == 0)
                    decide<P>(P1, sig, kp, uni[site - u_begin], uni[site + 1 - u_begin], &dec, &min_margin);
                __syncthreads();
                sig = dec.sig_next;  // 1: the Kraus pass below stores the true, renormalised state
                const int code = dec.ad_jump | (dec.pd_jump << 1);
                T.kraus_apply(q, &dec);
                if (threadIdx.x == 0 && T.rank == 0 && jump_log)
                    jump_log[(int64_t)tt * log_stride + (int64_t)(site >> 1)] = (uint8_t)code;
                jumps += (code & 1) + (code >> 1);
                site += 2;
            }
        }
        double z = ob.nterms > 0 ? T.observable(ob, part2) : T.reduce(0, true, part2);
        if (sig != 1.0) z *= sig * sig;  // factors carried past the last site
        if (threadIdx.x == 0 && T.rank == 0) {
            z0_out[tt] = z;
            if (jumps_out) jumps_out[tt] = jumps;
        }
        group_sync<CL>();
    }
    if (threadIdx.x == 0 && margin_out) margin_out[blockIdx.x] = min_margin;
}

template <class P>
__global__ void __launch_bounds__(kTrajThreads) k_traj1(int n, const TrajGate* gates, int ngates, KrausParams kp,
                                                        const ObsTerms* ob,
                                                        uint64_t traj_begin, uint64_t n_traj, double* z0, uint32_t* jumps,
                                                        uint8_t* log, int64_t log_stride, double* margins) {
    traj_kernel_body<P, 1>(n, gates, ngates, kp, ob, traj_begin, n_traj, z0, jumps, log, log_stride, margins);
}

template <class P>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(kTrajThreads)
    k_traj2(int n, const TrajGate* gates, int ngates, KrausParams kp, const ObsTerms* ob, uint64_t traj_begin, uint64_t n_traj,
            double* z0,
            uint32_t* jumps, uint8_t* log, int64_t log_stride, double* margins) {
    traj_kernel_body<P, 2>(n, gates, ngates, kp, ob, traj_begin, n_traj, z0, jumps, log, log_stride, margins);
}

template <class P>
const void* traj_kernel(int cl) {
    return cl == 2 ? reinterpret_cast<const void*>(&k_traj2<P>) : reinterpret_cast<const void*>(&k_traj1<P>);
}

template <class P>
size_t traj_elem() {
    return sizeof(typename P::S);
}

const void* kernel_for(int P, int cl) {
    switch (P) {
        case LLG_F64: return traj_kernel<PolF64>(cl);
        case LLG_F32: return traj_kernel<PolF32>(cl);
        default: return traj_kernel<PolDF64>(cl);
    }
}

}  // namespace

// A trajectory circuit planned once: gates on the device, output buffers for up to max_traj
// trajectories, and the persistent launch captured as a CUDA graph whose kernel-node arguments
// (seed, first trajectory, count, log) are updated before each replay.
struct llg_traj {
    int n = 0, P = LLG_DF64;
    int cl = 1, threads = 0, grid = 0;
    size_t smem = 0;
    int ngates = 0;
    int64_t sites = 0;
    KrausParams kp{};
    ObsTerms obs{};
    ObsTerms* d_obs = nullptr;  // device copy of obs, read by the kernel
    uint64_t max_traj = 0;
    uint64_t shape_key = 0;
    TrajGate* d_gates = nullptr;
    double* d_z0 = nullptr;
    uint32_t* d_jumps = nullptr;
    double* d_margin = nullptr;
    cudaStream_t stream = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaGraphNode_t node = nullptr;
};

namespace {

void drop_graph(llg_traj* h) {
    if (h->exec) cudaGraphExecDestroy(h->exec);
    if (h->graph) cudaGraphDestroy(h->graph);
    h->exec = nullptr;
    h->graph = nullptr;
    h->node = nullptr;
}

// The CTA threads a (cluster, threads) request resolves to, or 0 if it cannot run: the state
// slice must fit shared memory, and a cross-CTA step holds at most kMaxPerThread amplitudes per
// thread in registers.
int resolve_threads(int n, int P, int cl, int threads, size_t* smem_out) {
    if (cl != 1 && cl != 2) return 0;
    if (cl == 2 && n < 2) return 0;
    const int nl = cl == 2 ? n - 1 : n;
    const size_t smem = ((size_t)1 << nl) * elem_bytes(P);
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (smem > (size_t)optin) return 0;
    if (threads <= 0) threads = std::min(kTrajThreads, std::max(32, 1 << std::max(0, nl - 1)));
    if (threads < 32 || threads > kTrajThreads || (threads & 31)) return 0;
    if (cl == 2 && (((1u << nl) + threads - 1) / threads) > (unsigned)kMaxPerThread) return 0;
    *smem_out = smem;
    return threads;
}

// Sets (cluster, threads), sizes the persistent grid from the occupancy and captures the graph.
int configure(llg_traj* h, int cl, int threads) {
    size_t smem = 0;
    const int th = resolve_threads(h->n, h->P, cl, threads, &smem);
    if (!th) return set_error(LLG_EINVAL, "traj: cluster " + std::to_string(cl) + " with " + std::to_string(threads) +
                                              " threads cannot hold a " + std::to_string(h->n) + "-qubit state");
    const void* fn = kernel_for(h->P, cl);
    int dev = 0, sms = 1, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, th, smem);
    if (e != cudaSuccess) return cuda_fail(e, "trajectory kernel attributes");
    if (per_sm < 1) return set_error(LLG_EINVAL, "traj: configuration does not fit an SM");
    uint64_t groups = (uint64_t)sms * per_sm / cl;
    groups = std::max<uint64_t>(1, std::min<uint64_t>(groups, h->max_traj));
    groups = std::min<uint64_t>(groups, (uint64_t)(kMaxGrid / cl));  // margin buffer holds kMaxGrid CTAs
    drop_graph(h);
    h->cl = cl;
    h->threads = th;
    h->smem = smem;
    h->grid = (int)(groups * cl);
    // capture one launch; its arguments are replaced before every replay
    int n = h->n, ngates = h->ngates;
    uint64_t b0 = 0, c0 = 0;
    uint8_t* lg = nullptr;
    int64_t ls = 0;
    void* args[] = {&n, &h->d_gates, &ngates, &h->kp, &h->d_obs, &b0, &c0, &h->d_z0, &h->d_jumps, &lg, &ls, &h->d_margin};
    e = cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        cudaError_t le = cudaLaunchKernel(fn, dim3(h->grid), dim3(th), args, smem, h->stream);
        e = cudaStreamEndCapture(h->stream, &h->graph);
        if (le != cudaSuccess) e = le;
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&h->exec, h->graph, 0);
    size_t count = 1;
    if (e == cudaSuccess) e = cudaGraphGetNodes(h->graph, &h->node, &count);
    if (e == cudaSuccess && count != 1) return set_error(LLG_ECUDA, "traj: captured graph has an unexpected shape");
    if (e != cudaSuccess) {
        drop_graph(h);
        return cuda_fail(e, "trajectory graph capture");
    }
    return LLG_OK;
}

// Replays the graph for trajectories [begin, begin + count) (outputs stay on the device).
int replay(llg_traj* h, uint64_t seed, uint64_t begin, uint64_t count, uint8_t* d_log, int64_t log_stride) {
    int n = h->n, ngates = h->ngates;
    KrausParams kp = h->kp;
    kp.seed = seed;
    void* args[] = {&n,     &h->d_gates, &ngates,     &kp,        &h->d_obs,    &begin,
                    &count, &h->d_z0,    &h->d_jumps, &d_log,     &log_stride, &h->d_margin};
    cudaKernelNodeParams p;
    std::memset(&p, 0, sizeof(p));
    p.func = const_cast<void*>(kernel_for(h->P, h->cl));
    p.gridDim = dim3(h->grid);
    p.blockDim = dim3(h->threads);
    p.sharedMemBytes = (unsigned)h->smem;
    p.kernelParams = args;
    cudaError_t e = cudaGraphExecKernelNodeSetParams(h->exec, h->node, &p);
    if (e == cudaSuccess) e = cudaGraphLaunch(h->exec, h->stream);
    if (e != cudaSuccess) return cuda_fail(e, "trajectory launch");
    return LLG_OK;
}

int collect(llg_traj* h, uint64_t count, double* z0_out, uint32_t* jumps_out, double* min_margin) {
    cudaError_t e = cudaSuccess;
    if (z0_out) e = cudaMemcpyAsync(z0_out, h->d_z0, count * sizeof(double), cudaMemcpyDefault, h->stream);
    if (e == cudaSuccess && jumps_out)
        e = cudaMemcpyAsync(jumps_out, h->d_jumps, count * sizeof(uint32_t), cudaMemcpyDefault, h->stream);
    std::vector<double> margins(min_margin ? h->grid : 0);
    if (e == cudaSuccess && min_margin)
        e = cudaMemcpyAsync(margins.data(), h->d_margin, h->grid * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return cuda_fail(e, "trajectory kernel");
    if (min_margin) {
        double m = 1.0;
        for (double v : margins) m = std::min(m, v);
        *min_margin = m;
    }
    return LLG_OK;
}

// Lowers the circuit to trajectory gates with global qubits.  NOISE_KRAUS: one site per touched
// qubit (control then target; mcz qubits in increasing order).  NOISE_DEPOL: the gate list folded
// as U (U^+ U)^folds per gate, each application followed by its noise site(s): a 2-qubit site
// for cnot, cz and 2-qubit mcz, else a 1-qubit site per touched qubit (src/Mitigation.h:184-205).
bool build_gates(int n, const llg_op* ops, int nops, int precision, int mode, int folds, std::vector<TrajGate>& gates,
                 int64_t& sites, std::string& err) {
    gates.clear();
    sites = 0;
    for (int i = 0; i < nops; ++i) {
        const llg_op& o = ops[i];
        bool ok = o.q0 >= 0 && o.q0 < n;
        if (o.kind == LLG_OP_CNOT || o.kind == LLG_OP_CZ) ok = ok && o.q1 >= 0 && o.q1 < n && o.q1 != o.q0;
        if (o.kind == LLG_OP_MCZ) ok = o.mask != 0 && (o.mask >> n) == 0;
        if ((o.kind == LLG_OP_RX || o.kind == LLG_OP_RY || o.kind == LLG_OP_RZ) && !std::isfinite(o.theta)) ok = false;
        if (o.kind < 0 || o.kind > LLG_OP_U2) ok = false;
        if (!ok) {
            err = "traj_run: invalid op " + std::to_string(i);
            return false;
        }
        if (o.kind == LLG_OP_MCZ && __builtin_popcountll(o.mask) > 6) {
            err = "traj_run: mcz on more than 6 qubits";
            return false;
        }
        // the op and (for folding) its inverse: R(-t) for rotations, the adjoint for a 2x2
        llg_op inv = o;
        if (o.kind == LLG_OP_RX || o.kind == LLG_OP_RY || o.kind == LLG_OP_RZ) inv.theta = -o.theta;
        if (o.kind == LLG_OP_U2)
            for (int r = 0; r < 2; ++r)
                for (int c = 0; c < 2; ++c) {
                    inv.m[2 * (2 * r + c)] = o.m[2 * (2 * c + r)];
                    inv.m[2 * (2 * r + c) + 1] = -o.m[2 * (2 * c + r) + 1];
                }
        TrajGate g[2];
        for (int v = 0; v < 2; ++v) {
            std::vector<ExecOp> lowered;
            if (!lower_op(n, v ? inv : o, precision, lowered, err) || lowered.size() != 1) {
                err = "traj_run: " + err;
                return false;
            }
            std::memset(&g[v], 0, sizeof(TrajGate));
            g[v].op = lowered[0];
            g[v].f = 1.0;
            if (precision != LLG_F32 && (o.kind == LLG_OP_RX || o.kind == LLG_OP_RY)) {
                // the scale-free form (one multiply-add per real instead of two): the factor joins
                // the carried one, which the next Kraus site's renormalisation or the observable
                // takes (IEEE complex128 Kraus trajectories 10.8k -> 12.7k per second, double-float
                // 26.1k -> 26.5k once the Kraus factors were carried too; complex64 keeps the full
                // forms, which measured 2-3 % faster in its barrier-bound kernel)
                const double th = (v ? inv : o).theta;
                const double c = std::cos(0.5 * th), sn = std::sin(0.5 * th);
                const bool tan_form = std::fabs(c) >= std::fabs(sn);
                ExecOp e;
                std::memset(&e, 0, sizeof(e));
                e.kind = o.kind == LLG_OP_RX ? (tan_form ? EX_RXT : EX_RXC) : (tan_form ? EX_RT : EX_RC);
                e.q0 = o.q0;
                e.c[2] = pack_coef(precision, tan_form ? sn / c : c / sn);
                g[v].op = e;
                g[v].f = tan_form ? c : sn;
            }
            if (o.kind == LLG_OP_CNOT || o.kind == LLG_OP_CZ) {
                g[v].nt = 2;
                g[v].q[0] = o.q0;
                g[v].q[1] = o.q1;
            } else if (o.kind == LLG_OP_MCZ) {
                for (int q = 0; q < n && g[v].nt < 6; ++q)
                    if ((o.mask >> q) & 1) g[v].q[g[v].nt++] = q;
            } else {
                g[v].nt = 1;
                g[v].q[0] = o.q0;
            }
            g[v].pair = (mode == NOISE_DEPOL && g[v].nt == 2) ? 1 : 0;
        }
        const int64_t per_app = mode == NOISE_DEPOL ? (g[0].pair ? 1 : g[0].nt) : g[0].nt;
        gates.push_back(g[0]);
        for (int f = 0; f < folds; ++f) {
            gates.push_back(g[1]);
            gates.push_back(g[0]);
        }
        sites += per_app * (1 + 2 * (int64_t)folds);
    }
    return true;
}

// Groups observable terms into at most kObsClasses coefficient classes.
bool build_obs(int n, int nterms, const int* za, const int* zb, const double* zc, ObsTerms& ob, std::string& err) {
    std::memset(&ob, 0, sizeof(ob));
    if (nterms < 0 || nterms > kObsTerms || (nterms > 0 && (!za || !zb || !zc))) {
        err = "observable: at most 16 terms";
        return false;
    }
    for (int k = 0; k < nterms; ++k) {
        if (za[k] < 0 || za[k] >= n || zb[k] >= n || zb[k] == za[k] || !std::isfinite(zc[k])) {
            err = "observable: bad term " + std::to_string(k);
            return false;
        }
        int c = 0;
        while (c < ob.nclass && ob.coef[c] != zc[k]) ++c;
        if (c == ob.nclass) {
            if (ob.nclass == kObsClasses) {
                err = "observable: at most 3 distinct coefficients";
                return false;
            }
            ob.coef[ob.nclass++] = zc[k];
        }
        ob.a[k] = za[k];
        ob.b[k] = zb[k] < 0 ? -1 : zb[k];
        ob.cls[k] = c;
    }
    ob.nterms = nterms;
    return true;
}

// Allocates and configures a handle for already-lowered gates.
int create_handle(int n, int precision, const std::vector<TrajGate>& gates, int64_t sites, const KrausParams& kp,
                  const ObsTerms& ob, uint64_t shape_key, uint64_t max_traj, int cluster, int cta_threads, llg_traj** out) {
    llg_traj* h = new llg_traj();
    h->n = n;
    h->P = precision;
    h->ngates = (int)gates.size();
    h->sites = sites;
    h->max_traj = max_traj;
    h->kp = kp;
    h->obs = ob;
    h->shape_key = shape_key;
    int rc = LLG_OK;
    cudaError_t e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&h->d_gates, std::max<size_t>(gates.size(), 1) * sizeof(TrajGate));
    if (e == cudaSuccess) e = cudaMalloc(&h->d_z0, max_traj * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&h->d_jumps, max_traj * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMalloc(&h->d_margin, kMaxGrid * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&h->d_obs, sizeof(ObsTerms));
    if (e == cudaSuccess) e = cudaMemcpy(h->d_obs, &h->obs, sizeof(ObsTerms), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !gates.empty())
        e = cudaMemcpy(h->d_gates, gates.data(), gates.size() * sizeof(TrajGate), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaGetLastError();
        rc = set_error(LLG_ENOMEM, std::string("traj_create: ") + cudaGetErrorString(e));
    }
    if (!rc) {
        // default: one CTA per trajectory, a 2-CTA cluster when the state does not fit one CTA
        size_t smem = 0;
        const int cl_default = resolve_threads(n, precision, 1, 0, &smem) ? 1 : 2;
        const int cl = cluster > 0 ? cluster : cl_default;
        rc = configure(h, cl, cta_threads > 0 ? cta_threads : 0);
        if (!rc && (cluster == LLG_TUNE_AUTO || cta_threads == LLG_TUNE_AUTO)) rc = llg_traj_autotune(h, 0, nullptr);
    }
    if (rc) {
        llg_traj_destroy(h);
        return rc;
    }
    *out = h;
    return LLG_OK;
}

}  // namespace

extern "C" {

int llg_traj_destroy(llg_traj* h) {
    if (!h) return LLG_OK;
    if (h->stream) cudaStreamSynchronize(h->stream);
    drop_graph(h);
    cudaFree(h->d_gates);
    cudaFree(h->d_z0);
    cudaFree(h->d_jumps);
    cudaFree(h->d_margin);
    cudaFree(h->d_obs);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return LLG_OK;
}

int llg_traj_create(int n, const llg_op* ops, int nops, double gamma_ad, double lambda_pd, int precision,
                    uint64_t max_traj, int cluster, int cta_threads, llg_traj** out) {
    if (!out) return set_error(LLG_EINVAL, "traj_create: out is NULL");
    *out = nullptr;
    if (n < 1 || n > 14) return set_error(LLG_EINVAL, "traj_run: n must be in [1, 14]");
    if (precision != LLG_F64 && precision != LLG_DF64 && precision != LLG_F32)
        return set_error(LLG_EINVAL, "traj_run: unknown precision");
    if (nops < 0 || (nops > 0 && !ops)) return set_error(LLG_EINVAL, "traj_run: NULL argument");
    if (!(gamma_ad >= 0.0 && gamma_ad <= 1.0) || !(lambda_pd >= 0.0 && lambda_pd <= 1.0))
        return set_error(LLG_EINVAL, "traj_run: gamma and lambda must be in [0, 1]");
    if (max_traj == 0) return set_error(LLG_EINVAL, "traj_create: max_traj must be positive");
    if (cluster < LLG_TUNE_AUTO || cluster > 2 || cta_threads < LLG_TUNE_AUTO)
        return set_error(LLG_EINVAL, "traj_create: cluster must be -1, 0, 1 or 2 and cta_threads >= -1");
    std::vector<TrajGate> gates;
    int64_t sites = 0;
    std::string err;
    if (!build_gates(n, ops, nops, precision, NOISE_KRAUS, 0, gates, sites, err)) return set_error(LLG_EINVAL, err);
    KrausParams kp;
    std::memset(&kp, 0, sizeof(kp));
    kp.gamma = gamma_ad;
    kp.lambda = lambda_pd;
    kp.sq1mg = std::sqrt(1.0 - gamma_ad);
    kp.sq1ml = std::sqrt(1.0 - lambda_pd);
    kp.mode = NOISE_KRAUS;
    ObsTerms ob;
    std::memset(&ob, 0, sizeof(ob));
    const uint64_t key =
        tune_hash_ops(tune_hash(tune_hash(1469598103934665603ULL, 0x54524a), (uint64_t)n << 8 | (uint64_t)precision), ops, nops);
    return create_handle(n, precision, gates, sites, kp, ob, key, max_traj, cluster, cta_threads, out);
}

int llg_noisy_create(int n, const llg_op* ops, int nops, double p, int scale, int precision, uint64_t max_traj,
                     int nterms, const int* za, const int* zb, const double* zcoeff, int cluster, int cta_threads,
                     llg_traj** out) {
    if (!out) return set_error(LLG_EINVAL, "noisy_create: out is NULL");
    *out = nullptr;
    if (n < 1 || n > 14) return set_error(LLG_EINVAL, "noisy_create: n must be in [1, 14]");
    if (precision != LLG_F64 && precision != LLG_DF64 && precision != LLG_F32)
        return set_error(LLG_EINVAL, "noisy_create: unknown precision");
    if (nops < 0 || (nops > 0 && !ops)) return set_error(LLG_EINVAL, "noisy_create: NULL argument");
    if (!(p >= 0.0 && p <= 1.0)) return set_error(LLG_EINVAL, "NoisyBackend: p must be in [0, 1]");
    if (scale < 1 || scale > 99 || scale % 2 == 0)
        return set_error(LLG_EINVAL, "NoisyBackend::set_scale: scale must be an odd integer in [1, 99]");
    if (max_traj == 0) return set_error(LLG_EINVAL, "noisy_create: max_traj must be positive");
    if (cluster < LLG_TUNE_AUTO || cluster > 2 || cta_threads < LLG_TUNE_AUTO)
        return set_error(LLG_EINVAL, "noisy_create: cluster must be -1, 0, 1 or 2 and cta_threads >= -1");
    std::vector<TrajGate> gates;
    int64_t sites = 0;
    std::string err;
    if (!build_gates(n, ops, nops, precision, NOISE_DEPOL, (scale - 1) / 2, gates, sites, err))
        return set_error(LLG_EINVAL, err);
    ObsTerms ob;
    if (!build_obs(n, nterms, za, zb, zcoeff, ob, err)) return set_error(LLG_EINVAL, "noisy_create: " + err);
    KrausParams kp;
    std::memset(&kp, 0, sizeof(kp));
    kp.gamma = p;
    kp.mode = NOISE_DEPOL;
    uint64_t key = tune_hash(tune_hash(tune_hash(1469598103934665603ULL, 0x44504c), (uint64_t)n << 8 | (uint64_t)precision),
                             (uint64_t)scale);
    key = tune_hash_ops(key, ops, nops);
    return create_handle(n, precision, gates, sites, kp, ob, key, max_traj, cluster, cta_threads, out);
}

int llg_richardson_weights(const double* scales, int nscales, double* weights) {
    if (!scales || !weights || nscales < 2) return set_error(LLG_EINVAL, "ZNE::richardson_weights: need at least 2 scales");
    for (int k = 0; k < nscales; ++k)
        if (!std::isfinite(scales[k]) || scales[k] == 0.0)
            return set_error(LLG_EINVAL, "ZNE::richardson_weights: scales must be finite and nonzero");
    for (int k = 0; k < nscales; ++k) {
        double c = 1.0;
        for (int j = 0; j < nscales; ++j) {
            if (j == k) continue;
            if (scales[j] == scales[k]) return set_error(LLG_EINVAL, "ZNE::richardson_weights: scales must be distinct");
            c *= scales[j] / (scales[j] - scales[k]);
        }
        weights[k] = c;
    }
    return LLG_OK;
}

int llg_zne_run(int n, const llg_op* ops, int nops, double p, int precision, const double* scales, int nscales,
                int64_t trajectories, uint64_t seed, int nterms, const int* za, const int* zb, const double* zcoeff,
                llg_zne_result* out) {
    if (!out || !scales) return set_error(LLG_EINVAL, "ZNE::extrapolate: NULL argument");
    if (trajectories < 1) return set_error(LLG_EINVAL, "ZNE: trajectories must be >= 1");
    if (nscales < 2 || nscales > LLG_ZNE_MAX_SCALES)
        return set_error(LLG_EINVAL, "ZNE::validate_scales: need between 2 and 8 noise scales");
    for (int k = 0; k < nscales; ++k) {
        const double v = scales[k];
        if (!std::isfinite(v) || v < 1.0 || v > 99.0 || v != std::floor(v) || std::fmod(v, 2.0) != 1.0)
            return set_error(LLG_EINVAL, "ZNE::validate_scales: each scale must be an odd integer in [1, 99]");
        for (int j = 0; j < k; ++j)
            if (scales[j] == v) return set_error(LLG_EINVAL, "ZNE::validate_scales: scales must be distinct");
    }
    if (!(p >= 0.0 && p <= 1.0)) return set_error(LLG_EINVAL, "NoisyBackend: p must be in [0, 1]");
    llg_zne_result r;
    std::memset(&r, 0, sizeof(r));
    int rc = llg_richardson_weights(scales, nscales, r.weights);
    if (rc) return rc;
    if (nops < 1) return set_error(LLG_ERUNTIME, "ZNE::extrapolate: circuit_fn applied no gates to the backend");
    const bool noisy = p > 0.0;
    const int64_t nt = noisy ? trajectories : 1;
    r.nscales = nscales;
    r.trajectories = nt;
    std::vector<double> vals((size_t)nt);
    for (int k = 0; k < nscales && !rc; ++k) {
        llg_traj* h = nullptr;
        rc = llg_noisy_create(n, ops, nops, p, (int)scales[k], precision, (uint64_t)nt, nterms, za, zb, zcoeff, 0, 0, &h);
        if (!rc) rc = llg_traj_launch(h, seed, (uint64_t)k * (uint64_t)nt, (uint64_t)nt, vals.data(), nullptr, nullptr);
        llg_traj_destroy(h);
        if (rc) break;
        double mean = 0.0, m2 = 0.0;  // Welford, as the reference (src/Mitigation.h:350-353)
        for (int64_t t = 0; t < nt; ++t) {
            if (!std::isfinite(vals[t])) return set_error(LLG_EINVAL, "ZNE::extrapolate: observable returned a non-finite value");
            const double d = vals[t] - mean;
            mean += d / (double)(t + 1);
            m2 += d * (vals[t] - mean);
        }
        double se = 0.0;
        if (nt > 1) se = std::sqrt(std::max(0.0, m2 / (double)(nt - 1)) / (double)nt);
        else if (noisy) se = std::nan("");
        r.scales[k] = scales[k];
        r.values[k] = mean;
        r.std_errors[k] = se;
    }
    if (rc) return rc;
    double var = 0.0;
    for (int k = 0; k < nscales; ++k) {
        r.value += r.weights[k] * r.values[k];
        var += r.weights[k] * r.weights[k] * r.std_errors[k] * r.std_errors[k];
    }
    r.std_error = std::sqrt(var);
    *out = r;
    return LLG_OK;
}

int llg_traj_launch(llg_traj* h, uint64_t seed, uint64_t traj_begin, uint64_t n_traj, double* z0_out, uint32_t* jumps_out,
                    double* min_margin) {
    if (!h) return set_error(LLG_EINVAL, "traj_launch: NULL handle");
    if (n_traj > h->max_traj) return set_error(LLG_EINVAL, "traj_launch: n_traj exceeds the handle's max_traj");
    if (n_traj == 0) return LLG_OK;
    int rc = replay(h, seed, traj_begin, n_traj, nullptr, 0);
    if (rc) return rc;
    return collect(h, n_traj, z0_out, jumps_out, min_margin);
}

int llg_traj_config(const llg_traj* h, int* cluster, int* cta_threads, int* grid, int64_t* sites) {
    if (!h) return set_error(LLG_EINVAL, "traj_config: NULL handle");
    if (cluster) *cluster = h->cl;
    if (cta_threads) *cta_threads = h->threads;
    if (grid) *grid = h->grid;
    if (sites) *sites = h->sites;
    return LLG_OK;
}

int llg_traj_stream(const llg_traj* h, void** out) {
    if (!h || !out) return set_error(LLG_EINVAL, "traj_stream: NULL argument");
    *out = h->stream;
    return LLG_OK;
}

int llg_traj_autotune(llg_traj* h, uint64_t sample_traj, llg_tune_result* out) {
    if (!h) return set_error(LLG_EINVAL, "traj_autotune: NULL handle");
    llg_tune_result res;
    std::memset(&res, 0, sizeof(res));
    const int cl0 = h->cl, th0 = h->threads;
    if (!tune_cache_get(h->shape_key, &res)) {
        const uint64_t sample = std::min<uint64_t>(h->max_traj, sample_traj > 0 ? sample_traj : 2ULL * (h->grid / h->cl));
        cudaEvent_t a = nullptr, b = nullptr;
        cudaError_t e = cudaEventCreate(&a);
        if (e == cudaSuccess) e = cudaEventCreate(&b);
        if (e != cudaSuccess) return cuda_fail(e, "traj autotune events");
        auto time_it = [&](double* ms) -> int {
            int rc = replay(h, 0, 0, sample, nullptr, 0);  // untimed
            if (rc) return rc;
            cudaError_t ee = cudaEventRecord(a, h->stream);
            if (ee == cudaSuccess) {
                rc = replay(h, 0, 0, sample, nullptr, 0);
                if (rc) return rc;
                ee = cudaEventRecord(b, h->stream);
            }
            if (ee == cudaSuccess) ee = cudaEventSynchronize(b);
            float t = 0.f;
            if (ee == cudaSuccess) ee = cudaEventElapsedTime(&t, a, b);
            if (ee != cudaSuccess) return cuda_fail(ee, "traj autotune timing");
            *ms = t;
            return LLG_OK;
        };
        int rc = time_it(&res.default_ms);
        double best = 1e300;
        int best_cl = cl0, best_th = th0;
        for (int cl = 1; cl <= 2 && !rc; ++cl) {
            for (int th : {256, 512, 1024}) {
                size_t smem = 0;
                if (resolve_threads(h->n, h->P, cl, th, &smem) != th) continue;
                if (th > std::max(32, 1 << std::max(0, (cl == 2 ? h->n - 1 : h->n) - 1))) continue;
                rc = configure(h, cl, th);
                double ms = 0.0;
                if (!rc) rc = time_it(&ms);
                if (rc) break;
                ++res.candidates;
                if (ms < best) {
                    best = ms;
                    best_cl = cl;
                    best_th = th;
                    res.best_ms = ms;
                }
            }
        }
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        if (rc) {
            configure(h, cl0, th0);
            return rc;
        }
        res.cluster = best_cl;
        res.cta_threads = best_th;
        res.tile_qubits = h->cl == 2 ? h->n - 1 : h->n;
        res.fuse_mode = LLG_FUSE_TILE;
        tune_cache_put(h->shape_key, res);
    }
    int rc = configure(h, res.cluster, res.cta_threads);
    if (rc) return rc;
    res.tile_qubits = h->cl == 2 ? h->n - 1 : h->n;
    if (out) *out = res;
    return LLG_OK;
}

int llg_traj_run(int n, const llg_op* ops, int nops, double gamma_ad, double lambda_pd, uint64_t seed, uint64_t traj_begin,
                 uint64_t n_traj, int precision, double* z0_out, uint32_t* jumps_out, uint8_t* jump_log, int64_t log_stride,
                 double* min_margin) {
    if (!z0_out) return set_error(LLG_EINVAL, "traj_run: NULL argument");
    if (n_traj == 0) {
        // validate the arguments all the same
        llg_traj* h = nullptr;
        int rc = llg_traj_create(n, ops, nops, gamma_ad, lambda_pd, precision, 1, 0, 0, &h);
        llg_traj_destroy(h);
        return rc;
    }
    llg_traj* h = nullptr;
    int rc = llg_traj_create(n, ops, nops, gamma_ad, lambda_pd, precision, n_traj, 0, 0, &h);
    if (rc) return rc;
    uint8_t* d_log = nullptr;
    if (jump_log && log_stride < h->sites) rc = set_error(LLG_EINVAL, "traj_run: log_stride smaller than the site count");
    if (!rc && jump_log) {
        cudaError_t e = cudaMalloc(&d_log, n_traj * (size_t)log_stride);
        if (e != cudaSuccess) rc = cuda_fail(e, "cudaMalloc(jump log)");
    }
    if (!rc) rc = replay(h, seed, traj_begin, n_traj, d_log, jump_log ? log_stride : 0);
    if (!rc && jump_log) {
        cudaError_t e = cudaMemcpyAsync(jump_log, d_log, n_traj * (size_t)log_stride, cudaMemcpyDefault, h->stream);
        if (e != cudaSuccess) rc = cuda_fail(e, "jump log copy");
    }
    if (!rc) rc = collect(h, n_traj, z0_out, jumps_out, min_margin);
    if (d_log) {
        cudaStreamSynchronize(h->stream);
        cudaFree(d_log);
    }
    llg_traj_destroy(h);
    return rc;
}

}  // extern "C"
