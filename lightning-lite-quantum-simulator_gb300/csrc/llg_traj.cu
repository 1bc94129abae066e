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
// Every cluster barrier is executed unconditionally in the same sequence by both CTAs.
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
constexpr int kMaxPerThread = 16;  // amplitudes per thread in a cross-CTA step (2^14 / 1024)
constexpr int kMaxGrid = 4096;     // persistent CTAs at most (per-CTA margin slots)

// one gate of a trajectory circuit: the executor op (global qubits) and the touched qubits
struct TrajGate {
    ExecOp op;
    int32_t nt;
    int32_t q[6];
    int32_t pad;
};

struct KrausParams {
    double gamma, lambda;
    double sq1mg, sq1ml;  // sqrt(1 - gamma), sqrt(1 - lambda)
    uint64_t seed;
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

template <class P>
__device__ __forceinline__ uint64_t packk(double x) {
    if (P::kPrecision == 0) return (uint64_t)__double_as_longlong(x);
    if (P::kPrecision == 2) return (uint64_t)__float_as_uint(__double2float_rn(x));
    const df d = double_to_df(x);
    return (uint64_t)__float_as_uint(d.hi) | ((uint64_t)__float_as_uint(d.lo) << 32);
}

// shared decision record written by thread 0
struct Decision {
    uint64_t f_ad0, f_ad1, f_pd0, f_pd1;  // packed scale factors
    int ad_jump, pd_jump;
    double p1;
};

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
            group_sync<CL>();
            return;
        }
        const PairMath<P, KIND> m(o);
        C out[kMaxPerThread];
        int cnt = 0;
        for (uint32_t l = threadIdx.x; l < NL; l += blockDim.x, ++cnt) {
            C mine = P::load(s[l]), other = P::load(remote[l]);
            C a0 = rank ? other : mine, a1 = rank ? mine : other;
            m.apply(a0, a1);
            out[cnt] = rank ? a1 : a0;
        }
        group_sync<CL>();  // the partner has read this CTA's half
        cnt = 0;
        for (uint32_t l = threadIdx.x; l < NL; l += blockDim.x, ++cnt) s[l] = P::store(out[cnt]);
        group_sync<CL>();
    }

    __device__ void gate(const ExecOp& o) {
        switch (o.kind) {
            case EX_U2: pair_gate<EX_U2>(o.q0, o); break;
            case EX_RX: pair_gate<EX_RX>(o.q0, o); break;
            case EX_RY: pair_gate<EX_RY>(o.q0, o); break;
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
                group_sync<CL>();
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
                            const uint32_t j = (uint32_t)insert0(insert0(r, lo), hi) | cbit;
                            const S x = s[j];
                            s[j] = s[j | tbit];
                            s[j | tbit] = x;
                        }
                    }
                    group_sync<CL>();
                } else {  // target is the top qubit: swap the control = 1 halves across the CTAs
                    S out[kMaxPerThread];
                    int cnt = 0;
                    for (uint32_t l = threadIdx.x; l < NL; l += blockDim.x, ++cnt) out[cnt] = ((l >> c) & 1) ? remote[l] : s[l];
                    group_sync<CL>();
                    cnt = 0;
                    for (uint32_t l = threadIdx.x; l < NL; l += blockDim.x, ++cnt) s[l] = out[cnt];
                    group_sync<CL>();
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
                group_sync<CL>();
                break;
            }
            default: group_sync<CL>(); break;
        }
    }

    // sum over the group of |a|^2 for amplitudes with (global bit q) == 1 (q < 0: all), or of
    // (1 - 2 bit0)|a|^2 when z0 is set; identical in every CTA of the group
    __device__ double reduce(int q, bool z0, typename P::Acc* red, typename P::Acc* slot) {
        typename P::Acc pos = P::acc_zero(), neg = P::acc_zero();
        for (uint32_t l = threadIdx.x; l < NL; l += blockDim.x) {
            const auto a = P::load(s[l]);
            if (z0) {
                if (l & 1) neg = P::acc_norm(neg, a);
                else pos = P::acc_norm(pos, a);
            } else {
                const int bit = cross(q) ? rank : (int)((l >> q) & 1);
                if (bit) pos = P::acc_norm(pos, a);
            }
        }
        using A = typename P::Acc;
        const A v = block_sum_acc(acc_minus(pos, neg), red);
        if (threadIdx.x == 0) *slot = v;
        group_sync<CL>();
        double total;
        if (CL == 1) {
            total = acc_value(*slot);
        } else {
            cg::cluster_group cl = cg::this_cluster();
            const A* s0 = cl.map_shared_rank(slot, 0);
            const A* s1 = cl.map_shared_rank(slot, 1);
            total = acc_value(acc_plus(*s0, *s1));  // the same order on both CTAs
        }
        return total;
    }

    // amplitude damping then phase damping on qubit q, decisions in *d (already filled)
    __device__ void kraus_apply(int q, const Decision* d) {
        const K fa0 = P::k_from_bits(d->f_ad0), fa1 = P::k_from_bits(d->f_ad1);
        const K fp0 = P::k_from_bits(d->f_pd0), fp1 = P::k_from_bits(d->f_pd1);
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
        if (!cross(q)) {
            const uint32_t bit = 1u << q;
            for (uint32_t p = threadIdx.x; p < (NL >> 1); p += blockDim.x) {
                const uint32_t j0 = (uint32_t)insert0(p, q), j1 = j0 | bit;
                C a0 = P::load(s[j0]), a1 = P::load(s[j1]);
                C t0, t1;
                if (adj) {
                    t0 = scale(a1, fa0);
                    t1 = zero();
                } else {
                    t0 = scale(a0, fa0);
                    t1 = scale(a1, fa1);
                }
                if (pdj) {
                    t0 = zero();
                    t1 = scale(t1, fp1);
                } else {
                    t0 = scale(t0, fp0);
                    t1 = scale(t1, fp1);
                }
                s[j0] = P::store(t0);
                s[j1] = P::store(t1);
            }
            group_sync<CL>();
            return;
        }
        // top qubit across the cluster: rank 0 holds the bit-0 half, rank 1 the bit-1 half
        C out[kMaxPerThread];
        int cnt = 0;
        for (uint32_t l = threadIdx.x; l < NL; l += blockDim.x, ++cnt) {
            C t;
            if (rank == 0) {
                t = adj ? scale(P::load(remote[l]), fa0) : scale(P::load(s[l]), fa0);
                t = pdj ? zero() : scale(t, fp0);
            } else {
                t = adj ? zero() : scale(P::load(s[l]), fa1);
                t = scale(t, fp1);
                if (pdj && adj) t = zero();
            }
            out[cnt] = t;
        }
        group_sync<CL>();
        cnt = 0;
        for (uint32_t l = threadIdx.x; l < NL; l += blockDim.x, ++cnt) s[l] = P::store(out[cnt]);
        group_sync<CL>();
    }
};

// thread 0: draw and decide one site pair (AD at `site`, PD at site + 1), as the oracle does
template <class P>
__device__ void decide(double P1, const KrausParams& kp, uint64_t traj, uint64_t site, Decision* d, double* min_margin) {
    // amplitude damping
    const double u1 = philox_u1(kp.seed, traj, site);
    double s_ad = 1.0 - kp.gamma * P1;
    const double tot_ad = kp.gamma * P1;
    double m = fabs(u1 - s_ad);
    if (m < *min_margin) *min_margin = m;
    double p1;
    if (u1 >= s_ad && tot_ad > 0.0) {
        d->ad_jump = 1;
        d->f_ad0 = packk<P>(1.0 / sqrt(P1));
        d->f_ad1 = packk<P>(0.0);
        p1 = 0.0;
    } else {
        d->ad_jump = 0;
        const double s0 = 1.0 / sqrt(s_ad);
        d->f_ad0 = packk<P>(s0);
        d->f_ad1 = packk<P>(kp.sq1mg * s0);
        p1 = (1.0 - kp.gamma) * P1 / s_ad;
    }
    // phase damping
    const double u2 = philox_u1(kp.seed, traj, site + 1);
    const double s_pd = 1.0 - kp.lambda * p1;
    const double tot_pd = kp.lambda * p1;
    m = fabs(u2 - s_pd);
    if (m < *min_margin) *min_margin = m;
    if (u2 >= s_pd && tot_pd > 0.0) {
        d->pd_jump = 1;
        d->f_pd0 = packk<P>(0.0);
        d->f_pd1 = packk<P>(1.0 / sqrt(p1));
    } else {
        d->pd_jump = 0;
        const double s0 = 1.0 / sqrt(s_pd);
        d->f_pd0 = packk<P>(s0);
        d->f_pd1 = packk<P>(kp.sq1ml * s0);
    }
    d->p1 = p1;
}

template <class P, int CL>
__device__ void traj_kernel_body(int n, const TrajGate* __restrict__ gates, int ngates, KrausParams kp, uint64_t traj_begin,
                                 uint64_t n_traj, double* __restrict__ z0_out, uint32_t* __restrict__ jumps_out,
                                 uint8_t* __restrict__ jump_log, int64_t log_stride, double* __restrict__ margin_out) {
    using S = typename P::S;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ typename P::Acc red[32];
    __shared__ typename P::Acc slot;
    __shared__ Decision dec;
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
        for (int g = 0; g < ngates; ++g) {
            const TrajGate& G = gates[g];
            T.gate(G.op);
            for (int k = 0; k < G.nt; ++k) {
                const int q = G.q[k];
                const double P1 = T.reduce(q, false, red, &slot);
                if (threadIdx.x == 0) decide<P>(P1, kp, traj, site, &dec, &min_margin);
                __syncthreads();
                const int code = dec.ad_jump | (dec.pd_jump << 1);
                T.kraus_apply(q, &dec);
                if (threadIdx.x == 0 && T.rank == 0 && jump_log)
                    jump_log[(int64_t)tt * log_stride + (int64_t)(site >> 1)] = (uint8_t)code;
                jumps += (code & 1) + (code >> 1);
                site += 2;
            }
        }
        const double z = T.reduce(0, true, red, &slot);
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
                                                        uint64_t traj_begin, uint64_t n_traj, double* z0, uint32_t* jumps,
                                                        uint8_t* log, int64_t log_stride, double* margins) {
    traj_kernel_body<P, 1>(n, gates, ngates, kp, traj_begin, n_traj, z0, jumps, log, log_stride, margins);
}

template <class P>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(kTrajThreads)
    k_traj2(int n, const TrajGate* gates, int ngates, KrausParams kp, uint64_t traj_begin, uint64_t n_traj, double* z0,
            uint32_t* jumps, uint8_t* log, int64_t log_stride, double* margins) {
    traj_kernel_body<P, 2>(n, gates, ngates, kp, traj_begin, n_traj, z0, jumps, log, log_stride, margins);
}

template <class P>
int launch_traj(int n, int cl, const TrajGate* d_gates, int ngates, const KrausParams& kp, uint64_t traj_begin,
                uint64_t n_traj, double* d_z0, uint32_t* d_jumps, uint8_t* d_log, int64_t log_stride, double* d_margin,
                int* grid_out, cudaStream_t s) {
    using S = typename P::S;
    const int nl = cl == 2 ? n - 1 : n;
    const size_t smem = ((size_t)1 << nl) * sizeof(S);
    const int threads = std::min(kTrajThreads, std::max(32, 1 << std::max(0, nl - 1)));
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaError_t e;
    int per_sm = 1;
    if (cl == 1) {
        e = cudaFuncSetAttribute(k_traj1<P>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_traj1<P>, threads, smem);
    } else {
        e = cudaFuncSetAttribute(k_traj2<P>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_traj2<P>, threads, smem);
    }
    if (e != cudaSuccess) return cuda_fail(e, "trajectory kernel attributes");
    per_sm = std::max(per_sm, 1);
    uint64_t groups = (uint64_t)sms * per_sm / cl;
    groups = std::max<uint64_t>(1, std::min<uint64_t>(groups, n_traj));
    groups = std::min<uint64_t>(groups, (uint64_t)(kMaxGrid / cl));  // margin buffer holds kMaxGrid CTAs
    const unsigned grid = (unsigned)(groups * cl);
    *grid_out = (int)grid;
    if (cl == 1)
        k_traj1<P><<<grid, threads, smem, s>>>(n, d_gates, ngates, kp, traj_begin, n_traj, d_z0, d_jumps, d_log, log_stride,
                                               d_margin);
    else
        k_traj2<P><<<grid, threads, smem, s>>>(n, d_gates, ngates, kp, traj_begin, n_traj, d_z0, d_jumps, d_log, log_stride,
                                               d_margin);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "trajectory kernel");
    return LLG_OK;
}

bool is_dev(const void* p) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

}  // namespace

extern "C" int llg_traj_run(int n, const llg_op* ops, int nops, double gamma_ad, double lambda_pd, uint64_t seed,
                            uint64_t traj_begin, uint64_t n_traj, int precision, double* z0_out, uint32_t* jumps_out,
                            uint8_t* jump_log, int64_t log_stride, double* min_margin) {
    if (n < 1 || n > 14) return set_error(LLG_EINVAL, "traj_run: n must be in [1, 14]");
    if (precision != LLG_F64 && precision != LLG_DF64 && precision != LLG_F32)
        return set_error(LLG_EINVAL, "traj_run: unknown precision");
    if (nops < 0 || (nops > 0 && !ops) || !z0_out) return set_error(LLG_EINVAL, "traj_run: NULL argument");
    if (!(gamma_ad >= 0.0 && gamma_ad <= 1.0) || !(lambda_pd >= 0.0 && lambda_pd <= 1.0))
        return set_error(LLG_EINVAL, "traj_run: gamma and lambda must be in [0, 1]");
    if (n_traj == 0) return LLG_OK;
    // lower the gates with global qubits and record the touched qubits of each
    std::vector<TrajGate> gates;
    gates.reserve(nops);
    int64_t sites = 0;
    for (int i = 0; i < nops; ++i) {
        const llg_op& o = ops[i];
        bool ok = o.q0 >= 0 && o.q0 < n;
        if (o.kind == LLG_OP_CNOT || o.kind == LLG_OP_CZ) ok = ok && o.q1 >= 0 && o.q1 < n && o.q1 != o.q0;
        if (o.kind == LLG_OP_MCZ) ok = o.mask != 0 && (o.mask >> n) == 0;
        if ((o.kind == LLG_OP_RX || o.kind == LLG_OP_RY || o.kind == LLG_OP_RZ) && !std::isfinite(o.theta)) ok = false;
        if (o.kind < 0 || o.kind > LLG_OP_U2) ok = false;
        if (!ok) return set_error(LLG_EINVAL, "traj_run: invalid op " + std::to_string(i));
        std::vector<ExecOp> lowered;
        std::string err;
        if (!lower_op(n, o, precision, lowered, err) || lowered.size() != 1) return set_error(LLG_EINVAL, "traj_run: " + err);
        TrajGate g;
        std::memset(&g, 0, sizeof(g));
        g.op = lowered[0];
        if (o.kind == LLG_OP_CNOT || o.kind == LLG_OP_CZ) {
            g.nt = 2;
            g.q[0] = o.q0;
            g.q[1] = o.q1;
        } else if (o.kind == LLG_OP_MCZ) {
            for (int q = 0; q < n && g.nt < 6; ++q)
                if ((o.mask >> q) & 1) g.q[g.nt++] = q;
            if (__builtin_popcountll(o.mask) > 6) return set_error(LLG_EINVAL, "traj_run: mcz on more than 6 qubits");
        } else {
            g.nt = 1;
            g.q[0] = o.q0;
        }
        sites += g.nt;
        gates.push_back(g);
    }
    if (jump_log && log_stride < sites) return set_error(LLG_EINVAL, "traj_run: log_stride smaller than the site count");
    const int cl = (precision != LLG_F32 && n == 14) ? 2 : 1;
    KrausParams kp;
    kp.gamma = gamma_ad;
    kp.lambda = lambda_pd;
    kp.sq1mg = std::sqrt(1.0 - gamma_ad);
    kp.sq1ml = std::sqrt(1.0 - lambda_pd);
    kp.seed = seed;

    TrajGate* d_gates = nullptr;
    double *d_z0 = nullptr, *d_margin = nullptr;
    uint32_t* d_jumps = nullptr;
    uint8_t* d_log = nullptr;
    cudaStream_t s = nullptr;
    int rc = LLG_OK;
    auto fail = [&](cudaError_t e, const char* what) {
        rc = cuda_fail(e, what);
    };
    cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (e) fail(e, "cudaStreamCreate");
    const bool z_dev = is_dev(z0_out);
    if (!rc && (e = cudaMalloc(&d_gates, std::max<size_t>(gates.size(), 1) * sizeof(TrajGate)))) fail(e, "cudaMalloc");
    if (!rc && !z_dev && (e = cudaMalloc(&d_z0, n_traj * sizeof(double)))) fail(e, "cudaMalloc");
    if (!rc && jumps_out && (e = cudaMalloc(&d_jumps, n_traj * sizeof(uint32_t)))) fail(e, "cudaMalloc");
    if (!rc && jump_log && (e = cudaMalloc(&d_log, n_traj * (size_t)log_stride))) fail(e, "cudaMalloc");
    if (!rc && (e = cudaMalloc(&d_margin, kMaxGrid * sizeof(double)))) fail(e, "cudaMalloc");
    if (!rc && !gates.empty() &&
        (e = cudaMemcpyAsync(d_gates, gates.data(), gates.size() * sizeof(TrajGate), cudaMemcpyHostToDevice, s)))
        fail(e, "gate upload");
    int grid = 0;
    if (!rc) {
        double* zt = z_dev ? z0_out : d_z0;
        switch (precision) {
            case LLG_F64:
                rc = launch_traj<PolF64>(n, cl, d_gates, (int)gates.size(), kp, traj_begin, n_traj, zt, d_jumps, d_log,
                                         log_stride, d_margin, &grid, s);
                break;
            case LLG_F32:
                rc = launch_traj<PolF32>(n, cl, d_gates, (int)gates.size(), kp, traj_begin, n_traj, zt, d_jumps, d_log,
                                         log_stride, d_margin, &grid, s);
                break;
            default:
                rc = launch_traj<PolDF64>(n, cl, d_gates, (int)gates.size(), kp, traj_begin, n_traj, zt, d_jumps, d_log,
                                          log_stride, d_margin, &grid, s);
        }
    }
    std::vector<double> margins;
    if (!rc && !z_dev && (e = cudaMemcpyAsync(z0_out, d_z0, n_traj * sizeof(double), cudaMemcpyDeviceToHost, s)))
        fail(e, "z0 copy");
    if (!rc && jumps_out &&
        (e = cudaMemcpyAsync(jumps_out, d_jumps, n_traj * sizeof(uint32_t),
                             is_dev(jumps_out) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, s)))
        fail(e, "jumps copy");
    if (!rc && jump_log &&
        (e = cudaMemcpyAsync(jump_log, d_log, n_traj * (size_t)log_stride,
                             is_dev(jump_log) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, s)))
        fail(e, "log copy");
    if (!rc && min_margin) {
        margins.resize(grid);
        if ((e = cudaMemcpyAsync(margins.data(), d_margin, grid * sizeof(double), cudaMemcpyDeviceToHost, s)))
            fail(e, "margin copy");
    }
    if (!rc && (e = cudaStreamSynchronize(s))) fail(e, "trajectory kernel");
    if (!rc && min_margin) {
        double m = 1.0;
        for (double v : margins) m = std::min(m, v);
        *min_margin = m;
    }
    cudaFree(d_gates);
    cudaFree(d_z0);
    cudaFree(d_jumps);
    cudaFree(d_log);
    cudaFree(d_margin);
    if (s) cudaStreamDestroy(s);
    return rc;
}
