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
    void* args[] = {&n, &h->d_gates, &ngates, &h->kp, &b0, &c0, &h->d_z0, &h->d_jumps, &lg, &ls, &h->d_margin};
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
    void* args[] = {&n, &h->d_gates, &ngates, &kp, &begin, &count, &h->d_z0, &h->d_jumps, &d_log, &log_stride, &h->d_margin};
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
            if (__builtin_popcountll(o.mask) > 6) return set_error(LLG_EINVAL, "traj_run: mcz on more than 6 qubits");
            for (int q = 0; q < n && g.nt < 6; ++q)
                if ((o.mask >> q) & 1) g.q[g.nt++] = q;
        } else {
            g.nt = 1;
            g.q[0] = o.q0;
        }
        sites += g.nt;
        gates.push_back(g);
    }
    llg_traj* h = new llg_traj();
    h->n = n;
    h->P = precision;
    h->ngates = (int)gates.size();
    h->sites = sites;
    h->max_traj = max_traj;
    h->kp.gamma = gamma_ad;
    h->kp.lambda = lambda_pd;
    h->kp.sq1mg = std::sqrt(1.0 - gamma_ad);
    h->kp.sq1ml = std::sqrt(1.0 - lambda_pd);
    h->kp.seed = 0;
    h->shape_key = tune_hash_ops(tune_hash(tune_hash(1469598103934665603ULL, 0x54524a), (uint64_t)n << 8 | (uint64_t)precision),
                                 ops, nops);
    int rc = LLG_OK;
    cudaError_t e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&h->d_gates, std::max<size_t>(gates.size(), 1) * sizeof(TrajGate));
    if (e == cudaSuccess) e = cudaMalloc(&h->d_z0, max_traj * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&h->d_jumps, max_traj * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMalloc(&h->d_margin, kMaxGrid * sizeof(double));
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
