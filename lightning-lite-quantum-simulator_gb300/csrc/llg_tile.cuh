// llg_tile.cuh -- per-pair gate math and shared-memory helpers used by every kernel family
// (single-state streaming and tile passes, batched forward/adjoint passes).
#pragma once

#include "llg_common.cuh"
#include "llg_internal.h"

namespace llg {

// ------------------------------------------------------------------------------------------
// the per-pair / per-amplitude math, shared by streaming and tile kernels
// ------------------------------------------------------------------------------------------
template <class P, int KIND>
struct PairMath {
    using K = typename P::K;
    using C = typename P::C;
    K k[8];
    __device__ explicit PairMath(const ExecOp& o) {
#pragma unroll
        for (int i = 0; i < 8; ++i) k[i] = P::k_from_bits(o.c[i]);
        if (KIND == EX_U2) {
            // pre-negate the imaginary parts used with a minus sign
            k[1] = P::kneg(k[1]);  // -g00i  (re rows use -gi)
            k[3] = P::kneg(k[3]);
            k[5] = P::kneg(k[5]);
            k[7] = P::kneg(k[7]);
        }
    }
    // Results are stored unnormalised (the _raw double-float forms; the same values, lo in full).
    __device__ __forceinline__ void apply(C& a0, C& a1) const {
        const auto x0 = a0.re, y0 = a0.im, x1 = a1.re, y1 = a1.im;
        if (KIND == EX_U2) {
            // k[0] = g00r, k[1] = -g00i, k[2] = g01r, k[3] = -g01i, ...
            a0.re = P::lin4_raw(k[0], x0, k[1], y0, k[2], x1, k[3], y1);
            a0.im = P::lin4_raw(k[0], y0, P::kneg(k[1]), x0, k[2], y1, P::kneg(k[3]), x1);
            a1.re = P::lin4_raw(k[4], x0, k[5], y0, k[6], x1, k[7], y1);
            a1.im = P::lin4_raw(k[4], y0, P::kneg(k[5]), x0, k[6], y1, P::kneg(k[7]), x1);
        } else if (KIND == EX_RX) {  // [c, -is; -is, c]
            const auto c = k[0], s = k[1], ms = P::kneg(k[1]);
            a0.re = P::lin2_raw(c, x0, s, y1);
            a0.im = P::lin2_raw(c, y0, ms, x1);
            a1.re = P::lin2_raw(s, y0, c, x1);
            a1.im = P::lin2_raw(ms, x0, c, y1);
        } else if (KIND == EX_RY) {  // [c, -s; s, c]
            const auto c = k[0], s = k[1], ms = P::kneg(k[1]);
            a0.re = P::lin2_raw(c, x0, ms, x1);
            a0.im = P::lin2_raw(c, y0, ms, y1);
            a1.re = P::lin2_raw(s, x0, c, x1);
            a1.im = P::lin2_raw(s, y0, c, y1);
        } else if (KIND == EX_ZYZ) {  // diag(1, ea) [c, -s; s, c] diag(1, eg)
            const auto gr = k[0], gi = k[1], c = k[2], s = k[3], ar = k[4], ai = k[5];
            const auto tr = P::lin2_raw(gr, x1, P::kneg(gi), y1);  // eg * a1
            const auto ti = P::lin2_raw(gr, y1, gi, x1);
            a0.re = P::lin2_raw(c, x0, P::kneg(s), tr);
            a0.im = P::lin2_raw(c, y0, P::kneg(s), ti);
            const auto ur = P::lin2_raw(s, x0, c, tr);
            const auto ui = P::lin2_raw(s, y0, c, ti);
            a1.re = P::lin2_raw(ar, ur, P::kneg(ai), ui);  // ea * u
            a1.im = P::lin2_raw(ar, ui, ai, ur);
        } else if (KIND == EX_ZY) {  // [c, -s; s, c] diag(1, eg)
            const auto gr = k[0], gi = k[1], c = k[2], s = k[3];
            const auto tr = P::lin2_raw(gr, x1, P::kneg(gi), y1);  // eg * a1
            const auto ti = P::lin2_raw(gr, y1, gi, x1);
            a0.re = P::lin2_raw(c, x0, P::kneg(s), tr);
            a0.im = P::lin2_raw(c, y0, P::kneg(s), ti);
            a1.re = P::lin2_raw(s, x0, c, tr);
            a1.im = P::lin2_raw(s, y0, c, ti);
        } else if (KIND == EX_ZT) {  // [1, -t; t, 1] diag(1, eg)
            const auto gr = k[0], gi = k[1], t = k[2];
            const auto zr = P::lin2_raw(gr, x1, P::kneg(gi), y1);  // z = eg * a1
            const auto zi = P::lin2_raw(gr, y1, gi, x1);
            a0.re = P::fma1_raw(P::kneg(t), zr, x0);
            a0.im = P::fma1_raw(P::kneg(t), zi, y0);
            a1.re = P::fma1_raw(t, x0, zr);
            a1.im = P::fma1_raw(t, y0, zi);
        } else if (KIND == EX_ZC) {  // [u, -1; 1, u] diag(1, eg)
            const auto gr = k[0], gi = k[1], u = k[2];
            const auto zr = P::lin2_raw(gr, x1, P::kneg(gi), y1);
            const auto zi = P::lin2_raw(gr, y1, gi, x1);
            a0.re = P::fma1_raw(u, x0, P::neg(zr));
            a0.im = P::fma1_raw(u, y0, P::neg(zi));
            a1.re = P::fma1_raw(u, zr, x0);
            a1.im = P::fma1_raw(u, zi, y0);
        } else if (KIND == EX_RT) {  // [1, -t; t, 1] (input phase applied by a phase table)
            const auto t = k[2], mt = P::kneg(k[2]);
            a0.re = P::fma1_raw(mt, x1, x0);
            a0.im = P::fma1_raw(mt, y1, y0);
            a1.re = P::fma1_raw(t, x0, x1);
            a1.im = P::fma1_raw(t, y0, y1);
        } else if (KIND == EX_RC) {  // [u, -1; 1, u]
            const auto u = k[2];
            a0.re = P::fma1_raw(u, x0, P::neg(x1));
            a0.im = P::fma1_raw(u, y0, P::neg(y1));
            a1.re = P::fma1_raw(u, x1, x0);
            a1.im = P::fma1_raw(u, y1, y0);
        } else if (KIND == EX_RXT) {  // [1, -it; -it, 1]
            const auto t = k[2], mt = P::kneg(k[2]);
            a0.re = P::fma1_raw(t, y1, x0);
            a0.im = P::fma1_raw(mt, x1, y0);
            a1.re = P::fma1_raw(t, y0, x1);
            a1.im = P::fma1_raw(mt, x0, y1);
        } else if (KIND == EX_RXC) {  // [u, -i; -i, u]
            const auto u = k[2];
            a0.re = P::fma1_raw(u, x0, y1);
            a0.im = P::fma1_raw(u, y0, P::neg(x1));
            a1.re = P::fma1_raw(u, x1, y0);
            a1.im = P::fma1_raw(u, y1, P::neg(x0));
        } else if (KIND == EX_ZTZ) {  // diag(1, ea) [1, -t; t, 1] diag(1, eg)
            const auto gr = k[0], gi = k[1], t = k[2], mt = P::kneg(k[2]), ar = k[4], ai = k[5];
            const auto zr = P::lin2_raw(gr, x1, P::kneg(gi), y1);  // z = eg a1
            const auto zi = P::lin2_raw(gr, y1, gi, x1);
            a0.re = P::fma1_raw(mt, zr, x0);
            a0.im = P::fma1_raw(mt, zi, y0);
            const auto ur = P::fma1_raw(t, x0, zr);
            const auto ui = P::fma1_raw(t, y0, zi);
            a1.re = P::lin2_raw(ar, ur, P::kneg(ai), ui);  // ea u
            a1.im = P::lin2_raw(ar, ui, ai, ur);
        } else if (KIND == EX_ZCZ) {  // diag(1, ea) [u, -1; 1, u] diag(1, eg)
            const auto gr = k[0], gi = k[1], u = k[2], ar = k[4], ai = k[5];
            const auto zr = P::lin2_raw(gr, x1, P::kneg(gi), y1);
            const auto zi = P::lin2_raw(gr, y1, gi, x1);
            a0.re = P::fma1_raw(u, x0, P::neg(zr));
            a0.im = P::fma1_raw(u, y0, P::neg(zi));
            const auto vr = P::fma1_raw(u, zr, x0);
            const auto vi = P::fma1_raw(u, zi, y0);
            a1.re = P::lin2_raw(ar, vr, P::kneg(ai), vi);
            a1.im = P::lin2_raw(ar, vi, ai, vr);
        } else if (KIND == EX_HS) {  // [1, 1; 1, -1]
            a0.re = P::add(x0, x1);
            a0.im = P::add(y0, y1);
            a1.re = P::sub(x0, x1);
            a1.im = P::sub(y0, y1);
        } else if (KIND == EX_H) {  // r [1, 1; 1, -1]
            const auto r = k[0], mr = P::kneg(k[0]);
            a0.re = P::lin2_raw(r, x0, r, x1);
            a0.im = P::lin2_raw(r, y0, r, y1);
            a1.re = P::lin2_raw(r, x0, mr, x1);
            a1.im = P::lin2_raw(r, y0, mr, y1);
        } else {  // EX_X
            const C t = a0;
            a0 = a1;
            a1 = t;
        }
    }
};

// a <- d * a for a complex constant d = (dr, di), stored unnormalised
template <class P>
__device__ __forceinline__ void cmul_const(typename P::C& a, typename P::K dr, typename P::K di, typename P::K mdi) {
    const auto x = a.re, y = a.im;
    a.re = P::lin2_raw(dr, x, mdi, y);
    a.im = P::lin2_raw(dr, y, di, x);
}

// Apply a pair op over the 2^t-amplitude shared-memory tile (pairs along local qubit q).
template <class P, int KIND>
__device__ __forceinline__ void tile_pairs(typename P::S* tile, uint32_t npairs, int q, const ExecOp& o) {
    const PairMath<P, KIND> m(o);
    const uint32_t bit = 1u << q;
    for (uint32_t p = threadIdx.x; p < npairs; p += blockDim.x) {
        const uint32_t j0 = ins0(p, bit), j1 = j0 | bit;
        auto a0 = P::load(tile[j0]);
        auto a1 = P::load(tile[j1]);
        m.apply(a0, a1);
        tile[j0] = P::store(a0);
        tile[j1] = P::store(a1);
    }
}


// diag(1, ph) on tile qubit q (or on the tile-uniform global qubit q when it is not local)
template <class P>
__device__ __forceinline__ void tile_phase1(typename P::S* tile, uint32_t tsize, uint64_t base, const ExecOp& o) {
    using K = typename P::K;
    const K pr = P::k_from_bits(o.c[0]), pi = P::k_from_bits(o.c[1]), mpi = P::kneg(pi);
    if (o.flags & OPF_NONLOCAL_Q0) {
        if ((base >> o.q0) & 1)
            for (uint32_t l = threadIdx.x; l < tsize; l += blockDim.x) {
                auto a = P::load(tile[l]);
                cmul_const<P>(a, pr, pi, mpi);
                tile[l] = P::store(a);
            }
        return;
    }
    const uint32_t bit = 1u << o.q0;
    for (uint32_t p = threadIdx.x; p < (tsize >> 1); p += blockDim.x) {
        const uint32_t j = ins0(p, bit) | bit;
        auto a = P::load(tile[j]);
        cmul_const<P>(a, pr, pi, mpi);
        tile[j] = P::store(a);
    }
}

// EX_PTAB: every amplitude l of the tile times the phase-table entry T[l] (the table starts at
// entry o.mask of `tables`; two coefficient slots (re, im) per entry, read through the L2 cache)
template <class P>
__device__ __forceinline__ void tile_ptab(typename P::S* tile, uint32_t tsize, const ExecOp& o,
                                          const uint64_t* __restrict__ tables) {
    using K = typename P::K;
    const ulonglong2* tb = reinterpret_cast<const ulonglong2*>(tables) + o.mask;
    for (uint32_t l = threadIdx.x; l < tsize; l += blockDim.x) {
        const ulonglong2 w = __ldg(tb + l);
        const K tr = P::k_from_bits(w.x), ti = P::k_from_bits(w.y);
        auto a = P::load(tile[l]);
        cmul_const<P>(a, tr, ti, P::kneg(ti));
        tile[l] = P::store(a);
    }
}

// CNOT (control q0, possibly a tile-uniform global qubit; target q1 local); with OPF_PHASE the
// amplitudes that end with control = target = 1 are then multiplied by c[0] + i c[1]
template <class P>
__device__ __forceinline__ void tile_cnot(typename P::S* tile, uint32_t tsize, uint64_t base, const ExecOp& o) {
    using K = typename P::K;
    using S = typename P::S;
    const int tq = o.q1;
    const bool phased = (o.flags & OPF_PHASE) != 0;
    const K pr = P::k_from_bits(o.c[0]), pi = P::k_from_bits(o.c[1]), mpi = P::kneg(pi);
    if (o.flags & OPF_NONLOCAL_Q0) {
        if (!((base >> o.q0) & 1)) return;
        const uint32_t tbit = 1u << tq;
        for (uint32_t p = threadIdx.x; p < (tsize >> 1); p += blockDim.x) {
            const uint32_t j0 = ins0(p, tbit), j1 = j0 | tbit;
            const S x = tile[j0];
            tile[j0] = tile[j1];
            if (phased) {
                auto a = P::load(x);
                cmul_const<P>(a, pr, pi, mpi);
                tile[j1] = P::store(a);
            } else {
                tile[j1] = x;
            }
        }
        return;
    }
    const int c = o.q0;
    const int lo = c < tq ? c : tq, hi = c < tq ? tq : c;
    const uint32_t cbit = 1u << c, tbit = 1u << tq;
    for (uint32_t r = threadIdx.x; r < (tsize >> 2); r += blockDim.x) {
        const uint32_t j = ins0(ins0(r, 1u << lo), 1u << hi) | cbit;
        const S x = tile[j];
        tile[j] = tile[j | tbit];
        if (phased) {
            auto a = P::load(x);
            cmul_const<P>(a, pr, pi, mpi);
            tile[j | tbit] = P::store(a);
        } else {
            tile[j | tbit] = x;
        }
    }
}

// ------------------------------------------------------------------------------------------
// one op on a shared-memory tile (all kinds, parametrised ones read their table row)
// ------------------------------------------------------------------------------------------
template <class P>
__device__ void tile_apply(typename P::S* tile, uint32_t tsize, uint64_t base, const ExecOp& o,
                           const uint64_t* __restrict__ trow, const uint64_t* __restrict__ tables = nullptr) {
    using K = typename P::K;
    using S = typename P::S;
    switch (o.kind) {
        case EX_U2: tile_pairs<P, EX_U2>(tile, tsize >> 1, o.q0, o); break;
        case EX_ZYZ: tile_pairs<P, EX_ZYZ>(tile, tsize >> 1, o.q0, o); break;
        case EX_ZY: tile_pairs<P, EX_ZY>(tile, tsize >> 1, o.q0, o); break;
        case EX_ZT: tile_pairs<P, EX_ZT>(tile, tsize >> 1, o.q0, o); break;
        case EX_ZC: tile_pairs<P, EX_ZC>(tile, tsize >> 1, o.q0, o); break;
        case EX_RT: tile_pairs<P, EX_RT>(tile, tsize >> 1, o.q0, o); break;
        case EX_RC: tile_pairs<P, EX_RC>(tile, tsize >> 1, o.q0, o); break;
        case EX_PTAB:  // plans with phase tables run only where the kernel passes them
            if (tables) tile_ptab<P>(tile, tsize, o, tables);
            break;
        case EX_PHASE1: tile_phase1<P>(tile, tsize, base, o); break;
        case EX_RX: tile_pairs<P, EX_RX>(tile, tsize >> 1, o.q0, o); break;
        case EX_RY: tile_pairs<P, EX_RY>(tile, tsize >> 1, o.q0, o); break;
        case EX_H: tile_pairs<P, EX_H>(tile, tsize >> 1, o.q0, o); break;
        case EX_X: tile_pairs<P, EX_X>(tile, tsize >> 1, o.q0, o); break;
        case EX_RX_P:
        case EX_RY_P: {  // (the adjoint kernels run IEEE complex128 occurrences in scale-free form)
            ExecOp r = o;
            r.c[0] = trow[2 * o.q1];
            const K s = P::k_from_bits(trow[2 * o.q1 + 1]);
            K sv = (o.flags & OPF_ADJOINT) ? P::kneg(s) : s;
            // re-pack the (possibly negated) sine through a local copy of the op
            if (o.kind == EX_RX_P) {
                PairMath<P, EX_RX> m(r);
                m.k[1] = sv;
                const uint32_t bit = 1u << o.q0;
                for (uint32_t p = threadIdx.x; p < (tsize >> 1); p += blockDim.x) {
                    const uint32_t j0 = ins0(p, bit), j1 = j0 | bit;
                    auto a0 = P::load(tile[j0]);
                    auto a1 = P::load(tile[j1]);
                    m.apply(a0, a1);
                    tile[j0] = P::store(a0);
                    tile[j1] = P::store(a1);
                }
            } else {
                PairMath<P, EX_RY> m(r);
                m.k[1] = sv;
                const uint32_t bit = 1u << o.q0;
                for (uint32_t p = threadIdx.x; p < (tsize >> 1); p += blockDim.x) {
                    const uint32_t j0 = ins0(p, bit), j1 = j0 | bit;
                    auto a0 = P::load(tile[j0]);
                    auto a1 = P::load(tile[j1]);
                    m.apply(a0, a1);
                    tile[j0] = P::store(a0);
                    tile[j1] = P::store(a1);
                }
            }
            break;
        }
        case EX_RZ_P: {
            // RZ(t) up to its global phase e^{-it/2}: diag(1, e^{it}), the table row holding
            // (cos t, sin t); the inverse conjugates
            const K pr = P::k_from_bits(trow[2 * o.q1]);
            K pi = P::k_from_bits(trow[2 * o.q1 + 1]);
            if (o.flags & OPF_ADJOINT) pi = P::kneg(pi);
            const K mpi = P::kneg(pi);
            if (o.flags & OPF_NONLOCAL_Q0) {
                if ((base >> o.q0) & 1)
                    for (uint32_t l = threadIdx.x; l < tsize; l += blockDim.x) {
                        auto a = P::load(tile[l]);
                        cmul_const<P>(a, pr, pi, mpi);
                        tile[l] = P::store(a);
                    }
            } else {
                const uint32_t bit = 1u << o.q0;
                for (uint32_t p = threadIdx.x; p < (tsize >> 1); p += blockDim.x) {
                    const uint32_t j = ins0(p, bit) | bit;
                    auto a = P::load(tile[j]);
                    cmul_const<P>(a, pr, pi, mpi);
                    tile[j] = P::store(a);
                }
            }
            break;
        }
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
                for (uint32_t l = threadIdx.x; l < tsize; l += blockDim.x) {
                    auto a = P::load(tile[l]);
                    if ((l >> o.q0) & 1) cmul_const<P>(a, d1r, d1i, md1i);
                    else cmul_const<P>(a, d0r, d0i, md0i);
                    tile[l] = P::store(a);
                }
            }
            break;
        }
        case EX_CNOT: tile_cnot<P>(tile, tsize, base, o); break;
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
}

}  // namespace llg
