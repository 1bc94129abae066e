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
    __device__ __forceinline__ void apply(C& a0, C& a1) const {
        const auto x0 = a0.re, y0 = a0.im, x1 = a1.re, y1 = a1.im;
        if (KIND == EX_U2) {
            // k[0] = g00r, k[1] = -g00i, k[2] = g01r, k[3] = -g01i, ...
            a0.re = P::lin4(k[0], x0, k[1], y0, k[2], x1, k[3], y1);
            a0.im = P::lin4(k[0], y0, P::kneg(k[1]), x0, k[2], y1, P::kneg(k[3]), x1);
            a1.re = P::lin4(k[4], x0, k[5], y0, k[6], x1, k[7], y1);
            a1.im = P::lin4(k[4], y0, P::kneg(k[5]), x0, k[6], y1, P::kneg(k[7]), x1);
        } else if (KIND == EX_RX) {  // [c, -is; -is, c]
            const auto c = k[0], s = k[1], ms = P::kneg(k[1]);
            a0.re = P::lin2(c, x0, s, y1);
            a0.im = P::lin2(c, y0, ms, x1);
            a1.re = P::lin2(s, y0, c, x1);
            a1.im = P::lin2(ms, x0, c, y1);
        } else if (KIND == EX_RY) {  // [c, -s; s, c]
            const auto c = k[0], s = k[1], ms = P::kneg(k[1]);
            a0.re = P::lin2(c, x0, ms, x1);
            a0.im = P::lin2(c, y0, ms, y1);
            a1.re = P::lin2(s, x0, c, x1);
            a1.im = P::lin2(s, y0, c, y1);
        } else if (KIND == EX_H) {  // r [1, 1; 1, -1]
            const auto r = k[0], mr = P::kneg(k[0]);
            a0.re = P::lin2(r, x0, r, x1);
            a0.im = P::lin2(r, y0, r, y1);
            a1.re = P::lin2(r, x0, mr, x1);
            a1.im = P::lin2(r, y0, mr, y1);
        } else {  // EX_X
            const C t = a0;
            a0 = a1;
            a1 = t;
        }
    }
};

// a <- d * a for a complex constant d = (dr, di)
template <class P>
__device__ __forceinline__ void cmul_const(typename P::C& a, typename P::K dr, typename P::K di, typename P::K mdi) {
    const auto x = a.re, y = a.im;
    a.re = P::lin2(dr, x, mdi, y);
    a.im = P::lin2(dr, y, di, x);
}

// Apply a pair op over the 2^t-amplitude shared-memory tile (pairs along local qubit q).
template <class P, int KIND>
__device__ __forceinline__ void tile_pairs(typename P::S* tile, uint32_t npairs, int q, const ExecOp& o) {
    const PairMath<P, KIND> m(o);
    const uint32_t bit = 1u << q;
    for (uint32_t p = threadIdx.x; p < npairs; p += blockDim.x) {
        const uint32_t j0 = (uint32_t)insert0(p, q), j1 = j0 | bit;
        auto a0 = P::load(tile[j0]);
        auto a1 = P::load(tile[j1]);
        m.apply(a0, a1);
        tile[j0] = P::store(a0);
        tile[j1] = P::store(a1);
    }
}


}  // namespace llg
