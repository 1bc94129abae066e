// llg_common_host.h -- host-side helpers shared by the planner and the engine (no CUDA types).
#pragma once

#include <cstdint>
#include <cstring>

namespace llg {

// Split a double into an fp32 pair with hi + lo == x to ~48 bits (hi = RN(x), lo = RN(x - hi)).
inline void split_double(double x, float* hi, float* lo) {
    const float h = (float)x;
    *hi = h;
    *lo = (float)(x - (double)h);
}

// Gate coefficients travel to the kernels as 64-bit slots: a double (LLG_F64), an fp32 in the
// low word (LLG_F32), or an fp32 hi/lo pair (LLG_DF64, hi in the low word).
inline uint64_t pack_coef(int precision, double x) {
    uint64_t out = 0;
    if (precision == 0) {
        std::memcpy(&out, &x, 8);
    } else if (precision == 2) {
        const float f = (float)x;
        uint32_t b;
        std::memcpy(&b, &f, 4);
        out = b;
    } else {
        float h, l;
        split_double(x, &h, &l);
        uint32_t bh, bl;
        std::memcpy(&bh, &h, 4);
        std::memcpy(&bl, &l, 4);
        out = (uint64_t)bh | ((uint64_t)bl << 32);
    }
    return out;
}

inline int popcount64(uint64_t x) { return __builtin_popcountll(x); }

}  // namespace llg
