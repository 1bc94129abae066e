// llg_tsolver.cu -- the dense trajectory solver on the GPU (include/llgpu.h, "dense trajectory
// solver" section): the reference's TrajectorySolver (src/TrajectorySolver.h) for the Lindblad
// equation with dense dim x dim operators (dim = 2^n <= 1024), thousands of trajectories in one
// persistent launch.
//
// Plan (host, once per run, src/TrajectorySolver.h:400-441): steps and h; jump operators
// J_k = sqrt(gamma) L, or sqrt(g) (1 - P) for Pauli-like channels under PROJECTOR; H_eff =
// H - i/2 sum J^+ J for the jump unravelings; a constant H gives one propagator exp(-i H_eff h)
// by scaling and squaring with an 18-term Taylor series (:95-110, evaluated by Paterson-Stockmeyer),
// a time-dependent H the RK4 nodes -i (H(t_j) + hnh).  The matrix products of the plan (powers,
// J^+ J, L^2) run on a tiled FP64 GEMM kernel.
//
// Trajectories (k_tsolve): one CTA per trajectory at a time (persistent over the trajectory
// range), the state and its work vectors in shared memory.  A matrix-vector product is one thread
// per row streaming the matrix column-major (coalesced, L2-resident across CTAs) against the
// vector broadcast from shared memory.  The matrices are stored and multiplied in double-float
// (rows accumulated with the Dot2 scheme on the FP32 pipe, ~2^-46 relative), states stay FP64:
// this GPU issues ~1.6 FP64 operations per clock per SM against ~115 FP32, and the FP64 product
// was FP64-bound.  Norm reductions are FP64 block sums.  Uniforms come from
// Philox4x32-10 (key = seed, counter = (draw, trajectory)): a jump step s uses draw s (u1, and
// u2 for the channel pick), a diffusive step channel k draw s * nch + k (Box-Muller).
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/llgpu.h"
#include "llg_common.cuh"

namespace llg {
int set_error(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);
}  // namespace llg

using namespace llg;
typedef std::complex<double> cd;

namespace {

constexpr int kTsMaxQubits = 10;
constexpr int kTsThreads = 256;

// ------------------------------------------------------------------------------------------
// plan-time dense algebra: C = op(A) B, row-major dim x dim, op = A or A^+
// ------------------------------------------------------------------------------------------
constexpr int kTile = 16;

__global__ void k_zgemm(const double2* __restrict__ a, const double2* __restrict__ b, double2* __restrict__ c, int d,
                        int adjoint_a) {
    __shared__ double2 ta[kTile][kTile + 1];
    __shared__ double2 tb[kTile][kTile + 1];
    const int row = blockIdx.y * kTile + threadIdx.y, col = blockIdx.x * kTile + threadIdx.x;
    double sr = 0.0, si = 0.0;
    for (int k0 = 0; k0 < d; k0 += kTile) {
        const int ka = k0 + threadIdx.x, kb = k0 + threadIdx.y;
        double2 va = make_double2(0.0, 0.0), vb = make_double2(0.0, 0.0);
        if (row < d && ka < d) {
            if (adjoint_a) {
                const double2 t = a[(size_t)ka * d + row];
                va = make_double2(t.x, -t.y);
            } else {
                va = a[(size_t)row * d + ka];
            }
        }
        if (kb < d && col < d) vb = b[(size_t)kb * d + col];
        ta[threadIdx.y][threadIdx.x] = va;
        tb[threadIdx.y][threadIdx.x] = vb;
        __syncthreads();
        for (int k = 0; k < kTile; ++k) {
            const double2 x = ta[threadIdx.y][k], y = tb[k][threadIdx.x];
            sr = fma(x.x, y.x, fma(-x.y, y.y, sr));
            si = fma(x.x, y.y, fma(x.y, y.x, si));
        }
        __syncthreads();
    }
    if (row < d && col < d) c[(size_t)row * d + col] = make_double2(sr, si);
}

// Host helper owning three device matrices for the plan products.
struct Gemm {
    int d = 0;
    double2 *a = nullptr, *b = nullptr, *c = nullptr;
    cudaStream_t s = nullptr;
    ~Gemm() {
        cudaFree(a);
        cudaFree(b);
        cudaFree(c);
    }
    cudaError_t init(int dim, cudaStream_t st) {
        d = dim;
        s = st;
        const size_t bytes = (size_t)d * d * sizeof(double2);
        cudaError_t e = cudaMalloc(&a, bytes);
        if (e == cudaSuccess) e = cudaMalloc(&b, bytes);
        if (e == cudaSuccess) e = cudaMalloc(&c, bytes);
        return e;
    }
    // out = op(x) y on device buffers of d x d row-major complex (out may not alias x or y)
    cudaError_t mul_dev(const double2* x, const double2* y, double2* out, bool adj_x) {
        const dim3 grid((d + kTile - 1) / kTile, (d + kTile - 1) / kTile), block(kTile, kTile);
        k_zgemm<<<grid, block, 0, s>>>(x, y, out, d, adj_x ? 1 : 0);
        return cudaGetLastError();
    }
    // out = op(x) y
    cudaError_t mul(const std::vector<cd>& x, const std::vector<cd>& y, std::vector<cd>& out, bool adj_x) {
        const size_t bytes = (size_t)d * d * sizeof(double2);
        cudaError_t e = cudaMemcpyAsync(a, x.data(), bytes, cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(b, y.data(), bytes, cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) return e;
        const dim3 grid((d + kTile - 1) / kTile, (d + kTile - 1) / kTile), block(kTile, kTile);
        k_zgemm<<<grid, block, 0, s>>>(a, b, c, d, adj_x ? 1 : 0);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        out.resize((size_t)d * d);
        e = cudaMemcpyAsync(out.data(), c, bytes, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        return e;
    }
};

double fro(const std::vector<cd>& m) {
    double s = 0.0;
    for (const cd& v : m) s += std::norm(v);
    return std::sqrt(s);
}

std::vector<cd> adjoint(const std::vector<cd>& m, int d) {
    std::vector<cd> r((size_t)d * d);
    for (int i = 0; i < d; ++i)
        for (int j = 0; j < d; ++j) r[(size_t)i * d + j] = std::conj(m[(size_t)j * d + i]);
    return r;
}

// acc[i] = (tmp ? tmp[i] : 0) + c0 [row == col] + c1 p1[i] + c2 p2[i] + c3 p3[i] over a d x d
// row-major matrix: one Paterson-Stockmeyer step of expm (FP64)
__global__ void k_ps_step(const double2* __restrict__ tmp, const double2* __restrict__ p1, const double2* __restrict__ p2,
                          const double2* __restrict__ p3, double2* __restrict__ acc, int d, double c0, double c1, double c2,
                          double c3) {
    const size_t count = (size_t)d * d, step = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += step) {
        double re = tmp ? tmp[i].x : 0.0, im = tmp ? tmp[i].y : 0.0;
        if (i / d == i % d) re += c0;
        re = fma(c1, p1[i].x, re);
        im = fma(c1, p1[i].y, im);
        re = fma(c2, p2[i].x, re);
        im = fma(c2, p2[i].y, im);
        re = fma(c3, p3[i].x, re);
        im = fma(c3, p3[i].y, im);
        acc[i] = make_double2(re, im);
    }
}

// exp(A) by the reference's scaling and squaring with an 18-term Taylor series
// (src/TrajectorySolver.h:95-110).  The degree-18 polynomial of B = A / 2^s is evaluated on the
// device by Paterson-Stockmeyer with blocks of four: B^2, B^3, B^4, then
//     p(B) = (((C_4 B^4 + C_3) B^4 + C_2) B^4 + C_1) B^4 + C_0,  C_j = sum_i B^i / (4j + i)!,
// 7 products instead of 18 (FP64 throughout; only the rounding order differs from term-by-term
// summation), then s squarings.  One copy in, one out.
cudaError_t expm(Gemm& g, const std::vector<cd>& a, std::vector<cd>& out) {
    const int d = g.d;
    double nrm = 0.0;
    for (int i = 0; i < d; ++i) {
        double row = 0.0;
        for (int j = 0; j < d; ++j) row += std::abs(a[(size_t)i * d + j]);
        nrm = std::max(nrm, row);
    }
    int s = 0;
    if (nrm > 0.5) s = std::max(0, (int)std::ceil(std::log2(nrm / 0.5)));
    const double scale = std::pow(2.0, s);
    const size_t count = (size_t)d * d, bytes = count * sizeof(double2);
    std::vector<cd> b(a.size());
    for (size_t i = 0; i < a.size(); ++i) b[i] = a[i] / scale;
    double coef[19];  // 1 / k!
    coef[0] = 1.0;
    for (int k = 1; k <= 18; ++k) coef[k] = coef[k - 1] / (double)k;
    double2 *p2 = nullptr, *p3 = nullptr, *p4 = nullptr, *acc = nullptr;
    cudaError_t e = cudaMalloc(&p2, bytes);
    if (e == cudaSuccess) e = cudaMalloc(&p3, bytes);
    if (e == cudaSuccess) e = cudaMalloc(&p4, bytes);
    if (e == cudaSuccess) e = cudaMalloc(&acc, bytes);
    double2* p1 = g.b;
    double2* tmp = g.c;
    if (e == cudaSuccess) e = cudaMemcpyAsync(p1, b.data(), bytes, cudaMemcpyHostToDevice, g.s);
    if (e == cudaSuccess) e = g.mul_dev(p1, p1, p2, false);
    if (e == cudaSuccess) e = g.mul_dev(p2, p1, p3, false);
    if (e == cudaSuccess) e = g.mul_dev(p2, p2, p4, false);
    const unsigned blocks = (unsigned)std::min<size_t>((count + 255) / 256, 4096);
    auto c = [&](int k) { return k <= 18 ? coef[k] : 0.0; };
    for (int j = 4; j >= 0 && e == cudaSuccess; --j) {
        if (j < 4) e = g.mul_dev(acc, p4, tmp, false);  // acc B^4
        if (e == cudaSuccess) {
            k_ps_step<<<blocks, 256, 0, g.s>>>(j < 4 ? tmp : nullptr, p1, p2, p3, acc, d, c(4 * j), c(4 * j + 1),
                                                c(4 * j + 2), c(4 * j + 3));
            e = cudaGetLastError();
        }
    }
    for (int i = 0; i < s && e == cudaSuccess; ++i) {
        e = g.mul_dev(acc, acc, tmp, false);
        if (e == cudaSuccess) e = cudaMemcpyAsync(acc, tmp, bytes, cudaMemcpyDeviceToDevice, g.s);
    }
    out.resize(count);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out.data(), acc, bytes, cudaMemcpyDeviceToHost, g.s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g.s);
    cudaFree(p2);
    cudaFree(p3);
    cudaFree(p4);
    cudaFree(acc);
    return e;
}

std::vector<cd> col_major(const std::vector<cd>& m, int d) {
    std::vector<cd> r((size_t)d * d);
    for (int i = 0; i < d; ++i)
        for (int j = 0; j < d; ++j) r[(size_t)j * d + i] = m[(size_t)i * d + j];
    return r;
}

// ------------------------------------------------------------------------------------------
// the trajectory kernel
// ------------------------------------------------------------------------------------------
struct TsParams {
    int32_t dim, nch, kind, constant;
    long long steps;
    double h;
    // matrices column-major, each entry double-float {re.hi, im.hi, re.lo, im.lo}
    const float4* prop;      // dim x dim
    const float4* nodes;     // n_nodes x dim x dim
    const float4* ops;       // nch x dim x dim
    const float4* ops_dop;   // nch x dim x dim (ANALOG)
    const double2* psi0;     // dim, normalised
    const float4* obs;       // dim x dim, or null
    uint64_t seed;
    uint64_t traj_begin, n_traj;
    double2* states;         // n_traj x dim, or null
    double* obs_out;         // n_traj, or null
    int* err;
};

__device__ __forceinline__ void philox_pair(uint64_t seed, uint64_t traj, uint64_t draw, double* u1, double* u2) {
    uint32_t c0 = (uint32_t)draw, c1 = (uint32_t)(draw >> 32), c2 = (uint32_t)traj, c3 = (uint32_t)(traj >> 32);
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

// y = A x, A column-major dim x dim in double-float; one thread per row.  x is converted to
// double-float into xs (shared memory, dim entries) first; each row's real and imaginary parts
// are Dot2 sums, converted to double once.
__device__ __forceinline__ void matvec(const float4* __restrict__ a, const double2* x, double2* y, int d, float4* xs) {
    for (int c = threadIdx.x; c < d; c += blockDim.x) {
        const df xr = double_to_df(x[c].x), xi = double_to_df(x[c].y);
        xs[c] = make_float4(xr.hi, xi.hi, xr.lo, xi.lo);
    }
    __syncthreads();
    for (int r = threadIdx.x; r < d; r += blockDim.x) {
        DotDF re, im;
        for (int c = 0; c < d; ++c) {
            const float4 m = a[(size_t)c * d + r], v = xs[c];
            const df mr{m.x, m.z}, mi{m.y, m.w}, vr{v.x, v.z}, vi{v.y, v.w};
            re.add(mr, vr);
            re.add(df_neg(mi), vi);
            im.add(mr, vi);
            im.add(mi, vr);
        }
        y[r] = make_double2(df_to_double(re.value()), df_to_double(im.value()));
    }
    __syncthreads();
}

// FP64 block sum (valid in every thread); `red` holds one double per warp plus one slot
__device__ double block_sum(double v, double* red) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) red[warp] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
        red[32] = t;
    }
    __syncthreads();
    const double t = red[32];
    __syncthreads();  // red is reused by the next call
    return t;
}

__device__ double norm2(const double2* x, int d, double* red) {
    double s = 0.0;
    for (int r = threadIdx.x; r < d; r += blockDim.x) s = fma(x[r].x, x[r].x, fma(x[r].y, x[r].y, s));
    return block_sum(s, red);
}

__global__ void __launch_bounds__(kTsThreads) k_tsolve(TsParams p) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ double red[33];
    __shared__ double weight[64];
    const int d = p.dim;
    double2* psi = reinterpret_cast<double2*>(smem_raw);
    double2* tmp = psi + d;
    double2* w = tmp + d;
    double2* k = w + d;
    double2* acc = k + d;
    float4* xs = reinterpret_cast<float4*>(acc + d);  // matvec scratch
    const size_t dd = (size_t)d * d;
    for (uint64_t tt = blockIdx.x; tt < p.n_traj; tt += gridDim.x) {
        const uint64_t traj = p.traj_begin + tt;
        for (int r = threadIdx.x; r < d; r += blockDim.x) psi[r] = p.psi0[r];
        __syncthreads();
        bool failed = false;
        for (long long s = 0; s < p.steps && !failed; ++s) {
            if (p.kind == 2) {  // diffusive
                if (p.constant) {
                    matvec(p.prop, psi, tmp, d, xs);
                    for (int r = threadIdx.x; r < d; r += blockDim.x) {
                        psi[r] = tmp[r];
                        acc[r] = make_double2(0.0, 0.0);  // drift
                    }
                } else {
                    matvec(p.nodes + (size_t)s * dd, psi, acc, d, xs);
                }
                for (int r = threadIdx.x; r < d; r += blockDim.x) tmp[r] = make_double2(0.0, 0.0);  // noise
                __syncthreads();
                for (int c = 0; c < p.nch; ++c) {
                    matvec(p.ops + (size_t)c * dd, psi, w, d, xs);      // cp
                    matvec(p.ops_dop + (size_t)c * dd, psi, k, d, xs);  // t2
                    double part = 0.0;
                    for (int r = threadIdx.x; r < d; r += blockDim.x) part = fma(psi[r].x, w[r].x, fma(psi[r].y, w[r].y, part));
                    const double x = 2.0 * block_sum(part, red);
                    double u1, u2;
                    philox_pair(p.seed, traj, (uint64_t)s * (uint64_t)p.nch + (uint64_t)c, &u1, &u2);
                    const double dw = sqrt(p.h) * (sqrt(-2.0 * log(1.0 - u1)) * cos(6.283185307179586 * u2));
                    for (int r = threadIdx.x; r < d; r += blockDim.x) {
                        acc[r].x += -0.5 * (k[r].x - x * w[r].x + 0.25 * x * x * psi[r].x);
                        acc[r].y += -0.5 * (k[r].y - x * w[r].y + 0.25 * x * x * psi[r].y);
                        tmp[r].x += (w[r].x - 0.5 * x * psi[r].x) * dw;
                        tmp[r].y += (w[r].y - 0.5 * x * psi[r].y) * dw;
                    }
                    __syncthreads();
                }
                for (int r = threadIdx.x; r < d; r += blockDim.x) {
                    psi[r].x += p.h * acc[r].x + tmp[r].x;
                    psi[r].y += p.h * acc[r].y + tmp[r].y;
                }
                __syncthreads();
                const double nrm = sqrt(norm2(psi, d, red));
                if (!(nrm > 0.0) || !isfinite(nrm)) {
                    failed = true;
                    break;
                }
                for (int r = threadIdx.x; r < d; r += blockDim.x) {
                    psi[r].x /= nrm;
                    psi[r].y /= nrm;
                }
                __syncthreads();
                continue;
            }
            // jump unravelings: tmp = psi~
            if (p.constant) {
                matvec(p.prop, psi, tmp, d, xs);
            } else {
                const float4* a0 = p.nodes + (size_t)(2 * s) * dd;
                const float4* a1 = a0 + dd;
                const float4* a2 = a1 + dd;
                const double h = p.h;
                matvec(a0, psi, k, d, xs);  // k1
                for (int r = threadIdx.x; r < d; r += blockDim.x) {
                    acc[r] = make_double2(k[r].x, k[r].y);  // k1 + 2 k2 + 2 k3 + k4, accumulated
                    w[r] = make_double2(psi[r].x + 0.5 * h * k[r].x, psi[r].y + 0.5 * h * k[r].y);
                }
                __syncthreads();
                matvec(a1, w, k, d, xs);  // k2
                for (int r = threadIdx.x; r < d; r += blockDim.x) {
                    acc[r].x += 2.0 * k[r].x;
                    acc[r].y += 2.0 * k[r].y;
                    w[r] = make_double2(psi[r].x + 0.5 * h * k[r].x, psi[r].y + 0.5 * h * k[r].y);
                }
                __syncthreads();
                matvec(a1, w, k, d, xs);  // k3
                for (int r = threadIdx.x; r < d; r += blockDim.x) {
                    acc[r].x += 2.0 * k[r].x;
                    acc[r].y += 2.0 * k[r].y;
                    w[r] = make_double2(psi[r].x + h * k[r].x, psi[r].y + h * k[r].y);
                }
                __syncthreads();
                matvec(a2, w, k, d, xs);  // k4
                for (int r = threadIdx.x; r < d; r += blockDim.x) {
                    tmp[r].x = psi[r].x + (h / 6.0) * (acc[r].x + k[r].x);
                    tmp[r].y = psi[r].y + (h / 6.0) * (acc[r].y + k[r].y);
                }
                __syncthreads();
            }
            const double survive = norm2(tmp, d, red);
            if (!(survive > 0.0) || !isfinite(survive)) {
                failed = true;
                break;
            }
            double u1, u2;
            philox_pair(p.seed, traj, (uint64_t)s, &u1, &u2);
            bool jumped = false;
            if (p.nch > 0 && u1 >= survive) {  // uniform across the block
                double total = 0.0;
                for (int c = 0; c < p.nch; ++c) {
                    matvec(p.ops + (size_t)c * dd, tmp, w, d, xs);
                    const double wc = norm2(w, d, red);
                    if (threadIdx.x == 0) weight[c] = wc;
                    total += wc;
                }
                __syncthreads();
                if (total > 0.0) {
                    const double rr = u2 * total;
                    int pick = p.nch;
                    double run = 0.0;
                    for (int c = 0; c < p.nch; ++c) {
                        run += weight[c];
                        if (rr < run && weight[c] > 0.0) {
                            pick = c;
                            break;
                        }
                    }
                    if (pick == p.nch)
                        for (int c = p.nch - 1; c >= 0; --c)
                            if (weight[c] > 0.0) {
                                pick = c;
                                break;
                            }
                    matvec(p.ops + (size_t)pick * dd, tmp, psi, d, xs);
                    const double inv = 1.0 / sqrt(weight[pick]);
                    for (int r = threadIdx.x; r < d; r += blockDim.x) {
                        psi[r].x *= inv;
                        psi[r].y *= inv;
                    }
                    __syncthreads();
                    jumped = true;
                }
            }
            if (!jumped) {
                const double inv = 1.0 / sqrt(survive);
                for (int r = threadIdx.x; r < d; r += blockDim.x) psi[r] = make_double2(tmp[r].x * inv, tmp[r].y * inv);
                __syncthreads();
            }
        }
        if (failed) {
            if (threadIdx.x == 0) atomicExch(p.err, 1);
            __syncthreads();
            continue;
        }
        if (p.states)
            for (int r = threadIdx.x; r < d; r += blockDim.x) p.states[tt * (uint64_t)d + r] = psi[r];
        if (p.obs) {
            matvec(p.obs, psi, w, d, xs);
            double part = 0.0;
            for (int r = threadIdx.x; r < d; r += blockDim.x) part = fma(psi[r].x, w[r].x, fma(psi[r].y, w[r].y, part));
            const double v = block_sum(part, red);
            if (threadIdx.x == 0) p.obs_out[tt] = v;
        }
        __syncthreads();
    }
}

// rho = (1/N) sum_t psi_t psi_t^+, in trajectory order
__global__ void k_rho(const double2* __restrict__ states, uint64_t n_traj, int d, double2* __restrict__ rho) {
    const int i = blockIdx.y * blockDim.y + threadIdx.y, j = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d || j >= d) return;
    double sr = 0.0, si = 0.0;
    for (uint64_t t = 0; t < n_traj; ++t) {
        const double2 a = states[t * (uint64_t)d + i], b = states[t * (uint64_t)d + j];
        sr = fma(a.x, b.x, fma(a.y, b.y, sr));
        si = fma(a.y, b.x, fma(-a.x, b.y, si));
    }
    const double inv = 1.0 / (double)n_traj;
    rho[(size_t)i * d + j] = make_double2(sr * inv, si * inv);
}

}  // namespace

struct llg_tsolver {
    int n = 0, dim = 0;
    std::vector<cd> h_const;
    llg_hamiltonian_fn h_fn = nullptr;
    void* h_user = nullptr;
    struct Channel {
        std::vector<cd> l;
        double gamma = 0.0;
        bool pauli = false;
        std::vector<cd> p;  // L / sqrt(c)
        double g = 0.0;     // gamma c
    };
    std::vector<Channel> channels;
    cudaStream_t stream = nullptr;
    // the last run's plan, host copies (row-major), for llg_tsolver_plan_export
    long long steps = 0;
    double h = 0.0;
    int constant = 1, kind = 0;
    std::vector<cd> prop, nodes, ops, ops_dop;
};

namespace {

bool hermitian(const std::vector<cd>& m, int d) {
    const std::vector<cd> a = adjoint(m, d);
    std::vector<cd> diff(m.size());
    for (size_t i = 0; i < m.size(); ++i) diff[i] = m[i] - a[i];
    return fro(diff) <= 1e-9 * std::max(1.0, fro(m));
}

bool finite(const std::vector<cd>& m) {
    for (const cd& v : m)
        if (!std::isfinite(v.real()) || !std::isfinite(v.imag())) return false;
    return true;
}

std::vector<cd> read_matrix(const double* m, int d) {
    std::vector<cd> r((size_t)d * d);
    for (size_t i = 0; i < r.size(); ++i) r[i] = cd(m[2 * i], m[2 * i + 1]);
    return r;
}

// Builds the plan into s (host copies) for `kind` over `duration` / `dt`.
int make_plan(llg_tsolver* s, int kind, double duration, double dt, Gemm& g) {
    const int d = s->dim;
    const cd I(0.0, 1.0);
    if (s->channels.empty()) kind = LLG_UNRAVEL_STANDARD;  // unitary evolution: exact propagator
    s->kind = kind;
    s->steps = std::max<long long>(1, (long long)std::ceil(duration / dt - 1e-9));
    s->h = duration / (double)s->steps;
    s->ops.clear();
    s->ops_dop.clear();
    std::vector<cd> hnh((size_t)d * d, 0.0), jdj;
    for (const auto& ch : s->channels) {
        std::vector<cd> j((size_t)d * d);
        if (kind == LLG_UNRAVEL_PROJECTOR && ch.pauli) {
            const double sg = std::sqrt(ch.g);
            for (int r = 0; r < d; ++r)
                for (int c = 0; c < d; ++c)
                    j[(size_t)r * d + c] = sg * ((r == c ? 1.0 : 0.0) - ch.p[(size_t)r * d + c]);
        } else {
            const double sg = std::sqrt(ch.gamma);
            for (size_t i = 0; i < j.size(); ++i) j[i] = sg * ch.l[i];
        }
        cudaError_t e = g.mul(j, j, jdj, true);
        if (e != cudaSuccess) return cuda_fail(e, "trajectory plan");
        s->ops.insert(s->ops.end(), j.begin(), j.end());
        s->ops_dop.insert(s->ops_dop.end(), jdj.begin(), jdj.end());
        if (kind != LLG_UNRAVEL_ANALOG)
            for (size_t i = 0; i < hnh.size(); ++i) hnh[i] -= cd(0.0, 0.5) * jdj[i];
    }
    s->constant = s->h_fn ? 0 : 1;
    s->prop.clear();
    s->nodes.clear();
    if (s->constant) {
        std::vector<cd> a((size_t)d * d);
        for (size_t i = 0; i < a.size(); ++i) a[i] = -I * (s->h_const[i] + hnh[i]) * s->h;
        cudaError_t e = expm(g, a, s->prop);
        if (e != cudaSuccess) return cuda_fail(e, "trajectory plan (expm)");
        return LLG_OK;
    }
    const bool jump = kind != LLG_UNRAVEL_ANALOG;
    const long long n_nodes = jump ? 2 * s->steps + 1 : s->steps;
    if ((double)n_nodes * d * d * 16.0 > 1.0e9)
        return set_error(LLG_EINVAL, "TrajectorySolver: time-dependent H(t) samples exceed 1 GB; increase dt");
    s->nodes.resize((size_t)n_nodes * d * d);
    std::vector<double> buf((size_t)2 * d * d);
    for (long long j = 0; j < n_nodes; ++j) {
        const double t = jump ? 0.5 * s->h * (double)j : s->h * (double)j;
        s->h_fn(t, buf.data(), s->h_user);
        for (size_t i = 0; i < (size_t)d * d; ++i) {
            const cd hv(buf[2 * i], buf[2 * i + 1]);
            if (!std::isfinite(hv.real()) || !std::isfinite(hv.imag()))
                return set_error(LLG_EINVAL, "H(t): returned non-finite values");
            s->nodes[(size_t)j * d * d + i] = -I * (hv + hnh[i]);
        }
    }
    return LLG_OK;
}

}  // namespace

extern "C" {

int llg_tsolver_create(int n_qubits, llg_tsolver** out) {
    if (!out) return set_error(LLG_EINVAL, "TrajectorySolver: out is NULL");
    *out = nullptr;
    if (n_qubits < 1 || n_qubits > kTsMaxQubits)
        return set_error(LLG_EINVAL, "TrajectorySolver: n_qubits must be in [1, 10]");
    llg_tsolver* s = new llg_tsolver();
    s->n = n_qubits;
    s->dim = 1 << n_qubits;
    s->h_const.assign((size_t)s->dim * s->dim, 0.0);
    cudaError_t e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete s;
        return cuda_fail(e, "cudaStreamCreate");
    }
    *out = s;
    return LLG_OK;
}

int llg_tsolver_destroy(llg_tsolver* s) {
    if (!s) return LLG_OK;
    if (s->stream) {
        cudaStreamSynchronize(s->stream);
        cudaStreamDestroy(s->stream);
    }
    delete s;
    return LLG_OK;
}

int llg_tsolver_set_hamiltonian(llg_tsolver* s, const double* h) {
    if (!s || !h) return set_error(LLG_EINVAL, "set_hamiltonian: NULL argument");
    std::vector<cd> m = read_matrix(h, s->dim);
    if (!finite(m)) return set_error(LLG_EINVAL, "set_hamiltonian: non-finite H");
    if (!hermitian(m, s->dim)) return set_error(LLG_EINVAL, "set_hamiltonian: H is not Hermitian");
    s->h_const.swap(m);
    s->h_fn = nullptr;
    s->h_user = nullptr;
    return LLG_OK;
}

int llg_tsolver_set_hamiltonian_fn(llg_tsolver* s, llg_hamiltonian_fn fn, void* user) {
    if (!s || !fn) return set_error(LLG_EINVAL, "set_hamiltonian: empty function");
    std::vector<double> buf((size_t)2 * s->dim * s->dim);
    fn(0.0, buf.data(), user);
    std::vector<cd> m = read_matrix(buf.data(), s->dim);
    if (!finite(m)) return set_error(LLG_EINVAL, "set_hamiltonian: non-finite H");
    if (!hermitian(m, s->dim)) return set_error(LLG_EINVAL, "set_hamiltonian: H is not Hermitian");
    s->h_fn = fn;
    s->h_user = user;
    return LLG_OK;
}

int llg_tsolver_add_lindblad(llg_tsolver* s, const double* l, double gamma) {
    if (!s || !l) return set_error(LLG_EINVAL, "add_lindblad: NULL argument");
    std::vector<cd> m = read_matrix(l, s->dim);
    if (!finite(m)) return set_error(LLG_EINVAL, "add_lindblad: non-finite operator");
    if (!(std::isfinite(gamma) && gamma >= 0.0)) return set_error(LLG_EINVAL, "add_lindblad: gamma must be finite and >= 0");
    if (gamma == 0.0) return LLG_OK;
    if ((int)s->channels.size() >= 64) return set_error(LLG_EINVAL, "add_lindblad: at most 64 channels");
    llg_tsolver::Channel ch;
    ch.l = m;
    ch.gamma = gamma;
    // Pauli-like: Hermitian with L^2 = c 1, c > 0 (src/TrajectorySolver.h:363-373)
    const int d = s->dim;
    if (hermitian(m, d)) {
        Gemm g;
        cudaError_t e = g.init(d, s->stream);
        std::vector<cd> l2;
        if (e == cudaSuccess) e = g.mul(adjoint(m, d), m, l2, true);  // (L^+)^+ L = L L
        if (e != cudaSuccess) return cuda_fail(e, "add_lindblad");
        const double c = l2[0].real();
        if (c > 1e-12) {
            std::vector<cd> diff(l2);
            for (int i = 0; i < d; ++i) diff[(size_t)i * d + i] -= c;
            if (fro(diff) <= 1e-9 * std::max(1.0, fro(l2))) {
                ch.pauli = true;
                ch.p.resize(m.size());
                for (size_t i = 0; i < m.size(); ++i) ch.p[i] = m[i] / std::sqrt(c);
                ch.g = gamma * c;
            }
        }
    }
    s->channels.push_back(std::move(ch));
    return LLG_OK;
}

int llg_tsolver_clear_lindblad(llg_tsolver* s) {
    if (!s) return set_error(LLG_EINVAL, "clear_lindblad: NULL solver");
    s->channels.clear();
    return LLG_OK;
}

int llg_tsolver_info(const llg_tsolver* s, int* n_channels, int* dim) {
    if (!s) return set_error(LLG_EINVAL, "tsolver_info: NULL solver");
    if (n_channels) *n_channels = (int)s->channels.size();
    if (dim) *dim = s->dim;
    return LLG_OK;
}

int llg_tsolver_projector_applies(const llg_tsolver* s, int channel, int* out) {
    if (!s || !out || channel < 0 || channel >= (int)s->channels.size())
        return set_error(LLG_EINVAL, "projector_applies: channel out of range");
    *out = s->channels[channel].pauli ? 1 : 0;
    return LLG_OK;
}

int llg_tsolver_run(llg_tsolver* s, const double* psi0, double duration, double dt, int64_t n_traj, int kind,
                    uint64_t seed, double* states_out, double* rho_out, const double* obs, double* obs_out) {
    if (!s || !psi0) return set_error(LLG_EINVAL, "TrajectorySolver: NULL argument");
    const int d = s->dim;
    if (kind < LLG_UNRAVEL_STANDARD || kind > LLG_UNRAVEL_ANALOG) return set_error(LLG_EINVAL, "TrajectorySolver: unknown unraveling");
    if (n_traj < 1) return set_error(LLG_EINVAL, "evolve_ensemble: n_trajectories must be >= 1");
    if (!(std::isfinite(duration) && duration >= 0.0)) return set_error(LLG_EINVAL, "TrajectorySolver: duration must be finite and >= 0");
    if (!(std::isfinite(dt) && dt > 0.0)) return set_error(LLG_EINVAL, "TrajectorySolver: dt must be finite and > 0");
    if (duration / dt > 2e9) return set_error(LLG_EINVAL, "TrajectorySolver: too many time steps");
    if ((obs == nullptr) != (obs_out == nullptr)) return set_error(LLG_EINVAL, "TrajectorySolver: obs and obs_out go together");
    std::vector<cd> start(d);
    double nrm = 0.0;
    for (int i = 0; i < d; ++i) {
        start[i] = cd(psi0[2 * i], psi0[2 * i + 1]);
        if (!std::isfinite(psi0[2 * i]) || !std::isfinite(psi0[2 * i + 1])) return set_error(LLG_EINVAL, "TrajectorySolver: non-finite psi0");
        nrm += std::norm(start[i]);
    }
    nrm = std::sqrt(nrm);
    if (!(nrm > 1e-12)) return set_error(LLG_EINVAL, "TrajectorySolver: psi0 has zero norm");
    for (cd& v : start) v /= nrm;
    std::vector<cd> obs_m;
    if (obs) {
        obs_m = read_matrix(obs, d);
        if (!finite(obs_m)) return set_error(LLG_EINVAL, "TrajectorySolver: non-finite observable");
    }

    Gemm g;
    cudaError_t e = g.init(d, s->stream);
    if (e != cudaSuccess) return cuda_fail(e, "TrajectorySolver");
    int rc = LLG_OK;
    const bool evolve = duration > 0.0;
    if (evolve) rc = make_plan(s, kind, duration, dt, g);
    if (rc) return rc;

    // device buffers
    const size_t dd = (size_t)d * d;
    float4 *d_prop = nullptr, *d_nodes = nullptr, *d_ops = nullptr, *d_dop = nullptr, *d_obs = nullptr;
    double2 *d_psi0 = nullptr, *d_states = nullptr, *d_rho = nullptr;
    double* d_obs_out = nullptr;
    int* d_err = nullptr;
    auto up = [&](double2** dst, const std::vector<cd>& src) {
        if (e != cudaSuccess || src.empty()) return;
        e = cudaMalloc(dst, src.size() * sizeof(double2));
        if (e == cudaSuccess) e = cudaMemcpyAsync(*dst, src.data(), src.size() * sizeof(double2), cudaMemcpyHostToDevice, s->stream);
    };
    std::vector<std::vector<float4>> staged;  // host copies alive until the stream synchronises
    auto up_df = [&](float4** dst, const std::vector<cd>& src) {  // matrices: double-float entries
        if (e != cudaSuccess || src.empty()) return;
        staged.emplace_back(src.size());
        std::vector<float4>& h = staged.back();
        for (size_t i = 0; i < src.size(); ++i) {
            float rh, rl, ih, il;
            split_double(src[i].real(), &rh, &rl);
            split_double(src[i].imag(), &ih, &il);
            h[i] = make_float4(rh, ih, rl, il);
        }
        e = cudaMalloc(dst, h.size() * sizeof(float4));
        if (e == cudaSuccess) e = cudaMemcpyAsync(*dst, h.data(), h.size() * sizeof(float4), cudaMemcpyHostToDevice, s->stream);
    };
    auto colmajor_list = [&](const std::vector<cd>& list) {
        std::vector<cd> r(list.size());
        for (size_t b = 0; b < list.size() / dd; ++b) {
            std::vector<cd> one(list.begin() + b * dd, list.begin() + (b + 1) * dd);
            std::vector<cd> cm = col_major(one, d);
            std::copy(cm.begin(), cm.end(), r.begin() + b * dd);
        }
        return r;
    };
    std::vector<cd> prop_cm, nodes_cm, ops_cm, dop_cm, obs_cm;
    if (evolve) {
        prop_cm = s->constant ? col_major(s->prop, d) : std::vector<cd>();
        nodes_cm = colmajor_list(s->nodes);
        ops_cm = colmajor_list(s->ops);
        dop_cm = colmajor_list(s->ops_dop);
    }
    if (obs) obs_cm = col_major(obs_m, d);
    up_df(&d_prop, prop_cm);
    up_df(&d_nodes, nodes_cm);
    up_df(&d_ops, ops_cm);
    up_df(&d_dop, dop_cm);
    up(&d_psi0, start);
    up_df(&d_obs, obs_cm);
    const bool need_states = states_out || rho_out;
    if (e == cudaSuccess && need_states) e = cudaMalloc(&d_states, (size_t)n_traj * d * sizeof(double2));
    if (e == cudaSuccess && obs) e = cudaMalloc(&d_obs_out, (size_t)n_traj * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&d_err, sizeof(int));
    if (e == cudaSuccess) e = cudaMemsetAsync(d_err, 0, sizeof(int), s->stream);
    if (e == cudaSuccess) {
        TsParams p;
        std::memset(&p, 0, sizeof(p));
        p.dim = d;
        p.nch = evolve ? (int)(s->ops.size() / dd) : 0;
        p.kind = evolve ? s->kind : 0;
        p.constant = evolve ? s->constant : 1;
        p.steps = evolve ? s->steps : 0;
        p.h = evolve ? s->h : 0.0;
        p.prop = d_prop;
        p.nodes = d_nodes;
        p.ops = d_ops;
        p.ops_dop = d_dop;
        p.psi0 = d_psi0;
        p.obs = d_obs;
        p.seed = seed;
        p.traj_begin = 0;
        p.n_traj = (uint64_t)n_traj;
        p.states = d_states;
        p.obs_out = d_obs_out;
        p.err = d_err;
        const int threads = std::min(kTsThreads, std::max(32, ((d + 31) / 32) * 32));
        const size_t smem = 5 * (size_t)d * sizeof(double2) + (size_t)d * sizeof(float4);
        int dev = 0, sms = 1, per_sm = 1;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        e = cudaFuncSetAttribute(k_tsolve, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_tsolve, threads, smem);
        if (e == cudaSuccess) {
            const uint64_t grid = std::min<uint64_t>((uint64_t)n_traj, (uint64_t)sms * std::max(per_sm, 1));
            k_tsolve<<<(unsigned)grid, threads, smem, s->stream>>>(p);
            e = cudaGetLastError();
        }
    }
    if (e == cudaSuccess && rho_out) {
        e = cudaMalloc(&d_rho, dd * sizeof(double2));
        if (e == cudaSuccess) {
            const dim3 block(16, 16), grid((d + 15) / 16, (d + 15) / 16);
            k_rho<<<grid, block, 0, s->stream>>>(d_states, (uint64_t)n_traj, d, d_rho);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaMemcpyAsync(rho_out, d_rho, dd * sizeof(double2), cudaMemcpyDefault, s->stream);
    }
    if (e == cudaSuccess && states_out)
        e = cudaMemcpyAsync(states_out, d_states, (size_t)n_traj * d * sizeof(double2), cudaMemcpyDefault, s->stream);
    if (e == cudaSuccess && obs)
        e = cudaMemcpyAsync(obs_out, d_obs_out, (size_t)n_traj * sizeof(double), cudaMemcpyDefault, s->stream);
    int err = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&err, d_err, sizeof(int), cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    cudaFree(d_prop);
    cudaFree(d_nodes);
    cudaFree(d_ops);
    cudaFree(d_dop);
    cudaFree(d_psi0);
    cudaFree(d_obs);
    cudaFree(d_states);
    cudaFree(d_rho);
    cudaFree(d_obs_out);
    cudaFree(d_err);
    if (e != cudaSuccess) return cuda_fail(e, "TrajectorySolver");
    if (err) return set_error(LLG_ERUNTIME, "TrajectorySolver: state norm vanished; reduce dt");
    return LLG_OK;
}

int llg_tsolver_plan_export(const llg_tsolver* s, long long* steps, double* h, int* constant, int* kind, double* prop,
                            double* nodes, int64_t max_nodes, double* ops, double* ops_dop, int* n_ops, int64_t* n_nodes) {
    if (!s) return set_error(LLG_EINVAL, "tsolver_plan_export: NULL solver");
    const size_t dd = (size_t)s->dim * s->dim;
    if (steps) *steps = s->steps;
    if (h) *h = s->h;
    if (constant) *constant = s->constant;
    if (kind) *kind = s->kind;
    if (n_ops) *n_ops = (int)(s->ops.size() / dd);
    if (n_nodes) *n_nodes = (int64_t)(s->nodes.size() / dd);
    if (prop && !s->prop.empty()) std::memcpy(prop, s->prop.data(), dd * sizeof(cd));
    if (nodes && (int64_t)(s->nodes.size() / dd) <= max_nodes) std::memcpy(nodes, s->nodes.data(), s->nodes.size() * sizeof(cd));
    if (ops) std::memcpy(ops, s->ops.data(), s->ops.size() * sizeof(cd));
    if (ops_dop) std::memcpy(ops_dop, s->ops_dop.data(), s->ops_dop.size() * sizeof(cd));
    return LLG_OK;
}

}  // extern "C"
