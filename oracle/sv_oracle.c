/*
 * sv_oracle.c -- the ORACLE: a plain-C restatement of the reference's CPU state-vector path.
 *
 * TEST INFRASTRUCTURE ONLY.  It is the checker, never the product: only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline / reference legs may load it.  The GPU
 * engine never calls, links or falls back to this file.
 *
 * Every function cites the reference lines it follows (paths inside the reference project).
 * Conventions (src/Backend.h:3-8): qubit q is bit q of the basis index; RX/RY/RZ(t) =
 * exp(-i t P/2); mcz negates every amplitude whose bits are all 1 on the listed qubits.
 *
 * A state is 2^n complex128 stored interleaved (re, im) as 2*2^n doubles, exactly the
 * std::complex<double> layout the reference uses.  Arithmetic is written out in real
 * operations in the same order as the reference and the file is compiled with
 * -ffp-contract=off, as the reference's ISO C++17 builds are, so results match the reference
 * build bit for bit.
 *
 * OpenMP: the loops over pairs follow StateVectorBackend's contiguous-thread-range scheme so
 * the CPU baseline timed from this file does the same work the reference does.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "sv_oracle.h"

typedef long long ll;

/* src/StateVectorBackend.h:170: below 2^15 amplitudes a single thread is used. */
#define ORC_PAR_MIN (1LL << 15)

static int g_threads = 0; /* 0 = OpenMP default */

void orc_set_threads(int t) { g_threads = t; }

int orc_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

static int nthreads_for(ll size) {
    if (size < ORC_PAR_MIN) return 1;
#ifdef _OPENMP
    return g_threads > 0 ? g_threads : omp_get_max_threads();
#else
    return 1;
#endif
}

/* src/StateVectorBackend.h:188-196: contiguous share [lo, hi) of n items for thread t of nt. */
static void thread_range(ll n, int t, int nt, ll* lo, ll* hi) {
    *lo = n * t / nt;
    *hi = n * (t + 1) / nt;
}

static int cur_thread(void) {
#ifdef _OPENMP
    return omp_get_thread_num();
#else
    return 0;
#endif
}
static int cur_nthreads(void) {
#ifdef _OPENMP
    return omp_get_num_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------------------------------
 * State construction
 * ---------------------------------------------------------------------------------------- */

/* src/StateVectorOptimized.cpp:17-24 (and Backend.h:55-62): |0...0>. */
void orc_init_zero(double* psi, int n) {
    const ll size = 1LL << n;
    memset(psi, 0, (size_t)size * 2 * sizeof(double));
    psi[0] = 1.0;
}

/* ------------------------------------------------------------------------------------------
 * quantum_sim_v3 generic 2x2 gate
 * ---------------------------------------------------------------------------------------- */

/* One std::complex<double> product x*y for finite operands: (ac - bd) + (ad + bc) i.
 * src/StateVectorOptimized.cpp:74-75 uses operator*, whose finite-operand result is this. */
static inline void cmul(double a, double b, double c, double d, double* re, double* im) {
    *re = a * c - b * d;
    *im = a * d + b * c;
}

/* src/StateVectorOptimized.cpp:56-78 apply_gate_cache_optimized: blocks of 2^(k+1), inner run
 * of 2^k contiguous pairs, a0' = g0 a0 + g1 a1, a1' = g2 a0 + g3 a1.  A target >= n is a no-op
 * (num_blocks = size >> (k+1) = 0).  g = {re0, im0, re1, im1, re2, im2, re3, im3}. */
void orc_apply_gate_v3(double* psi, int n, int target, const double* g) {
    if (target < 0 || target >= n) return;
    const ll size = 1LL << n;
    const ll stride = 1LL << target;
    const ll num_blocks = size >> (target + 1);
    const ll block_size = 1LL << (target + 1);
    const int nt = nthreads_for(size);
#pragma omp parallel for schedule(static) num_threads(nt)
    for (ll block = 0; block < num_blocks; block++) {
        const ll base = block * block_size;
        for (ll j = 0; j < stride; j++) {
            double* p0 = psi + 2 * (base + j);
            double* p1 = psi + 2 * (base + j + stride);
            const double x0 = p0[0], y0 = p0[1], x1 = p1[0], y1 = p1[1];
            double r0, i0, r1, i1;
            cmul(g[0], g[1], x0, y0, &r0, &i0);
            cmul(g[2], g[3], x1, y1, &r1, &i1);
            const double n0r = r0 + r1, n0i = i0 + i1;
            cmul(g[4], g[5], x0, y0, &r0, &i0);
            cmul(g[6], g[7], x1, y1, &r1, &i1);
            p0[0] = n0r;
            p0[1] = n0i;
            p1[0] = r0 + r1;
            p1[1] = i0 + i1;
        }
    }
}

/* src/StateVectorOptimized.cpp:81-97 apply_gate_standard (and bindings_v2.cpp:56-72): mask scan
 * over all indices.  Same arithmetic as above, different traversal. */
void orc_apply_gate_standard(double* psi, int n, int target, const double* g) {
    if (target < 0 || target >= n) return;
    const ll size = 1LL << n;
    const ll mask = 1LL << target;
    const int nt = nthreads_for(size);
#pragma omp parallel for num_threads(nt)
    for (ll i = 0; i < size; i++) {
        if ((i & mask) == 0) {
            double* p0 = psi + 2 * i;
            double* p1 = psi + 2 * (i | mask);
            const double x0 = p0[0], y0 = p0[1], x1 = p1[0], y1 = p1[1];
            double r0, i0, r1, i1;
            cmul(g[0], g[1], x0, y0, &r0, &i0);
            cmul(g[2], g[3], x1, y1, &r1, &i1);
            const double n0r = r0 + r1, n0i = i0 + i1;
            cmul(g[4], g[5], x0, y0, &r0, &i0);
            cmul(g[6], g[7], x1, y1, &r1, &i1);
            p0[0] = n0r;
            p0[1] = n0i;
            p1[0] = r0 + r1;
            p1[1] = i0 + i1;
        }
    }
}

/* ------------------------------------------------------------------------------------------
 * ll::StateVectorBackend specialised gates
 * ---------------------------------------------------------------------------------------- */

enum { K_H = 0, K_X = 1, K_RX = 2, K_RY = 3, K_RZ = 4 };

/* src/StateVectorBackend.h:198-218 for_pairs with the kernels of :61-105.
 * Pair p -> i0 = ((p >> q) << (q+1)) | (p & (2^q - 1)), i1 = i0 + 2^q; each thread walks its
 * contiguous pair range in runs that end where p >> q changes. */
static void for_pairs(double* psi, int n, int q, int kind, double c, double s) {
    const ll size = 1LL << n;
    const ll stride = 1LL << q;
    const ll n_pairs = size >> 1;
    const int nt = nthreads_for(size);
    const double r = 1.0 / sqrt(2.0);
#pragma omp parallel num_threads(nt)
    {
        ll p, end;
        thread_range(n_pairs, cur_thread(), cur_nthreads(), &p, &end);
        while (p < end) {
            ll run_end = ((p >> q) + 1) << q;
            if (run_end > end) run_end = end;
            double* p0 = psi + 2 * (((p >> q) << (q + 1)) | (p & (stride - 1)));
            double* p1 = p0 + 2 * stride;
            const ll len = run_end - p;
            for (ll j = 0; j < len; ++j) {
                double* a0 = p0 + 2 * j;
                double* a1 = p1 + 2 * j;
                const double x0 = a0[0], y0 = a0[1], x1 = a1[0], y1 = a1[1];
                switch (kind) {
                    case K_H: /* :61-68 */
                        a0[0] = r * (x0 + x1);
                        a0[1] = r * (y0 + y1);
                        a1[0] = r * (x0 - x1);
                        a1[1] = r * (y0 - y1);
                        break;
                    case K_X: /* :70-72 */
                        a0[0] = x1;
                        a0[1] = y1;
                        a1[0] = x0;
                        a1[1] = y0;
                        break;
                    case K_RX: /* :74-84  [c, -is; -is, c] */
                        a0[0] = c * x0 + s * y1;
                        a0[1] = c * y0 - s * x1;
                        a1[0] = s * y0 + c * x1;
                        a1[1] = -s * x0 + c * y1;
                        break;
                    case K_RY: /* :86-95  [c, -s; s, c] */
                        a0[0] = c * x0 - s * x1;
                        a0[1] = c * y0 - s * y1;
                        a1[0] = s * x0 + c * x1;
                        a1[1] = s * y0 + c * y1;
                        break;
                    default: /* K_RZ :97-105  diag(e^{-it/2}, e^{+it/2}) */
                        a0[0] = c * x0 + s * y0;
                        a0[1] = c * y0 - s * x0;
                        a1[0] = c * x1 - s * y1;
                        a1[1] = c * y1 + s * x1;
                        break;
                }
            }
            p = run_end;
        }
    }
}

static int bad_qubit(int n, int q) { return q < 0 || q >= n; }

int orc_h(double* psi, int n, int q) {
    if (bad_qubit(n, q)) return ORC_EINVAL;
    for_pairs(psi, n, q, K_H, 0.0, 0.0);
    return 0;
}
int orc_x(double* psi, int n, int q) {
    if (bad_qubit(n, q)) return ORC_EINVAL;
    for_pairs(psi, n, q, K_X, 0.0, 0.0);
    return 0;
}
/* :75-77, :87-89, :98-100: c = cos(t/2), s = sin(t/2); non-finite angles are rejected. */
int orc_rx(double* psi, int n, int q, double t) {
    if (bad_qubit(n, q) || !isfinite(t)) return ORC_EINVAL;
    for_pairs(psi, n, q, K_RX, cos(0.5 * t), sin(0.5 * t));
    return 0;
}
int orc_ry(double* psi, int n, int q, double t) {
    if (bad_qubit(n, q) || !isfinite(t)) return ORC_EINVAL;
    for_pairs(psi, n, q, K_RY, cos(0.5 * t), sin(0.5 * t));
    return 0;
}
int orc_rz(double* psi, int n, int q, double t) {
    if (bad_qubit(n, q) || !isfinite(t)) return ORC_EINVAL;
    for_pairs(psi, n, q, K_RZ, cos(0.5 * t), sin(0.5 * t));
    return 0;
}

/* src/StateVectorBackend.h:109-135 cnot: N/4 quads in runs of 2^lo; swap the control = 1
 * amplitudes between target = 0 and target = 1. */
int orc_cnot(double* psi, int n, int control, int target) {
    if (bad_qubit(n, control) || bad_qubit(n, target) || control == target) return ORC_EINVAL;
    const ll size = 1LL << n;
    const int lo = control < target ? control : target;
    const int hi = control < target ? target : control;
    const int mid_bits = hi - lo - 1;
    const ll n_mid = 1LL << mid_bits;
    const ll n_pairs = size >> 2;
    const ll cbit = 1LL << control, tbit = 1LL << target;
    const int nt = nthreads_for(size);
#pragma omp parallel num_threads(nt)
    {
        ll p, end;
        thread_range(n_pairs, cur_thread(), cur_nthreads(), &p, &end);
        while (p < end) {
            const ll g = p >> lo;
            ll run_end = (g + 1) << lo;
            if (run_end > end) run_end = end;
            const ll base = ((g >> mid_bits) << (hi + 1)) | ((g & (n_mid - 1)) << (lo + 1));
            double* p0 = psi + 2 * (base | cbit | (p & ((1LL << lo) - 1)));
            double* p1 = p0 + 2 * tbit;
            const ll len = run_end - p;
            for (ll j = 0; j < len; ++j) {
                const double x = p0[2 * j], y = p0[2 * j + 1];
                p0[2 * j] = p1[2 * j];
                p0[2 * j + 1] = p1[2 * j + 1];
                p1[2 * j] = x;
                p1[2 * j + 1] = y;
            }
            p = run_end;
        }
    }
    return 0;
}

/* src/StateVectorBackend.h:137-151 mcz: negate amplitudes whose index has every mask bit set.
 * The caller builds the mask; orc_mcz_list validates a qubit list the way :138-145 does. */
void orc_mcz_mask(double* psi, int n, uint64_t mask) {
    const ll size = 1LL << n;
    const ll m = (ll)mask;
    const int nt = nthreads_for(size);
#pragma omp parallel for schedule(static) num_threads(nt)
    for (ll i = 0; i < size; ++i)
        if ((i & m) == m) {
            psi[2 * i] = -psi[2 * i];
            psi[2 * i + 1] = -psi[2 * i + 1];
        }
}

int orc_mcz_list(double* psi, int n, const int* qubits, int nq) {
    if (nq <= 0) return ORC_EINVAL;
    uint64_t mask = 0;
    for (int i = 0; i < nq; ++i) {
        if (bad_qubit(n, qubits[i])) return ORC_EINVAL;
        const uint64_t b = 1ULL << qubits[i];
        if (mask & b) return ORC_EINVAL;
        mask |= b;
    }
    orc_mcz_mask(psi, n, mask);
    return 0;
}

/* src/StateVectorBackend.h:153-161 probabilities: |a|^2 = re*re + im*im. */
void orc_probabilities(const double* psi, int n, double* out) {
    const ll size = 1LL << n;
    const int nt = nthreads_for(size);
#pragma omp parallel for schedule(static) num_threads(nt)
    for (ll i = 0; i < size; ++i) out[i] = psi[2 * i] * psi[2 * i] + psi[2 * i + 1] * psi[2 * i + 1];
}

/* ------------------------------------------------------------------------------------------
 * Op lists (the record format shared with the GPU engine; kinds 0..6 follow the Op kinds of
 * the reference's random-circuit test, tests/test_backends.cpp:78-83)
 * ---------------------------------------------------------------------------------------- */

int orc_apply_op(double* psi, int n, const orc_op* op) {
    switch (op->kind) {
        case ORC_OP_H: return orc_h(psi, n, op->q0);
        case ORC_OP_X: return orc_x(psi, n, op->q0);
        case ORC_OP_RX: return orc_rx(psi, n, op->q0, op->theta);
        case ORC_OP_RY: return orc_ry(psi, n, op->q0, op->theta);
        case ORC_OP_RZ: return orc_rz(psi, n, op->q0, op->theta);
        case ORC_OP_CNOT: return orc_cnot(psi, n, op->q0, op->q1);
        case ORC_OP_MCZ:
            if (op->mask == 0 || (n < 64 && (op->mask >> n) != 0)) return ORC_EINVAL;
            orc_mcz_mask(psi, n, op->mask);
            return 0;
        case ORC_OP_CZ: {
            const int qs[2] = {op->q0, op->q1};
            return orc_mcz_list(psi, n, qs, 2);
        }
        case ORC_OP_U2:
            if (bad_qubit(n, op->q0)) return ORC_EINVAL;
            orc_apply_gate_v3(psi, n, op->q0, op->m);
            return 0;
        default: return ORC_EINVAL;
    }
}

int orc_run_ops(double* psi, int n, const orc_op* ops, int nops) {
    for (int i = 0; i < nops; ++i) {
        const int rc = orc_apply_op(psi, n, &ops[i]);
        if (rc) return rc;
    }
    return 0;
}

/* Dense k-qubit matrix (2^k x 2^k complex, row-major, interleaved) on qubits qs[0..k-1]; qs[0]
 * is the least-significant bit of the local index.  This is the fused-block generalisation of
 * python/gate_fusion.py:7-12 (g2 @ g1 products) to k qubits; it is the oracle for fused passes. */
int orc_apply_matrix(double* psi, int n, int k, const int* qs, const double* m) {
    if (k < 1 || k > 10) return ORC_EINVAL;
    uint64_t mask = 0;
    for (int i = 0; i < k; ++i) {
        if (bad_qubit(n, qs[i]) || (mask >> qs[i] & 1)) return ORC_EINVAL;
        mask |= 1ULL << qs[i];
    }
    const ll size = 1LL << n, dim = 1LL << k;
    const ll groups = size >> k;
    double* in = (double*)malloc(sizeof(double) * 2 * dim);
    ll* idx = (ll*)malloc(sizeof(ll) * dim);
    if (!in || !idx) {
        free(in);
        free(idx);
        return ORC_ENOMEM;
    }
    for (ll gi = 0; gi < groups; ++gi) {
        /* deposit the bits of gi into the positions not in mask */
        ll base = 0, rest = gi;
        for (int b = 0; b < n; ++b) {
            if (mask >> b & 1) continue;
            if (rest & 1) base |= 1LL << b;
            rest >>= 1;
        }
        for (ll l = 0; l < dim; ++l) {
            ll i = base;
            for (int b = 0; b < k; ++b)
                if (l >> b & 1) i |= 1LL << qs[b];
            idx[l] = i;
            in[2 * l] = psi[2 * i];
            in[2 * l + 1] = psi[2 * i + 1];
        }
        for (ll r = 0; r < dim; ++r) {
            double sr = 0.0, si = 0.0;
            for (ll c = 0; c < dim; ++c) {
                const double a = m[2 * (r * dim + c)], b = m[2 * (r * dim + c) + 1];
                sr += a * in[2 * c] - b * in[2 * c + 1];
                si += a * in[2 * c + 1] + b * in[2 * c];
            }
            psi[2 * idx[r]] = sr;
            psi[2 * idx[r] + 1] = si;
        }
    }
    free(in);
    free(idx);
    return 0;
}

/* Sum_k coeff_k <Z_{a_k} Z_{b_k}> (b_k < 0: single <Z_{a_k}>), accumulated over basis states
 * with the Z eigenvalue 1 - 2 bit_q of python/algorithms.py:141-153 (ising_diagonal). */
double orc_expect_zz(const double* psi, int n, int nterms, const int* a, const int* b, const double* coeff) {
    const ll size = 1LL << n;
    double total = 0.0;
    for (ll i = 0; i < size; ++i) {
        const double p = psi[2 * i] * psi[2 * i] + psi[2 * i + 1] * psi[2 * i + 1];
        double d = 0.0;
        for (int k = 0; k < nterms; ++k) {
            int par = (int)(i >> a[k] & 1);
            if (b[k] >= 0) par ^= (int)(i >> b[k] & 1);
            d += par ? -coeff[k] : coeff[k];
        }
        total += p * d;
    }
    return total;
}

double orc_norm2(const double* psi, int n) {
    const ll size = 1LL << n;
    double s = 0.0;
    for (ll i = 0; i < size; ++i) s += psi[2 * i] * psi[2 * i] + psi[2 * i + 1] * psi[2 * i + 1];
    return s;
}
