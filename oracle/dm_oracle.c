/*
 * dm_oracle.c -- the ORACLE for density-matrix channels (test infrastructure only).
 *
 * Restates the reference's KrausChannel::apply (src/Noise.cpp:174-258): for every block (r1, r2)
 * of the non-target bits, the 2^m x 2^m sub-matrix B of rho over the target bits (bit j of a block
 * index on targets[j]) becomes sum_k K_k B K_k^+.  Also the trace-preservation test
 * (src/Noise.cpp:166-172) and a gate U applied as U rho U^+.
 *
 * rho is dim x dim complex, element (row, col) at index row + col * dim (interleaved re, im): the
 * layout of a 2n-qubit state vector whose qubit q is bit q of the row and qubit n + q bit q of
 * the column, the layout the GPU engine keeps.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "sv_oracle.h"

#define RE(p, i) (p)[2 * (i)]
#define IM(p, i) (p)[2 * (i) + 1]

/* max |sum_k K_k^+ K_k - I| <= tol over 2^m x 2^m operators (row-major, interleaved) */
int orc_kraus_trace_preserving(int nk, const double* ops, int m, double tol) {
    const int d = 1 << m;
    double worst = 0.0;
    for (int i = 0; i < d; ++i)
        for (int j = 0; j < d; ++j) {
            double sr = 0.0, si = 0.0;
            for (int k = 0; k < nk; ++k) {
                const double* K = ops + (size_t)2 * k * d * d;
                for (int r = 0; r < d; ++r) { /* (K^+ K)_{ij} = sum_r conj(K_{ri}) K_{rj} */
                    const double ar = RE(K, r * d + i), ai = -IM(K, r * d + i);
                    const double br = RE(K, r * d + j), bi = IM(K, r * d + j);
                    sr += ar * br - ai * bi;
                    si += ar * bi + ai * br;
                }
            }
            if (i == j) sr -= 1.0;
            const double v = sqrt(sr * sr + si * si);
            if (v > worst) worst = v;
        }
    return worst <= tol;
}

int orc_kraus_apply(double* rho, int n, int nk, const double* ops, int m, const int* targets) {
    if (n < 0 || n > 10 || m < 1 || m > n || nk < 1) return ORC_EINVAL;
    for (int j = 0; j < m; ++j) {
        if (targets[j] < 0 || targets[j] >= n) return ORC_EINVAL;
        for (int i = 0; i < j; ++i)
            if (targets[i] == targets[j]) return ORC_EINVAL;
    }
    const int64_t dim = 1LL << n;
    const int blk = 1 << m;
    const int64_t n_rest = 1LL << (n - m);
    int64_t* rest_base = (int64_t*)malloc(sizeof(int64_t) * (size_t)n_rest);
    int64_t* tgt_off = (int64_t*)malloc(sizeof(int64_t) * (size_t)blk);
    double* out = (double*)malloc(sizeof(double) * 2 * (size_t)(dim * dim));
    double* B = (double*)malloc(sizeof(double) * 2 * (size_t)(blk * blk));
    double* T = (double*)malloc(sizeof(double) * 2 * (size_t)(blk * blk));
    double* A = (double*)malloc(sizeof(double) * 2 * (size_t)(blk * blk));
    if (!rest_base || !tgt_off || !out || !B || !T || !A) {
        free(rest_base);
        free(tgt_off);
        free(out);
        free(B);
        free(T);
        free(A);
        return ORC_ENOMEM;
    }
    /* non-target bit positions ascending; block bases; target offsets (bit j -> targets[j]) */
    for (int64_t r = 0; r < n_rest; ++r) {
        int64_t base = 0, bits = r;
        for (int q = 0; q < n; ++q) {
            int is_t = 0;
            for (int j = 0; j < m; ++j) is_t |= targets[j] == q;
            if (is_t) continue;
            if (bits & 1) base |= 1LL << q;
            bits >>= 1;
        }
        rest_base[r] = base;
    }
    for (int t = 0; t < blk; ++t) {
        int64_t off = 0;
        for (int j = 0; j < m; ++j)
            if ((t >> j) & 1) off |= 1LL << targets[j];
        tgt_off[t] = off;
    }
    for (int64_t r1 = 0; r1 < n_rest; ++r1)
        for (int64_t r2 = 0; r2 < n_rest; ++r2) {
            const int64_t row0 = rest_base[r1], col0 = rest_base[r2];
            for (int a = 0; a < blk; ++a)
                for (int b = 0; b < blk; ++b) {
                    const int64_t e = (row0 | tgt_off[a]) + (col0 | tgt_off[b]) * dim;
                    RE(B, a * blk + b) = RE(rho, e);
                    IM(B, a * blk + b) = IM(rho, e);
                }
            memset(A, 0, sizeof(double) * 2 * (size_t)(blk * blk));
            for (int k = 0; k < nk; ++k) {
                const double* K = ops + (size_t)2 * k * blk * blk;
                /* T = K B */
                for (int a = 0; a < blk; ++a)
                    for (int b = 0; b < blk; ++b) {
                        double sr = 0.0, si = 0.0;
                        for (int c = 0; c < blk; ++c) {
                            const double kr = RE(K, a * blk + c), ki = IM(K, a * blk + c);
                            const double br = RE(B, c * blk + b), bi = IM(B, c * blk + b);
                            sr += kr * br - ki * bi;
                            si += kr * bi + ki * br;
                        }
                        RE(T, a * blk + b) = sr;
                        IM(T, a * blk + b) = si;
                    }
                /* A += T K^+ */
                for (int a = 0; a < blk; ++a)
                    for (int b = 0; b < blk; ++b) {
                        double sr = 0.0, si = 0.0;
                        for (int c = 0; c < blk; ++c) {
                            const double tr = RE(T, a * blk + c), ti = IM(T, a * blk + c);
                            const double kr = RE(K, b * blk + c), ki = -IM(K, b * blk + c);
                            sr += tr * kr - ti * ki;
                            si += tr * ki + ti * kr;
                        }
                        RE(A, a * blk + b) += sr;
                        IM(A, a * blk + b) += si;
                    }
            }
            for (int a = 0; a < blk; ++a)
                for (int b = 0; b < blk; ++b) {
                    const int64_t e = (row0 | tgt_off[a]) + (col0 | tgt_off[b]) * dim;
                    RE(out, e) = RE(A, a * blk + b);
                    IM(out, e) = IM(A, a * blk + b);
                }
        }
    memcpy(rho, out, sizeof(double) * 2 * (size_t)(dim * dim));
    free(rest_base);
    free(tgt_off);
    free(out);
    free(B);
    free(T);
    free(A);
    return 0;
}

/* U rho U^+ for one gate record: U on the row qubits, conj(U) on the column qubits. */
int orc_dm_apply_op(double* rho, int n, const orc_op* op) {
    if (n < 1 || n > 10) return ORC_EINVAL;
    const int two = op->kind == ORC_OP_CNOT || op->kind == ORC_OP_CZ;
    if (op->kind == ORC_OP_MCZ) {
        if (op->mask == 0 || (op->mask >> n) != 0) return ORC_EINVAL;
    } else if (op->q0 < 0 || op->q0 >= n || (two && (op->q1 < 0 || op->q1 >= n))) {
        return ORC_EINVAL;
    }
    orc_op row = *op, col = *op;
    col.q0 = op->q0 + n;
    col.q1 = op->q1 + n;
    col.mask = op->mask << n;
    if (op->kind == ORC_OP_RX || op->kind == ORC_OP_RZ) col.theta = -op->theta;
    if (op->kind == ORC_OP_U2)
        for (int i = 0; i < 4; ++i) col.m[2 * i + 1] = -op->m[2 * i + 1];
    int rc = orc_apply_op(rho, 2 * n, &row);
    if (!rc) rc = orc_apply_op(rho, 2 * n, &col);
    return rc;
}
