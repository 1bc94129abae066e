/*
 * adjoint_oracle.c -- the ORACLE for circuit gradients (test infrastructure only).
 *
 * The reference has no adjoint method; its gradient is the parameter-shift rule of
 * src/Algorithms.h:210-212 and :277-292:
 *     dE/dtheta_k = [ E(theta + (pi/2) e_k) - E(theta - (pi/2) e_k) ] / 2,
 * exact for RX/RY/RZ (generator eigenvalues +-1/2).  E is the diagonal observable
 * sum_k c_k Z_{a_k} Z_{b_k} evaluated from the probabilities, as python/algorithms.py:177-179
 * does with ising_diagonal (:141-153).  When one parameter drives several rotations the rule is
 * applied to each occurrence and the results summed (chain rule).
 */
#include <stdlib.h>
#include <string.h>

#include "sv_oracle.h"

static const double HALF_PI = 1.57079632679489661923;

static int energy_of(int n, orc_op* ops, int nops, double* psi, int nterms, const int* a, const int* b,
                     const double* coeff, double* e) {
    orc_init_zero(psi, n);
    const int rc = orc_run_ops(psi, n, ops, nops);
    if (rc) return rc;
    *e = orc_expect_zz(psi, n, nterms, a, b, coeff);
    return 0;
}

int orc_param_shift(int n, const orc_op* ops_in, int nops, const double* params, int nparams, int nterms,
                    const int* a, const int* b, const double* coeff, double* energy, double* grad) {
    if (n < 1 || n > 26) return ORC_EINVAL;
    orc_op* ops = (orc_op*)malloc(sizeof(orc_op) * (size_t)(nops > 0 ? nops : 1));
    double* psi = (double*)malloc(sizeof(double) * 2 * ((size_t)1 << n));
    if (!ops || !psi) {
        free(ops);
        free(psi);
        return ORC_ENOMEM;
    }
    memcpy(ops, ops_in, sizeof(orc_op) * (size_t)nops);
    for (int g = 0; g < nops; ++g)
        if (ops[g].param >= 0) {
            if (ops[g].param >= nparams) {
                free(ops);
                free(psi);
                return ORC_EINVAL;
            }
            ops[g].theta = params[ops[g].param];
        }
    int rc = energy_of(n, ops, nops, psi, nterms, a, b, coeff, energy);
    if (grad) {
        for (int k = 0; k < nparams; ++k) grad[k] = 0.0;
        for (int g = 0; g < nops && !rc; ++g) {
            const int k = ops[g].param;
            if (k < 0) continue;
            const double t0 = ops[g].theta;
            double ep = 0.0, em = 0.0;
            ops[g].theta = t0 + HALF_PI;
            rc = energy_of(n, ops, nops, psi, nterms, a, b, coeff, &ep);
            ops[g].theta = t0 - HALF_PI;
            if (!rc) rc = energy_of(n, ops, nops, psi, nterms, a, b, coeff, &em);
            ops[g].theta = t0;
            grad[k] += 0.5 * (ep - em);
        }
    }
    free(ops);
    free(psi);
    return rc;
}
