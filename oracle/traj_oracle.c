/*
 * traj_oracle.c -- the ORACLE for batched noisy trajectories (test infrastructure only).
 *
 * Restates the per-gate Kraus-jump trajectory step the GPU engine runs:
 *   - noise sites: after every gate application, one site per touched qubit in the order the
 *     reference's NoisyBackend lists them (src/Mitigation.h:146-176: {q} for 1-qubit gates,
 *     {control, target} for cnot), as in its fold/noise placement (src/Mitigation.h:183-204);
 *   - at each site two single-qubit Kraus channels, amplitude damping then phase damping
 *     (src/Noise.cpp:274-298 for the operators, src/Noise.cpp:366-372 for the AD-then-PD order);
 *   - each channel is unravelled with the jump-selection rule of the reference's trajectory
 *     solver (src/TrajectorySolver.h:421-455): no-jump branch weight `survive` = ||K0 psi||^2,
 *     jump if u1 >= survive, a second uniform r = u2 * total picks the channel (one jump
 *     operator here, so the pick is always K1), psi <- K psi / sqrt(weight);
 *   - uniforms are 53-bit doubles (x >> 11) * 2^-53 (src/Mitigation.h:207), drawn from a
 *     counter-based Philox4x32-10 stream (Salmon, Moraes, Dror, Shaw, SC'11) with
 *     key = seed and counter = (site, trajectory): one Philox call per site gives u1 and u2.
 *
 * The weights use the analytic marginals of the single-qubit channels: with P1 = P(bit q = 1),
 *   AD: survive = 1 - gamma * P1,   jump weight gamma * P1;
 *   PD: survive = 1 - lambda * P1', jump weight lambda * P1', where P1' is P1 after the AD
 *       update: (1 - gamma) P1 / survive_AD on no jump, 0 after a jump.
 * The GPU kernels evaluate exactly these expressions in FP64, so jump choices agree bit for bit
 * except on ties |u1 - survive| below the rounding of the P1 reduction; orc_traj_run returns the
 * smallest margin seen so the tests can tell a tie from a disagreement.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "sv_oracle.h"

/* Philox4x32 constants from the SC'11 paper (multipliers and Weyl key increments). */
#define PHILOX_M0 0xD2511F53u
#define PHILOX_M1 0xCD9E8D57u
#define PHILOX_W0 0x9E3779B9u
#define PHILOX_W1 0xBB67AE85u

void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
        if (r > 0) {
            k0 += PHILOX_W0;
            k1 += PHILOX_W1;
        }
        const uint64_t p0 = (uint64_t)PHILOX_M0 * c0;
        const uint64_t p1 = (uint64_t)PHILOX_M1 * c2;
        const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        const uint32_t n0 = hi1 ^ c1 ^ k0;
        const uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0;
        c1 = lo1;
        c2 = n2;
        c3 = lo0;
    }
    out[0] = c0;
    out[1] = c1;
    out[2] = c2;
    out[3] = c3;
}

void orc_uniform_pair(uint64_t seed, uint64_t traj, uint64_t site, double* u1, double* u2) {
    const uint32_t ctr[4] = {(uint32_t)site, (uint32_t)(site >> 32), (uint32_t)traj, (uint32_t)(traj >> 32)};
    const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    uint32_t o[4];
    orc_philox4x32_10(ctr, key, o);
    const uint64_t a = ((uint64_t)o[1] << 32) | o[0];
    const uint64_t b = ((uint64_t)o[3] << 32) | o[2];
    *u1 = (double)(a >> 11) * (1.0 / 9007199254740992.0);
    *u2 = (double)(b >> 11) * (1.0 / 9007199254740992.0);
}

static double p1_of(const double* psi, int n, int q) {
    const int64_t size = 1LL << n;
    const int64_t bit = 1LL << q;
    double s = 0.0;
    for (int64_t i = 0; i < size; ++i)
        if (i & bit) s += psi[2 * i] * psi[2 * i] + psi[2 * i + 1] * psi[2 * i + 1];
    return s;
}

/* One Kraus channel {K0 = diag(1, sqrt(1-g)), K1} on qubit q.  ad != 0: K1 = sqrt(g)|0><1|;
 * ad == 0: K1 = sqrt(g)|1><1|.  Returns 1 on a jump; *p1 is updated to the post-channel P1. */
static int kraus_site(double* psi, int n, int q, double g, int ad, double u1, double* p1, double* margin) {
    const int64_t size = 1LL << n;
    const int64_t bit = 1LL << q;
    const double P1 = *p1;
    const double survive = 1.0 - g * P1;
    const double total = g * P1;
    const double m = fabs(u1 - survive);
    if (m < *margin) *margin = m;
    if (u1 >= survive && total > 0.0) {
        const double inv = 1.0 / sqrt(P1);
        for (int64_t i = 0; i < size; ++i) {
            if (i & bit) continue;
            double* a0 = psi + 2 * i;
            double* a1 = psi + 2 * (i | bit);
            if (ad) {
                a0[0] = a1[0] * inv;
                a0[1] = a1[1] * inv;
            } else {
                a0[0] = 0.0;
                a0[1] = 0.0;
                a1[0] = a1[0] * inv;
                a1[1] = a1[1] * inv;
                continue;
            }
            a1[0] = 0.0;
            a1[1] = 0.0;
        }
        *p1 = ad ? 0.0 : 1.0;
        return 1;
    }
    const double s0 = 1.0 / sqrt(survive);
    const double s1 = sqrt(1.0 - g) * s0;
    for (int64_t i = 0; i < size; ++i) {
        if (i & bit) continue;
        double* a0 = psi + 2 * i;
        double* a1 = psi + 2 * (i | bit);
        a0[0] *= s0;
        a0[1] *= s0;
        a1[0] *= s1;
        a1[1] *= s1;
    }
    *p1 = (1.0 - g) * P1 / survive;
    return 0;
}

/* Touched qubits of a gate, in noise-site order: its qubit for 1-qubit gates, control then target
 * for cnot / cz, and every listed qubit in increasing order for mcz (src/Mitigation.h:196-204
 * puts one single-qubit site on each qubit of a gate wider than two). */
static int touched(const orc_op* op, int qs[64]) {
    if (op->kind == ORC_OP_CNOT || op->kind == ORC_OP_CZ) {
        qs[0] = op->q0;
        qs[1] = op->q1;
        return 2;
    }
    if (op->kind == ORC_OP_MCZ) {
        int k = 0;
        for (int q = 0; q < 64; ++q)
            if (op->mask >> q & 1) qs[k++] = q;
        return k;
    }
    qs[0] = op->q0;
    return 1;
}

/* Runs trajectories [traj_begin, traj_end).  z0_out[t] = <Z_0> of trajectory t's final state;
 * jump_counts[t] = number of jumps; jump_log (optional) gets one byte per site and trajectory:
 * bit 0 = AD jumped, bit 1 = PD jumped.  margin_out = min |u1 - survive| over all draws. */
int orc_traj_run(int n, const orc_op* ops, int nops, double gamma_ad, double lambda_pd, uint64_t seed,
                 uint64_t traj_begin, uint64_t traj_end, double* z0_out, uint32_t* jump_counts,
                 uint8_t* jump_log, int64_t jump_log_stride, double* margin_out) {
    if (n < 1 || n > 24) return ORC_EINVAL;
    const int64_t size = 1LL << n;
    /* validate the circuit once, serially, on a scratch state */
    {
        double* scratch = (double*)malloc(sizeof(double) * 2 * (size_t)size);
        if (!scratch) return ORC_ENOMEM;
        orc_init_zero(scratch, n);
        const int rc = orc_run_ops(scratch, n, ops, nops);
        free(scratch);
        if (rc) return rc;
    }
    double margin = 1.0;
    int failed = 0;
    /* trajectories are independent: spread them over the host threads, as the reference's
     * trajectory solver does (src/TrajectorySolver.h:211-229); each trajectory's state is small
     * enough that its own loops run single-threaded */
#pragma omp parallel
    {
        double* psi = (double*)malloc(sizeof(double) * 2 * (size_t)size);
        double local_margin = 1.0;
        if (!psi) {
#pragma omp atomic write
            failed = 1;
        }
#pragma omp for schedule(dynamic, 4)
        for (int64_t tt = (int64_t)traj_begin; tt < (int64_t)traj_end; ++tt) {
            if (!psi) continue;
            const uint64_t t = (uint64_t)tt;
            orc_init_zero(psi, n);
            uint64_t site = 0;
            uint32_t jumps = 0;
            for (int g = 0; g < nops; ++g) {
                orc_apply_op(psi, n, &ops[g]);
                int qs[64];
                const int nq = touched(&ops[g], qs);
                for (int k = 0; k < nq; ++k) {
                    double p1 = p1_of(psi, n, qs[k]);
                    double u1, u2;
                    uint8_t code = 0;
                    orc_uniform_pair(seed, t, site, &u1, &u2);
                    if (kraus_site(psi, n, qs[k], gamma_ad, 1, u1, &p1, &local_margin)) code |= 1;
                    ++site;
                    orc_uniform_pair(seed, t, site, &u1, &u2);
                    if (kraus_site(psi, n, qs[k], lambda_pd, 0, u1, &p1, &local_margin)) code |= 2;
                    ++site;
                    jumps += (code & 1) + (code >> 1);
                    if (jump_log) jump_log[(int64_t)(t - traj_begin) * jump_log_stride + (int64_t)(site / 2 - 1)] = code;
                }
            }
            double z = 0.0;
            for (int64_t i = 0; i < size; ++i) {
                const double p = psi[2 * i] * psi[2 * i] + psi[2 * i + 1] * psi[2 * i + 1];
                z += (i & 1) ? -p : p;
            }
            z0_out[t - traj_begin] = z;
            if (jump_counts) jump_counts[t - traj_begin] = jumps;
        }
#pragma omp critical
        {
            if (local_margin < margin) margin = local_margin;
        }
        free(psi);
    }
    if (failed) return ORC_ENOMEM;
    if (margin_out) *margin_out = margin;
    return 0;
}

/* Exact density-matrix evolution of the same noisy circuit for small n (the mean the trajectory
 * ensemble estimates).  rho is stored as a 2n-qubit vector: row index in the low n bits, column
 * index in the high n bits; U rho U^+ is U on qubit q and conj(U) on qubit n + q.  The Kraus
 * channels follow src/Noise.cpp:174-258 (rho <- sum_k K rho K^+) with the operators of
 * src/Noise.cpp:274-298. */
static void apply_2x2(double* v, int nn, int q, const double* u) {
    orc_apply_gate_v3(v, nn, q, u);
}

static void conj2(const double* u, double* c) {
    for (int i = 0; i < 4; ++i) {
        c[2 * i] = u[2 * i];
        c[2 * i + 1] = -u[2 * i + 1];
    }
}

static void gate_matrix(const orc_op* op, double* u) {
    memset(u, 0, 8 * sizeof(double));
    const double c = cos(0.5 * op->theta), s = sin(0.5 * op->theta);
    const double r = 1.0 / sqrt(2.0);
    switch (op->kind) {
        case ORC_OP_H: u[0] = r; u[2] = r; u[4] = r; u[6] = -r; break;
        case ORC_OP_X: u[2] = 1; u[4] = 1; break;
        case ORC_OP_RX: u[0] = c; u[3] = -s; u[5] = -s; u[6] = c; break;
        case ORC_OP_RY: u[0] = c; u[2] = -s; u[4] = s; u[6] = c; break;
        case ORC_OP_RZ: u[0] = c; u[1] = -s; u[6] = c; u[7] = s; break;
        default: memcpy(u, op->m, 8 * sizeof(double)); break;
    }
}

static int channel(double* rho, double* tmp, double* acc, int n, int q, double g, int ad) {
    const int nn = 2 * n;
    const int64_t len = 2 * (1LL << nn);
    double k0[8] = {1, 0, 0, 0, 0, 0, sqrt(1.0 - g), 0};
    double k1[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (ad) k1[2] = sqrt(g); /* sqrt(g)|0><1| : row 0, col 1 */
    else k1[6] = sqrt(g);    /* sqrt(g)|1><1| */
    double c[8];
    memcpy(tmp, rho, sizeof(double) * (size_t)len);
    apply_2x2(tmp, nn, q, k0);
    conj2(k0, c);
    apply_2x2(tmp, nn, n + q, c);
    memcpy(acc, tmp, sizeof(double) * (size_t)len);
    memcpy(tmp, rho, sizeof(double) * (size_t)len);
    apply_2x2(tmp, nn, q, k1);
    conj2(k1, c);
    apply_2x2(tmp, nn, n + q, c);
    for (int64_t i = 0; i < len; ++i) rho[i] = acc[i] + tmp[i];
    return 0;
}

int orc_density_z0(int n, const orc_op* ops, int nops, double gamma_ad, double lambda_pd, double* z0_out) {
    if (n < 1 || n > 8) return ORC_EINVAL;
    const int nn = 2 * n;
    const int64_t dim = 1LL << n;
    const int64_t len = 2 * (1LL << nn);
    double* rho = (double*)calloc((size_t)len, sizeof(double));
    double* tmp = (double*)malloc(sizeof(double) * (size_t)len);
    double* acc = (double*)malloc(sizeof(double) * (size_t)len);
    if (!rho || !tmp || !acc) {
        free(rho);
        free(tmp);
        free(acc);
        return ORC_ENOMEM;
    }
    rho[0] = 1.0;
    for (int g = 0; g < nops; ++g) {
        const orc_op* op = &ops[g];
        if (op->kind == ORC_OP_CNOT) {
            orc_cnot(rho, nn, op->q0, op->q1);
            orc_cnot(rho, nn, n + op->q0, n + op->q1);
        } else if (op->kind == ORC_OP_CZ) {
            const int qa[2] = {op->q0, op->q1}, qb[2] = {n + op->q0, n + op->q1};
            orc_mcz_list(rho, nn, qa, 2);
            orc_mcz_list(rho, nn, qb, 2);
        } else {
            double u[8], c[8];
            gate_matrix(op, u);
            apply_2x2(rho, nn, op->q0, u);
            conj2(u, c);
            apply_2x2(rho, nn, n + op->q0, c);
        }
        int qs[64];
        const int nq = touched(op, qs);
        for (int k = 0; k < nq; ++k) {
            channel(rho, tmp, acc, n, qs[k], gamma_ad, 1);
            channel(rho, tmp, acc, n, qs[k], lambda_pd, 0);
        }
    }
    double z = 0.0;
    for (int64_t i = 0; i < dim; ++i) {
        const double p = rho[2 * (i + i * dim)];
        z += (i & 1) ? -p : p;
    }
    *z0_out = z;
    free(rho);
    free(tmp);
    free(acc);
    return 0;
}
