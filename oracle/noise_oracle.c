/*
 * noise_oracle.c -- the ORACLE for depolarizing-noise trajectories with gate folding and
 * zero-noise extrapolation (test infrastructure only).
 *
 * Restates the reference's NoisyBackend and ZNE (src/Mitigation.h):
 *   - folding: every logical gate U runs as U (U^+ U)^k for scale 2k + 1, with a noise site after
 *     every application (src/Mitigation.h:184-196); inverses are R(-t) for rotations, the
 *     adjoint for a generic 2x2, and the gate itself for H, X, CNOT, CZ and MCZ;
 *   - noise sites (src/Mitigation.h:198-205): 1-qubit gates one 1-qubit channel; cnot and
 *     2-qubit mcz one 2-qubit channel over (first, second) qubit; wider mcz one 1-qubit channel
 *     per qubit in increasing order;
 *   - a site draws u; u >= p does nothing; otherwise a second uniform u2 picks the Pauli:
 *     1 + floor(3 u2) in {X, Y, Z} for one qubit (src/Mitigation.h:210-213); 1 + floor(15 u2)
 *     for two, low two bits on the first qubit, high two on the second (:216-221);
 *     X = x(q), Z = mcz({q}), Y = Z then X (:224-241);
 *   - ZNE (src/Mitigation.h:313-377): per scale, `trajectories` runs from |0..0>, Welford mean
 *     and standard error sigma / sqrt(N) (NaN when p > 0 and N = 1, 0 when p = 0, where one
 *     run is used), Richardson weights c_k = prod_{j != k} l_j / (l_j - l_k) (:287-301), value
 *     sum c_k E_k and error sqrt(sum c_k^2 se_k^2).
 * Uniforms are 53-bit doubles (x >> 11) * 2^-53 (src/Mitigation.h:207).  Two streams:
 *   ORC_RNG_MT     -- the reference's: one MT19937-64 engine seeded once (std::mt19937_64,
 *                     Matsumoto and Nishimura, ACM TOMACS 2000 / the 64-bit variant of 2004),
 *                     drawn sequentially across sites, trajectories and scales, u2 only when
 *                     u < p.  Used to pin this restatement against the reference's own build.
 *   ORC_RNG_PHILOX -- the GPU engine's: Philox4x32-10 with key = seed and counter = (site,
 *                     trajectory); one call per site gives u (low 64 bits) and u2 (high 64
 *                     bits); scale k of a ZNE run uses trajectories [k N, (k + 1) N).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "sv_oracle.h"

/* ---- MT19937-64 (the published 64-bit Mersenne Twister) ---- */
#define MT_N 312
#define MT_M 156
#define MT_MATRIX_A 0xB5026F5AA96619E9ULL
#define MT_UPPER 0xFFFFFFFF80000000ULL
#define MT_LOWER 0x7FFFFFFFULL

typedef struct {
    uint64_t mt[MT_N];
    int idx;
} mt64;

static void mt64_seed(mt64* g, uint64_t seed) {
    g->mt[0] = seed;
    for (int i = 1; i < MT_N; ++i) g->mt[i] = 6364136223846793005ULL * (g->mt[i - 1] ^ (g->mt[i - 1] >> 62)) + (uint64_t)i;
    g->idx = MT_N;
}

static uint64_t mt64_next(mt64* g) {
    if (g->idx >= MT_N) {
        for (int i = 0; i < MT_N; ++i) {
            const uint64_t x = (g->mt[i] & MT_UPPER) | (g->mt[(i + 1) % MT_N] & MT_LOWER);
            uint64_t xa = x >> 1;
            if (x & 1ULL) xa ^= MT_MATRIX_A;
            g->mt[i] = g->mt[(i + MT_M) % MT_N] ^ xa;
        }
        g->idx = 0;
    }
    uint64_t x = g->mt[g->idx++];
    x ^= (x >> 29) & 0x5555555555555555ULL;
    x ^= (x << 17) & 0x71D67FFFEDA60000ULL;
    x ^= (x << 37) & 0xFFF7EEE000000000ULL;
    x ^= x >> 43;
    return x;
}

static double mt64_u01(mt64* g) { return (double)(mt64_next(g) >> 11) * (1.0 / 9007199254740992.0); }

uint64_t orc_mt64_first(uint64_t seed, int k) {
    mt64 g;
    mt64_seed(&g, seed);
    uint64_t x = 0;
    for (int i = 0; i <= k; ++i) x = mt64_next(&g);
    return x;
}

/* ---- one trajectory ---- */
typedef struct {
    int kind; /* ORC_RNG_* */
    mt64* mt;
    uint64_t seed, traj, site;
} noise_rng;

/* the site's u (and, for Philox, its u2 from the same call); the MT stream draws u2 separately, only when u < p */
static double draw_u(noise_rng* r, double* u2_philox) {
    if (r->kind == ORC_RNG_PHILOX) {
        double u1, u2;
        orc_uniform_pair(r->seed, r->traj, r->site, &u1, &u2);
        *u2_philox = u2;
        return u1;
    }
    return mt64_u01(r->mt);
}

static double draw_u2(noise_rng* r, double u2_philox) {
    return r->kind == ORC_RNG_PHILOX ? u2_philox : mt64_u01(r->mt);
}

static void pauli(double* psi, int n, int q, int which) {
    if (which == 2 || which == 3) orc_mcz_mask(psi, n, 1ULL << q);
    if (which == 1 || which == 2) orc_x(psi, n, q);
}

/* returns the number of non-identity Paulis applied at this site (0 or 1) */
static int depolarize1(double* psi, int n, int q, double p, noise_rng* r) {
    double u2p = 0.0;
    const double u = draw_u(r, &u2p);
    ++r->site;
    if (u >= p) return 0;
    pauli(psi, n, q, 1 + (int)(draw_u2(r, u2p) * 3.0));
    return 1;
}

static int depolarize2(double* psi, int n, int a, int b, double p, noise_rng* r) {
    double u2p = 0.0;
    const double u = draw_u(r, &u2p);
    ++r->site;
    if (u >= p) return 0;
    const int idx = 1 + (int)(draw_u2(r, u2p) * 15.0);
    pauli(psi, n, a, idx & 3);
    pauli(psi, n, b, idx >> 2);
    return 1;
}

static int noise_after(double* psi, int n, const orc_op* op, double p, noise_rng* r) {
    if (p == 0.0) return 0; /* src/Mitigation.h:199: no draw at all */
    if (op->kind == ORC_OP_CNOT || op->kind == ORC_OP_CZ) return depolarize2(psi, n, op->q0, op->q1, p, r);
    if (op->kind == ORC_OP_MCZ) {
        int qs[64], k = 0;
        for (int q = 0; q < 64; ++q)
            if (op->mask >> q & 1) qs[k++] = q;
        if (k == 1) return depolarize1(psi, n, qs[0], p, r);
        if (k == 2) return depolarize2(psi, n, qs[0], qs[1], p, r);
        int c = 0;
        for (int i = 0; i < k; ++i) c += depolarize1(psi, n, qs[i], p, r);
        return c;
    }
    return depolarize1(psi, n, op->q0, p, r);
}

static orc_op inverse_of(const orc_op* op) {
    orc_op v = *op;
    if (op->kind == ORC_OP_RX || op->kind == ORC_OP_RY || op->kind == ORC_OP_RZ) v.theta = -op->theta;
    if (op->kind == ORC_OP_U2) { /* adjoint: (g^+)_{rc} = conj(g_{cr}) */
        for (int r = 0; r < 2; ++r)
            for (int c = 0; c < 2; ++c) {
                v.m[2 * (2 * r + c)] = op->m[2 * (2 * c + r)];
                v.m[2 * (2 * r + c) + 1] = -op->m[2 * (2 * c + r) + 1];
            }
    }
    return v;
}

static int run_folded(double* psi, int n, const orc_op* ops, int nops, double p, int folds, noise_rng* r) {
    int paulis = 0;
    orc_init_zero(psi, n);
    for (int g = 0; g < nops; ++g) {
        const orc_op inv = inverse_of(&ops[g]);
        orc_apply_op(psi, n, &ops[g]);
        paulis += noise_after(psi, n, &ops[g], p, r);
        for (int f = 0; f < folds; ++f) {
            orc_apply_op(psi, n, &inv);
            paulis += noise_after(psi, n, &ops[g], p, r);
            orc_apply_op(psi, n, &ops[g]);
            paulis += noise_after(psi, n, &ops[g], p, r);
        }
    }
    return paulis;
}

static int check_circuit(int n, const orc_op* ops, int nops) {
    double* scratch = (double*)malloc(sizeof(double) * 2 * ((size_t)1 << n));
    if (!scratch) return ORC_ENOMEM;
    orc_init_zero(scratch, n);
    const int rc = orc_run_ops(scratch, n, ops, nops);
    free(scratch);
    return rc;
}

/* Observable sum_k coeff[k] Z_a[k] Z_b[k] (b < 0: Z_a alone) of trajectories
 * [traj_begin, traj_end) at fold scale `scale` (odd).  rng = ORC_RNG_PHILOX runs them in parallel
 * with per-(site, trajectory) uniforms; ORC_RNG_MT runs them in order on one engine seeded with
 * `seed`.  paulis_out (optional): non-identity Paulis applied per trajectory. */
int orc_noisy_run(int n, const orc_op* ops, int nops, double p, int scale, int rng, uint64_t seed, uint64_t traj_begin,
                  uint64_t traj_end, int nterms, const int* za, const int* zb, const double* zc, double* obs_out,
                  uint32_t* paulis_out) {
    if (n < 1 || n > 24 || !(p >= 0.0 && p <= 1.0) || scale < 1 || scale % 2 == 0) return ORC_EINVAL;
    int rc = check_circuit(n, ops, nops);
    if (rc) return rc;
    const size_t amps = (size_t)1 << n;
    const int folds = (scale - 1) / 2;
    if (rng == ORC_RNG_MT) {
        double* psi = (double*)malloc(sizeof(double) * 2 * amps);
        mt64* g = (mt64*)malloc(sizeof(mt64));
        if (!psi || !g) {
            free(psi);
            free(g);
            return ORC_ENOMEM;
        }
        mt64_seed(g, seed);
        noise_rng r = {ORC_RNG_MT, g, seed, 0, 0};
        for (uint64_t t = traj_begin; t < traj_end; ++t) {
            const int c = run_folded(psi, n, ops, nops, p, folds, &r);
            obs_out[t - traj_begin] = orc_expect_zz(psi, n, nterms, za, zb, zc);
            if (paulis_out) paulis_out[t - traj_begin] = (uint32_t)c;
        }
        free(psi);
        free(g);
        return 0;
    }
    int failed = 0;
#pragma omp parallel
    {
        double* psi = (double*)malloc(sizeof(double) * 2 * amps);
        if (!psi) {
#pragma omp atomic write
            failed = 1;
        }
#pragma omp for schedule(dynamic, 4)
        for (int64_t tt = (int64_t)traj_begin; tt < (int64_t)traj_end; ++tt) {
            if (!psi) continue;
            noise_rng r = {ORC_RNG_PHILOX, NULL, seed, (uint64_t)tt, 0};
            const int c = run_folded(psi, n, ops, nops, p, folds, &r);
            obs_out[(uint64_t)tt - traj_begin] = orc_expect_zz(psi, n, nterms, za, zb, zc);
            if (paulis_out) paulis_out[(uint64_t)tt - traj_begin] = (uint32_t)c;
        }
        free(psi);
    }
    return failed ? ORC_ENOMEM : 0;
}

/* Richardson weights (src/Mitigation.h:287-301).  Returns ORC_EINVAL on fewer than 2 scales or
 * a zero, non-finite or repeated scale. */
int orc_richardson_weights(const double* scales, int ns, double* w) {
    if (ns < 2) return ORC_EINVAL;
    for (int k = 0; k < ns; ++k)
        if (!isfinite(scales[k]) || scales[k] == 0.0) return ORC_EINVAL;
    for (int k = 0; k < ns; ++k) {
        w[k] = 1.0;
        for (int j = 0; j < ns; ++j) {
            if (j == k) continue;
            if (scales[j] == scales[k]) return ORC_EINVAL;
            w[k] *= scales[j] / (scales[j] - scales[k]);
        }
    }
    return 0;
}

/* ZNE::extrapolate over the folded noisy circuit.  out (4 * ns + 3 doubles): value, std_error,
 * trajectories used, then values[ns], std_errors[ns], weights[ns], scales[ns]. */
int orc_zne(int n, const orc_op* ops, int nops, double p, const double* scales, int ns, int trajectories, int rng,
            uint64_t seed, int nterms, const int* za, const int* zb, const double* zc, double* out) {
    if (trajectories < 1 || ns < 2 || ns > 8) return ORC_EINVAL;
    for (int k = 0; k < ns; ++k) {
        const double s = scales[k];
        if (!isfinite(s) || s < 1.0 || s > 99.0 || s != floor(s) || fmod(s, 2.0) != 1.0) return ORC_EINVAL;
        for (int j = 0; j < k; ++j)
            if (scales[j] == s) return ORC_EINVAL;
    }
    double* w = out + 3 + 2 * ns;
    int rc = orc_richardson_weights(scales, ns, w);
    if (rc) return rc;
    if (nops < 1) return ORC_ERUNTIME; /* "circuit_fn applied no gates", src/Mitigation.h:342-343 */
    rc = check_circuit(n, ops, nops);
    if (rc) return rc;
    const int noisy = p > 0.0;
    const int nt = noisy ? trajectories : 1;
    double* vals = (double*)malloc(sizeof(double) * (size_t)nt);
    mt64* g = (mt64*)malloc(sizeof(mt64));
    double* psi = (double*)malloc(sizeof(double) * 2 * ((size_t)1 << n));
    if (!vals || !g || !psi) {
        free(vals);
        free(g);
        free(psi);
        return ORC_ENOMEM;
    }
    mt64_seed(g, seed);
    double value = 0.0, var = 0.0;
    for (int k = 0; k < ns; ++k) {
        const int scale = (int)scales[k];
        if (rng == ORC_RNG_MT) {
            noise_rng r = {ORC_RNG_MT, g, seed, 0, 0};
            for (int t = 0; t < nt; ++t) {
                run_folded(psi, n, ops, nops, p, (scale - 1) / 2, &r);
                vals[t] = orc_expect_zz(psi, n, nterms, za, zb, zc);
            }
        } else {
            rc = orc_noisy_run(n, ops, nops, p, scale, ORC_RNG_PHILOX, seed, (uint64_t)k * (uint64_t)nt,
                               (uint64_t)(k + 1) * (uint64_t)nt, nterms, za, zb, zc, vals, NULL);
            if (rc) break;
        }
        double mean = 0.0, m2 = 0.0; /* Welford, as src/Mitigation.h:350-353 */
        for (int t = 0; t < nt; ++t) {
            const double d = vals[t] - mean;
            mean += d / (t + 1);
            m2 += d * (vals[t] - mean);
        }
        double se = 0.0;
        if (nt > 1) se = sqrt(fmax(0.0, m2 / (nt - 1)) / nt);
        else if (noisy) se = NAN;
        out[3 + k] = mean;
        out[3 + ns + k] = se;
        out[3 + 3 * ns + k] = scales[k];
    }
    free(vals);
    free(g);
    free(psi);
    if (rc) return rc;
    for (int k = 0; k < ns; ++k) {
        value += w[k] * out[3 + k];
        var += w[k] * w[k] * out[3 + ns + k] * out[3 + ns + k];
    }
    out[0] = value;
    out[1] = sqrt(var);
    out[2] = nt;
    return 0;
}
