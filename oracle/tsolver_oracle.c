/*
 * tsolver_oracle.c -- the ORACLE for the dense trajectory solver (test infrastructure only).
 *
 * Restates the reference's TrajectorySolver (src/TrajectorySolver.h):
 *   - exp(A) by scaling and squaring with an 18-term Taylor series, ||A / 2^s||_inf <= 1/2
 *     (:95-110);
 *   - the plan (:400-441): steps = max(1, ceil(duration / dt - 1e-9)), h = duration / steps;
 *     jump operators sqrt(gamma) L, or sqrt(g) (1 - P) for Pauli-like channels under PROJECTOR
 *     (L Hermitian with L^2 = c 1: P = L / sqrt(c), g = gamma c, :363-373); H_eff = H - i/2 sum
 *     J^+ J for the jump unravelings; constant H: one propagator exp(-i H_eff h); time-dependent
 *     H: nodes -i (H(t) + hnh) at t = j h / 2 (jumps, RK4) or t = j h (ANALOG);
 *   - the norm-loss jump step (:443-486): survive = |psi~|^2, jump if u1 >= survive, channel
 *     weights |J_k psi~|^2, r = u2 * total picks the first k with r < acc and w_k > 0 (last
 *     positive weight on rounding), psi <- J psi~ / sqrt(w); else psi~ / sqrt(survive);
 *   - the diffusive step (:489-514), Euler-Maruyama with renormalisation.
 * Uniforms: Philox4x32-10 with key = seed, counter = (draw, trajectory); step s of a jump
 * unraveling uses draw s (u1 from the low 64 bits; u2 for the channel pick from the high 64
 * bits); the diffusive step s draws channel k's Wiener increment from draw s * nch + k by
 * Box-Muller (sqrt(-2 ln u1) cos(2 pi u2), u1 taken in (0, 1]) scaled by sqrt(h).  The reference
 * draws from per-trajectory mt19937_64 streams instead; the two agree in distribution.
 *
 * Matrices are dim x dim complex, row-major, interleaved (re, im).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "sv_oracle.h"

typedef struct {
    double re, im;
} cpx;

/* C = A B (dim x dim) */
static void matmul(const cpx* a, const cpx* b, cpx* c, int d) {
    for (int i = 0; i < d; ++i)
        for (int j = 0; j < d; ++j) {
            double sr = 0.0, si = 0.0;
            for (int k = 0; k < d; ++k) {
                const cpx x = a[i * d + k], y = b[k * d + j];
                sr += x.re * y.re - x.im * y.im;
                si += x.re * y.im + x.im * y.re;
            }
            c[i * d + j] = (cpx){sr, si};
        }
}

int orc_expm(const double* ain, int d, double* out) {
    const cpx* a = (const cpx*)ain;
    cpx* res = (cpx*)out;
    double nrm = 0.0;
    for (int i = 0; i < d; ++i) {
        double row = 0.0;
        for (int j = 0; j < d; ++j) row += hypot(a[i * d + j].re, a[i * d + j].im);
        if (row > nrm) nrm = row;
    }
    int s = 0;
    if (nrm > 0.5) s = (int)fmax(0.0, ceil(log2(nrm / 0.5)));
    const double scale = pow(2.0, s);
    cpx* b = (cpx*)malloc(sizeof(cpx) * (size_t)d * d);
    cpx* term = (cpx*)malloc(sizeof(cpx) * (size_t)d * d);
    cpx* tmp = (cpx*)malloc(sizeof(cpx) * (size_t)d * d);
    if (!b || !term || !tmp) {
        free(b);
        free(term);
        free(tmp);
        return ORC_ENOMEM;
    }
    for (int i = 0; i < d * d; ++i) b[i] = (cpx){a[i].re / scale, a[i].im / scale};
    for (int i = 0; i < d * d; ++i) term[i] = res[i] = (cpx){(i / d == i % d) ? 1.0 : 0.0, 0.0};
    for (int k = 1; k <= 18; ++k) {
        matmul(term, b, tmp, d);
        for (int i = 0; i < d * d; ++i) {
            term[i] = (cpx){tmp[i].re / k, tmp[i].im / k};
            res[i].re += term[i].re;
            res[i].im += term[i].im;
        }
    }
    for (int i = 0; i < s; ++i) {
        matmul(res, res, tmp, d);
        memcpy(res, tmp, sizeof(cpx) * (size_t)d * d);
    }
    free(b);
    free(term);
    free(tmp);
    return 0;
}

/* y = A x */
static void matvec(const cpx* a, const cpx* x, cpx* y, int d) {
    for (int i = 0; i < d; ++i) {
        double sr = 0.0, si = 0.0;
        for (int k = 0; k < d; ++k) {
            const cpx m = a[i * d + k];
            sr += m.re * x[k].re - m.im * x[k].im;
            si += m.re * x[k].im + m.im * x[k].re;
        }
        y[i] = (cpx){sr, si};
    }
}

static double norm2(const cpx* x, int d) {
    double s = 0.0;
    for (int i = 0; i < d; ++i) s += x[i].re * x[i].re + x[i].im * x[i].im;
    return s;
}

static double gauss(uint64_t seed, uint64_t traj, uint64_t draw) {
    double u1, u2;
    orc_uniform_pair(seed, traj, draw, &u1, &u2);
    u1 = 1.0 - u1; /* (0, 1] */
    return sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
}

/* One trajectory per index in [traj_begin, traj_end) from psi0 (normalised by the caller).
 *   kind 0 STANDARD, 1 PROJECTOR, 2 ANALOG (the plan's jump operators already reflect it);
 *   constant: prop (dim x dim) is exp(-i H_eff h) (jump kinds) or exp(-i H h) (ANALOG);
 *   otherwise nodes (n_nodes x dim x dim) hold -i (H(t_j) + hnh).
 * ops / ops_dop: nch operators J_k and J_k^+ J_k.  states_out: (traj_end - traj_begin) x dim. */
int orc_tsolver_run(int d, int kind, long long steps, double h, int constant, const double* prop, const double* nodes,
                    int nch, const double* ops, const double* ops_dop, const double* psi0, uint64_t seed,
                    uint64_t traj_begin, uint64_t traj_end, double* states_out) {
    const cpx* P = (const cpx*)prop;
    const cpx* N = (const cpx*)nodes;
    const cpx* J = (const cpx*)ops;
    const cpx* JJ = (const cpx*)ops_dop;
    const size_t dd = (size_t)d * d;
    int failed = 0;
#pragma omp parallel
    {
        cpx* psi = (cpx*)malloc(sizeof(cpx) * d);
        cpx* tmp = (cpx*)malloc(sizeof(cpx) * d);
        cpx* w = (cpx*)malloc(sizeof(cpx) * d);
        cpx* k1 = (cpx*)malloc(sizeof(cpx) * d);
        cpx* k2 = (cpx*)malloc(sizeof(cpx) * d);
        cpx* k3 = (cpx*)malloc(sizeof(cpx) * d);
        cpx* k4 = (cpx*)malloc(sizeof(cpx) * d);
        cpx* drift = (cpx*)malloc(sizeof(cpx) * d);
        cpx* noise = (cpx*)malloc(sizeof(cpx) * d);
        double* weight = (double*)malloc(sizeof(double) * (size_t)(nch > 0 ? nch : 1));
        if (!psi || !tmp || !w || !k1 || !k2 || !k3 || !k4 || !drift || !noise || !weight) {
#pragma omp atomic write
            failed = ORC_ENOMEM;
        }
#pragma omp for schedule(dynamic, 4)
        for (int64_t tt = (int64_t)traj_begin; tt < (int64_t)traj_end; ++tt) {
            if (failed) continue;
            const uint64_t t = (uint64_t)tt;
            memcpy(psi, psi0, sizeof(cpx) * d);
            for (long long s = 0; s < steps && !failed; ++s) {
                if (kind == 2) {
                    if (constant) {
                        matvec(P, psi, tmp, d);
                        memcpy(psi, tmp, sizeof(cpx) * d);
                        memset(drift, 0, sizeof(cpx) * d);
                    } else {
                        matvec(N + (size_t)s * dd, psi, drift, d);
                    }
                    memset(noise, 0, sizeof(cpx) * d);
                    for (int k = 0; k < nch; ++k) {
                        matvec(J + (size_t)k * dd, psi, w, d); /* cp */
                        double x = 0.0;
                        for (int i = 0; i < d; ++i) x += psi[i].re * w[i].re + psi[i].im * w[i].im;
                        x *= 2.0; /* <C + C^+> = 2 Re <psi|C psi> */
                        matvec(JJ + (size_t)k * dd, psi, k1, d); /* t2 */
                        const double dw = sqrt(h) * gauss(seed, t, (uint64_t)s * (uint64_t)nch + (uint64_t)k);
                        for (int i = 0; i < d; ++i) {
                            drift[i].re += -0.5 * (k1[i].re - x * w[i].re + 0.25 * x * x * psi[i].re);
                            drift[i].im += -0.5 * (k1[i].im - x * w[i].im + 0.25 * x * x * psi[i].im);
                            noise[i].re += (w[i].re - 0.5 * x * psi[i].re) * dw;
                            noise[i].im += (w[i].im - 0.5 * x * psi[i].im) * dw;
                        }
                    }
                    for (int i = 0; i < d; ++i) {
                        psi[i].re += h * drift[i].re + noise[i].re;
                        psi[i].im += h * drift[i].im + noise[i].im;
                    }
                    const double nrm = sqrt(norm2(psi, d));
                    if (!(nrm > 0.0) || !isfinite(nrm)) {
#pragma omp atomic write
                        failed = ORC_ERUNTIME;
                        break;
                    }
                    for (int i = 0; i < d; ++i) {
                        psi[i].re /= nrm;
                        psi[i].im /= nrm;
                    }
                    continue;
                }
                if (constant) {
                    matvec(P, psi, tmp, d);
                } else {
                    const cpx* a0 = N + (size_t)(2 * s) * dd;
                    const cpx* a1 = N + (size_t)(2 * s + 1) * dd;
                    const cpx* a2 = N + (size_t)(2 * s + 2) * dd;
                    matvec(a0, psi, k1, d);
                    for (int i = 0; i < d; ++i) w[i] = (cpx){psi[i].re + 0.5 * h * k1[i].re, psi[i].im + 0.5 * h * k1[i].im};
                    matvec(a1, w, k2, d);
                    for (int i = 0; i < d; ++i) w[i] = (cpx){psi[i].re + 0.5 * h * k2[i].re, psi[i].im + 0.5 * h * k2[i].im};
                    matvec(a1, w, k3, d);
                    for (int i = 0; i < d; ++i) w[i] = (cpx){psi[i].re + h * k3[i].re, psi[i].im + h * k3[i].im};
                    matvec(a2, w, k4, d);
                    for (int i = 0; i < d; ++i) {
                        tmp[i].re = psi[i].re + (h / 6.0) * (k1[i].re + 2.0 * k2[i].re + 2.0 * k3[i].re + k4[i].re);
                        tmp[i].im = psi[i].im + (h / 6.0) * (k1[i].im + 2.0 * k2[i].im + 2.0 * k3[i].im + k4[i].im);
                    }
                }
                const double survive = norm2(tmp, d);
                if (!(survive > 0.0) || !isfinite(survive)) {
#pragma omp atomic write
                    failed = ORC_ERUNTIME;
                    break;
                }
                double u1, u2;
                orc_uniform_pair(seed, t, (uint64_t)s, &u1, &u2);
                int jumped = 0;
                if (nch > 0 && u1 >= survive) {
                    double total = 0.0;
                    for (int k = 0; k < nch; ++k) {
                        matvec(J + (size_t)k * dd, tmp, w, d);
                        weight[k] = norm2(w, d);
                        total += weight[k];
                    }
                    if (total > 0.0) {
                        const double r = u2 * total;
                        int pick = nch;
                        double acc = 0.0;
                        for (int k = 0; k < nch; ++k) {
                            acc += weight[k];
                            if (r < acc && weight[k] > 0.0) {
                                pick = k;
                                break;
                            }
                        }
                        if (pick == nch)
                            for (int k = nch - 1; k >= 0; --k)
                                if (weight[k] > 0.0) {
                                    pick = k;
                                    break;
                                }
                        matvec(J + (size_t)pick * dd, tmp, psi, d);
                        const double inv = 1.0 / sqrt(weight[pick]);
                        for (int i = 0; i < d; ++i) {
                            psi[i].re *= inv;
                            psi[i].im *= inv;
                        }
                        jumped = 1;
                    }
                }
                if (!jumped) {
                    const double inv = 1.0 / sqrt(survive);
                    for (int i = 0; i < d; ++i) psi[i] = (cpx){tmp[i].re * inv, tmp[i].im * inv};
                }
            }
            memcpy(states_out + (size_t)2 * d * (t - traj_begin), psi, sizeof(cpx) * d);
        }
        free(psi);
        free(tmp);
        free(w);
        free(k1);
        free(k2);
        free(k3);
        free(k4);
        free(drift);
        free(noise);
        free(weight);
    }
    return failed;
}

/* Exact density-matrix integration of the Lindblad equation by RK4 (the reference's own check,
 * src/TrajectorySolver.h:547-575): d rho/dt = -i [H, rho] + sum_k g_k (L rho L^+ - {L^+L, rho}/2),
 * constant H.  ls: nch operators L_k (not scaled), gs: rates. */
static void lindblad_rhs(const cpx* H, int nch, const cpx* L, const double* g, const cpx* rho, cpx* out, cpx* t1,
                         cpx* t2, int d) {
    const size_t dd = (size_t)d * d;
    /* -i (H rho - rho H) */
    matmul(H, rho, t1, d);
    matmul(rho, H, t2, d);
    for (size_t i = 0; i < dd; ++i) out[i] = (cpx){t1[i].im - t2[i].im, -(t1[i].re - t2[i].re)};
    cpx* ldag = (cpx*)malloc(sizeof(cpx) * dd);
    cpx* ldl = (cpx*)malloc(sizeof(cpx) * dd);
    for (int k = 0; k < nch; ++k) {
        const cpx* l = L + (size_t)k * dd;
        for (int i = 0; i < d; ++i)
            for (int j = 0; j < d; ++j) ldag[i * d + j] = (cpx){l[j * d + i].re, -l[j * d + i].im};
        matmul(ldag, l, ldl, d);
        matmul(l, rho, t1, d);
        matmul(t1, ldag, t2, d); /* L rho L^+ */
        for (size_t i = 0; i < dd; ++i) {
            out[i].re += g[k] * t2[i].re;
            out[i].im += g[k] * t2[i].im;
        }
        matmul(ldl, rho, t1, d);
        matmul(rho, ldl, t2, d);
        for (size_t i = 0; i < dd; ++i) {
            out[i].re -= 0.5 * g[k] * (t1[i].re + t2[i].re);
            out[i].im -= 0.5 * g[k] * (t1[i].im + t2[i].im);
        }
    }
    free(ldag);
    free(ldl);
}

int orc_lindblad_exact(int d, const double* h, int nch, const double* ls, const double* gs, const double* rho0,
                       double duration, int steps, double* rho_out) {
    const size_t dd = (size_t)d * d;
    cpx* rho = (cpx*)rho_out;
    memcpy(rho, rho0, sizeof(cpx) * dd);
    cpx *k1 = malloc(sizeof(cpx) * dd), *k2 = malloc(sizeof(cpx) * dd), *k3 = malloc(sizeof(cpx) * dd),
        *k4 = malloc(sizeof(cpx) * dd), *tmp = malloc(sizeof(cpx) * dd), *t1 = malloc(sizeof(cpx) * dd),
        *t2 = malloc(sizeof(cpx) * dd);
    const double hh = duration / steps;
    for (int s = 0; s < steps; ++s) {
        lindblad_rhs((const cpx*)h, nch, (const cpx*)ls, gs, rho, k1, t1, t2, d);
        for (size_t i = 0; i < dd; ++i) tmp[i] = (cpx){rho[i].re + 0.5 * hh * k1[i].re, rho[i].im + 0.5 * hh * k1[i].im};
        lindblad_rhs((const cpx*)h, nch, (const cpx*)ls, gs, tmp, k2, t1, t2, d);
        for (size_t i = 0; i < dd; ++i) tmp[i] = (cpx){rho[i].re + 0.5 * hh * k2[i].re, rho[i].im + 0.5 * hh * k2[i].im};
        lindblad_rhs((const cpx*)h, nch, (const cpx*)ls, gs, tmp, k3, t1, t2, d);
        for (size_t i = 0; i < dd; ++i) tmp[i] = (cpx){rho[i].re + hh * k3[i].re, rho[i].im + hh * k3[i].im};
        lindblad_rhs((const cpx*)h, nch, (const cpx*)ls, gs, tmp, k4, t1, t2, d);
        for (size_t i = 0; i < dd; ++i) {
            rho[i].re += (hh / 6.0) * (k1[i].re + 2.0 * k2[i].re + 2.0 * k3[i].re + k4[i].re);
            rho[i].im += (hh / 6.0) * (k1[i].im + 2.0 * k2[i].im + 2.0 * k3[i].im + k4[i].im);
        }
    }
    free(k1);
    free(k2);
    free(k3);
    free(k4);
    free(tmp);
    free(t1);
    free(t2);
    return 0;
}
