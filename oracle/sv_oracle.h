/*
 * sv_oracle.h -- the ORACLE (test infrastructure only; never linked into the GPU engine).
 * CPU restatement of the reference's state-vector path; see sv_oracle.c / traj_oracle.c.
 */
#ifndef SV_ORACLE_H
#define SV_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_EINVAL 1
#define ORC_ENOMEM 2
#define ORC_ERUNTIME 3

/* Op record.  Kinds 0..6 are the Op kinds of tests/test_backends.cpp:78-83 in the reference
 * (h, x, rx, ry, rz, cnot, mcz); 7 = cz, 8 = generic 2x2 (quantum_sim_v3 gate list). */
enum {
    ORC_OP_H = 0,
    ORC_OP_X = 1,
    ORC_OP_RX = 2,
    ORC_OP_RY = 3,
    ORC_OP_RZ = 4,
    ORC_OP_CNOT = 5,
    ORC_OP_MCZ = 6,
    ORC_OP_CZ = 7,
    ORC_OP_U2 = 8
};

/* Same layout as llg_op in include/llgpu.h (96 bytes). */
typedef struct orc_op {
    int32_t kind;
    int32_t q0;
    int32_t q1;
    int32_t param; /* parameter index for differentiable rotations, -1 otherwise */
    uint64_t mask; /* MCZ qubit mask */
    double theta;  /* rotation angle */
    double m[8];   /* generic 2x2, row-major, interleaved re/im */
} orc_op;

void orc_set_threads(int t);
int orc_max_threads(void);

void orc_init_zero(double* psi, int n);
void orc_apply_gate_v3(double* psi, int n, int target, const double* g);
void orc_apply_gate_standard(double* psi, int n, int target, const double* g);
int orc_h(double* psi, int n, int q);
int orc_x(double* psi, int n, int q);
int orc_rx(double* psi, int n, int q, double t);
int orc_ry(double* psi, int n, int q, double t);
int orc_rz(double* psi, int n, int q, double t);
int orc_cnot(double* psi, int n, int control, int target);
void orc_mcz_mask(double* psi, int n, uint64_t mask);
int orc_mcz_list(double* psi, int n, const int* qubits, int nq);
void orc_probabilities(const double* psi, int n, double* out);
int orc_apply_op(double* psi, int n, const orc_op* op);
int orc_run_ops(double* psi, int n, const orc_op* ops, int nops);
int orc_apply_matrix(double* psi, int n, int k, const int* qs, const double* m);
double orc_expect_zz(const double* psi, int n, int nterms, const int* a, const int* b, const double* coeff);
double orc_norm2(const double* psi, int n);

/* traj_oracle.c */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
void orc_uniform_pair(uint64_t seed, uint64_t traj, uint64_t site, double* u1, double* u2);
int orc_traj_run(int n, const orc_op* ops, int nops, double gamma_ad, double lambda_pd, uint64_t seed,
                 uint64_t traj_begin, uint64_t traj_end, double* z0_out, uint32_t* jump_counts,
                 uint8_t* jump_log, int64_t jump_log_stride, double* margin_out);
int orc_density_z0(int n, const orc_op* ops, int nops, double gamma_ad, double lambda_pd, double* z0_out);

/* dm_oracle.c: KrausChannel::apply restatement; rho(row, col) at row + col * 2^n */
int orc_kraus_trace_preserving(int nk, const double* ops, int m, double tol);
int orc_kraus_apply(double* rho, int n, int nk, const double* ops, int m, const int* targets);
int orc_dm_apply_op(double* rho, int n, const orc_op* op);

/* tsolver_oracle.c: TrajectorySolver restatement */
int orc_expm(const double* a, int d, double* out);
int orc_tsolver_run(int d, int kind, long long steps, double h, int constant, const double* prop, const double* nodes,
                    int nch, const double* ops, const double* ops_dop, const double* psi0, uint64_t seed,
                    uint64_t traj_begin, uint64_t traj_end, double* states_out);
int orc_lindblad_exact(int d, const double* h, int nch, const double* ls, const double* gs, const double* rho0,
                       double duration, int steps, double* rho_out);

/* noise_oracle.c: NoisyBackend + ZNE restatement */
#define ORC_RNG_PHILOX 0
#define ORC_RNG_MT 1
uint64_t orc_mt64_first(uint64_t seed, int k);
int orc_noisy_run(int n, const orc_op* ops, int nops, double p, int scale, int rng, uint64_t seed, uint64_t traj_begin,
                  uint64_t traj_end, int nterms, const int* za, const int* zb, const double* zc, double* obs_out,
                  uint32_t* paulis_out);
int orc_richardson_weights(const double* scales, int ns, double* w);
int orc_zne(int n, const orc_op* ops, int nops, double p, const double* scales, int ns, int trajectories, int rng,
            uint64_t seed, int nterms, const int* za, const int* zb, const double* zc, double* out);

/* adjoint_oracle.c */
int orc_param_shift(int n, const orc_op* ops, int nops, const double* params, int nparams, int nterms,
                    const int* a, const int* b, const double* coeff, double* energy, double* grad);

#ifdef __cplusplus
}
#endif

#endif
