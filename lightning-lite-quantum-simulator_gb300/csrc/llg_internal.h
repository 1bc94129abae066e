// llg_internal.h -- records shared by the host engine, the fusion planner and the kernels.
// Plain C++ (no CUDA types), so the planner compiles and is tested without a GPU.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/llgpu.h"

namespace llg {

// Executor op kinds (what a kernel actually runs; the planner lowers llg_op records to these).
enum ExecKind : int32_t {
    EX_U2 = 0,    // generic 2x2 on q0; c[0..7] = g00, g01, g10, g11 (re, im)
    EX_RX = 1,    // c[0] = cos(t/2), c[1] = sin(t/2)
    EX_RY = 2,    // same coefficients
    EX_H = 3,     // c[0] = 1/sqrt(2)
    EX_X = 4,     // swap
    EX_DIAG = 5,  // diag(d0, d1) on q0; c[0..3] = d0 (re, im), d1 (re, im); RZ(t) = diag(e^-it/2, e^it/2)
    EX_CNOT = 6,  // control q0, target q1
    EX_MCZ = 7,   // negate amplitudes with all `mask` bits set
    // parametrised rotations of the batched / adjoint engine: q1 = occurrence slot, the (cos, sin)
    // of the half angle come from a per-batch table; RZ_P is diagonal (q0 may be non-local)
    EX_RX_P = 8,
    EX_RY_P = 9,
    EX_RZ_P = 10,
    // unitary 2x2 without its global phase, as diag(1, e^{ia}) RY(b) diag(1, e^{ig}) on q0:
    // c[0..1] = cos g, sin g; c[2..3] = cos b/2, sin b/2; c[4..5] = cos a, sin a.  152 FP32
    // instructions per double-float pair against 172 for EX_U2; the plan carries the dropped
    // phases in one EX_U2 of the same flush.
    EX_ZYZ = 11,
    // EX_ZYZ without its output phase: RY(b) diag(1, e^{ig}) on q0, c[0..1] = cos g, sin g,
    // c[2..3] = cos b/2, sin b/2 (114 FP32 instructions per double-float pair); the planner carries
    // the dropped output phase forward to the next op on the qubit
    EX_ZY = 12,
    // diag(1, c[0] + i c[1]) on q0 (q0 may be non-local): the planner's flush of a carried phase
    EX_PHASE1 = 13,
    // EX_ZY divided by a real factor f the planner tracks (the amplitudes of a pass are scaled by
    // 1/prod f until one full EX_ZY absorbs the product): with z = e^{ig} a1,
    //   EX_ZT: f = cos b/2, c[2] = t = tan b/2, |t| <= 1:  a0' = a0 - t z,  a1' = z + t a0
    //   EX_ZC: f = sin b/2, c[2] = u = cot b/2, |u| < 1:   a0' = u a0 - z,  a1' = a0 + u z
    // c[0..1] = cos g, sin g.  92 FP32 instructions per double-float pair against 114 for EX_ZY.
    EX_ZT = 14,
    EX_ZC = 15,
    // EX_ZT / EX_ZC whose input phase diag(1, e^{ig}) was moved into a phase table (EX_PTAB) that
    // runs earlier in the pass: the real rotations a0' = a0 - t a1, a1' = a1 + t a0 (EX_RT,
    // c[2] = t) and a0' = u a0 - a1, a1' = a0 + u a1 (EX_RC, c[2] = u): 4 FMA per pair
    EX_RT = 16,
    EX_RC = 17,
    // multiply every tile amplitude l by the phase-table entry T[l] (a diagonal of the tile's
    // local qubits: the product of the input phases, controlled phases and carried phases the
    // planner gathered there); the table starts at entry `mask` of the plan's table buffer and
    // has 2^t entries of (re, im) coefficient slots
    EX_PTAB = 18,
    // register-tiled passes (to_register_program): switch the tile's register layout.  Each thread
    // holds 16 amplitudes whose local indices vary over 4 "register" positions (mask: 4 x 4 bits)
    // and are fixed by the thread index over the other t - 4 positions (nl_mask: 4 bits per thread
    // index bit, in order; q0 = t - 4).  The tile moves through shared memory once per layout.
    EX_LAYOUT = 19,
    // a dense two-qubit block (fuse_two_qubit): a CNOT together with the one-qubit ops next to it on
    // its two qubits, as one 4x4 matrix on local qubits q0 (index bit 0) and q1 (index bit 1); the
    // 16 entries (row-major, (re, im) coefficient slots) start at entry `mask` of the plan's table
    // buffer.  One shared-memory round trip for up to five ops.
    EX_U4 = 20,
    // a CNOT whose control q0 is a global qubit (outside the tile), merged with the one-qubit ops
    // next to it on its local target q1 (fuse_two_qubit): a 2x2 on q1 chosen by the control bit of
    // the tile's base index, entries (row-major, (re, im) slots) at table entry `mask` (control 0)
    // and `mask` + 4 (control 1)
    EX_U2C = 21,
    // Streaming forms for IEEE complex128 per-gate flushes (lower_stream_f64): the gate without
    // its real factor f, which the flush carries and absorbs once (4 FP64 operations per pair
    // instead of 8).  RX(b) = f [1, -it; -it, 1] (EX_RXT, c[2] = t = tan b/2, f = cos b/2) or
    // f [u, -i; -i, u] (EX_RXC, c[2] = u = cot b/2, f = sin b/2); H = 2^-1/2 [1, 1; 1, -1]
    // (EX_HS: sums and differences only).
    EX_RXT = 22,
    EX_RXC = 23,
    EX_HS = 24,
    // A unitary 2x2 z diag(1, ea) RY(b) diag(1, eg) in the same streaming lowering, without z and
    // the rotation's real factor: diag(1, ea) [1, -t; t, 1] diag(1, eg) (EX_ZTZ, c[2] = t) or
    // diag(1, ea) [u, -1; 1, u] diag(1, eg) (EX_ZCZ, c[2] = u); c[0..1] = eg, c[4..5] = ea.
    // 12 FP64 operations per pair against 16 for the generic form.
    EX_ZTZ = 25,
    EX_ZCZ = 26,
};

// Flags of a tile op.
enum : int32_t {
    OPF_NONLOCAL_Q0 = 1,  // q0 is a global qubit outside the tile (diagonal / control use only)
    OPF_ADJOINT = 2,      // parametrised op applied as its inverse (angle negated)
    OPF_GRAD = 4,         // backward pass: accumulate Im<lambda|P|psi> before applying the op
    OPF_PHASE = 8,        // EX_CNOT: multiply the amplitudes with control = target = 1 after the swap
                          // by c[0] + i c[1] (a carried target phase pushed through the CNOT)
    OPF_SLOT_Q0 = 16,     // register program: q0 (a CNOT control, a diagonal's qubit) is a register slot
};

// One executor op.  In a tile pass q0/q1/mask are LOCAL (tile) indices unless flagged; `nl_mask`
// holds the global bits that must all be set in the tile's base index for the op to act.
// Coefficients are 64-bit slots packed for the state's precision (see pack_coef).
struct ExecOp {
    int32_t kind;
    int32_t q0;
    int32_t q1;
    int32_t flags;
    uint64_t mask;
    uint64_t nl_mask;
    uint64_t c[8];
};
static_assert(sizeof(ExecOp) == 96, "ExecOp layout");

constexpr int kMaxTileQubits = 13;
constexpr int kMaxHiPos = 16;

// One fused pass: a tile of 2^t amplitudes whose index bits vary over `local` (the low `low`
// bits 0..low-1 plus hi_pos[0..t-low-1]), ops [op_begin, op_begin + nops).
struct PassDesc {
    uint64_t local_mask;
    int32_t t;
    int32_t low;
    int32_t op_begin;
    int32_t nops;
    int32_t hi_pos[kMaxHiPos];
};

struct Plan {
    std::vector<PassDesc> passes;
    std::vector<ExecOp> ops;
    std::vector<int> source_index;  // for each ExecOp, index of the llg_op it came from (-1: fused)
    // phase tables of the EX_PTAB ops: 2^t entries each, two coefficient slots (re, im) per
    // entry, packed for the plan's precision like ExecOp::c
    std::vector<uint64_t> tables;
};

// Lower and plan a gate list into tile passes (llg_plan.cpp).  Returns false with `err` set on
// invalid input.
// With use_params, rotations whose `param` >= 0 are kept unfused and lowered to EX_*_P ops whose
// q1 is the op's occurrence slot (the index of that op among all parametrised ops, in order).
// With zyz, fused unitary 2x2s are lowered to EX_ZYZ and their global phases folded into the
// first EX_U2 of the plan (default: on for double-float and FP64 states without parametrised ops).
enum PlanZyz : int { ZYZ_DEFAULT = -1, ZYZ_OFF = 0, ZYZ_ON = 1 };
// With tables, runs of diagonal factors inside a pass (the input phases of carried-phase
// rotations, the controlled phases of phased CNOTs, carried phases flushed at the end) are
// gathered into EX_PTAB phase tables where a table replaces more than two complex multiplies per
// amplitude pair; only kernels that execute EX_PTAB (the engine's tile pass) may run such plans.
// With fuse2, every CNOT whose control and target are local is merged with the one-qubit ops that
// can move next to it on those qubits (the last before it and the first after it on each, when
// they are pair or diagonal ops) into an EX_U4 block; only kernels that execute EX_U4 (the
// engine's tile pass) may run such plans.  Not combined with zyz or tables.
bool plan_tiles(int n, const llg_op* ops, int nops, int tile_qubits, int precision, Plan& out, std::string& err,
                bool use_params = false, int zyz = ZYZ_DEFAULT, bool tables = false, bool fuse2 = false);

// Rewrites a tile plan (without EX_PTAB ops) as register programs for the register-tiled pass
// kernel (tile widths 9..13): EX_LAYOUT ops are inserted so that the target of every non-diagonal
// 1-qubit op and every CNOT is a register position when it runs; those ops then name register
// slots 0..3 in q0 (CNOT: the target in q1, the control as a slot with OPF_SLOT_Q0, else a local
// position or a global qubit as before).  Every pass starts and ends in the layout whose register
// positions are the top four tile positions.  Returns the number of layout changes.
int to_register_program(Plan& plan);

// Per-gate lowering of a flush for IEEE complex128 states on the streaming path (one pass per
// gate): RX / RY / H in their scale-free forms (EX_RXT, EX_RXC, EX_RT, EX_RC, EX_HS) with the
// dropped real factors carried, RZ as its global phase (carried) times diag(1, e^{it}) on the
// |1> half (EX_PHASE1), unitary 2x2s as EX_ZTZ / EX_ZCZ with their global phase and real factor
// carried.  The carried factor is absorbed once: into a generic (non-unitary) 2x2 of the flush
// when there is one; else, when the phase has no EX_PHASE1 to take it, both into the last
// EX_ZTZ / EX_ZCZ (rewritten as a generic 2x2); else the real part into the last scale-free op
// (rewritten as its full form) and the phase into the last EX_PHASE1 (rewritten as an EX_DIAG
// over the whole state).  The real part is also absorbed whenever it would fall below 2^-300.
// Other gates lower as lower_op does.
bool lower_stream_f64(int n, const llg_op* ops, int nops, std::vector<ExecOp>& out, std::string& err);

// The EX_U4 fusion of plan_tiles(fuse2): returns the number of one-qubit ops merged into blocks.
int fuse_two_qubit(Plan& plan);

// Dense dispatch codes of register-program ops, in flags >> kRegCodeShift: one jump table in the
// kernel selects the kind and its register slots together.
constexpr int kRegCodeShift = 8;
enum RegCode : int32_t {
    RC_PAIR = 1,           // + 4 * (index of the kind in U2, ZYZ, ZY, ZT, ZC, RT, RC, RX, RY, H, X) + slot
    RC_CNOT_SLOT = 45,     // + 4 * target slot + control slot
    RC_CNOT_UNIFORM = 61,  // + target slot (control a thread-index position or a global qubit)
    RC_DIAG_SLOT = 65,     // + slot
    RC_PHASE_SLOT = 69,    // + slot
    RC_DIAG_UNIFORM = 73,  // EX_DIAG / EX_PHASE1 on a thread-index position or a global qubit
    RC_MCZ = 74,
    RC_LAYOUT = 75,
};
int32_t reg_dispatch_code(const ExecOp& x);

// Lower one gate record to executor ops with GLOBAL qubit indices (streaming path).
bool lower_op(int n, const llg_op& op, int precision, std::vector<ExecOp>& out, std::string& err);

// 2x2 matrix (row-major, interleaved) of a single-qubit gate record.
void op_matrix(const llg_op& op, double m[8]);

bool is_single_qubit(int kind);

}  // namespace llg
