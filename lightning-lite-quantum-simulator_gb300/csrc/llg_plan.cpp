// llg_plan.cpp -- lowers gate records to executor ops and plans them into shared-memory tile
// passes (the GPU form of the reference's cache blocking, src/StateVectorOptimized.cpp:55-78,
// and of its gate fuser, python/gate_fusion.py:15-37).
//
// A tile pass loads 2^t amplitudes whose index bits vary over a qubit set S -- always the `low`
// least-significant qubits, so every tile is made of contiguous 2^low-amplitude runs that load
// coalesced, plus up to t - low qubits anywhere in the register -- applies every op it owns in
// shared memory, and writes the tile back: one HBM read and write of the state per pass, however
// many gates the pass applies.  Choosing S per pass replaces an explicit qubit-remap sweep.
//
// Greedy plan: scan the remaining ops in order with the local set S starting as the low qubits.
// An op joins the pass if none of its qubits is blocked and the qubits it needs local (the target
// of a non-diagonal 1-qubit gate or of a CNOT; none for RZ/CZ/MCZ, which are diagonal and act
// tile-uniformly on non-local bits) fit in S (S grows up to t qubits).  Otherwise it is deferred
// and its qubits are blocked, so no later op on those qubits overtakes it.  The first remaining
// op always fits, so every pass makes progress.  Inside a pass, runs of 1-qubit gates on the same
// qubit with nothing else on that qubit between them are multiplied into one 2x2 (g2 @ g1, the
// fuser's rule) before lowering.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <string>
#include <vector>

#include "llg_common_host.h"
#include "llg_internal.h"

namespace llg {

// Smallest |product of dropped rotation factors| a flush may carry before a full EX_ZY absorbs it:
// double-float amplitudes then stay within 2^40 of their true scale (FP32 range to 2^127), IEEE
// double ones within 2^300 (range to 2^1023).
constexpr double kMinScaleDF64 = 0x1p-40;
constexpr double kMinScaleF64 = 0x1p-300;

bool is_single_qubit(int kind) {
    return kind == LLG_OP_H || kind == LLG_OP_X || kind == LLG_OP_RX || kind == LLG_OP_RY || kind == LLG_OP_RZ ||
           kind == LLG_OP_U2;
}

void op_matrix(const llg_op& op, double m[8]) {
    std::memset(m, 0, 8 * sizeof(double));
    const double c = std::cos(0.5 * op.theta), s = std::sin(0.5 * op.theta);
    const double r = 1.0 / std::sqrt(2.0);
    switch (op.kind) {
        case LLG_OP_H: m[0] = r; m[2] = r; m[4] = r; m[6] = -r; break;
        case LLG_OP_X: m[2] = 1.0; m[4] = 1.0; break;
        case LLG_OP_RX: m[0] = c; m[3] = -s; m[5] = -s; m[6] = c; break;
        case LLG_OP_RY: m[0] = c; m[2] = -s; m[4] = s; m[6] = c; break;
        case LLG_OP_RZ: m[0] = c; m[1] = -s; m[6] = c; m[7] = s; break;
        default: std::memcpy(m, op.m, 8 * sizeof(double)); break;
    }
}

// (a @ b) for row-major interleaved 2x2 complex matrices.
static void matmul2(const double* a, const double* b, double* out) {
    double t[8];
    for (int r = 0; r < 2; ++r)
        for (int c = 0; c < 2; ++c) {
            double re = 0.0, im = 0.0;
            for (int k = 0; k < 2; ++k) {
                const double ar = a[2 * (2 * r + k)], ai = a[2 * (2 * r + k) + 1];
                const double br = b[2 * (2 * k + c)], bi = b[2 * (2 * k + c) + 1];
                re += ar * br - ai * bi;
                im += ar * bi + ai * br;
            }
            t[2 * (2 * r + c)] = re;
            t[2 * (2 * r + c) + 1] = im;
        }
    std::memcpy(out, t, sizeof(t));
}

static ExecOp blank(int kind) {
    ExecOp e;
    std::memset(&e, 0, sizeof(e));
    e.kind = kind;
    return e;
}

// Lower one record with GLOBAL indices.  Validation of qubits/angles is done by the caller.
bool lower_op(int n, const llg_op& op, int P, std::vector<ExecOp>& out, std::string& err) {
    (void)n;
    const double c = std::cos(0.5 * op.theta), s = std::sin(0.5 * op.theta);
    switch (op.kind) {
        case LLG_OP_H: {
            ExecOp e = blank(EX_H);
            e.q0 = op.q0;
            e.c[0] = pack_coef(P, 1.0 / std::sqrt(2.0));
            out.push_back(e);
            return true;
        }
        case LLG_OP_X: {
            ExecOp e = blank(EX_X);
            e.q0 = op.q0;
            out.push_back(e);
            return true;
        }
        case LLG_OP_RX:
        case LLG_OP_RY: {
            ExecOp e = blank(op.kind == LLG_OP_RX ? EX_RX : EX_RY);
            e.q0 = op.q0;
            e.c[0] = pack_coef(P, c);
            e.c[1] = pack_coef(P, s);
            out.push_back(e);
            return true;
        }
        case LLG_OP_RZ: {
            ExecOp e = blank(EX_DIAG);
            e.q0 = op.q0;
            e.c[0] = pack_coef(P, c);
            e.c[1] = pack_coef(P, -s);
            e.c[2] = pack_coef(P, c);
            e.c[3] = pack_coef(P, s);
            out.push_back(e);
            return true;
        }
        case LLG_OP_U2: {
            ExecOp e = blank(EX_U2);
            e.q0 = op.q0;
            for (int k = 0; k < 8; ++k) e.c[k] = pack_coef(P, op.m[k]);
            out.push_back(e);
            return true;
        }
        case LLG_OP_CNOT: {
            ExecOp e = blank(EX_CNOT);
            e.q0 = op.q0;
            e.q1 = op.q1;
            out.push_back(e);
            return true;
        }
        case LLG_OP_CZ: {
            ExecOp e = blank(EX_MCZ);
            e.mask = (1ULL << op.q0) | (1ULL << op.q1);
            out.push_back(e);
            return true;
        }
        case LLG_OP_MCZ: {
            ExecOp e = blank(EX_MCZ);
            e.mask = op.mask;
            out.push_back(e);
            return true;
        }
        default:
            err = "unknown op kind " + std::to_string(op.kind);
            return false;
    }
}

namespace {

// qubits an op touches, and those it needs inside the tile
void op_qubits(const llg_op& op, std::vector<int>& touched, std::vector<int>& need) {
    touched.clear();
    need.clear();
    switch (op.kind) {
        case LLG_OP_RZ: touched.push_back(op.q0); break;
        case LLG_OP_CNOT:
            touched.push_back(op.q0);
            touched.push_back(op.q1);
            need.push_back(op.q1);
            break;
        case LLG_OP_CZ:
            touched.push_back(op.q0);
            touched.push_back(op.q1);
            break;
        case LLG_OP_MCZ:
            for (int q = 0; q < 64; ++q)
                if (op.mask >> q & 1) touched.push_back(q);
            break;
        default:
            touched.push_back(op.q0);
            need.push_back(op.q0);
            break;
    }
}

struct Pending {
    bool active = false;
    bool diag = true;
    int count = 0;
    int first = -1;
    double m[8];
};

}  // namespace

// The double held by a coefficient slot packed for LLG_F64.
static double coef_value(uint64_t bits) {
    double v;
    std::memcpy(&v, &bits, sizeof(v));
    return v;
}

// ------------------------------------------------------------------------------------------
// Phase tables.  A diagonal factor commutes with every op that leaves the Z basis of its qubits
// alone, so inside a pass it may slide to any slot between the ops that do not.  Three kinds of
// diagonal factors are gathered:
//   * the input phase diag(1, e^{ig}) of a carried-phase rotation (EX_ZT / EX_ZC / EX_ZY); it may
//     move earlier, back to the previous op that mixes its qubit;
//   * the controlled phase of a phased CNOT (control local), applied after the CNOT's swap; it
//     may move later, up to the next op that mixes its control or target;
//   * a local carried-phase flush (EX_PHASE1) or diagonal (EX_DIAG), in both directions.
// Each factor has an interval of slots (slot s = just before op s).  The fewest points that
// stab every interval are chosen greedily (intervals by right end); a point becomes one EX_PTAB
// when its factors save more complex multiplies per amplitude pair than the table costs (2: one
// multiply per amplitude), and the rotations it serves become the real forms EX_RT / EX_RC /
// EX_RY.  The table's entry l is the product of the point's factors at the tile's local index l.
// ------------------------------------------------------------------------------------------
namespace {

struct DiagFactor {
    int kind;       // 0 rotation input phase, 1 controlled phase, 2 one-qubit diagonal op
    int op;         // index of the op in the pass
    int q0, q1;     // local qubits: the phase's qubit; for 1 the control and the target
    std::complex<double> v0, v1;  // kind 2: the values on bit 0 and bit 1; else v1 only
    int lo, hi;     // slots it may move to
    double saves;   // complex multiplies per amplitude pair when applied on its own
    int point = -1;
};

// Does an op mix the Z basis of local qubit q (is it an op a diagonal on q cannot pass)?
bool mixes(const ExecOp& e, int q) {
    switch (e.kind) {
        case EX_CNOT: return e.q1 == q;
        case EX_DIAG:
        case EX_PHASE1:
        case EX_MCZ:
        case EX_RZ_P:
        case EX_PTAB: return false;
        default: return e.q0 == q;  // every other kind is a non-diagonal op on its target q0
    }
}

}  // namespace

static void gather_phase_tables(Plan& out) {
    using cd = std::complex<double>;
    std::vector<ExecOp> ops;
    std::vector<int> src;
    ops.reserve(out.ops.size());
    src.reserve(out.ops.size());
    for (PassDesc& pd : out.passes) {
        const int b = pd.op_begin, m = pd.nops, t = pd.t;
        // Reorder the pass by ASAP depth (an op's depth is one more than the deepest earlier op
        // sharing a qubit with it; ops keep their order within a depth).  Ops on shared qubits keep
        // their relative order, so the product is unchanged, and the rotations of one depth become
        // adjacent: one table point can then serve all of them.
        {
            std::vector<int> depth(m), last(t + 64, 0);
            auto res = [&](const ExecOp& x, std::vector<int>& r) {  // local q -> q, global q -> t + q
                r.clear();
                const bool nl = (x.flags & OPF_NONLOCAL_Q0) != 0;
                switch (x.kind) {
                    case EX_CNOT:
                        r.push_back(nl ? t + x.q0 : x.q0);
                        r.push_back(x.q1);
                        break;
                    case EX_MCZ:
                        for (int q = 0; q < t; ++q)
                            if (x.mask >> q & 1) r.push_back(q);
                        for (int q = 0; q < 64; ++q)
                            if (x.nl_mask >> q & 1) r.push_back(t + q);
                        break;
                    default: r.push_back(nl ? t + x.q0 : x.q0); break;
                }
            };
            std::vector<int> r;
            for (int i = 0; i < m; ++i) {
                res(out.ops[b + i], r);
                int d = 0;
                for (int q : r) d = std::max(d, last[q]);
                depth[i] = d + 1;
                for (int q : r) last[q] = d + 1;
            }
            std::vector<int> ord(m);
            for (int i = 0; i < m; ++i) ord[i] = i;
            std::stable_sort(ord.begin(), ord.end(), [&](int a, int c) { return depth[a] < depth[c]; });
            std::vector<ExecOp> tmp(m);
            std::vector<int> tsrc(m);
            for (int i = 0; i < m; ++i) {
                tmp[i] = out.ops[b + ord[i]];
                tsrc[i] = out.source_index[b + ord[i]];
            }
            for (int i = 0; i < m; ++i) {
                out.ops[b + i] = tmp[i];
                out.source_index[b + i] = tsrc[i];
            }
        }
        const ExecOp* e = out.ops.data() + b;
        std::vector<DiagFactor> fs;
        auto last_mix = [&](int i, int q) {  // last op before i that mixes q (-1: none)
            for (int j = i - 1; j >= 0; --j)
                if (mixes(e[j], q)) return j;
            return -1;
        };
        auto next_mix = [&](int i, int qa, int qb) {  // first op after i that mixes qa or qb (m: none)
            for (int j = i + 1; j < m; ++j)
                if (mixes(e[j], qa) || (qb >= 0 && mixes(e[j], qb))) return j;
            return m;
        };
        for (int i = 0; i < m; ++i) {
            const ExecOp& x = e[i];
            DiagFactor f{};
            f.op = i;
            if ((x.kind == EX_ZT || x.kind == EX_ZC || x.kind == EX_ZY) &&
                !(coef_value(x.c[0]) == 1.0 && coef_value(x.c[1]) == 0.0)) {
                f.kind = 0;
                f.q0 = x.q0;
                f.v1 = cd(coef_value(x.c[0]), coef_value(x.c[1]));
                f.lo = last_mix(i, x.q0) + 1;
                f.hi = i;
                f.saves = 1.0;  // a1 times e^{ig}: one multiply per pair
            } else if (x.kind == EX_CNOT && (x.flags & OPF_PHASE) && !(x.flags & OPF_NONLOCAL_Q0)) {
                f.kind = 1;
                f.q0 = x.q0;
                f.q1 = x.q1;
                f.v1 = cd(coef_value(x.c[0]), coef_value(x.c[1]));
                f.lo = i + 1;
                f.hi = next_mix(i, x.q0, x.q1);
                f.saves = 0.5;  // a quarter of the amplitudes
            } else if ((x.kind == EX_PHASE1 || x.kind == EX_DIAG) && !(x.flags & OPF_NONLOCAL_Q0)) {
                f.kind = 2;
                f.q0 = x.q0;
                if (x.kind == EX_PHASE1) {
                    f.v0 = 1.0;
                    f.v1 = cd(coef_value(x.c[0]), coef_value(x.c[1]));
                    f.saves = 1.0;
                } else {
                    f.v0 = cd(coef_value(x.c[0]), coef_value(x.c[1]));
                    f.v1 = cd(coef_value(x.c[2]), coef_value(x.c[3]));
                    f.saves = 2.0;
                }
                f.lo = last_mix(i, x.q0) + 1;
                f.hi = next_mix(i, x.q0, -1);
            } else {
                continue;
            }
            fs.push_back(f);
        }
        // greedy stabbing by right end, then keep the points that pay for their table
        std::vector<int> order(fs.size());
        for (size_t k = 0; k < fs.size(); ++k) order[k] = (int)k;
        std::stable_sort(order.begin(), order.end(), [&](int a, int c) { return fs[a].hi < fs[c].hi; });
        std::vector<int> pts;      // slot of each point
        std::vector<double> gain;  // multiplies saved per pair
        for (int k : order) {
            if (pts.empty() || pts.back() < fs[k].lo) {
                pts.push_back(fs[k].hi);
                gain.push_back(0.0);
            }
            fs[k].point = (int)pts.size() - 1;
            gain.back() += fs[k].saves;
        }
        std::vector<char> keep(pts.size());
        for (size_t p = 0; p < pts.size(); ++p) keep[p] = gain[p] > 2.0;
        // tables of the kept points
        std::vector<long> table_of(pts.size(), -1);
        const size_t entries = (size_t)1 << t;
        for (size_t p = 0; p < pts.size(); ++p) {
            if (!keep[p]) continue;
            std::vector<cd> qv(t, cd(1.0, 0.0)), q0v(t, cd(1.0, 0.0));  // per-qubit bit-1 / bit-0 factors
            std::vector<const DiagFactor*> cps;
            for (const DiagFactor& f : fs) {
                if (f.point != (int)p) continue;
                if (f.kind == 1) cps.push_back(&f);
                else {
                    qv[f.q0] *= f.v1;
                    if (f.kind == 2) q0v[f.q0] *= f.v0;
                }
            }
            std::vector<cd> tab(entries);
            tab[0] = 1.0;
            for (int q = 0; q < t; ++q) {  // doubling: entries with bit q set from those without
                const size_t half = (size_t)1 << q;
                const bool scale0 = !(q0v[q].real() == 1.0 && q0v[q].imag() == 0.0);
                for (size_t l = 0; l < half; ++l) {
                    tab[l | half] = tab[l] * qv[q];
                    if (scale0) tab[l] *= q0v[q];
                }
            }
            for (const DiagFactor* f : cps) {
                const size_t both = ((size_t)1 << f->q0) | ((size_t)1 << f->q1);
                for (size_t l = 0; l < entries; ++l)
                    if ((l & both) == both) tab[l] *= f->v1;
            }
            table_of[p] = (long)(out.tables.size() / 2);
            for (const cd& v : tab) {
                out.tables.push_back(pack_coef(LLG_F64, v.real()));
                out.tables.push_back(pack_coef(LLG_F64, v.imag()));
            }
        }
        // rewrite the pass
        std::vector<int> pt_at(m + 1, -1);
        for (size_t p = 0; p < pts.size(); ++p)
            if (keep[p]) pt_at[pts[p]] = (int)p;
        std::vector<int> absorbed(m, 0);  // 1: factor moved into a table
        for (const DiagFactor& f : fs)
            if (keep[f.point]) absorbed[f.op] = 1;
        const int begin = (int)ops.size();
        for (int i = 0; i <= m; ++i) {
            if (pt_at[i] >= 0) {
                ExecOp tp = blank(EX_PTAB);
                tp.mask = (uint64_t)table_of[pt_at[i]];
                ops.push_back(tp);
                src.push_back(-1);
            }
            if (i == m) break;
            ExecOp x = e[i];
            if (absorbed[i]) {
                switch (x.kind) {
                    case EX_ZT:
                    case EX_ZC:
                        x.kind = x.kind == EX_ZT ? EX_RT : EX_RC;
                        x.c[0] = pack_coef(LLG_F64, 1.0);
                        x.c[1] = 0;
                        break;
                    case EX_ZY:  // RY(b) with the pass scale folded into (c, s)
                        x.kind = EX_RY;
                        x.c[0] = x.c[2];
                        x.c[1] = x.c[3];
                        x.c[2] = x.c[3] = 0;
                        break;
                    case EX_CNOT:
                        x.flags &= ~OPF_PHASE;
                        x.c[0] = x.c[1] = 0;
                        break;
                    default: continue;  // EX_PHASE1 / EX_DIAG: wholly in the table
                }
            }
            ops.push_back(x);
            src.push_back(out.source_index[b + i]);
        }
        pd.op_begin = begin;
        pd.nops = (int)ops.size() - begin;
    }
    out.ops.swap(ops);
    out.source_index.swap(src);
}

// ------------------------------------------------------------------------------------------
// Register programs.  A thread of the register-tiled kernel holds 16 amplitudes of the tile: the
// ones whose local index varies over 4 register positions, its thread index fixing the others.
// An op whose target is a register position runs in registers; a layout change moves the tile
// through shared memory once.  Layouts are chosen greedily: when an op's target is not a register
// position, the next four distinct targets of the pass (in op order, from this op on) become the
// register positions.  The thread-index bits go to the other positions, the first four to
// positions of four different residues mod 4 where possible: the kernel's shared-memory swizzle
// folds every 4-bit group of a local index into its low 4 bits, so such lanes hit distinct banks.
// ------------------------------------------------------------------------------------------
namespace {

// the local position an op needs in a register (-1: none)
int reg_need(const ExecOp& e) {
    switch (e.kind) {
        case EX_CNOT: return e.q1;
        case EX_DIAG:
        case EX_PHASE1:
        case EX_MCZ: return -1;
        default: return e.q0;
    }
}

}  // namespace

// The register kernel's dense dispatch code of an encoded op (RegCode in llg_internal.h).
int32_t reg_dispatch_code(const ExecOp& x) {
    static const int kinds[] = {EX_U2, EX_ZYZ, EX_ZY, EX_ZT, EX_ZC, EX_RT, EX_RC, EX_RX, EX_RY, EX_H, EX_X};
    switch (x.kind) {
        case EX_CNOT:
            if (x.flags & OPF_SLOT_Q0) return RC_CNOT_SLOT + 4 * x.q1 + x.q0;
            return RC_CNOT_UNIFORM + x.q1;
        case EX_DIAG: return (x.flags & OPF_SLOT_Q0) ? RC_DIAG_SLOT + x.q0 : RC_DIAG_UNIFORM;
        case EX_PHASE1: return (x.flags & OPF_SLOT_Q0) ? RC_PHASE_SLOT + x.q0 : RC_DIAG_UNIFORM;
        case EX_MCZ: return RC_MCZ;
        case EX_LAYOUT: return RC_LAYOUT;
        default:
            for (int k = 0; k < (int)(sizeof(kinds) / sizeof(kinds[0])); ++k)
                if (kinds[k] == x.kind) return RC_PAIR + 4 * k + x.q0;
            return 0;
    }
}

namespace {

ExecOp layout_op(int t, const int regs[4]) {
    ExecOp e = blank(EX_LAYOUT);
    uint64_t rm = 0;
    bool is_reg[kMaxTileQubits + 2] = {};
    for (int j = 0; j < 4; ++j) {
        rm |= (uint64_t)regs[j] << (4 * j);
        is_reg[regs[j]] = true;
    }
    // thread-index bits: first four at distinct residues mod 4 (lowest first), then the rest ascending
    std::vector<int> order;
    bool used[kMaxTileQubits + 2] = {};
    bool res_used[4] = {false, false, false, false};
    for (int p = 0; p < t && order.size() < 4; ++p)
        if (!is_reg[p] && !res_used[p & 3]) {
            order.push_back(p);
            used[p] = true;
            res_used[p & 3] = true;
        }
    for (int p = 0; p < t; ++p)
        if (!is_reg[p] && !used[p]) order.push_back(p);
    uint64_t tm = 0;
    for (size_t k = 0; k < order.size(); ++k) tm |= (uint64_t)order[k] << (4 * k);
    e.mask = rm;
    e.nl_mask = tm;
    e.q0 = t - 4;
    e.flags = RC_LAYOUT << kRegCodeShift;
    return e;
}

}  // namespace

int to_register_program(Plan& out) {
    std::vector<ExecOp> ops;
    std::vector<int> src;
    int changes = 0;
    for (PassDesc& pd : out.passes) {
        const int t = pd.t, b = pd.op_begin, m = pd.nops;
        int base_regs[4], regs[4];
        for (int j = 0; j < 4; ++j) base_regs[j] = regs[j] = t - 4 + j;
        auto slot_of = [&](int q) {
            for (int j = 0; j < 4; ++j)
                if (regs[j] == q) return j;
            return -1;
        };
        const int begin = (int)ops.size();
        for (int i = 0; i < m; ++i) {
            ExecOp x = out.ops[b + i];
            const int q = reg_need(x);
            if (q >= 0 && slot_of(q) < 0) {
                // the next four distinct targets from here on
                std::vector<int> want;
                for (int k = i; k < m && want.size() < 4; ++k) {
                    const int w = reg_need(out.ops[b + k]);
                    if (w >= 0 && std::find(want.begin(), want.end(), w) == want.end()) want.push_back(w);
                }
                for (int j = 0; j < 4 && want.size() < 4; ++j)  // keep current registers in the free slots
                    if (std::find(want.begin(), want.end(), regs[j]) == want.end()) want.push_back(regs[j]);
                std::sort(want.begin(), want.end());
                for (int j = 0; j < 4; ++j) regs[j] = want[j];
                ops.push_back(layout_op(t, regs));
                src.push_back(-1);
                ++changes;
            }
            switch (x.kind) {
                case EX_CNOT: {
                    x.q1 = slot_of(x.q1);
                    if (!(x.flags & OPF_NONLOCAL_Q0)) {
                        const int c = slot_of(x.q0);
                        if (c >= 0) {
                            x.q0 = c;
                            x.flags |= OPF_SLOT_Q0;
                        }
                    }
                    break;
                }
                case EX_DIAG:
                case EX_PHASE1:
                    if (!(x.flags & OPF_NONLOCAL_Q0)) {
                        const int c = slot_of(x.q0);
                        if (c >= 0) {
                            x.q0 = c;
                            x.flags |= OPF_SLOT_Q0;
                        }
                    }
                    break;
                case EX_MCZ: break;
                default: x.q0 = slot_of(x.q0); break;
            }
            x.flags |= reg_dispatch_code(x) << kRegCodeShift;
            ops.push_back(x);
            src.push_back(out.source_index[b + i]);
        }
        bool same = true;
        for (int j = 0; j < 4; ++j) same &= regs[j] == base_regs[j];
        if (!same) {
            ops.push_back(layout_op(t, base_regs));
            src.push_back(-1);
            ++changes;
        }
        pd.op_begin = begin;
        pd.nops = (int)ops.size() - begin;
    }
    out.ops.swap(ops);
    out.source_index.swap(src);
    return changes;
}

// ------------------------------------------------------------------------------------------
// Two-qubit blocks.  A CNOT on local qubits c, t and the one-qubit ops next to it on c and t (the
// last op before it on each qubit and the first after it, when those are pair or local diagonal
// ops: nothing between them and the CNOT touches their qubit, so they may move to it) become one
// 4x4 matrix M = (A_c x A_t) CNOT (B_c x B_t), applied as EX_U4 in one shared-memory round trip.
// Coefficients are FP64 bits here (packed for the state's precision by plan_tiles afterwards).
// ------------------------------------------------------------------------------------------
namespace {

using cd2 = std::complex<double>;

// the 2x2 of a one-qubit executor op on a local qubit (false: not such an op)
bool op_2x2(const ExecOp& e, cd2 m[4]) {
    if (e.flags & OPF_NONLOCAL_Q0) return false;
    auto c = [&](int i) { return coef_value(e.c[i]); };
    switch (e.kind) {
        case EX_U2:
            for (int r = 0; r < 4; ++r) m[r] = cd2(c(2 * r), c(2 * r + 1));
            return true;
        case EX_RX: m[0] = m[3] = c(0); m[1] = m[2] = cd2(0.0, -c(1)); return true;
        case EX_RY: m[0] = m[3] = c(0); m[1] = -c(1); m[2] = c(1); return true;
        case EX_H: m[0] = m[1] = m[2] = c(0); m[3] = -c(0); return true;
        case EX_X: m[0] = m[3] = 0.0; m[1] = m[2] = 1.0; return true;
        case EX_DIAG: m[0] = cd2(c(0), c(1)); m[1] = m[2] = 0.0; m[3] = cd2(c(2), c(3)); return true;
        default: return false;
    }
}

bool touches(const ExecOp& e, int q) {
    switch (e.kind) {
        case EX_CNOT: return e.q1 == q || (!(e.flags & OPF_NONLOCAL_Q0) && e.q0 == q);
        case EX_U4: return e.q0 == q || e.q1 == q;
        case EX_U2C: return e.q1 == q;
        case EX_MCZ: return (e.mask >> q) & 1;
        default: return !(e.flags & OPF_NONLOCAL_Q0) && e.q0 == q;
    }
}

// M <- (U on index bit p) M, for 4x4 row-major M
void left_1q(cd2 M[16], const cd2 u[4], int p) {
    cd2 R[16];
    for (int r = 0; r < 4; ++r)
        for (int col = 0; col < 4; ++col) {
            const int br = (r >> p) & 1, r0 = r & ~(1 << p);
            R[r * 4 + col] = u[br * 2 + 0] * M[(r0) * 4 + col] + u[br * 2 + 1] * M[(r0 | (1 << p)) * 4 + col];
        }
    for (int i = 0; i < 16; ++i) M[i] = R[i];
}

}  // namespace

int fuse_two_qubit(Plan& out) {
    int fused = 0;
    for (PassDesc& pd : out.passes) {
        const int b = pd.op_begin, m = pd.nops;
        std::vector<char> gone(m, 0);
        for (int i = 0; i < m; ++i) {
            ExecOp& x = out.ops[b + i];
            if (x.kind != EX_CNOT) continue;
            if (x.flags & OPF_NONLOCAL_Q0) {
                // global control: only the target's neighbours can join; one 2x2 per control value
                const int tq = x.q1;
                int bj = -1, aj = -1;
                cd2 ub[4], ua[4];
                for (int j = i - 1; j >= 0; --j) {
                    if (gone[j] || !touches(out.ops[b + j], tq)) continue;
                    if (op_2x2(out.ops[b + j], ub)) bj = j;
                    break;
                }
                for (int j = i + 1; j < m; ++j) {
                    if (gone[j] || !touches(out.ops[b + j], tq)) continue;
                    if (op_2x2(out.ops[b + j], ua)) aj = j;
                    break;
                }
                if (bj < 0 && aj < 0) continue;
                const cd2 one(1.0, 0.0), zero(0.0, 0.0);
                const cd2 ph = (x.flags & OPF_PHASE) ? cd2(coef_value(x.c[0]), coef_value(x.c[1])) : one;
                cd2 B[4] = {one, zero, zero, one}, A[4] = {one, zero, zero, one};
                if (bj >= 0) std::copy(ub, ub + 4, B);
                if (aj >= 0) std::copy(ua, ua + 4, A);
                // control 0: A B; control 1: A diag(1, ph) X B (a phased CNOT multiplies target 1)
                const cd2 X1[4] = {zero, one, ph, zero};
                auto mul = [](const cd2* p, const cd2* q, cd2* r) {
                    r[0] = p[0] * q[0] + p[1] * q[2];
                    r[1] = p[0] * q[1] + p[1] * q[3];
                    r[2] = p[2] * q[0] + p[3] * q[2];
                    r[3] = p[2] * q[1] + p[3] * q[3];
                };
                cd2 M0[4], XB[4], M1[4];
                mul(A, B, M0);
                mul(X1, B, XB);
                mul(A, XB, M1);
                ExecOp u = blank(EX_U2C);
                u.q0 = x.q0;
                u.q1 = tq;
                u.flags = OPF_NONLOCAL_Q0;
                u.mask = out.tables.size() / 2;
                for (const cd2* mm : {M0, M1})
                    for (int r = 0; r < 4; ++r) {
                        out.tables.push_back(pack_coef(LLG_F64, mm[r].real()));
                        out.tables.push_back(pack_coef(LLG_F64, mm[r].imag()));
                    }
                x = u;
                if (bj >= 0) gone[bj] = 1, ++fused;
                if (aj >= 0) gone[aj] = 1, ++fused;
                continue;
            }
            const int q[2] = {x.q0, x.q1};  // index bit 0: the control, bit 1: the target
            int before[2] = {-1, -1}, after[2] = {-1, -1};
            cd2 ub[2][4], ua[2][4];
            for (int k = 0; k < 2; ++k) {
                for (int j = i - 1; j >= 0; --j) {
                    if (gone[j] || !touches(out.ops[b + j], q[k])) continue;
                    if (op_2x2(out.ops[b + j], ub[k])) before[k] = j;
                    break;
                }
                for (int j = i + 1; j < m; ++j) {
                    if (gone[j] || !touches(out.ops[b + j], q[k])) continue;
                    if (op_2x2(out.ops[b + j], ua[k])) after[k] = j;
                    break;
                }
            }
            if (before[0] < 0 && before[1] < 0 && after[0] < 0 && after[1] < 0) continue;
            cd2 M[16];
            for (int r = 0; r < 16; ++r) M[r] = 0.0;
            // CNOT: |c, t> -> |c, t ^ c>, index k = c + 2 t; a phased CNOT then multiplies |1, 1>
            const cd2 ph = (x.flags & OPF_PHASE) ? cd2(coef_value(x.c[0]), coef_value(x.c[1])) : cd2(1.0, 0.0);
            M[0 * 4 + 0] = 1.0;
            M[2 * 4 + 2] = 1.0;
            M[3 * 4 + 1] = ph;   // |1,0> -> |1,1>
            M[1 * 4 + 3] = 1.0;  // |1,1> -> |1,0>
            cd2 Mb[16];
            for (int r = 0; r < 16; ++r) Mb[r] = (r % 5 == 0) ? cd2(1.0, 0.0) : cd2(0.0, 0.0);
            for (int k = 0; k < 2; ++k)
                if (before[k] >= 0) left_1q(Mb, ub[k], k);
            // M <- M Mb
            cd2 R[16];
            for (int r = 0; r < 4; ++r)
                for (int col = 0; col < 4; ++col) {
                    cd2 v = 0.0;
                    for (int k = 0; k < 4; ++k) v += M[r * 4 + k] * Mb[k * 4 + col];
                    R[r * 4 + col] = v;
                }
            for (int k = 0; k < 2; ++k)
                if (after[k] >= 0) left_1q(R, ua[k], k);
            ExecOp u = blank(EX_U4);
            u.q0 = q[0];
            u.q1 = q[1];
            u.mask = out.tables.size() / 2;
            for (int r = 0; r < 16; ++r) {
                out.tables.push_back(pack_coef(LLG_F64, R[r].real()));
                out.tables.push_back(pack_coef(LLG_F64, R[r].imag()));
            }
            x = u;
            for (int k = 0; k < 2; ++k) {
                if (before[k] >= 0) gone[before[k]] = 1, ++fused;
                if (after[k] >= 0) gone[after[k]] = 1, ++fused;
            }
        }
        // compact the pass
        int w = b;
        for (int i = 0; i < m; ++i)
            if (!gone[i]) {
                out.ops[w] = out.ops[b + i];
                out.source_index[w] = out.source_index[b + i];
                ++w;
            }
        pd.nops = w - b;
    }
    // close the gaps between passes
    std::vector<ExecOp> ops;
    std::vector<int> src;
    for (PassDesc& pd : out.passes) {
        const int begin = (int)ops.size();
        ops.insert(ops.end(), out.ops.begin() + pd.op_begin, out.ops.begin() + pd.op_begin + pd.nops);
        src.insert(src.end(), out.source_index.begin() + pd.op_begin, out.source_index.begin() + pd.op_begin + pd.nops);
        pd.op_begin = begin;
    }
    out.ops.swap(ops);
    out.source_index.swap(src);
    return fused;
}

static bool is_param_op(const llg_op& op, bool use_params) {
    return use_params && op.param >= 0 && (op.kind == LLG_OP_RX || op.kind == LLG_OP_RY || op.kind == LLG_OP_RZ);
}

// Splits a unitary 2x2 m (row-major (re, im) pairs) as z * diag(1, ea) * [[c, -s], [s, c]] *
// diag(1, eg) with |z| = |ea| = |eg| = 1, c = |m00|, s = |m10|.  Returns false when m is not
// unitary to within 2e-15 (then the op stays a generic EX_U2).
static bool split_zyz(const double* m, std::complex<double>& z, double& c, double& s, std::complex<double>& ea,
                      std::complex<double>& eg) {
    using cd = std::complex<double>;
    const cd u00(m[0], m[1]), u01(m[2], m[3]), u10(m[4], m[5]), u11(m[6], m[7]);
    const double n0 = std::norm(u00) + std::norm(u10), n1 = std::norm(u01) + std::norm(u11);
    const cd cross = std::conj(u00) * u01 + std::conj(u10) * u11;
    const double tol = 2e-15;
    if (!(std::fabs(n0 - 1.0) <= tol && std::fabs(n1 - 1.0) <= tol && std::abs(cross) <= tol)) return false;
    c = std::abs(u00);
    s = std::abs(u10);
    if (c > 0.0 && s > 0.0) {
        z = u00 / c;
        ea = u10 * std::conj(z) / s;
        eg = -u01 * std::conj(z) / s;
    } else if (s > 0.0) {  // anti-diagonal: take a = 0
        z = u10 / s;
        ea = 1.0;
        eg = -u01 * std::conj(z) / s;
    } else if (c > 0.0) {  // diagonal: take g = 0
        z = u00 / c;
        ea = u11 * std::conj(z) / c;
        eg = 1.0;
    } else {
        return false;
    }
    return true;
}

bool plan_tiles(int n, const llg_op* ops, int nops, int tile_qubits, int P, Plan& out, std::string& err,
                bool use_params, int zyz, bool tables, bool fuse2) {
    out.passes.clear();
    out.ops.clear();
    out.source_index.clear();
    out.tables.clear();
    // coefficients are planned as FP64 bits and packed for the state's precision at the end
    constexpr int PP = LLG_F64;
    const bool use_zyz = zyz == ZYZ_DEFAULT ? ((P == LLG_DF64 || P == LLG_F64) && !use_params) : zyz == ZYZ_ON;
    // the phase carrier: the plan's first EX_U2, which also applies the global phases dropped by
    // every EX_ZYZ (a scalar factor commutes with every op, so any op of the flush may carry it)
    int carrier = -1;
    double carrier_m[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    std::complex<double> phase(1.0, 0.0);
    // carried phases: ph[q] is a pending diag(1, ph[q]) on global qubit q that has not been applied
    // yet.  A rotation's output phase is carried instead of applied; it commutes with diagonal
    // gates and CNOT controls, merges into the next rotation on the qubit, and is pushed through a
    // CNOT target as phases on both qubits plus a controlled phase folded into the CNOT:
    //   CNOT diag_t(1, p) = diag_t(1, p) diag_c(1, p) CP(c, t; p^-2) CNOT.
    using cd = std::complex<double>;
    std::vector<cd> ph(n, cd(1.0, 0.0));
    auto is_one = [](const cd& v) { return v.real() == 1.0 && v.imag() == 0.0; };
    const int t = std::min(n, tile_qubits);
    // the low qubits are always local; when the register is wider than the tile at least one slot
    // stays free, so the first remaining op (which needs at most one qubit local) always fits
    const int low = n > t ? std::min(4, t - 1) : std::min(4, t);
    if (t < 1 || t > kMaxTileQubits + 1) {
        err = "tile width out of range";
        return false;
    }
    const uint64_t low_mask = (low >= 64) ? ~0ULL : ((1ULL << low) - 1);

    std::vector<int> remaining(nops);
    for (int i = 0; i < nops; ++i) remaining[i] = i;
    std::vector<int> occ_of(nops, -1);
    {
        int occ = 0;
        for (int i = 0; i < nops; ++i)
            if (is_param_op(ops[i], use_params)) occ_of[i] = occ++;
    }
    std::vector<int> touched, need, deferred, included;
    std::vector<char> blocked(64, 0);

    // Rotations as EX_ZT / EX_ZC leave the amplitudes divided by sigma, the product of their
    // dropped factors f (|f| >= 1/sqrt 2 each).  Sigma is carried across the passes of the flush:
    // one full EX_ZY absorbs it mid-flush when |sigma| would fall below min_scale, and at the end
    // the flush's last EX_ZT / EX_ZC is rewritten as that EX_ZY, so the flush stores true
    // amplitudes (every op after it is unitary and scale-free).  A pass boundary is no absorption
    // point: tiles hold amplitudes scaled by the same 1 / sigma everywhere in the register.
    const double min_scale = P == LLG_F64 ? kMinScaleF64 : kMinScaleDF64;
    double sigma = 1.0;
    int last_t = -1;  // index in out.ops of the last EX_ZT / EX_ZC since sigma was 1
    double last_f = 1.0, last_c = 1.0, last_s = 0.0;
    std::complex<double> last_g(1.0, 0.0);

    // remaining[head..] are the ops still to place, in order.  A pass scans a prefix of them; its
    // deferred ops are written back right-aligned inside that prefix and head moves to the first,
    // so the unscanned tail is never copied.
    size_t head = 0;
    while (head < remaining.size()) {
        uint64_t local = low_mask;
        int local_count = low;
        std::fill(blocked.begin(), blocked.end(), 0);
        deferred.clear();
        included.clear();
        int nblocked = 0;
        size_t scanned = remaining.size();
        for (size_t r = head; r < remaining.size(); ++r) {
            const int idx = remaining[r];
            const llg_op& op = ops[idx];
            op_qubits(op, touched, need);
            bool is_blocked = false;
            for (int q : touched) is_blocked |= blocked[q] != 0;
            if (!is_blocked) {
                uint64_t add = 0;
                for (int q : need)
                    if (!(local >> q & 1)) add |= 1ULL << q;
                const int extra = __builtin_popcountll(add);
                if (local_count + extra <= t) {
                    local |= add;
                    local_count += extra;
                    included.push_back(idx);
                    continue;
                }
            }
            deferred.push_back(idx);
            for (int q : touched)
                if (!blocked[q]) {
                    blocked[q] = 1;
                    ++nblocked;
                }
            if (nblocked >= n) {  // every qubit is blocked: the rest of the list stays deferred as is
                scanned = r + 1;
                break;
            }
        }

        // Fill the local set up to t qubits with the lowest unused positions so every pass has
        // the same tile width (and therefore the same grid).
        for (int q = 0; q < n && local_count < t; ++q)
            if (!(local >> q & 1)) {
                local |= 1ULL << q;
                ++local_count;
            }

        PassDesc pd;
        std::memset(&pd, 0, sizeof(pd));
        pd.local_mask = local;
        pd.t = t;
        pd.low = low;
        pd.op_begin = (int)out.ops.size();
        int to_local[64];
        for (int q = 0; q < 64; ++q) to_local[q] = -1;
        {
            int j = 0, h = 0;
            for (int q = 0; q < n; ++q)
                if (local >> q & 1) {
                    to_local[q] = j++;
                    if (q >= low) pd.hi_pos[h++] = q;
                }
        }

        // Peephole fusion of same-qubit 1-qubit runs, then lowering to local indices.
        std::vector<Pending> pend(n);
        // local indices for one executor op (global qubits in), then append it
        auto emit_raw = [&](ExecOp e, int src) {
            switch (e.kind) {
                case EX_U2:
                case EX_ZYZ:
                case EX_ZY:
                case EX_ZT:
                case EX_ZC:
                case EX_RX:
                case EX_RY:
                case EX_H:
                case EX_X: e.q0 = to_local[e.q0]; break;
                case EX_DIAG:
                case EX_PHASE1:
                    if (to_local[e.q0] >= 0) e.q0 = to_local[e.q0];
                    else e.flags |= OPF_NONLOCAL_Q0;
                    break;
                case EX_CNOT:
                    e.q1 = to_local[e.q1];
                    if (to_local[e.q0] >= 0) e.q0 = to_local[e.q0];
                    else e.flags |= OPF_NONLOCAL_Q0;
                    break;
                case EX_MCZ: {
                    uint64_t lm = 0, nl = 0;
                    for (int q = 0; q < 64; ++q)
                        if (e.mask >> q & 1) {
                            if (to_local[q] >= 0) lm |= 1ULL << to_local[q];
                            else nl |= 1ULL << q;
                        }
                    e.mask = lm;
                    e.nl_mask = nl;
                    break;
                }
                default: break;
            }
            out.ops.push_back(e);
            out.source_index.push_back(src);
        };
        // a generic 2x2 on q after folding in the carried phase: the phase carrier (first one),
        // else RY diag(1, g) with the output phase carried, else (not unitary) a generic 2x2
        auto emit_u2 = [&](const double* m_in, int q, int src) {
            double m[8];
            std::memcpy(m, m_in, sizeof(m));
            const cd p = ph[q];
            if (!is_one(p)) {  // U diag(1, p): column 1 times p
                const cd m01 = cd(m[2], m[3]) * p, m11 = cd(m[6], m[7]) * p;
                m[2] = m01.real();
                m[3] = m01.imag();
                m[6] = m11.real();
                m[7] = m11.imag();
                ph[q] = 1.0;
            }
            ExecOp e = blank(EX_U2);
            e.q0 = q;
            cd z, ea, eg;
            double c = 0.0, sn = 0.0;
            if (carrier < 0) {
                carrier = (int)out.ops.size();
                std::memcpy(carrier_m, m, sizeof(carrier_m));
            } else if (split_zyz(m, z, c, sn, ea, eg)) {
                ph[q] = ea;
                phase *= z;
                const bool tan_form = std::fabs(c) >= std::fabs(sn);
                const double f = tan_form ? c : sn;
                if (std::fabs(sigma * f) < min_scale) {  // absorb sigma here: a full EX_ZY
                    e = blank(EX_ZY);
                    e.q0 = q;
                    const double v[4] = {eg.real(), eg.imag(), sigma * c, sigma * sn};
                    for (int k = 0; k < 4; ++k) e.c[k] = pack_coef(PP, v[k]);
                    sigma = 1.0;
                    last_t = -1;
                } else {
                    e = blank(tan_form ? EX_ZT : EX_ZC);
                    e.q0 = q;
                    const double v[3] = {eg.real(), eg.imag(), tan_form ? sn / c : c / sn};
                    for (int k = 0; k < 3; ++k) e.c[k] = pack_coef(PP, v[k]);
                    sigma *= f;
                    last_t = (int)out.ops.size();
                    last_f = f;
                    last_c = c;
                    last_s = sn;
                    last_g = eg;
                }
                emit_raw(e, src);
                return;
            }
            for (int k = 0; k < 8; ++k) e.c[k] = pack_coef(PP, m[k]);
            emit_raw(e, src);
        };
        auto emit_lowered = [&](const llg_op& gop, int src) -> bool {
            if (!use_zyz) {
                std::vector<ExecOp> tmp;
                if (!lower_op(n, gop, PP, tmp, err)) return false;
                for (ExecOp& e : tmp) emit_raw(e, src);
                return true;
            }
            const int q = gop.q0;
            switch (gop.kind) {
                case LLG_OP_RZ: {  // diag(e^-it/2, e^it/2) = e^-it/2 diag(1, e^it): global phase + carried phase
                    const cd d0(std::cos(0.5 * gop.theta), -std::sin(0.5 * gop.theta));
                    const cd d1(std::cos(0.5 * gop.theta), std::sin(0.5 * gop.theta));
                    phase *= d0;
                    ph[q] *= d1 / d0;
                    return true;
                }
                case LLG_OP_X: {  // X diag(1, p) = p diag(1, 1/p) X
                    const cd p = ph[q];
                    if (!is_one(p)) {
                        phase *= p;
                        ph[q] = 1.0 / p;
                    }
                    break;  // the swap itself below
                }
                case LLG_OP_H:
                case LLG_OP_RX:
                case LLG_OP_RY:
                    if (is_one(ph[q])) break;  // nothing carried: the cheaper specialised form
                    {
                        double m[8];
                        op_matrix(gop, m);
                        emit_u2(m, q, src);
                    }
                    return true;
                case LLG_OP_U2: emit_u2(gop.m, q, src); return true;
                case LLG_OP_CNOT: {
                    std::vector<ExecOp> tmp;
                    if (!lower_op(n, gop, PP, tmp, err)) return false;
                    const cd p = ph[gop.q1];
                    if (!is_one(p)) {
                        ph[gop.q0] *= p;
                        const cd cp = 1.0 / (p * p);
                        tmp[0].flags |= OPF_PHASE;
                        tmp[0].c[0] = pack_coef(PP, cp.real());
                        tmp[0].c[1] = pack_coef(PP, cp.imag());
                    }
                    emit_raw(tmp[0], src);
                    return true;
                }
                default: break;  // cz, mcz: diagonal, they commute with the carried phases
            }
            std::vector<ExecOp> tmp;
            if (!lower_op(n, gop, PP, tmp, err)) return false;
            for (ExecOp& e : tmp) emit_raw(e, src);
            return true;
        };
        auto flush_pending = [&](int q) -> bool {
            Pending& p = pend[q];
            if (!p.active) return true;
            p.active = false;
            if (p.count == 1) return emit_lowered(ops[p.first], p.first);
            llg_op u;
            std::memset(&u, 0, sizeof(u));
            u.kind = LLG_OP_U2;
            u.q0 = q;
            u.param = -1;
            std::memcpy(u.m, p.m, sizeof(p.m));
            if (p.diag && use_zyz) {  // diag(d0, d1) = d0 diag(1, d1 / d0): nothing to emit
                const cd d0(p.m[0], p.m[1]), d1(p.m[6], p.m[7]);
                phase *= d0;
                ph[q] *= d1 / d0;
                return true;
            }
            if (p.diag) {
                // product of diagonal gates stays diagonal: emit it as a diagonal op so it may act on
                // a non-local qubit
                std::vector<ExecOp> tmp;
                ExecOp e = blank(EX_DIAG);
                e.q0 = q;
                e.c[0] = pack_coef(PP, p.m[0]);
                e.c[1] = pack_coef(PP, p.m[1]);
                e.c[2] = pack_coef(PP, p.m[6]);
                e.c[3] = pack_coef(PP, p.m[7]);
                if (to_local[q] >= 0) e.q0 = to_local[q];
                else e.flags |= OPF_NONLOCAL_Q0;
                out.ops.push_back(e);
                out.source_index.push_back(-1);
                return true;
            }
            return emit_lowered(u, -1);
        };

        for (int idx : included) {
            const llg_op& op = ops[idx];
            if (occ_of[idx] >= 0) {
                // parametrised rotation: never fused, coefficients come from the batch table
                if (!flush_pending(op.q0)) return false;
                ExecOp e = blank(op.kind == LLG_OP_RX ? EX_RX_P : (op.kind == LLG_OP_RY ? EX_RY_P : EX_RZ_P));
                e.q1 = occ_of[idx];
                if (to_local[op.q0] >= 0) e.q0 = to_local[op.q0];
                else {
                    e.q0 = op.q0;
                    e.flags |= OPF_NONLOCAL_Q0;
                }
                out.ops.push_back(e);
                out.source_index.push_back(idx);
                continue;
            }
            if (is_single_qubit(op.kind)) {
                Pending& p = pend[op.q0];
                double m[8];
                op_matrix(op, m);
                if (!p.active) {
                    p.active = true;
                    p.diag = op.kind == LLG_OP_RZ;
                    p.count = 1;
                    p.first = idx;
                    std::memcpy(p.m, m, sizeof(m));
                } else {
                    matmul2(m, p.m, p.m);  // later gate on the left: g2 @ g1
                    p.diag = p.diag && op.kind == LLG_OP_RZ;
                    ++p.count;
                }
                continue;
            }
            op_qubits(op, touched, need);
            for (int q : touched)
                if (!flush_pending(q)) return false;
            if (!emit_lowered(op, idx)) return false;
        }
        for (int q = 0; q < n; ++q)
            if (!flush_pending(q)) return false;

        pd.nops = (int)out.ops.size() - pd.op_begin;
        if (included.empty()) {
            err = "planner made no progress";
            return false;
        }
        out.passes.push_back(pd);
        size_t w = scanned;
        for (size_t k = deferred.size(); k-- > 0;) remaining[--w] = deferred[k];
        head = w;
    }
    if (last_t >= 0 && sigma != 1.0) {
        // the flush's last EX_ZT / EX_ZC becomes the EX_ZY that absorbs sigma: before it the
        // amplitudes carry 1 / (sigma / last_f), so its rotation is scaled by sigma / last_f
        ExecOp& e = out.ops[last_t];
        const double g = sigma / last_f;
        e.kind = EX_ZY;
        const double v[4] = {last_g.real(), last_g.imag(), g * last_c, g * last_s};
        for (int k = 0; k < 4; ++k) e.c[k] = pack_coef(PP, v[k]);
    }
    if (use_zyz && !out.passes.empty()) {
        // the carried phases that reached the end, as diag(1, p) ops in the last pass; the global
        // phase goes there too when no generic 2x2 can carry it
        PassDesc& last = out.passes.back();
        int to_local[64];
        for (int q = 0; q < 64; ++q) to_local[q] = -1;
        for (int q = 0, j = 0; q < n; ++q)
            if (last.local_mask >> q & 1) to_local[q] = j++;
        auto append = [&](ExecOp e) {
            out.ops.push_back(e);
            out.source_index.push_back(-1);
            ++last.nops;
        };
        for (int q = 0; q < n; ++q) {
            if (is_one(ph[q])) continue;
            ExecOp e = blank(EX_PHASE1);
            e.c[0] = pack_coef(PP, ph[q].real());
            e.c[1] = pack_coef(PP, ph[q].imag());
            if (to_local[q] >= 0) e.q0 = to_local[q];
            else {
                e.q0 = q;
                e.flags |= OPF_NONLOCAL_Q0;
            }
            append(e);
            ph[q] = 1.0;
        }
        if (carrier < 0 && !is_one(phase)) {
            ExecOp e = blank(EX_DIAG);  // local qubit 0 of the tile, both entries the phase
            e.q0 = 0;
            e.c[0] = e.c[2] = pack_coef(PP, phase.real());
            e.c[1] = e.c[3] = pack_coef(PP, phase.imag());
            append(e);
            phase = 1.0;
        }
    }
    if (carrier >= 0 && (phase.real() != 1.0 || phase.imag() != 0.0)) {
        for (int r = 0; r < 4; ++r) {
            const std::complex<double> v = phase * std::complex<double>(carrier_m[2 * r], carrier_m[2 * r + 1]);
            out.ops[carrier].c[2 * r] = pack_coef(PP, v.real());
            out.ops[carrier].c[2 * r + 1] = pack_coef(PP, v.imag());
        }
    }
    if (tables) gather_phase_tables(out);
    if (fuse2 && !use_zyz && !tables) fuse_two_qubit(out);
    if (P != PP) {
        for (ExecOp& e : out.ops)
            for (uint64_t& c : e.c) c = pack_coef(P, coef_value(c));
        for (uint64_t& c : out.tables) c = pack_coef(P, coef_value(c));
    }
    return true;
}

bool lower_stream_f64(int n, const llg_op* ops, int nops, std::vector<ExecOp>& out, std::string& err) {
    using cd = std::complex<double>;
    constexpr int PP = LLG_F64;
    double r = 1.0;      // carried real factor: the state is r w times what the kernels hold
    cd w(1.0, 0.0);      // carried global phase (from RZ)
    int last_real = -1;  // index in out of the last scale-free op (absorbs r)
    int last_phase = -1; // index in out of the last EX_PHASE1 (absorbs w)
    int phase_q0 = -1;   // index in out of an EX_PHASE1 on qubit 0 (absorbs w first, see below)
    int last_u2 = -1;    // index in out of a generic 2x2 (absorbs r w for free)
    int last_zyz = -1;   // index in out of the last EX_ZTZ / EX_ZCZ (or the EX_ZYZ it became)
    // the scale-free op at index i rewritten as its full form times the real factor g
    auto absorb_real = [&](int i, double g) {
        ExecOp& e = out[i];
        const double a = coef_value(e.c[2]);
        double c = g, sn = g;
        if (e.kind == EX_ZTZ || e.kind == EX_ZCZ) {  // diag(1, ea) g T diag(1, eg) = EX_ZYZ (c, s)
            if (e.kind == EX_ZTZ) sn = g * a;
            else c = g * a;
            e.kind = EX_ZYZ;
            e.c[2] = pack_coef(PP, c);
            e.c[3] = pack_coef(PP, sn);
            return;
        }
        switch (e.kind) {
            case EX_RT: sn = g * a; e.kind = EX_RY; break;   // g [1, -t; t, 1] = RY-form (g, g t)
            case EX_RC: c = g * a; e.kind = EX_RY; break;    // g [u, -1; 1, u] = RY-form (g u, g)
            case EX_RXT: sn = g * a; e.kind = EX_RX; break;  // g [1, -it; -it, 1] = RX-form (g, g t)
            case EX_RXC: c = g * a; e.kind = EX_RX; break;   // g [u, -i; -i, u] = RX-form (g u, g)
            default: e.kind = EX_H; break;                   // g [1, 1; 1, -1]
        }
        std::memset(e.c, 0, sizeof(e.c));
        e.c[0] = pack_coef(PP, c);
        e.c[1] = pack_coef(PP, sn);
    };
    // the 2x2 of a unitary-form op (EX_ZTZ, EX_ZCZ, EX_ZYZ): diag(1, ea) R diag(1, eg)
    auto zyz_matrix = [&](const ExecOp& e, cd m[4]) {
        const cd eg(coef_value(e.c[0]), coef_value(e.c[1])), ea(coef_value(e.c[4]), coef_value(e.c[5]));
        const double a = coef_value(e.c[2]);
        double r00 = 1.0, r01 = -a, r10 = a, r11 = 1.0;  // EX_ZTZ: [1, -t; t, 1]
        if (e.kind == EX_ZCZ) {
            r00 = r11 = a;
            r01 = -1.0;
            r10 = 1.0;
        } else if (e.kind == EX_ZYZ) {
            const double sn = coef_value(e.c[3]);
            r00 = r11 = a;
            r01 = -sn;
            r10 = sn;
        }
        m[0] = r00;
        m[1] = r01 * eg;
        m[2] = ea * r10;
        m[3] = ea * r11 * eg;
    };
    for (int i = 0; i < nops; ++i) {
        const llg_op& op = ops[i];
        const double c = std::cos(0.5 * op.theta), s = std::sin(0.5 * op.theta);
        ExecOp e;
        std::memset(&e, 0, sizeof(e));
        e.q0 = op.q0;
        switch (op.kind) {
            case LLG_OP_RX:
            case LLG_OP_RY: {
                const bool tan_form = std::fabs(c) >= std::fabs(s);
                const bool rx = op.kind == LLG_OP_RX;
                e.kind = tan_form ? (rx ? EX_RXT : EX_RT) : (rx ? EX_RXC : EX_RC);
                e.c[2] = pack_coef(PP, tan_form ? s / c : c / s);
                r *= tan_form ? c : s;
                last_real = (int)out.size();
                out.push_back(e);
                break;
            }
            case LLG_OP_H:
                e.kind = EX_HS;
                r *= 1.0 / std::sqrt(2.0);
                last_real = (int)out.size();
                out.push_back(e);
                break;
            case LLG_OP_RZ: {  // diag(e^-it/2, e^it/2) = e^-it/2 diag(1, e^it)
                w *= cd(c, -s);
                const cd p(std::cos(op.theta), std::sin(op.theta));
                e.kind = EX_PHASE1;
                e.c[0] = pack_coef(PP, p.real());
                e.c[1] = pack_coef(PP, p.imag());
                last_phase = (int)out.size();
                if (op.q0 == 0) phase_q0 = last_phase;
                out.push_back(e);
                break;
            }
            case LLG_OP_U2: {
                cd z, ea, eg;
                double cc = 0.0, ss = 0.0;
                if (split_zyz(op.m, z, cc, ss, ea, eg)) {  // z diag(1, ea) [cc, -ss; ss, cc] diag(1, eg)
                    const bool tan_form = cc >= ss;         // cc, ss >= 0
                    e.kind = tan_form ? EX_ZTZ : EX_ZCZ;
                    e.c[0] = pack_coef(PP, eg.real());
                    e.c[1] = pack_coef(PP, eg.imag());
                    e.c[2] = pack_coef(PP, tan_form ? ss / cc : cc / ss);
                    e.c[4] = pack_coef(PP, ea.real());
                    e.c[5] = pack_coef(PP, ea.imag());
                    r *= tan_form ? cc : ss;
                    w *= z;
                    last_real = last_zyz = (int)out.size();
                    out.push_back(e);
                    break;
                }
                if (!lower_op(n, op, PP, out, err)) return false;  // not unitary: the generic form
                last_u2 = (int)out.size() - 1;
                break;
            }
            default: {
                const size_t before = out.size();
                if (!lower_op(n, op, PP, out, err)) return false;
                for (size_t k = before; k < out.size(); ++k)
                    if (out[k].kind == EX_U2) last_u2 = (int)k;
                break;
            }
        }
        // amplitudes held at 1 / r of their size: keep them within 2^300 (FP64 range to 2^1023)
        if (std::fabs(r) < 0x1p-300 && last_real >= 0) {
            absorb_real(last_real, r);
            r = 1.0;
            last_real = -1;
        }
    }
    if (r == 1.0 && w == cd(1.0, 0.0)) return true;
    if (last_u2 >= 0) {  // a scalar times a generic 2x2: free
        const cd z = r * w;
        ExecOp& e = out[last_u2];
        for (int k = 0; k < 4; ++k) {
            const cd v = z * cd(coef_value(e.c[2 * k]), coef_value(e.c[2 * k + 1]));
            e.c[2 * k] = pack_coef(PP, v.real());
            e.c[2 * k + 1] = pack_coef(PP, v.imag());
        }
        return true;
    }
    if (w != cd(1.0, 0.0) && last_phase < 0 && last_zyz >= 0) {
        // a phase from unitary 2x2s and no phase op to take it: the last of them becomes the
        // generic 2x2 r w diag(1, ea) R diag(1, eg)
        ExecOp& e = out[last_zyz];
        cd m[4];
        zyz_matrix(e, m);
        const int q = e.q0;
        std::memset(&e, 0, sizeof(e));
        e.kind = EX_U2;
        e.q0 = q;
        for (int k = 0; k < 4; ++k) {
            const cd v = r * w * m[k];
            e.c[2 * k] = pack_coef(PP, v.real());
            e.c[2 * k + 1] = pack_coef(PP, v.imag());
        }
        return true;
    }
    if (r != 1.0) {
        if (last_real < 0) {
            err = "stream lowering: a carried factor without a scale-free op";
            return false;
        }
        absorb_real(last_real, r);
    }
    if (w != cd(1.0, 0.0)) {
        if (last_phase < 0) {
            err = "stream lowering: a carried phase without a phase op";
            return false;
        }
        // w diag(1, p) = diag(w, w p) over the whole state.  A phase on qubit 0 takes it when there
        // is one: its |1> amplitudes share every 32-byte sector with |0> ones, so its half-state
        // pass already moves the whole state, and the other phases keep their half-state passes.
        ExecOp& e = out[phase_q0 >= 0 ? phase_q0 : last_phase];
        const cd p(coef_value(e.c[0]), coef_value(e.c[1]));
        const cd d1 = w * p;
        e.kind = EX_DIAG;
        e.c[0] = pack_coef(PP, w.real());
        e.c[1] = pack_coef(PP, w.imag());
        e.c[2] = pack_coef(PP, d1.real());
        e.c[3] = pack_coef(PP, d1.imag());
    }
    return true;
}

}  // namespace llg
