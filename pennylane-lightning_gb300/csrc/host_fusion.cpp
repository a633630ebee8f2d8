// Gate fusion: lowered primitives -> shared-memory tile passes.
//
// 1. Rewrite (exact algebra, rounding-level differences only):
//    * a dense one-wire unitary U is written D1 R D2 with D diagonal and R a
//      real rotation, and the rotation as s [[a,-b],[b,a]] with one of a, b
//      equal to 1 (|other| <= 1): two fused multiply-adds per amplitude
//      instead of eight, which is what the FP64 pipe of a GB300 (1.25
//      TFLOP/s) makes decisive for complex128.  The scalar s of every
//      rotation in a pass is applied once, at the tile store.
//    * RY-shaped real rotations take the same scaled form.
// 2. Schedule: in program order, a primitive joins the current pass when
//    every earlier primitive it does not commute with is already placed and
//    its mixing targets fit the pass's local bit set (diagonal primitives
//    commute with each other and need no local bits).  Per-bit "blocked"
//    flags make this linear in the number of primitives per pass.
// 3. Translate: consecutive diagonals of a pass merge into one op: factors on
//    local bits multiply into a table over the local index, factors on
//    global bits into one scalar per tile, and two-bit factors across the
//    boundary into integer sign flips (CZ) or a per-tile local factor.
//
// Primitives a tile cannot run (dense blocks on 3+ wires, Pauli rotations,
// projections, wide diagonals across the tile boundary) run unfused
// between passes.
#include "df.cuh"
#include "fusion.hpp"

#include <algorithm>
#include <atomic>
#include <cstring>
#include <type_traits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <map>

namespace plgb {

namespace {

constexpr int kModeSrotA = 100; // [[1,-b],[b,1]]
constexpr int kModeSrotB = 101; // [[a,-1],[1,a]]

bool pair_is_diag(int mode) { return mode == M1_DIAG || mode == M1_PHASE1 || mode == M1_NEG1; }

// Runs of uncontrolled one-wire gates on the same bit, with nothing else
// touching that bit in between, become one 2x2 (composed in double
// precision).  RX RY RZ on a wire then costs one rotation instead of two.
template <class T> std::vector<Prim<T>> merge1q(const std::vector<Prim<T>> &in) {
    using C2 = std::complex<double>;
    struct Pend {
        int count{0};
        size_t first{0}; // index in `in` of the first gate of the run
        C2 m[4];
    };
    std::vector<Pend> pend(64);
    std::vector<Prim<T>> out;
    out.reserve(in.size());
    auto single = [](const Prim<T> &p) {
        return p.kind == Prim<T>::Pair && p.tbits.size() == 1 && p.cbits.empty() && p.o0 == 0 &&
               p.o1 == (u64{1} << p.tbits[0]) && p.mode >= M1_DENSE && p.mode <= M1_NEG1;
    };
    auto matrix = [](const Prim<T> &p, C2 (&m)[4]) {
        auto c = [](cx<T> v) { return C2(v.x, v.y); };
        switch (p.mode) {
        case M1_DENSE: m[0] = c(p.m[0]); m[1] = c(p.m[1]); m[2] = c(p.m[2]); m[3] = c(p.m[3]); break;
        case M1_REAL: m[0] = p.m[0].x; m[1] = p.m[1].x; m[2] = p.m[2].x; m[3] = p.m[3].x; break;
        case M1_RXF:
            m[0] = m[3] = p.m[0].x;
            m[1] = m[2] = C2(0, p.m[1].y);
            break;
        case M1_DIAG: m[0] = c(p.m[0]); m[1] = m[2] = 0; m[3] = c(p.m[3]); break;
        case M1_PHASE1: m[0] = 1; m[1] = m[2] = 0; m[3] = c(p.m[3]); break;
        case M1_SWAP: m[0] = m[3] = 0; m[1] = m[2] = 1; break;
        case M1_ANTI: m[0] = m[3] = 0; m[1] = c(p.m[1]); m[2] = c(p.m[2]); break;
        default: m[0] = 1; m[1] = m[2] = 0; m[3] = -1; break; // M1_NEG1
        }
    };
    auto flush = [&](int b) {
        Pend &pd = pend[static_cast<size_t>(b)];
        if (pd.count == 0) {
            return;
        }
        if (pd.count == 1) {
            out.push_back(in[pd.first]);
        } else {
            Prim<T> p = in[pd.first];
            auto t = [](C2 v) { return cx<T>{static_cast<T>(v.real()), static_cast<T>(v.imag())}; };
            const bool offz = pd.m[1] == C2(0) && pd.m[2] == C2(0);
            const bool diagz = pd.m[0] == C2(0) && pd.m[3] == C2(0);
            p.m = {t(pd.m[0]), t(pd.m[1]), t(pd.m[2]), t(pd.m[3])};
            p.mode = offz ? (pd.m[0] == C2(1) ? M1_PHASE1 : M1_DIAG) : diagz ? M1_ANTI : M1_DENSE;
            out.push_back(std::move(p));
        }
        pd.count = 0;
    };
    for (size_t i = 0; i < in.size(); i++) {
        const Prim<T> &p = in[i];
        if (single(p)) {
            const int b = p.tbits[0];
            Pend &pd = pend[static_cast<size_t>(b)];
            C2 g[4];
            matrix(p, g);
            if (pd.count == 0) {
                pd.first = i;
                std::copy(g, g + 4, pd.m);
            } else { // later gate on the left: m <- g m
                const C2 r0 = g[0] * pd.m[0] + g[1] * pd.m[2], r1 = g[0] * pd.m[1] + g[1] * pd.m[3];
                const C2 r2 = g[2] * pd.m[0] + g[3] * pd.m[2], r3 = g[2] * pd.m[1] + g[3] * pd.m[3];
                pd.m[0] = r0;
                pd.m[1] = r1;
                pd.m[2] = r2;
                pd.m[3] = r3;
            }
            pd.count++;
            continue;
        }
        for (u64 r = p.touched(); r; r &= r - 1) {
            flush(__builtin_ctzll(r));
        }
        out.push_back(p);
    }
    for (int b = 0; b < 64; b++) {
        flush(b);
    }
    return out;
}

template <class T> std::vector<Prim<T>> rewrite(const std::vector<Prim<T>> &in) {
    std::vector<Prim<T>> out;
    out.reserve(in.size() * 2);
    for (const auto &p : in) {
        const bool single = p.kind == Prim<T>::Pair && p.tbits.size() == 1 && p.cbits.empty() && p.o0 == 0 &&
                            p.o1 == (u64{1} << p.tbits[0]);
        if (single && p.mode == M1_REAL && p.m[0].x == p.m[3].x && p.m[1].x == -p.m[2].x) {
            // real rotation [[c, -s], [s, c]]
            const double c = p.m[0].x, s = p.m[2].x;
            Prim<T> r = p;
            if (std::fabs(c) >= std::fabs(s)) {
                r.mode = kModeSrotA;
                r.m = {cx<T>{1, static_cast<T>(s / c)}};
                r.c = static_cast<T>(c);
            } else {
                r.mode = kModeSrotB;
                r.m = {cx<T>{static_cast<T>(c / s), 1}};
                r.c = static_cast<T>(s);
            }
            out.push_back(std::move(r));
            continue;
        }
        if (single && (p.mode == M1_DENSE || p.mode == M1_RXF)) {
            // U = diag(e^{i a0}, e^{i a1}) [[c, -s], [s, c]] diag(e^{i b0}, e^{i b1}), b0 = 0
            // RX-form coefficients are stored as (c, s): U = [[c, i s], [i s, c]]
            const bool rxf = p.mode == M1_RXF;
            const std::complex<double> u00(p.m[0].x, rxf ? 0.0 : p.m[0].y),
                u01(rxf ? 0.0 : p.m[1].x, p.m[1].y), u10(rxf ? 0.0 : p.m[2].x, rxf ? p.m[1].y : p.m[2].y),
                u11(p.m[rxf ? 0 : 3].x, rxf ? 0.0 : p.m[3].y);
            const double cm = std::abs(u00), sm = std::abs(u10);
            const double a0 = std::arg(u00), a1 = std::arg(u10);
            const double b1 = cm >= sm ? std::arg(u11) - a1 : std::arg(-u01) - a0;
            const double th = std::atan2(sm, cm);
            const double c = std::cos(th), s = std::sin(th);
            auto ph = [](double a) { return cx<T>{static_cast<T>(std::cos(a)), static_cast<T>(std::sin(a))}; };
            Prim<T> d2 = p;
            d2.mode = M1_PHASE1;
            d2.m = {cx<T>{1, 0}, cx<T>{0, 0}, cx<T>{0, 0}, ph(b1)};
            Prim<T> r = p;
            if (c >= s) {
                r.mode = kModeSrotA;
                r.m = {cx<T>{1, static_cast<T>(s / c)}};
                r.c = static_cast<T>(c);
            } else {
                r.mode = kModeSrotB;
                r.m = {cx<T>{static_cast<T>(c / s), 1}};
                r.c = static_cast<T>(s);
            }
            Prim<T> d1 = p;
            d1.mode = M1_DIAG;
            d1.m = {ph(a0), cx<T>{0, 0}, cx<T>{0, 0}, ph(a1)};
            out.push_back(std::move(d2));
            out.push_back(std::move(r));
            out.push_back(std::move(d1));
            continue;
        }
        out.push_back(p);
    }
    return out;
}

// Canonical diagonal: factor tab[k], k over `bits` (first = MSB).
template <class T> struct Diag {
    std::vector<int> bits;
    std::vector<std::complex<double>> tab;
};

template <class T> bool to_diag(const Prim<T> &p, Diag<T> &d) {
    auto ctrl_table = [&](const std::vector<int> &tb, auto factor) {
        d.bits = tb;
        d.bits.insert(d.bits.end(), p.cbits.begin(), p.cbits.end());
        const size_t k = d.bits.size();
        d.tab.assign(size_t{1} << k, {1.0, 0.0});
        for (size_t idx = 0; idx < d.tab.size(); idx++) {
            bool match = true;
            for (size_t c = 0; c < p.cbits.size(); c++) {
                const size_t pos = tb.size() + c;
                const u64 bitval = (idx >> (k - 1 - pos)) & 1U;
                const u64 want = (p.cval >> p.cbits[c]) & 1U;
                match = match && bitval == want;
            }
            if (match) {
                d.tab[idx] = factor(idx >> p.cbits.size());
            }
        }
    };
    auto C = [](cx<T> v) { return std::complex<double>(v.x, v.y); };
    if (p.kind == Prim<T>::Pair && pair_is_diag(p.mode) && p.tbits.size() == 1 && p.o0 == 0 &&
        p.o1 == (u64{1} << p.tbits[0])) {
        std::complex<double> d0{1, 0}, d1{-1, 0};
        if (p.mode == M1_DIAG) {
            d0 = C(p.m[0]);
            d1 = C(p.m[3]);
        } else if (p.mode == M1_PHASE1) {
            d1 = C(p.m[3]);
        }
        ctrl_table(p.tbits, [&](size_t t) { return t ? d1 : d0; });
        return true;
    }
    if (p.kind == Prim<T>::DiagK) {
        ctrl_table(p.tbits, [&](size_t t) { return C(p.m[t]); });
        return true;
    }
    if (p.kind == Prim<T>::Scale) {
        ctrl_table({}, [&](size_t) { return C(p.m[0]); });
        return true;
    }
    return false;
}

struct PassPlan {
    bool fused{false};
    std::vector<size_t> prims; // indices into the rewritten list
    u64 local{0};
};

// Order the primitives of one pass for execution; per position, levels_out
// gets the merge group of a diagonal (diagonals of one group run as one
// merged op) and the dependency depth of any other primitive.
//
// Dependencies, in program order: two non-diagonal primitives that share a
// touched bit; a diagonal and a non-diagonal primitive that changes one of
// its bits (tmask: touched minus control bits; a diagonal commutes with an op
// that only uses its bits as controls).  Diagonals commute with each other.
// The order is a list schedule that postpones diagonals: every ready
// non-diagonal primitive is emitted first (lowest dependency depth, then
// program order); only when none is left are all ready diagonals emitted as
// one group.  A diagonal thus waits until a primitive needs it, and every
// diagonal ready by then joins it: in a layer of one-wire rotations followed
// by a CNOT chain, the diagonal halves of the rotations merge into one group
// before the chain and one after it, where depth levels would stagger them
// along the chain.
std::vector<size_t> order_by_levels(const std::vector<size_t> &prims, const std::vector<u64> &touch,
                                    const std::vector<u64> &tmask, const std::vector<char> &diag,
                                    std::vector<int> *levels_out) {
    const size_t np = prims.size();
    // dependency depth of the non-diagonal primitives (emission priority)
    std::vector<int> depth(np, 0);
    {
        int ndl[64] = {0};
        for (size_t k = 0; k < np; k++) {
            const size_t pi = prims[k];
            if (diag[pi]) {
                continue;
            }
            int lv = 0;
            for (u64 r = touch[pi]; r; r &= r - 1) {
                lv = std::max(lv, ndl[__builtin_ctzll(r)]);
            }
            lv += 1;
            for (u64 r = touch[pi]; r; r &= r - 1) {
                ndl[__builtin_ctzll(r)] = lv;
            }
            depth[k] = lv;
        }
    }
    auto depends = [&](size_t a, size_t b) { // a before b in program order
        const size_t pa = prims[a], pb = prims[b];
        if (diag[pa] && diag[pb]) {
            return false;
        }
        if (diag[pa]) {
            return (touch[pa] & tmask[pb]) != 0;
        }
        if (diag[pb]) {
            return (tmask[pa] & touch[pb]) != 0;
        }
        return (touch[pa] & touch[pb]) != 0;
    };
    std::vector<int> npred(np, 0);
    std::vector<std::vector<size_t>> succ(np);
    for (size_t b = 0; b < np; b++) {
        for (size_t a = 0; a < b; a++) {
            if (depends(a, b)) {
                npred[b]++;
                succ[a].push_back(b);
            }
        }
    }
    std::vector<size_t> ordered;
    ordered.reserve(np);
    std::vector<int> lv_of(np, 0);
    std::vector<char> emitted(np, 0);
    auto emit = [&](size_t k, int lv) {
        emitted[k] = 1;
        ordered.push_back(prims[k]);
        lv_of[ordered.size() - 1] = lv;
        for (size_t q : succ[k]) {
            npred[q]--;
        }
    };
    int group = 0;
    while (ordered.size() < np) {
        // the ready non-diagonal primitive of lowest depth, else a group of
        // every ready diagonal
        size_t best = np;
        for (size_t k = 0; k < np; k++) {
            if (!emitted[k] && npred[k] == 0 && !diag[prims[k]] && (best == np || depth[k] < depth[best])) {
                best = k;
            }
        }
        if (best != np) {
            emit(best, depth[best]);
            continue;
        }
        std::vector<size_t> ready;
        for (size_t k = 0; k < np; k++) {
            if (!emitted[k] && npred[k] == 0) {
                ready.push_back(k); // diagonals only: no non-diagonal one is ready
            }
        }
        if (ready.empty()) {
            // not reachable: program order is a topological order
            throw PLError("fusion plan: cyclic dependencies in a pass");
        }
        for (size_t k : ready) {
            emit(k, group);
        }
        group++;
    }
    if (levels_out) {
        levels_out->assign(lv_of.begin(), lv_of.end());
    }
    return ordered;
}

} // namespace

// Split a pass's op range into register / shared-memory stages for the
// register-blocked kernel and rewrite the ops' modes for it.  Returns false
// when the pass needs the plain tile kernel.
template <class T>
bool plan_stages(std::vector<TileOp<T>> &ops, const std::vector<DiagForm<T>> &forms, TilePassDesc &d,
                 std::vector<StageDesc> &stages, int rbits) {
    if (d.t < kMinRegTileBits || d.t > 12) { // 2^(t-4) <= 256 threads
        return false;
    }
    if (d.nops > kMaxOpsPerPass) {
        return false; // the register kernel stages at most kMaxOpsPerPass op records
    }
    // Adjoint passes (with reductions) run on the two-register kernel
    // (k_tile_reg_adj): a reduction sits in a register stage whose register
    // bits hold its flip bit, so both amplitudes of every pair it sums are in
    // the same thread; flips of two or more bits keep the pass on the
    // shared-memory two-register kernel.
    for (int i = d.op_begin; i < d.op_begin + d.nops; i++) {
        const auto &op = ops[static_cast<size_t>(i)];
        if (op.kind == TK_REDUCE && __builtin_popcount(op.lo1) > 1) {
            return false;
        }
    }
    const int begin = d.op_begin, end = d.op_begin + d.nops;
    auto single_target = [&](const TileOp<T> &op, int &q) {
        if (op.kind == TK_REDUCE && op.lo1 != 0) {
            q = __builtin_ctz(op.lo1);
            return true;
        }
        if ((op.kind != TK_PAIR && op.kind != TK_SROT) || op.lo0 != 0 || __builtin_popcount(op.lo1) != 1) {
            return false;
        }
        q = __builtin_ctz(op.lo1);
        return true;
    };
    auto is_diag = [](const TileOp<T> &op) {
        return op.kind == TK_DIAGTAB || op.kind == TK_PARITY || (op.kind == TK_REDUCE && op.lo1 == 0);
    };
    // limits of the register kernel's per-tile prologue
    int ndiag = 0;
    for (int i = begin; i < end; i++) {
        if (ops[static_cast<size_t>(i)].kind != TK_DIAGTAB) {
            continue;
        }
        const auto &op = ops[static_cast<size_t>(i)];
        int general = 0;
        for (int f = 0; f < op.nmforms; f++) {
            const auto &mf = forms[static_cast<size_t>(op.mform_begin + f)];
            for (int gb = 0; gb < 2; gb++) {
                const cx<T> d0 = mf.tab[2 * gb], d1 = mf.tab[2 * gb + 1];
                const bool same = d1.x == d0.x && d1.y == d0.y;
                const bool neg = d1.x == -d0.x && d1.y == -d0.y;
                if (!same && !neg) {
                    general++;
                    break;
                }
            }
        }
        if (general > 4) {
            return false;
        }
        ndiag++;
    }
    if (ndiag > kMaxDiagOpsPerPass) {
        return false;
    }
    const int w = d.t - rbits;
    auto layout_from = [&](int i0, int first_q) {
        StageDesc st{};
        st.kind = 0;
        std::vector<int> rb;
        if (first_q >= 0) {
            rb.push_back(first_q);
        }
        for (int i = i0; i < end && static_cast<int>(rb.size()) < rbits; i++) {
            const auto &op = ops[static_cast<size_t>(i)];
            int q;
            if (single_target(op, q)) {
                if (std::find(rb.begin(), rb.end(), q) == rb.end()) {
                    rb.push_back(q);
                }
            } else if (!is_diag(op)) {
                break;
            }
        }
        for (int b = d.t - 1; b >= 0 && static_cast<int>(rb.size()) < rbits; b--) {
            if (std::find(rb.begin(), rb.end(), b) == rb.end()) {
                rb.push_back(b);
            }
        }
        for (int k = 0; k < kRegBits; k++) {
            st.rb[k] = k < rbits ? rb[static_cast<size_t>(k)] : d.t; // unused slots: never selected
        }
        int m = 0;
        for (int b = 0; b < d.t; b++) {
            if (std::find(rb.begin(), rb.end(), b) == rb.end()) {
                st.tb[m++] = b;
            }
        }
        (void)w;
        return st;
    };
    std::vector<StageDesc> local;
    int cur = -1;
    int slot = 0;
    for (int i = begin; i < end; i++) {
        auto &op = ops[static_cast<size_t>(i)];
        int q;
        if (is_diag(op)) {
            if (cur < 0 || local[static_cast<size_t>(cur)].kind != 0) {
                local.push_back(layout_from(i, -1));
                local.back().op_begin = i;
                cur = static_cast<int>(local.size()) - 1;
            }
            if (op.kind == TK_DIAGTAB) {
                op.diag_slot = slot++;
            }
            if (op.kind == TK_REDUCE) {
                op.tcmask = 0;     // no flip
                op.tcval = slot;   // merged diagonals before it in the pass
            }
        } else if (single_target(op, q)) {
            bool in = false;
            if (cur >= 0 && local[static_cast<size_t>(cur)].kind == 0) {
                for (int k = 0; k < rbits; k++) {
                    in = in || local[static_cast<size_t>(cur)].rb[k] == q;
                }
            }
            if (!in) {
                local.push_back(layout_from(i, q));
                local.back().op_begin = i;
                cur = static_cast<int>(local.size()) - 1;
            }
            const auto &st = local[static_cast<size_t>(cur)];
            for (int k = 0; k < rbits; k++) {
                if (st.rb[k] == q) {
                    op.rk = k;
                }
            }
            if (op.kind == TK_REDUCE) {
                // the flip as a register-slot mask; rcmask / lcval stay the
                // local projector
                op.tcmask = 1u << op.rk;
                op.tcval = slot;
                local[static_cast<size_t>(cur)].nops = i - local[static_cast<size_t>(cur)].op_begin + 1;
                continue;
            }
            // controls: every local insert bit except the target
            op.rcmask = 0;
            for (int k = 0; k < op.nlins; k++) {
                if (op.lins[k] != q) {
                    op.rcmask |= 1u << op.lins[k];
                }
            }
            op.rcval = op.lcval;
        } else {
            if (cur < 0 || local[static_cast<size_t>(cur)].kind != 1) {
                StageDesc st{};
                st.kind = 1;
                st.op_begin = i;
                local.push_back(st);
                cur = static_cast<int>(local.size()) - 1;
            }
        }
        local[static_cast<size_t>(cur)].nops = i - local[static_cast<size_t>(cur)].op_begin + 1;
        // register-kernel mode codes
        if (op.kind == TK_SROT) {
            op.mode = op.mode == 0 ? RM_SROT_A : RM_SROT_B;
        } else if (op.kind == TK_PAIR) {
            if (op.mode == M1_SWAP) {
                op.mode = RM_SWAP;
            } else {
                if (op.mode == M1_NEG1) {
                    op.m[0] = cx<T>{1, 0};
                    op.m[1] = op.m[2] = cx<T>{0, 0};
                    op.m[3] = cx<T>{-1, 0};
                } else if (op.mode == M1_PHASE1) {
                    op.m[0] = cx<T>{1, 0};
                    op.m[1] = op.m[2] = cx<T>{0, 0};
                } else if (op.mode == M1_DIAG) {
                    op.m[1] = op.m[2] = cx<T>{0, 0};
                } else if (op.mode == M1_SWAP) {
                    op.m[0] = op.m[3] = cx<T>{0, 0};
                    op.m[1] = op.m[2] = cx<T>{1, 0};
                }
                op.mode = RM_DENSE;
            }
        }
    }
    d.stage_begin = static_cast<int>(stages.size());
    d.nstages = static_cast<int>(local.size());
    d.ndiag = ndiag;
    stages.insert(stages.end(), local.begin(), local.end());
    return true;
}

template <class T>
std::shared_ptr<FusedProgram<T>> compile_fused(int n, const std::vector<Prim<T>> &in, int tile_bits, bool upload,
                                               bool recipes) {
    // Uploaded programs also describe their merged-diagonal tables by
    // factors: expanding 2^t-entry tables on the host cost several times the
    // rest of the compilation.
    const bool use_recipes = recipes || upload;
    auto prog = std::make_shared<FusedProgram<T>>();
    prog->n = n;
    // a tile of 2^t amplitudes must fit the 200 KiB of shared memory the tile
    // kernel requests: t <= 13 for complex128, t <= 14 for complex64
    const int tsmem = sizeof(T) == 8 ? 13 : 14;
    const int tmax = std::max(1, std::min({tile_bits, n, kMaxTileBits, tsmem}));
    const int Lbase = sizeof(T) == 8 ? 4 : 5;
    const int L = std::min(Lbase, tmax);
    const u64 lowmask = (u64{1} << L) - 1;
    const std::vector<Prim<T>> P = rewrite(merge1q(in));
    prog->prims = P.size();

    // per-primitive properties
    const size_t m = P.size();
    std::vector<u64> need(m), touch(m), tmask(m);
    std::vector<char> diag(m), fusible(m);
    for (size_t i = 0; i < m; i++) {
        const auto &p = P[i];
        touch[i] = p.touched();
        tmask[i] = touch[i] & ~p.cmask;
        Diag<T> dd;
        const bool isd = to_diag(p, dd) || p.kind == Prim<T>::Parity;
        diag[i] = isd;
        u64 nb = 0;
        if (!isd) {
            for (int b : p.tbits) {
                nb |= u64{1} << b;
            }
        }
        if (p.kind == Prim<T>::Reduce) {
            nb = p.rx; // the flip bits must be local; Y|Z and projector bits may be global
        }
        need[i] = nb;
        bool ok = false;
        if (p.kind == Prim<T>::Reduce) {
            ok = __builtin_popcountll(nb | lowmask) <= tmax;
        } else if (p.kind == Prim<T>::Pair || p.kind == Prim<T>::Dense2) {
            ok = __builtin_popcountll(nb | lowmask) <= tmax && p.tbits.size() <= 12;
        } else if (p.kind == Prim<T>::Parity) {
            ok = true;
        } else if (isd) {
            ok = dd.bits.size() <= 16;
        }
        fusible[i] = ok;
    }

    // ---- schedule
    std::vector<PassPlan> plan;
    std::vector<char> done(m, 0);
    size_t seg_start = 0;
    while (seg_start < m) {
        size_t seg_end = seg_start;
        while (seg_end < m && fusible[seg_end]) {
            seg_end++;
        }
        // fused passes over [seg_start, seg_end)
        size_t remaining = seg_end - seg_start;
        while (remaining > 0) {
            PassPlan pp;
            pp.fused = true;
            pp.local = lowmask;
            u64 blocked_nd = 0, blocked_d = 0;
            // global bits of placed cross-boundary diagonals must stay global
            // (their fused form was chosen for that split)
            u64 frozen = 0;
            for (size_t i = seg_start; i < seg_end; i++) {
                if (done[i]) {
                    continue;
                }
                bool ok = !(touch[i] & blocked_nd) && (diag[i] || !(touch[i] & blocked_d));
                if (ok) {
                    const u64 nl = pp.local | need[i];
                    if (__builtin_popcountll(nl) <= tmax && !(need[i] & ~pp.local & frozen)) {
                        pp.local = nl;
                    } else {
                        ok = false;
                    }
                }
                if (ok && diag[i]) {
                    // a diagonal across the tile boundary must have a fused form
                    Diag<T> dd;
                    if (to_diag(P[i], dd)) {
                        int nglob = 0, nloc = 0;
                        u64 gbits = 0;
                        for (int b : dd.bits) {
                            if ((pp.local >> b) & 1U) {
                                nloc++;
                            } else {
                                nglob++;
                                gbits |= u64{1} << b;
                            }
                        }
                        ok = nglob == 0 || (nloc == 0 && nglob <= 4) || (nglob == 1 && nloc == 1);
                        if (!ok && __builtin_popcountll(pp.local | gbits) <= tmax && !(gbits & frozen)) {
                            // no fused form across the boundary: make its bits local
                            pp.local |= gbits;
                            gbits = 0;
                            ok = true;
                        }
                        // one- and two-bit diagonals stay valid when a bit turns
                        // local; wider ones pin their global bits
                        if (ok && dd.bits.size() >= 3) {
                            frozen |= gbits;
                        }
                    }
                }
                if (ok) {
                    pp.prims.push_back(i);
                    done[i] = 1;
                    remaining--;
                } else if (diag[i]) {
                    blocked_d |= touch[i];
                } else {
                    blocked_nd |= touch[i];
                }
            }
            // full tiles: pad the local set with free (non-frozen) bits
            for (int b = L; b < n && __builtin_popcountll(pp.local) < tmax; b++) {
                if (!((pp.local >> b) & 1U) && !((frozen >> b) & 1U)) {
                    pp.local |= u64{1} << b;
                }
            }
            if (pp.prims.empty()) {
                // cannot place the first open primitive in a tile: run it unfused
                for (size_t i = seg_start; i < seg_end; i++) {
                    if (!done[i]) {
                        PassPlan up;
                        up.prims = {i};
                        plan.push_back(up);
                        done[i] = 1;
                        remaining--;
                        break;
                    }
                }
                continue;
            }
            plan.push_back(std::move(pp));
        }
        if (seg_end < m) {
            PassPlan up;
            up.prims = {seg_end};
            plan.push_back(up);
            done[seg_end] = 1;
            seg_end++;
        }
        seg_start = seg_end;
    }

    // Split passes whose merged diagonals would outgrow the tile prologue:
    // a prefix of a pass's level order is itself a valid pass on the same
    // local bits.
    {
        constexpr int kDiagLevelsPerPass = kMaxDiagOpsPerPass - 8; // slack for split form lists
        std::vector<PassPlan> split;
        for (auto &pp : plan) {
            if (!pp.fused) {
                split.push_back(std::move(pp));
                continue;
            }
            std::vector<int> lv;
            const std::vector<size_t> ord = order_by_levels(pp.prims, touch, tmask, diag, &lv);
            PassPlan cur;
            cur.fused = true;
            cur.local = pp.local;
            int ndl = 0, last_dl = -1, nred = 0, nprim = 0;
            for (size_t k = 0; k < ord.size(); k++) {
                const bool dg = diag[ord[k]] != 0;
                const bool rd = P[ord[k]].kind == Prim<T>::Reduce;
                // (a primitive becomes at most one op, merged diagonals fewer)
                if ((dg && lv[k] != last_dl && ndl == kDiagLevelsPerPass) || (rd && nred == kMaxReducePerPass) ||
                    nprim == kMaxOpsPerPass - kMaxDiagOpsPerPass) {
                    split.push_back(std::move(cur));
                    cur = PassPlan{};
                    cur.fused = true;
                    cur.local = pp.local;
                    ndl = 0;
                    nred = 0;
                    nprim = 0;
                    last_dl = -1;
                }
                if (dg && lv[k] != last_dl) {
                    ndl++;
                    last_dl = lv[k];
                }
                nred += rd ? 1 : 0;
                nprim += (dg && P[ord[k]].kind != Prim<T>::Parity) ? 0 : 1;
                cur.prims.push_back(ord[k]);
            }
            if (!cur.prims.empty()) {
                split.push_back(std::move(cur));
            }
        }
        plan.swap(split);
    }

    // ---- translate
    std::vector<TileOp<T>> ops;
    std::vector<DiagForm<T>> forms;
    std::vector<cx<T>> tables;
    std::vector<StageDesc> stages;
    for (auto &pp : plan) {
        typename FusedProgram<T>::Seg seg;
        if (!pp.fused) {
            seg.tile = false;
            seg.prim = P[pp.prims[0]];
            if (seg.prim.kind == Prim<T>::Pair && (seg.prim.mode == kModeSrotA || seg.prim.mode == kModeSrotB)) {
                // a scaled rotation outside a tile: back to s [[a,-b],[b,a]]
                const T sc = seg.prim.c;
                const T a = seg.prim.mode == kModeSrotA ? T(1) : seg.prim.m[0].x;
                const T b = seg.prim.mode == kModeSrotA ? seg.prim.m[0].y : T(1);
                seg.prim.mode = M1_REAL;
                seg.prim.m = {cx<T>{sc * a, 0}, cx<T>{-sc * b, 0}, cx<T>{sc * b, 0}, cx<T>{sc * a, 0}};
            }
            prog->segs.push_back(std::move(seg));
            prog->unfused++;
            continue;
        }
        seg.tile = true;
        TilePassDesc &d = seg.desc;
        d.L = L;
        std::vector<int> hb;
        for (int b = L; b < n; b++) {
            if ((pp.local >> b) & 1U) {
                hb.push_back(b);
            }
        }
        d.H = static_cast<int>(hb.size());
        d.t = L + d.H;
        for (int i = 0; i < d.H; i++) {
            d.hb[i] = hb[static_cast<size_t>(i)];
        }
        d.ntiles = u64{1} << (n - d.t);
        d.op_begin = static_cast<int>(ops.size());
        d.pass_scale = 1.0;
        d.rslot_begin = 0;
        d.nrslots = 0;
        auto lpos = [&](int b) -> int {
            if (b < L) {
                return b;
            }
            for (int i = 0; i < d.H; i++) {
                if (d.hb[i] == b) {
                    return L + i;
                }
            }
            return -1;
        };
        auto is_local = [&](int b) { return ((pp.local >> b) & 1U) != 0; };
        auto local_mask = [&](u64 gm) {
            u32 lm = 0;
            for (int b = 0; b < n; b++) {
                if ((gm >> b) & 1U) {
                    const int lp = lpos(b);
                    if (lp >= 0) {
                        lm |= 1u << lp;
                    }
                }
            }
            return lm;
        };
        // pending merged diagonal
        std::vector<Diag<T>> pend;
        auto flush = [&]() {
            if (pend.empty()) {
                return;
            }
            TileOp<T> op;
            op.kind = TK_DIAGTAB;
            std::vector<std::complex<double>> tab;
            bool has_table = false;
            std::vector<DiagForm<T>> gforms, mforms;
            // one-bit local factors collapse to one 2-entry factor per local
            // bit; the table is then their tensor product, built by doubling
            std::complex<double> bitf[kMaxTileBits][2];
            u32 bitf_used = 0;
            for (auto &dg : pend) {
                if (dg.bits.size() == 1 && is_local(dg.bits[0])) {
                    const int lp = lpos(dg.bits[0]);
                    if (!((bitf_used >> lp) & 1U)) {
                        bitf[lp][0] = bitf[lp][1] = {1.0, 0.0};
                        bitf_used |= 1u << lp;
                    }
                    bitf[lp][0] *= dg.tab[0];
                    bitf[lp][1] *= dg.tab[1];
                }
            }
            // recipe mode: the table's factors instead of its 2^t values
            // (possible while every multi-bit local factor has <= 4 bits)
            bool as_recipe = use_recipes;
            for (auto &dg : pend) {
                bool all_local = true;
                for (int b : dg.bits) {
                    all_local = all_local && is_local(b);
                }
                if (all_local && dg.bits.size() > 4) {
                    as_recipe = false;
                }
            }
            TableRecipe rec{0, d.t, static_cast<int>(prog->h_factors.size()), 0};
            if (as_recipe) {
                auto C = [](std::complex<double> v) { return cx<double>{v.real(), v.imag()}; };
                for (int lp = 0; lp < d.t; lp++) {
                    if ((bitf_used >> lp) & 1U) {
                        TableFactor f{};
                        f.nb = 1;
                        f.pos[0] = lp;
                        f.val[0] = C(bitf[lp][0]);
                        f.val[1] = C(bitf[lp][1]);
                        prog->h_factors.push_back(f);
                    }
                }
                for (auto &dg : pend) {
                    bool all_local = true;
                    for (int b : dg.bits) {
                        all_local = all_local && is_local(b);
                    }
                    if (!all_local || dg.bits.size() == 1) {
                        continue;
                    }
                    TableFactor f{};
                    f.nb = static_cast<int>(dg.bits.size());
                    for (int i = 0; i < f.nb; i++) {
                        f.pos[i] = lpos(dg.bits[static_cast<size_t>(i)]);
                    }
                    for (size_t i = 0; i < dg.tab.size(); i++) {
                        f.val[i] = C(dg.tab[i]);
                    }
                    prog->h_factors.push_back(f);
                }
                rec.nfac = static_cast<int>(prog->h_factors.size()) - rec.fac_begin;
            }
            const bool table_needed = [&] {
                if (bitf_used) {
                    return true;
                }
                for (auto &dg : pend) {
                    bool all_local = true;
                    for (int b : dg.bits) {
                        all_local = all_local && is_local(b);
                    }
                    if (all_local) {
                        return true;
                    }
                }
                return false;
            }();
            if (as_recipe) {
                bitf_used = 0; // nothing to materialise on the host
            }
            if (bitf_used) {
                tab.assign(size_t{1} << d.t, {1.0, 0.0});
                has_table = true;
                size_t len = 1;
                for (int lp = 0; lp < d.t; lp++) {
                    if ((bitf_used >> lp) & 1U) {
                        for (size_t j = 0; j < len; j++) {
                            tab[j + len] = tab[j] * bitf[lp][1];
                            tab[j] *= bitf[lp][0];
                        }
                    } else {
                        std::copy(tab.begin(), tab.begin() + static_cast<std::ptrdiff_t>(len),
                                  tab.begin() + static_cast<std::ptrdiff_t>(len));
                    }
                    len <<= 1;
                }
            }
            for (auto &dg : pend) {
                int nloc = 0, nglob = 0;
                for (int b : dg.bits) {
                    is_local(b) ? nloc++ : nglob++;
                }
                if (nglob == 0 && dg.bits.size() == 1) {
                    continue; // in the per-bit factors above
                }
                if (nglob == 0 && as_recipe) {
                    continue; // a recipe factor
                }
                if (nglob == 0) {
                    if (!has_table) {
                        tab.assign(size_t{1} << d.t, {1.0, 0.0});
                        has_table = true;
                    }
                    const size_t k = dg.bits.size();
                    std::vector<int> lp(k);
                    for (size_t i = 0; i < k; i++) {
                        lp[i] = lpos(dg.bits[i]);
                    }
                    for (size_t j = 0; j < tab.size(); j++) {
                        size_t idx = 0;
                        for (size_t i = 0; i < k; i++) {
                            idx = (idx << 1) | ((j >> lp[i]) & 1U);
                        }
                        tab[j] *= dg.tab[idx];
                    }
                } else if (nloc == 0) {
                    DiagForm<T> f;
                    f.nb = static_cast<int>(dg.bits.size());
                    for (int i = 0; i < f.nb; i++) {
                        f.bits[i] = dg.bits[static_cast<size_t>(i)];
                    }
                    for (size_t i = 0; i < dg.tab.size(); i++) {
                        f.tab[i] = cx<T>{static_cast<T>(dg.tab[i].real()), static_cast<T>(dg.tab[i].imag())};
                    }
                    gforms.push_back(f);
                } else {
                    // one global, one local bit: reorder as [global][local]
                    DiagForm<T> f;
                    f.nb = 2;
                    const bool g_first = !is_local(dg.bits[0]);
                    f.bits[0] = g_first ? dg.bits[0] : dg.bits[1];
                    f.local_bit = lpos(g_first ? dg.bits[1] : dg.bits[0]);
                    for (int gbv = 0; gbv < 2; gbv++) {
                        for (int lbv = 0; lbv < 2; lbv++) {
                            const int idx = g_first ? (gbv << 1 | lbv) : (lbv << 1 | gbv);
                            const auto v = dg.tab[static_cast<size_t>(idx)];
                            f.tab[gbv * 2 + lbv] = cx<T>{static_cast<T>(v.real()), static_cast<T>(v.imag())};
                        }
                    }
                    mforms.push_back(f);
                }
            }
            // split the form lists into ops of bounded size
            size_t gi = 0, mi = 0;
            bool first = true;
            while (first || gi < gforms.size() || mi < mforms.size()) {
                TileOp<T> o = op;
                o.has_table = first && (has_table || (as_recipe && table_needed)) ? 1 : 0;
                if (o.has_table && as_recipe) {
                    o.table_off = static_cast<int>(prog->table_entries);
                    rec.table_off = o.table_off;
                    prog->h_recipes.push_back(rec);
                    prog->table_entries += size_t{1} << d.t;
                } else if (o.has_table) {
                    o.table_off = static_cast<int>(prog->table_entries);
                    prog->h_table_chunks.push_back({prog->table_entries, tables.size(), tab.size()});
                    for (auto &v : tab) {
                        tables.push_back(cx<T>{static_cast<T>(v.real()), static_cast<T>(v.imag())});
                    }
                    prog->table_entries += tab.size();
                }
                o.gform_begin = static_cast<int>(forms.size());
                const size_t gtake = std::min<size_t>(gforms.size() - gi, 64);
                for (size_t i = 0; i < gtake; i++) {
                    forms.push_back(gforms[gi++]);
                }
                o.ngforms = static_cast<int>(gtake);
                o.mform_begin = static_cast<int>(forms.size());
                const size_t mtake = std::min<size_t>(mforms.size() - mi, kMaxMixedForms);
                for (size_t i = 0; i < mtake; i++) {
                    forms.push_back(mforms[mi++]);
                }
                o.nmforms = static_cast<int>(mtake);
                if (o.has_table || o.ngforms || o.nmforms) {
                    ops.push_back(o);
                }
                first = false;
            }
            pend.clear();
        };

        const std::vector<size_t> ordered = order_by_levels(pp.prims, touch, tmask, diag, nullptr);
        for (size_t pi : ordered) {
            const auto &p = P[pi];
            Diag<T> dg;
            if (to_diag(p, dg)) {
                pend.push_back(std::move(dg));
                continue;
            }
            if (p.kind == Prim<T>::Reduce) {
                flush(); // diagonals before the reduction point apply first
                TileOp<T> o;
                o.kind = TK_REDUCE;
                o.lo1 = local_mask(p.rx);   // flip bits (all local)
                o.lo0 = local_mask(p.ryz);  // Y|Z bits inside the tile
                o.pmask = p.ryz;            // with gbase: the tile's share of the sign parity
                o.rcmask = local_mask(p.rpm);
                o.lcval = local_mask(p.rpv);
                {
                    u64 gm = 0; // projector bits outside the tile gate the whole tile
                    for (int b = 0; b < n; b++) {
                        if (((p.rpm >> b) & 1U) && !is_local(b)) {
                            gm |= u64{1} << b;
                        }
                    }
                    o.gcmask = gm;
                    o.gcval = p.rpv & gm;
                }
                o.mode = p.rny4;
                o.rslot = p.rslot;
                o.rmul = d.pass_scale * d.pass_scale;
                o.diag_slot = d.nrslots++; // the CTA's accumulator for this op
                PLGB_REQUIRE(d.nrslots <= kMaxReducePerPass, "fusion: too many reductions in one pass");
                ops.push_back(o);
                continue;
            }
            if (p.kind == Prim<T>::Parity) {
                TileOp<T> o;
                o.kind = TK_PARITY;
                o.pmask = p.pmask;
                o.cmask = p.cmask;
                o.cval = p.cval;
                o.zero_outside = p.zero_outside ? 1 : 0;
                o.m[0] = p.m[0];
                o.m[1] = p.m[1];
                ops.push_back(o);
                continue;
            }
            flush();
            TileOp<T> o;
            // controls: local ones enumerate, global ones gate the whole tile
            std::vector<int> lins;
            for (int b : p.tbits) {
                lins.push_back(lpos(b));
            }
            for (int b : p.cbits) {
                if (is_local(b)) {
                    lins.push_back(lpos(b));
                    if ((p.cval >> b) & 1U) {
                        o.lcval |= 1u << lpos(b);
                    }
                } else {
                    o.gcmask |= u64{1} << b;
                    o.gcval |= p.cval & (u64{1} << b);
                }
            }
            std::sort(lins.begin(), lins.end());
            PLGB_REQUIRE(lins.size() <= 12, "fusion: too many local bits in one op");
            o.nlins = static_cast<int>(lins.size());
            for (size_t i = 0; i < lins.size(); i++) {
                o.lins[i] = lins[i];
            }
            if (p.kind == Prim<T>::Pair) {
                o.lo0 = local_mask(p.o0);
                o.lo1 = local_mask(p.o1);
                if (p.mode == kModeSrotA || p.mode == kModeSrotB) {
                    o.kind = TK_SROT;
                    o.mode = p.mode == kModeSrotA ? 0 : 1;
                    o.m[0] = p.m[0];
                    d.pass_scale *= static_cast<double>(p.c);
                } else {
                    o.kind = TK_PAIR;
                    o.mode = p.mode;
                    for (int i = 0; i < 4; i++) {
                        o.m[i] = p.m[static_cast<size_t>(i)];
                    }
                }
            } else { // Dense2
                o.kind = TK_DENSE2;
                o.lo0 = 1u << lpos(p.tbits[0]);
                o.lo1 = 1u << lpos(p.tbits[1]);
                for (int i = 0; i < 16; i++) {
                    o.m[i] = p.m[static_cast<size_t>(i)];
                }
            }
            ops.push_back(o);
        }
        flush();
        d.nops = static_cast<int>(ops.size()) - d.op_begin;
        // passes with reductions (adjoint sweeps) run two registers per
        // thread: 8 amplitudes of each (3 register bits) instead of 16
        bool has_reduce = false;
        for (int i = d.op_begin; i < d.op_begin + d.nops; i++) {
            has_reduce = has_reduce || ops[static_cast<size_t>(i)].kind == TK_REDUCE;
        }
        seg.reg = plan_stages<T>(ops, forms, d, stages, has_reduce ? kAdjRegBits : kRegBits);
        prog->segs.push_back(std::move(seg));
        prog->passes++;
    }

    // plan description: one JSON object per segment
    {
        std::string js = "[";
        for (size_t si = 0; si < prog->segs.size(); si++) {
            const auto &seg = prog->segs[si];
            char buf[256];
            if (!seg.tile) {
                std::snprintf(buf, sizeof(buf), "%s{\"tile\": false, \"prim\": %d}", si ? ", " : "",
                              static_cast<int>(seg.prim.kind));
                js += buf;
                continue;
            }
            const auto &d = seg.desc;
            int nreg = 0, nsm = 0, ndg = 0, nrot = 0, npair = 0;
            for (int i = d.op_begin; i < d.op_begin + d.nops; i++) {
                const int k = ops[static_cast<size_t>(i)].kind;
                ndg += (k == TK_DIAGTAB || k == TK_PARITY) ? 1 : 0;
                nrot += (k == TK_SROT) ? 1 : 0;
                npair += (k == TK_PAIR || k == TK_DENSE2) ? 1 : 0;
            }
            for (int sidx = d.stage_begin; seg.reg && sidx < d.stage_begin + d.nstages; sidx++) {
                (stages[static_cast<size_t>(sidx)].kind == 0 ? nreg : nsm)++;
            }
            std::snprintf(buf, sizeof(buf),
                          "%s{\"tile\": true, \"t\": %d, \"ops\": %d, \"rotations\": %d, \"pairs\": %d, "
                          "\"diagonals\": %d, \"register_kernel\": %s, \"reg_stages\": %d, \"smem_stages\": %d}",
                          si ? ", " : "", d.t, d.nops, nrot, npair, ndg, seg.reg ? "true" : "false", nreg, nsm);
            js += buf;
        }
        prog->plan = js + "]";
    }
    if (!upload) {
        prog->h_ops = std::move(ops);
        prog->h_forms = std::move(forms);
        prog->h_tables = std::move(tables);
        prog->h_stages = std::move(stages);
        return prog;
    }

    // ---- upload: one block [ops][forms][stages][recipes][df recipes][factors][tables],
    // the first five in one copy; host-built table chunks copied in place;
    // recipe tables expanded on the device
    bool all_tile = !prog->segs.empty(), all_reg = !prog->segs.empty();
    for (const auto &seg : prog->segs) {
        all_reg = all_reg && seg.tile && seg.reg;
        all_tile = all_tile && seg.tile;
    }
    const bool want_df = std::is_same_v<T, double> && all_tile;
    const size_t nrec = prog->h_recipes.size();
    const size_t nfac = prog->h_factors.size();
    const size_t b_ops = align_up(std::max<size_t>(1, ops.size()) * sizeof(TileOp<T>));
    const size_t b_forms = align_up(std::max<size_t>(1, forms.size()) * sizeof(DiagForm<T>));
    const size_t b_st = align_up(std::max<size_t>(1, stages.size()) * sizeof(StageDesc));
    const size_t b_rec = align_up(std::max<size_t>(1, 2 * nrec) * sizeof(DevRecipe));
    const size_t b_fac = align_up(std::max<size_t>(1, nfac) * sizeof(TableFactor));
    const size_t b_tab = align_up(std::max<size_t>(1, prog->table_entries) * sizeof(cx<T>));
    const size_t b_head = b_ops + b_forms + b_st + b_rec + b_fac;
    prog->dev = dev_alloc(b_head + b_tab);
    char *base = static_cast<char *>(prog->dev);
    prog->d_ops = reinterpret_cast<TileOp<T> *>(base);
    prog->d_forms = reinterpret_cast<DiagForm<T> *>(base + b_ops);
    prog->d_stages = reinterpret_cast<StageDesc *>(base + b_ops + b_forms);
    auto *d_rec = reinterpret_cast<DevRecipe *>(base + b_ops + b_forms + b_st);
    auto *d_fac = reinterpret_cast<TableFactor *>(base + b_ops + b_forms + b_st + b_rec);
    prog->d_tables = reinterpret_cast<cx<T> *>(base + b_head);
    char *bd = nullptr;
    if (want_df) {
        // the same tables re-encoded as double-float (same 16-byte layout)
        static_assert(sizeof(TileOp<double>) == sizeof(TileOp<df>) && sizeof(DiagForm<double>) == sizeof(DiagForm<df>) &&
                          sizeof(cx<double>) == sizeof(cx<df>),
                      "double-float op tables must share the double layout");
        prog->dev_df = dev_alloc(b_ops + b_forms + b_tab);
        bd = static_cast<char *>(prog->dev_df);
        prog->d_ops_df = bd;
        prog->d_forms_df = bd + b_ops;
        prog->d_tables_df = bd + b_ops + b_forms;
    }
    std::vector<char> head(b_head, 0);
    auto put = [](char *dst, const auto &v) {
        if (!v.empty()) {
            std::memcpy(static_cast<void *>(dst), v.data(), v.size() * sizeof(v[0]));
        }
    };
    put(head.data(), ops);
    put(head.data() + b_ops, forms);
    put(head.data() + b_ops + b_forms, stages);
    u64 rec_entries = 0;
    {
        auto *hr = reinterpret_cast<DevRecipe *>(head.data() + b_ops + b_forms + b_st);
        for (size_t i = 0; i < nrec; i++) {
            const TableRecipe &r = prog->h_recipes[i];
            DevRecipe d{};
            d.dst = prog->d_tables + r.table_off;
            d.fac = d_fac + r.fac_begin;
            d.t = r.t;
            d.nfac = r.nfac;
            d.entry_begin = rec_entries;
            rec_entries += u64{1} << r.t;
            hr[i] = d;
            if (want_df) {
                d.dst = reinterpret_cast<cx<df> *>(bd + b_ops + b_forms) + r.table_off;
                hr[nrec + i] = d;
            }
        }
        put(head.data() + b_ops + b_forms + b_st + b_rec, prog->h_factors);
    }
    cuda_check(cudaMemcpy(base, head.data(), b_head, cudaMemcpyHostToDevice), "H2D");
    for (const auto &ch : prog->h_table_chunks) {
        cuda_check(cudaMemcpy(prog->d_tables + ch[0], tables.data() + ch[1], ch[2] * sizeof(cx<T>),
                              cudaMemcpyHostToDevice), "H2D");
    }
    if (nrec) {
        launch_expand_tables(nullptr, d_rec, static_cast<int>(nrec), rec_entries, std::is_same_v<T, float> ? 0 : 1);
    }
    if constexpr (std::is_same_v<T, double>) {
        prog->df_reg = all_reg;
        if (want_df) {
            auto cdf = [](cx<double> v) { return cx<df>{df(v.x), df(v.y)}; };
            std::vector<char> hd(b_ops + b_forms, 0);
            auto *ops_df = reinterpret_cast<TileOp<df> *>(hd.data());
            for (size_t i = 0; i < ops.size(); i++) {
                std::memcpy(static_cast<void *>(&ops_df[i]), &ops[i], sizeof(TileOp<double>));
                for (int k = 0; k < 16; k++) {
                    ops_df[i].m[k] = cdf(ops[i].m[k]);
                }
            }
            auto *forms_df = reinterpret_cast<DiagForm<df> *>(hd.data() + b_ops);
            for (size_t i = 0; i < forms.size(); i++) {
                std::memcpy(static_cast<void *>(&forms_df[i]), &forms[i], sizeof(DiagForm<double>));
                for (int k = 0; k < 16; k++) {
                    forms_df[i].tab[k] = cdf(forms[i].tab[k]);
                }
            }
            cuda_check(cudaMemcpy(bd, hd.data(), hd.size(), cudaMemcpyHostToDevice), "H2D");
            auto *tdf = reinterpret_cast<cx<df> *>(bd + b_ops + b_forms);
            for (const auto &ch : prog->h_table_chunks) {
                std::vector<cx<df>> c(ch[2]);
                for (size_t i = 0; i < ch[2]; i++) {
                    c[i] = cdf(tables[ch[1] + i]);
                }
                cuda_check(cudaMemcpy(tdf + ch[0], c.data(), c.size() * sizeof(cx<df>), cudaMemcpyHostToDevice), "H2D");
            }
            if (nrec) {
                launch_expand_tables(nullptr, d_rec + nrec, static_cast<int>(nrec), rec_entries, 2);
            }
            prog->df_ok = true;
        }
    }
    if (nrec) {
        // the passes run on the register's own (non-blocking) stream
        cuda_check(cudaStreamSynchronize(nullptr), "table expansion");
    }
    return prog;
}

namespace {
// complex128 fused passes compute in FP64 unless a caller opts into the
// double-float arithmetic (about 48 significant bits, FP32 exponent range)
std::atomic<bool> g_c128_fp64{true};
}
void set_c128_fp64_passes(bool on) { g_c128_fp64 = on; }
bool c128_fp64_passes() { return g_c128_fp64; }

template <class T> void run_fused(StateVector<T> &sv, const FusedProgram<T> &prog) {
    PLGB_REQUIRE(prog.n == sv.num_qubits(), "fused program compiled for a different register size");
    if constexpr (std::is_same_v<T, double>) {
        if (prog.df_reg && prog.df_ok && !c128_fp64_passes()) {
            // the register holds df values between the first and the last pass
            const size_t np = prog.segs.size();
            for (size_t k = 0; k < np; k++) {
                const int io = np == 1 ? 0 : k == 0 ? 1 : k + 1 == np ? 3 : 2;
                launch_tile_pass_reg_df(sv.stream(), sv.data(), io, prog.segs[k].desc,
                                        static_cast<const TileOp<df> *>(prog.d_ops_df),
                                        static_cast<const DiagForm<df> *>(prog.d_forms_df),
                                        static_cast<const cx<df> *>(prog.d_tables_df), prog.d_stages);
            }
            return;
        }
    }
    for (const auto &seg : prog.segs) {
        if (seg.tile && seg.reg) {
            launch_tile_pass_reg<T>(sv.stream(), sv.data(), seg.desc, prog.d_ops, prog.d_forms, prog.d_tables,
                                    prog.d_stages);
        } else if (seg.tile) {
            launch_tile_pass<T>(sv.stream(), sv.data(), seg.desc, prog.d_ops, prog.d_forms, prog.d_tables);
        } else {
            sv.run_prim(seg.prim);
        }
    }
}

template <class T>
void run_fused_adjoint(StateVector<T> &lam, StateVector<T> &hlam, const FusedProgram<T> &prog, double *partials,
                       int G) {
    PLGB_REQUIRE(prog.n == lam.num_qubits() && prog.n == hlam.num_qubits(),
                 "adjoint program compiled for a different register size");
    PLGB_REQUIRE(lam.stream() == hlam.stream(), "adjoint registers must share a stream");
    if constexpr (std::is_same_v<T, double>) {
        if (prog.df_ok && !c128_fp64_passes()) {
            // both registers hold df values between the first and the last pass
            const size_t np = prog.segs.size();
            for (size_t k = 0; k < np; k++) {
                const int io = np == 1 ? 0 : k == 0 ? 1 : k + 1 == np ? 3 : 2;
                if (prog.segs[k].reg) {
                    launch_tile_pass_reg_adj_df(lam.stream(), lam.data(), hlam.data(), io, prog.segs[k].desc,
                                                static_cast<const TileOp<df> *>(prog.d_ops_df),
                                                static_cast<const DiagForm<df> *>(prog.d_forms_df),
                                                static_cast<const cx<df> *>(prog.d_tables_df), prog.d_stages,
                                                partials, G);
                } else {
                    launch_tile_pass_adj_df(lam.stream(), lam.data(), hlam.data(), io, prog.segs[k].desc,
                                            static_cast<const TileOp<df> *>(prog.d_ops_df),
                                            static_cast<const DiagForm<df> *>(prog.d_forms_df),
                                            static_cast<const cx<df> *>(prog.d_tables_df), partials, G);
                }
            }
            return;
        }
    }
    for (const auto &seg : prog.segs) {
        if (seg.tile && seg.reg) {
            launch_tile_pass_reg_adj<T>(lam.stream(), lam.data(), hlam.data(), seg.desc, prog.d_ops, prog.d_forms,
                                        prog.d_tables, prog.d_stages, partials, G);
        } else if (seg.tile) {
            launch_tile_pass_adj<T>(lam.stream(), lam.data(), hlam.data(), seg.desc, prog.d_ops, prog.d_forms,
                                    prog.d_tables, partials, G);
        } else {
            PLGB_REQUIRE(seg.prim.kind != Prim<T>::Reduce, "adjoint program: reduction outside a tile pass");
            lam.run_prim(seg.prim);
            hlam.run_prim(seg.prim);
        }
    }
}

template <class T>
void StateVector<T>::apply_prims_fused(const std::vector<Prim<T>> &prims, int tile_bits) {
    auto prog = compile_fused<T>(n_, prims, tile_bits);
    run_fused<T>(*this, *prog);
    synchronize(); // the program's device buffer is freed on return
}

template <class T> std::string fused_plan_json(const FusedProgram<T> &prog) { return prog.plan; }
template std::string fused_plan_json<float>(const FusedProgram<float> &);
template std::string fused_plan_json<double>(const FusedProgram<double> &);

template <class T> FusedStats fused_stats(const FusedProgram<T> &prog) {
    return FusedStats{prog.passes, prog.unfused, prog.prims};
}
template FusedStats fused_stats<float>(const FusedProgram<float> &);
template FusedStats fused_stats<double>(const FusedProgram<double> &);

template struct FusedProgram<float>;
template struct FusedProgram<double>;
template std::shared_ptr<FusedProgram<float>> compile_fused<float>(int, const std::vector<Prim<float>> &, int, bool,
                                                                   bool);
template std::shared_ptr<FusedProgram<double>> compile_fused<double>(int, const std::vector<Prim<double>> &, int,
                                                                     bool, bool);
template void run_fused_adjoint<float>(StateVector<float> &, StateVector<float> &, const FusedProgram<float> &,
                                       double *, int);
template void run_fused_adjoint<double>(StateVector<double> &, StateVector<double> &, const FusedProgram<double> &,
                                        double *, int);
template void run_fused<float>(StateVector<float> &, const FusedProgram<float> &);
template void run_fused<double>(StateVector<double> &, const FusedProgram<double> &);
template void StateVector<float>::apply_prims_fused(const std::vector<Prim<float>> &, int);
template void StateVector<double>::apply_prims_fused(const std::vector<Prim<double>> &, int);

} // namespace plgb
