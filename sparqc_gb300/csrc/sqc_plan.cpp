// Host-side gate planning: see sqc_plan.h.
#include "sqc_plan.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

namespace sqc {

const char* check_gate(const sqc_gate& g, uint32_t nq) {
    if (g.kind > SQC_U) return "unknown gate kind";
    if (g.target >= nq) return "target qubit out of range";
    if (nq < 64 && (g.controls >> nq)) return "control qubit out of range";
    if ((g.controls >> g.target) & 1ULL) return "target qubit among the controls";
    return nullptr;
}

GateDesc make_desc(const Planner& p, uint32_t kind, uint32_t target, unsigned long long ctrl, const sqc_gate& g) {
    GateDesc d;
    std::memset(&d, 0, sizeof d);
    d.kind = kind;
    d.target = target;
    d.ctrl = ctrl;
    d.cval = ctrl & ~p.frame;
    d.flip = (uint32_t)((p.frame >> target) & 1ULL);
    switch (kind) {
    case KPHASE: d.c = std::cos(g.theta); d.s = std::sin(g.theta); break;
    case KRZ: case KRX: case KRY: {
        const double h = g.theta / 2.;   // the reference passes par/2 (table_manager.cuh:333-336)
        d.c = std::cos(h);
        d.s = std::sin(h);
        break;
    }
    case KT: d.c = 0.70710678118654752440; d.s = 0.70710678118654752440; break;
    case KTDG: d.c = 0.70710678118654752440; d.s = -0.70710678118654752440; break;
    case KH: d.c = 1. / std::sqrt(2.); break;   // as in h_core (device_data.cuh:205)
    case KU: {
        const double c = std::cos(g.theta / 2.), s = std::sin(g.theta / 2.);
        const double cl = std::cos(g.lambda), sl = std::sin(g.lambda);
        const double cp = std::cos(g.phi), sp = std::sin(g.phi);
        const double cpl = std::cos(g.phi + g.lambda), spl = std::sin(g.phi + g.lambda);
        d.m[0] = c;         d.m[1] = 0.;
        d.m[2] = -(cl * s); d.m[3] = -(sl * s);
        d.m[4] = cp * s;    d.m[5] = sp * s;
        d.m[6] = cpl * c;   d.m[7] = spl * c;
        break;
    }
    default: break;
    }
    d.cf = (float)d.c;
    d.sf = (float)d.s;
    for (int i = 0; i < 8; ++i) d.mf[i] = (float)d.m[i];
    return d;
}

bool plan_gate(Planner& p, const sqc_gate& g, GateDesc* out) {
    const unsigned long long bq = 1ULL << g.target;
    const unsigned long long kc = g.controls & p.kmask;
    if ((p.kval & kc) != kc) { ++p.credit; return false; }   // a control is known to be 0
    const unsigned long long ctrl = g.controls & ~p.kmask;   // controls still to test per key
    if (is_swap_kind(g.kind) && ctrl == 0) {
        p.frame ^= bq;
        if (p.kmask & bq) p.kval ^= bq;
        if (g.kind == KX) { ++p.credit; return false; }
        *out = make_desc(p, KYPH, g.target, 0, g);   // Y = relabel + diag(-i, +i)
        return true;
    }
    if (is_one_sided_kind(g.kind) && (p.kmask & bq) && !(p.kval & bq)) { ++p.credit; return false; }
    *out = make_desc(p, g.kind, g.target, ctrl, g);
    if (is_branch_kind(g.kind) || is_swap_kind(g.kind)) p.kmask &= ~bq;
    return true;
}

void encode_pass(GateDesc* d, size_t g0, size_t g1, uint32_t q1, uint32_t q3) {
    for (size_t k = g0; k < g1; ++k) {
        GateDesc& g = d[k];
        uint32_t op = g.flip & kOpFlip;
        const bool branch = is_branch_kind(g.kind), swap = is_swap_kind(g.kind);
        if (g.ctrl) op |= kOpCtrl;
        if (branch) op |= kOpBranch;
        if (swap) op |= kOpSwap;
        if (is_one_sided_kind(g.kind)) op |= kOpOneSided;
        if (g.target < (uint32_t)kSlotBits) op |= kOpLowBit;
        if (branch || swap) {
            if (g.target == q1 && g.target >= (uint32_t)kSlotBits) {
                op |= kOpPair;
            } else if (g.target == q3 && g.target >= (uint32_t)kSlotBits) {
                op |= kOpPair3;
            } else {
                // qubits 0..3: a lane of the same half; the pass's second cross-group qubit:
                // the other half of the warp
                const uint32_t off_log2 = g.target < (uint32_t)kSlotBits ? g.target : 4u;
                op |= kOpShfl | (off_log2 << kOpOffShift);
            }
        }
        g.flip = op;
    }
}

namespace {

// The gates of a scheduling window, as the scheduler sees them: the qubits each touches (target
// and controls), the qubit it changes (its target, unless it is diagonal), its target bit when
// the device pairs keys across groups for it, and whether the device runs it at all.
struct SchedWindow {
    std::vector<unsigned long long> sup, moves, cross;
    std::vector<unsigned char> dev;
    std::vector<uint32_t> idx;   // the gates' positions in the input
    void clear() {
        sup.clear();
        moves.clear();
        cross.clear();
        dev.clear();
        idx.clear();
    }
};

// One pass over the window's gates (in order, the first one first): a gate joins when it
// commutes with every gate left behind so far and fits the pass (cross-group qubits: those of
// fixed_q when nonzero, else the first max_nx used; at most max_run device gates), over the
// first nscan gates. Two gates commute when neither changes a qubit the other touches: gates
// act diagonally on their controls, and a diagonal gate on its target too, and operators that
// are diagonal on their shared qubits and change disjoint ones commute. Appends the positions
// taken to *took (if given) and returns the number of device gates among them; *limited (if
// given) tells whether a gate was refused for want of a cross-group qubit.
size_t sched_pass(const SchedWindow& w, size_t nscan, uint32_t max_nx, size_t max_run, unsigned long long fixed_q,
                  std::vector<uint32_t>* took, bool* limited) {
    unsigned long long qmask = fixed_q;
    uint32_t nx = 0;
    const bool fixed = fixed_q != 0;
    size_t run = 0;
    bool lim = false;
    unsigned long long left_sup = 0, left_moves = 0;   // of the gates left behind
    // written without data-dependent branches: whether a gate joins is close to a coin flip
    for (size_t r = 0; r < nscan && run < max_run; ++r) {
        const unsigned long long blocked = (w.moves[r] & left_sup) | (w.sup[r] & left_moves);
        const unsigned long long new_q = w.cross[r] & ~qmask;
        const bool refused = (new_q != 0) & (fixed | (nx >= max_nx));
        const bool take = (blocked == 0) & !refused;
        lim |= (blocked == 0) & refused;
        const unsigned long long behind = take ? 0ULL : ~0ULL;
        left_sup |= w.sup[r] & behind;
        left_moves |= w.moves[r] & behind;
        qmask |= new_q & ~behind;
        nx += (unsigned)(take & (new_q != 0));
        run += (size_t)(take & (w.dev[r] != 0));
        if (took && take) took->push_back(w.idx[r]);
    }
    if (limited) *limited = lim;
    return run;
}

}  // namespace

void schedule_gates(const sqc_gate* g, size_t n, uint32_t max_nx, size_t max_run, size_t window, uint32_t* perm) {
    // what each gate is, planned in the given order: a move below only passes gates that change
    // none of the key bits the moved gate's planning reads (its target and controls), and the
    // moved gate changes none of theirs, so every gate plans the same in the new order
    std::vector<unsigned long long> sup(n), moves(n), cross(n);
    std::vector<unsigned char> dev(n), done(n, 0);
    Planner p;
    for (size_t i = 0; i < n; ++i) {
        GateDesc d;
        const unsigned long long t = 1ULL << g[i].target;
        dev[i] = plan_gate(p, g[i], &d) ? 1 : 0;
        cross[i] = dev[i] && !streamable(d) ? t : 0ULL;
        sup[i] = t | g[i].controls;
        moves[i] = is_diag_kind(g[i].kind) ? 0ULL : t;
    }
    if (max_nx > 3) max_nx = 3;
    size_t out = 0, first = 0;
    SchedWindow w;
    std::vector<uint32_t> best;
    while (first < n) {
        if (done[first]) {
            ++first;
            continue;
        }
        w.clear();   // the window's gates not yet placed
        for (size_t i = first, end = std::min(n, first + window); i < end; ++i) {
            if (done[i]) continue;
            w.sup.push_back(sup[i]);
            w.moves.push_back(moves[i]);
            w.cross.push_back(cross[i]);
            w.dev.push_back(dev[i]);
            w.idx.push_back((uint32_t)i);
        }
        // the pass's cross-group qubits: the first-use choice, or any max_nx of the first
        // kSchedCandidates qubits the window's gates pair across, whichever takes the most
        // device gates over the first kSchedTrialWindow gates (earliest choice on ties). A
        // first-use pass that refused no gate for want of a qubit took every gate it reached (the
        // first refusal of any other kind needs a gate left behind), so no choice does better.
        const size_t ntrial = std::min(w.idx.size(), (size_t)kSchedTrialWindow);
        bool limited = false;
        size_t best_run = sched_pass(w, ntrial, max_nx, max_run, 0ULL, nullptr, &limited);
        unsigned long long best_q = 0;
        if (limited) {
            unsigned long long cand[kSchedCandidates];
            uint32_t m = 0;
            unsigned long long seen = 0;
            for (size_t r = 0; r < w.idx.size() && m < kSchedCandidates; ++r) {
                if (w.cross[r] & ~seen) cand[m++] = w.cross[r];
                seen |= w.cross[r];
            }
            const uint32_t k = std::min(max_nx, m);
            if (k > 0 && m > k) {
                uint32_t ix[3] = {0, 1, 2};
                for (;;) {   // every k-subset of the candidates, in lexicographic order
                    unsigned long long set = 0;
                    for (uint32_t a = 0; a < k; ++a) set |= cand[ix[a]];
                    const size_t r = sched_pass(w, ntrial, max_nx, max_run, set, nullptr, nullptr);
                    if (r > best_run) {   // earliest choice on ties, the first-use one first
                        best_run = r;
                        best_q = set;
                    }
                    int a = (int)k - 1;
                    while (a >= 0 && ix[a] == m - k + (uint32_t)a) --a;
                    if (a < 0) break;
                    ++ix[a];
                    for (uint32_t b = (uint32_t)a + 1; b < k; ++b) ix[b] = ix[b - 1] + 1;
                }
            }
        }
        best.clear();   // the chosen pass over the whole window
        sched_pass(w, w.idx.size(), max_nx, max_run, best_q, &best, nullptr);
        if (best.empty()) best.push_back((uint32_t)first);   // (never: the first gate always fits the first-use pass)
        for (uint32_t i : best) {
            done[i] = 1;
            perm[out++] = i;
        }
    }
}

unsigned long long group_bound(const Planner& p, uint32_t nq) {
    const unsigned long long reg = nq >= 64 ? ~0ULL : ((1ULL << nq) - 1);
    const unsigned long long var = ~p.kmask & reg & ~15ULL;
    const int bits = __builtin_popcountll(var);
    return bits >= 63 ? (1ULL << 63) : (1ULL << bits);
}

}  // namespace sqc
