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

// A gate as the scheduler sees it: its qubits (target and controls), the qubit it changes (its
// target, unless it is diagonal), and whether the device runs it and pairs keys across groups.
struct SchedGate {
    unsigned long long sup, moves;
    uint32_t target;
    bool dev, cross;
};

// One pass built from gate `first` over [first, end): a gate joins when it commutes with every
// gate left behind so far and fits the pass (cross-group qubits: the nfixed given ones, or with
// nfixed == 0 the first max_nx used; at most max_run device gates). Two gates commute when
// neither changes a qubit the other touches: gates act diagonally on their controls, and a
// diagonal gate on its target too, and operators that are diagonal on their shared qubits and
// change disjoint ones commute. Appends the gates taken to *took (if given); returns the number
// of device gates among them.
size_t sched_pass(const std::vector<SchedGate>& s, const std::vector<unsigned char>& done, size_t first, size_t end,
                  uint32_t max_nx, size_t max_run, const uint32_t* fixed, uint32_t nfixed, std::vector<uint32_t>* took) {
    uint32_t q[3] = {kNoQubit, kNoQubit, kNoQubit};
    uint32_t nx = 0;
    for (; nx < nfixed; ++nx) q[nx] = fixed[nx];
    size_t run = 0;
    unsigned long long left_sup = 0, left_moves = 0;   // of the gates left behind
    for (size_t i = first; i < end && run < max_run; ++i) {
        if (done[i]) continue;
        const SchedGate& x = s[i];
        bool take = (x.moves & left_sup) == 0 && (x.sup & left_moves) == 0;
        const bool new_q = x.cross && x.target != q[0] && x.target != q[1] && x.target != q[2];
        if (take && new_q && (nfixed || nx >= max_nx)) take = false;
        if (!take) {
            left_sup |= x.sup;
            left_moves |= x.moves;
            continue;
        }
        if (new_q) q[nx++] = x.target;
        run += x.dev ? 1 : 0;
        if (took) took->push_back((uint32_t)i);
    }
    return run;
}

}  // namespace

void schedule_gates(const sqc_gate* g, size_t n, uint32_t max_nx, size_t max_run, size_t window, uint32_t* perm) {
    // what each gate is, planned in the given order: a move below only passes gates that change
    // none of the key bits the moved gate's planning reads (its target and controls), and the
    // moved gate changes none of theirs, so every gate plans the same in the new order
    std::vector<SchedGate> s(n);
    std::vector<unsigned char> done(n, 0);
    Planner p;
    for (size_t i = 0; i < n; ++i) {
        GateDesc d;
        SchedGate& x = s[i];
        x.dev = plan_gate(p, g[i], &d);
        x.cross = x.dev && !streamable(d);
        x.target = g[i].target;
        x.sup = (1ULL << g[i].target) | g[i].controls;
        x.moves = is_diag_kind(g[i].kind) ? 0ULL : (1ULL << g[i].target);
    }
    if (max_nx > 3) max_nx = 3;
    size_t out = 0, first = 0;
    std::vector<uint32_t> took, best;
    while (first < n) {
        if (done[first]) {
            ++first;
            continue;
        }
        const size_t end = std::min(n, first + window);
        // the pass's cross-group qubits: the first-use choice, or any max_nx of the first
        // kSchedCandidates qubits the remaining gates pair across, whichever takes the most
        // device gates (earliest choice on ties)
        best.clear();
        size_t best_run = sched_pass(s, done, first, end, max_nx, max_run, nullptr, 0, &best);
        uint32_t cand[kSchedCandidates];
        uint32_t m = 0;
        for (size_t i = first; i < end && m < kSchedCandidates; ++i) {
            if (done[i] || !s[i].cross) continue;
            bool seen = false;
            for (uint32_t c = 0; c < m; ++c) seen = seen || cand[c] == s[i].target;
            if (!seen) cand[m++] = s[i].target;
        }
        const uint32_t k = std::min(max_nx, m);
        if (k > 0 && m > k) {   // (m == k: the first-use choice already holds them all)
            uint32_t idx[3] = {0, 1, 2};
            for (;;) {
                uint32_t set[3];
                for (uint32_t a = 0; a < k; ++a) set[a] = cand[idx[a]];
                const size_t r = sched_pass(s, done, first, end, max_nx, max_run, set, k, nullptr);
                if (r > best_run) {
                    best_run = r;
                    best.clear();
                    sched_pass(s, done, first, end, max_nx, max_run, set, k, &best);
                }
                int a = (int)k - 1;   // next k-subset of [0, m) in lexicographic order
                while (a >= 0 && idx[a] == m - k + (uint32_t)a) --a;
                if (a < 0) break;
                ++idx[a];
                for (uint32_t b = (uint32_t)a + 1; b < k; ++b) idx[b] = idx[b - 1] + 1;
            }
        }
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
