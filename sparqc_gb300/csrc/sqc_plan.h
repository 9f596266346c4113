// Host-side gate planning shared by the single-state engine and the many-circuit batch:
// resolution of gates against what is known about the keys, descriptor construction
// (coefficients on the host) and the split of a descriptor sequence into passes.
#pragma once
#include <cstddef>
#include <cstdint>

#include "../../include/sparqc.h"
#include "sqc_types.h"

namespace sqc {

// What the host knows about the keys without looking at them: stored key = actual key ^
// frame; bits in kmask are identical across all keys and equal kval. Gates whose effect
// follows from this are resolved here: an uncontrolled X flips a frame bit, a gate with a
// known-zero control or a one-sided diagonal gate on a known-zero bit is the identity.
// kmask only loses bits, so ~kmask is every bit that has ever differed between keys.
struct Planner {
    unsigned long long frame = 0;
    unsigned long long kmask = ~0ULL;
    unsigned long long kval = 0;
    uint32_t credit = 0;   // resolved gates not yet credited to a device gate
};

inline bool is_diag_kind(uint32_t k) {
    return k == KZ || k == KPHASE || k == KRZ || k == KS || k == KSDG || k == KT || k == KTDG || k == KYPH;
}
inline bool is_one_sided_kind(uint32_t k) {
    return k == KZ || k == KPHASE || k == KS || k == KSDG || k == KT || k == KTDG;
}
inline bool is_branch_kind(uint32_t k) { return k == KH || k == KRX || k == KRY || k == KU; }
inline bool is_swap_kind(uint32_t k) { return k == KX || k == KY; }
// A gate that never pairs keys of different 16-key groups.
inline bool streamable(const GateDesc& d) { return d.target < (uint32_t)kSlotBits || is_diag_kind(d.kind); }

// Check one gate against a register of nq qubits; nullptr when valid, else the reason.
const char* check_gate(const sqc_gate& g, uint32_t nq);

// Descriptor of one device gate in the stored-key frame of p, coefficients resolved here.
GateDesc make_desc(const Planner& p, uint32_t kind, uint32_t target, unsigned long long ctrl, const sqc_gate& g);

// Resolve one gate against p. Returns true and a descriptor when the gate needs the device;
// otherwise the gate was applied here (identity, or an uncontrolled X as a frame flip) and
// is counted in p.credit, to be credited to the next device gate.
bool plan_gate(Planner& p, const sqc_gate& g, GateDesc* out);

// Passes of a descriptor sequence. A pass is a run of at most max_run consecutive gates whose
// cross-group gates (gates that pair keys of different 16-key groups) target at most
// max_nx (<= 3) distinct qubits; streamable gates may sit anywhere in it. Passes are cut
// greedily. f(g0, g1, nx, q1, q2, q3, keys_fixed) is called per pass, q1..q3 the cross-group
// qubits in order of first use (kNoQubit when absent).
template <class F>
void split_passes(const GateDesc* d, size_t n, size_t max_run, uint32_t max_nx, F&& f) {
    size_t i = 0;
    while (i < n) {
        const size_t start = i;
        uint32_t q[3] = {kNoQubit, kNoQubit, kNoQubit};
        uint32_t nx = 0;
        while (i < n && i - start < max_run) {
            if (!streamable(d[i])) {
                const uint32_t t = d[i].target;
                if (t != q[0] && t != q[1] && t != q[2]) {
                    if (nx >= max_nx || nx >= 3) break;
                    q[nx++] = t;
                }
            }
            ++i;
        }
        bool fixed = true;
        for (size_t k = start; k < i; ++k) fixed = fixed && is_diag_kind(d[k].kind);
        f(start, i, nx, q[0], q[1], q[2], fixed);
    }
}

// Record in descriptors [g0, g1) -- one pass with cross-group qubits q1, q2, q3 (in order of
// first use; kNoQubit when absent) -- how the pass applies each gate (GateDesc.flip kOp*
// bits): gates on q1 and q3 pair slots held by the same lane, gates on q2 and on qubits 0..3
// pair lanes (shuffles).
void encode_pass(GateDesc* d, size_t g0, size_t g1, uint32_t q1, uint32_t q3 = kNoQubit);

// An order of gates g[0..n) that passes fuse better, as a permutation: perm[i] is the index of
// the i-th gate to apply. Passes are built greedily from the first gate not yet placed: a gate
// within the next `window` joins the pass when it commutes with every gate it moves ahead of
// (neither changes a qubit the other touches: a gate changes its target, unless it is
// diagonal, and only reads its controls) and the pass still has room for it (at most max_nx
// cross-group qubits, max_run device gates). The pass's cross-group qubits are the set, among
// the first-use choice and the max_nx-subsets of the first kSchedCandidates qubits gates pair
// across, that takes the most device gates over the first kSchedTrialWindow gates of the
// window. Commuting gates give the same state in either order; rounding and pruning follow the
// new order. Deterministic: a function of the gates.
void schedule_gates(const sqc_gate* g, size_t n, uint32_t max_nx, size_t max_run, size_t window, uint32_t* perm);
constexpr uint32_t kSchedCandidates = 6;
constexpr uint32_t kSchedTrialWindow = 64;   // gates the candidate choices are compared over
constexpr size_t kScheduleWindow = 256;
// Longer gate arrays (indices no longer fit 32 bits) keep the order given.
constexpr uint64_t kScheduleMaxGates = 0xFFFFFFFFULL;

// Largest number of 16-key groups a state can ever hold while running a gate sequence whose
// planning ended in p (starting from keys that agreed on every bit of the starting kmask):
// 2^(bits >= 4 that have ever differed between keys).
unsigned long long group_bound(const Planner& p, uint32_t nq);

}  // namespace sqc
