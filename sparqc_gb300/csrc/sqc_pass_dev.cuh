// Per-slot device code of a gate pass, shared by the single-state passes (sqc_pass.cu) and
// the many-circuit persistent kernel (sqc_batch.cu): a warp holds two slots per lane (two
// buckets, or both groups of a pair), applies a run of gates in registers and writes the
// slots back in place.
#pragma once
#include "sqc_device.cuh"

namespace sqc {
namespace {

template <class T> struct AmpT;
template <> struct AmpT<double> { using V = double2; };
template <> struct AmpT<float> { using V = float2; };

template <class T> __device__ __forceinline__ Cx<T> czero() { return Cx<T>{T(0), T(0)}; }

__device__ __forceinline__ unsigned long long umin64(unsigned long long a, unsigned long long b) { return a < b ? a : b; }

template <class T>
__device__ __forceinline__ void store_amp(void* amps, size_t s, Cx<T> a) {
    typename AmpT<T>::V v;
    v.x = a.r;
    v.y = a.i;
    reinterpret_cast<typename AmpT<T>::V*>(amps)[s] = v;
}

__device__ __forceinline__ bool slot_present(unsigned long long key, int j) { return (int)(key & 15ULL) == j; }

// One slot held by a lane: its key ((group << 4) | slot), amplitude and presence, where it
// lives (b = -1 for a group absent at the start of the pass) and whether the pass changed it.
template <class T> struct Val {
    unsigned long long key;
    int b;   // bucket index (< 2^31: far more buckets than any device holds), -1 when absent
    Cx<T> amp;
    bool pres, pres0, dirty;
};

struct GateHead {
    uint32_t kind, target, op, credit;
    unsigned long long ctrl, cval;
};

// The descriptor's first 32 bytes in two vector loads: {kind, target, ctrl}, {cval, op, credit}.
__device__ __forceinline__ GateHead gate_head(const GateDesc* g) {
    const uint4 v0 = ld_desc4(g);
    const uint4 v1 = ld_desc4(reinterpret_cast<const uint4*>(g) + 1);
    GateHead h;
    h.kind = v0.x;
    h.target = v0.y;
    h.ctrl = (unsigned long long)v0.z | ((unsigned long long)v0.w << 32);
    h.cval = (unsigned long long)v1.x | ((unsigned long long)v1.y << 32);
    h.op = v1.z;
    h.credit = v1.w;
    return h;
}

// FP64 arithmetic issues on the slow FP64 pipe: skip it when no lane of the warp needs it.
// FP32 arithmetic is cheaper than the vote.
template <class T> struct Vote { static constexpr bool kSkip = sizeof(T) == 8; };

template <class T>
__device__ __forceinline__ bool warp_needs(bool need) {
    return Vote<T>::kSkip ? __any_sync(kFull, need) : true;
}

// Whether the gate acts on the slot's key (its controls hold) and the slot's logical target bit.
__device__ __forceinline__ bool slot_sat(const GateHead& h, unsigned long long key) {
    return !(h.op & kOpCtrl) || (key & h.ctrl) == h.cval;
}

__device__ __forceinline__ bool slot_bit(const GateHead& h, unsigned long long key) {
    return (((unsigned)(key >> h.target) ^ h.op) & 1u) != 0;   // kOpFlip is bit 0
}

// Absent slots hold amplitude +-0 (loads zero them, branching updates zero what they prune,
// swaps move them), and the prune threshold is positive, so a branching update of two absent
// slots gives a negligible result: "keep iff not negligible" needs no presence test. FP64
// still forms it, for the warp vote that skips FP64 work no lane needs.
template <class T> struct NeedAny { static constexpr bool kOn = Vote<T>::kSkip; };

// FP64 steps update a slot with selects on the per-lane conditions (controls, presence)
// rather than branches around them: the warp runs the arithmetic once for all its lanes either
// way, and the selects spare the divergent branches (64-qubit FP64 workload 0.6% faster).
// FP32 steps keep the branches: their selects made the octet kernels' code larger, and the
// instruction-fetch stalls cost more than the branches (64-qubit FP32 workload 3% slower).
// Only the FP64 warp vote (warp_needs) branches in the select form, uniformly across the warp.
template <class T> struct SelectForm { static constexpr bool kOn = sizeof(T) == 8; };

template <class T>
__device__ __forceinline__ Cx<T> pick(bool c, Cx<T> x, Cx<T> y) {
    return Cx<T>{c ? x.r : y.r, c ? x.i : y.i};
}

// A branching or swap gate of kind K whose partner slot sits in lane ^ off; bit is the slot's
// logical target bit.
template <class T, uint32_t K, class G>
__device__ __forceinline__ void shfl_step(const G& g, const GateHead& h, int off, bool bit, Val<T>& v,
                                          const PruneBits& pb) {
    const bool sat = slot_sat(h, v.key);
    Cx<T> pa;
    pa.r = __shfl_xor_sync(kFull, v.amp.r, off);
    pa.i = __shfl_xor_sync(kFull, v.amp.i, off);
    const bool swap = K == KANY ? (h.op & kOpSwap) != 0 : swap_kind(K);
    bool pp = false;
    if (swap || NeedAny<T>::kOn) pp = __shfl_xor_sync(kFull, (int)v.pres, off) != 0;   // warp-uniform
    if (swap) {
        const Cx<T> o = K == KANY ? swap_update_rt<T>(h.kind, bit, pa) : swap_update<T, K == KANY ? KX : K>(bit, pa);
        if constexpr (SelectForm<T>::kOn) {
            v.amp = pick(sat, o, v.amp);
            v.pres = sat ? pp : v.pres;
            v.dirty = v.dirty || sat;
        } else if (sat) {
            v.amp = o;
            v.pres = pp;
            v.dirty = true;
        }
    } else {
        const bool any = !NeedAny<T>::kOn || v.pres || pp;
        if (warp_needs<T>(sat && any)) {
            const Cx<T> o = K == KANY ? branch_update_rt<T>(h.kind, g, bit, v.amp, pa)
                                      : branch_update<T, K == KANY ? KH : K>(g, bit, v.amp, pa);
            if constexpr (SelectForm<T>::kOn) {
                const bool keep = any && !negligible(o, pb);
                v.amp = pick(sat, pick(keep, o, czero<T>()), v.amp);
                v.pres = sat ? keep : v.pres;
                v.dirty = v.dirty || sat;
            } else if (sat) {
                const bool keep = any && !negligible(o, pb);
                v.pres = keep;
                v.amp = keep ? o : czero<T>();
                v.dirty = true;
            }
        }
    }
}

// A diagonal gate of kind K on one slot (lane-local).
template <class T, uint32_t K, class G>
__device__ __forceinline__ void diag_step(const G& g, const GateHead& h, Val<T>& v) {
    const bool bit = slot_bit(h, v.key);
    const bool one_sided = K == KANY ? (h.op & kOpOneSided) != 0 : one_sided_kind(K);
    const bool need = v.pres && (!one_sided || bit) && slot_sat(h, v.key);
    if (warp_needs<T>(need)) {
        Cx<T> o = K == KANY ? diag_update_rt<T>(h.kind, g, bit, v.amp)
                            : diag_update<T, K == KANY ? KZ : K>(g, bit, v.amp);
        if constexpr (K == KS) {   // Sdg runs S's code: its result is S's negated (exact)
            if (h.kind == KSDG) o = Cx<T>{neg(o.r), neg(o.i)};
        }
        if constexpr (SelectForm<T>::kOn) {
            v.amp = pick(need, o, v.amp);
            v.dirty = v.dirty || need;
        } else if (need) {
            v.amp = o;
            v.dirty = true;
        }
    }
}

// A branching or swap gate of kind K on the pass's first cross-group qubit, lane-local:
// a = slot of the group with stored target bit 0, b = slot of its partner group.
template <class T, uint32_t K, class G>
__device__ __forceinline__ void pair_step(const G& g, const GateHead& h, Val<T>& a, Val<T>& b,
                                          const PruneBits& pb) {
    const bool sat = slot_sat(h, a.key);
    const bool bit_a = (h.op & kOpFlip) != 0, bit_b = !bit_a;
    const bool swap = K == KANY ? (h.op & kOpSwap) != 0 : swap_kind(K);
    constexpr uint32_t KS_ = K == KANY ? KX : K;
    if (swap) {
        const Cx<T> na = K == KANY ? swap_update_rt<T>(h.kind, bit_a, b.amp) : swap_update<T, KS_>(bit_a, b.amp);
        const Cx<T> nb = K == KANY ? swap_update_rt<T>(h.kind, bit_b, a.amp) : swap_update<T, KS_>(bit_b, a.amp);
        const bool pa = b.pres, pbr = a.pres;
        if constexpr (SelectForm<T>::kOn) {
            a.amp = pick(sat, na, a.amp);
            b.amp = pick(sat, nb, b.amp);
            a.pres = sat ? pa : a.pres;
            b.pres = sat ? pbr : b.pres;
            a.dirty = a.dirty || sat;
            b.dirty = b.dirty || sat;
        } else if (sat) {
            a.amp = na; b.amp = nb;
            a.pres = pa; b.pres = pbr;
            a.dirty = b.dirty = true;
        }
    } else {
        const bool any = !NeedAny<T>::kOn || a.pres || b.pres;
        if (warp_needs<T>(sat && any)) {
            constexpr uint32_t KB_ = K == KANY ? KH : K;
            const Cx<T> oa = K == KANY ? branch_update_rt<T>(h.kind, g, bit_a, a.amp, b.amp)
                                       : branch_update<T, KB_>(g, bit_a, a.amp, b.amp);
            const Cx<T> ob = K == KANY ? branch_update_rt<T>(h.kind, g, bit_b, b.amp, a.amp)
                                       : branch_update<T, KB_>(g, bit_b, b.amp, a.amp);
            if constexpr (SelectForm<T>::kOn) {
                const bool ka = any && !negligible(oa, pb), kb = any && !negligible(ob, pb);
                a.amp = pick(sat, pick(ka, oa, czero<T>()), a.amp);
                b.amp = pick(sat, pick(kb, ob, czero<T>()), b.amp);
                a.pres = sat ? ka : a.pres;
                b.pres = sat ? kb : b.pres;
                a.dirty = a.dirty || sat;
                b.dirty = b.dirty || sat;
            } else if (sat) {
                const bool ka = any && !negligible(oa, pb), kb = any && !negligible(ob, pb);
                a.pres = ka; a.amp = ka ? oa : czero<T>();
                b.pres = kb; b.amp = kb ? ob : czero<T>();
                a.dirty = b.dirty = true;
            }
        }
    }
}

// One gate of kind K on the lane's two slots, as its pass encoded it (encode_pass).
template <class T, uint32_t K, class G>
__device__ __forceinline__ void gate_on(const G& g, const GateHead& h, Val<T>& a, Val<T>& b,
                                        const PruneBits& pb) {
    // A shuffled gate targets a qubit below 4 (a bit of the slot index, shared by a and b) or
    // the quad's second cross-group qubit (whose bit a and b, one unit's groups in one half of
    // the warp, also share): its target bit is computed once for both slots.
    if constexpr (K == KANY) {   // kind known at run time: category from the encoded op bits
        if (h.op & kOpPair) {
            pair_step<T, KANY>(g, h, a, b, pb);
        } else if (h.op & kOpShfl) {
            const int off = 1 << ((h.op >> kOpOffShift) & 7u);
            const bool bit = slot_bit(h, a.key);
            shfl_step<T, KANY>(g, h, off, bit, a, pb);
            shfl_step<T, KANY>(g, h, off, bit, b, pb);
        } else {
            diag_step<T, KANY>(g, h, a);
            diag_step<T, KANY>(g, h, b);
        }
    } else if constexpr (branch_kind(K) || swap_kind(K)) {
        if (h.op & kOpPair) {
            pair_step<T, K>(g, h, a, b, pb);
        } else {
            const int off = 1 << ((h.op >> kOpOffShift) & 7u);
            const bool bit = slot_bit(h, a.key);
            shfl_step<T, K>(g, h, off, bit, a, pb);
            shfl_step<T, K>(g, h, off, bit, b, pb);
        }
    } else {
        diag_step<T, K>(g, h, a);
        diag_step<T, K>(g, h, b);
    }
}

// Apply gates [g0, g1) to the two held slots. With SPEC each gate is dispatched once on its
// (warp-uniform) kind to code specialised for that kind; without, its category is read from
// the encoded op bits and the kind is switched on inside the arithmetic -- less code, for the
// persistent batch kernel whose every pass type shares one instruction cache. Each gate is
// applied as its pass encoded it:
// branching and swap gates on the pass's first cross-group qubit pair a with b (lane-local),
// those on qubits 0..3 or on the second cross-group qubit pair each lane with lane ^ off (the
// other half of the warp holds the groups with the second qubit's bit set), diagonal gates are
// lane-local. Every lane accumulates the amp-update count of its own slots (the pass sums the
// lanes): every gate is credited with the present slots it sees, and host-resolved gates
// recorded in a descriptor's credit with the same count.
template <class T, bool SPEC = true>
__device__ __forceinline__ void run_gates(const GateDesc* __restrict__ gates, uint32_t g0, uint32_t g1, Val<T>& a,
                                          Val<T>& b, int lane, const PruneBits& pb, unsigned long long& upd) {
    // present slots in the warp: only a branching gate changes the count (swap gates permute
    // presence among slots that satisfy the same controls, diagonal gates keep it)
    unsigned n = (unsigned)a.pres + (unsigned)b.pres;
    bool recount = false;
    for (uint32_t gi = g0; gi < g1; ++gi) {
        const GateDesc* g = gates + gi;
        const GateHead h = gate_head(g);
        if (recount) n = (unsigned)a.pres + (unsigned)b.pres;
        recount = (h.op & kOpBranch) != 0;
        upd += (unsigned long long)n * (1ULL + h.credit);
        if constexpr (!SPEC) {
            gate_on<T, KANY>(g, h, a, b, pb);
            continue;
        }
        switch (h.kind) {
        case KX: gate_on<T, KX>(g, h, a, b, pb); break;
        case KY: gate_on<T, KY>(g, h, a, b, pb); break;
        case KZ: gate_on<T, KZ>(g, h, a, b, pb); break;
        case KH: gate_on<T, KH>(g, h, a, b, pb); break;
        case KPHASE:
        case KT:
        case KTDG: gate_on<T, KPHASE>(g, h, a, b, pb); break;   // T, Tdg: Phase with their (c, s)
        case KRZ: gate_on<T, KRZ>(g, h, a, b, pb); break;
        case KRX: gate_on<T, KRX>(g, h, a, b, pb); break;
        case KRY: gate_on<T, KRY>(g, h, a, b, pb); break;
        case KS:
        case KSDG: gate_on<T, KS>(g, h, a, b, pb); break;   // Sdg: S negated
        case KU: gate_on<T, KU>(g, h, a, b, pb); break;
        default: gate_on<T, KYPH>(g, h, a, b, pb); break;
        }
    }
}

// A pass's gate, staged in shared memory by its block: the descriptor's first 32 bytes (kind,
// target, ctrl, cval, op, credit) and its (c, s) pair in both precisions. Gates are read once
// per slot held by every warp; from shared memory they never wait on L1 misses.
struct alignas(16) SmemGate {
    uint4 h0, h1;
    double c, s;
    float cf, sf;
    uint32_t pad[2];
};

// Copy gate g into its shared-memory form.
__device__ __forceinline__ void stage_gate(SmemGate* d, const GateDesc* g) {
    SmemGate x;
    x.h0 = ld_desc4(g);
    x.h1 = ld_desc4(reinterpret_cast<const uint4*>(g) + 1);
    x.c = ld_desc(&g->c);
    x.s = ld_desc(&g->s);
    x.cf = ld_desc(&g->cf);
    x.sf = ld_desc(&g->sf);
    x.pad[0] = x.pad[1] = 0;
    *d = x;
}

// Copy gates [g0, g1) (at most kMaxRun) of the pass into shared memory; every thread of the
// block calls it, and it ends with a barrier.
__device__ __forceinline__ void stage_gates(SmemGate* sg, const GateDesc* __restrict__ gates, uint32_t g0,
                                            uint32_t g1) {
    for (uint32_t i = threadIdx.x; g0 + i < g1; i += blockDim.x) stage_gate(sg + i, gates + g0 + i);
    __syncthreads();
}

// The same for one warp's own copy (every lane calls it; it ends with a warp barrier).
__device__ __forceinline__ void stage_gates_warp(SmemGate* sg, const GateDesc* __restrict__ gates, uint32_t g0,
                                                 uint32_t g1, int lane) {
    for (uint32_t i = (uint32_t)lane; g0 + i < g1; i += 32) stage_gate(sg + i, gates + g0 + i);
    __syncwarp();
}

template <class T> struct SmemPair;
template <> struct SmemPair<double> {
    __device__ static __forceinline__ SmemCoef<double> of(const SmemGate& x, const GateDesc* g) {
        return SmemCoef<double>{x.c, x.s, g};
    }
};
template <> struct SmemPair<float> {
    __device__ static __forceinline__ SmemCoef<float> of(const SmemGate& x, const GateDesc* g) {
        return SmemCoef<float>{x.cf, x.sf, g};
    }
};

// run_gates with the pass's gates staged in shared memory (sg[i] is gate g0 + i).
template <class T, bool SPEC = true>
__device__ __forceinline__ void run_gates_s(const SmemGate* sg, const GateDesc* __restrict__ gates, uint32_t g0,
                                            uint32_t g1, Val<T>& a, Val<T>& b, int lane, const PruneBits& pb,
                                            unsigned long long& upd) {
    unsigned n = (unsigned)a.pres + (unsigned)b.pres;
    bool recount = false;
    for (uint32_t gi = g0; gi < g1; ++gi) {
        const SmemGate& x = sg[gi - g0];
        const uint4 v0 = x.h0, v1 = x.h1;
        GateHead h;
        h.kind = v0.x;
        h.target = v0.y;
        h.ctrl = (unsigned long long)v0.z | ((unsigned long long)v0.w << 32);
        h.cval = (unsigned long long)v1.x | ((unsigned long long)v1.y << 32);
        h.op = v1.z;
        h.credit = v1.w;
        const SmemCoef<T> g = SmemPair<T>::of(x, gates + gi);
        if (recount) n = (unsigned)a.pres + (unsigned)b.pres;
        recount = (h.op & kOpBranch) != 0;
        upd += (unsigned long long)n * (1ULL + h.credit);
        if constexpr (!SPEC) {
            gate_on<T, KANY>(g, h, a, b, pb);
            continue;
        }
        switch (h.kind) {
        case KX: gate_on<T, KX>(g, h, a, b, pb); break;
        case KY: gate_on<T, KY>(g, h, a, b, pb); break;
        case KZ: gate_on<T, KZ>(g, h, a, b, pb); break;
        case KH: gate_on<T, KH>(g, h, a, b, pb); break;
        case KPHASE:
        case KT:
        case KTDG: gate_on<T, KPHASE>(g, h, a, b, pb); break;   // T, Tdg: Phase with their (c, s)
        case KRZ: gate_on<T, KRZ>(g, h, a, b, pb); break;
        case KRX: gate_on<T, KRX>(g, h, a, b, pb); break;
        case KRY: gate_on<T, KRY>(g, h, a, b, pb); break;
        case KS:
        case KSDG: gate_on<T, KS>(g, h, a, b, pb); break;   // Sdg: S negated
        case KU: gate_on<T, KU>(g, h, a, b, pb); break;
        default: gate_on<T, KYPH>(g, h, a, b, pb); break;
        }
    }
}

// Ownership of the unit of list entry group G (bucket b) in a pass with nx cross-group qubits
// (masks m1, m2, m3): the unit's members are G0 | i0*m1 | i1*m2 | i2*m3 (G0 = G with those bits
// cleared); the owner is the member with the smallest index i0 + 2*i1 + 4*i2 among those live at
// the start of the pass -- for a pair this is the reference's rule (the bit-0 key owns the pair unless it
// is absent, emulator/device/device_table_FC.cuh:62-110) lifted to groups. Fills the members'
// buckets (-1 when absent) and returns whether G owns its unit. Members a pass creates are
// only ever created by the unit's owner, after its own check, so the lookups are consistent.
template <int NX>
__device__ __forceinline__ bool unit_owner(const TableDev& t, unsigned ep, unsigned long long G, long long b,
                                           unsigned long long m1, unsigned long long m2, unsigned long long m3,
                                           long long bk[8], unsigned long long* G0) {
    constexpr int K = 1 << NX;
    const int idx = ((G & m1) ? 1 : 0) | ((NX >= 2 && (G & m2)) ? 2 : 0) | ((NX == 3 && (G & m3)) ? 4 : 0);
    *G0 = G & ~(m1 | (NX >= 2 ? m2 : 0ULL) | (NX == 3 ? m3 : 0ULL));
    auto member = [&](int k) { return *G0 | ((k & 1) ? m1 : 0ULL) | ((k & 2) ? m2 : 0ULL) | ((k & 4) ? m3 : 0ULL); };
#pragma unroll
    for (int k = 0; k < 8; ++k) bk[k] = -1;
#pragma unroll
    for (int k = 0; k < K; ++k) {   // a live member of smaller index owns the unit
        if (k < idx && lookup_group(t, ep, member(k)) >= 0) return false;
    }
#pragma unroll
    for (int k = 0; k < K; ++k) {
        if (k == idx) bk[k] = b;
        else if (k > idx) bk[k] = lookup_group(t, ep, member(k));
    }
    return true;
}

// Write a held slot back in place. A group absent at the start of the pass gets a bucket
// (claimed by lane 0 of the half) when it ends up with a present key; every slot of a new
// bucket is written. Returns the new bucket index on lane 0 of the half, else -1.
template <class T>
__device__ __forceinline__ long long write_val(const TableDev& t, unsigned ep, Val<T>& v, int lane,
                                               unsigned int* status, unsigned long long& cnt_nnz,
                                               unsigned long long& cnt_empty) {
    const int j = lane & 15, half = lane >> 4;
    const unsigned bal = __ballot_sync(kFull, v.pres);
    const unsigned hm = half ? (bal >> 16) : (bal & 0xFFFFu);
    long long b = v.b;
    bool created = false;
    long long fresh = -1;
    if (__any_sync(kFull, b < 0 && hm != 0)) {
        long long cb = -1;
        if (b < 0 && hm && j == 0) cb = claim_group(t, ep, v.key >> kSlotBits, status, &created);
        cb = (long long)shfl64((unsigned long long)cb, half << 4);
        created = __shfl_sync(kFull, (int)created, half << 4) != 0;
        if (b < 0 && hm) {
            b = cb;
            if (created && j == 0) fresh = b;
        }
    }
    if (b >= 0) {
        const size_t s = (size_t)b * kSlots + j;
        if (created || v.pres != v.pres0)
            t.keys[s] = v.pres ? v.key : empty_key(j);
        if (v.pres && v.dirty) store_amp<T>(t.amps, s, v.amp);
        cnt_nnz += v.pres ? 1 : 0;
        if (j == 0 && !hm) cnt_empty += 1;
    }
    return fresh;
}

// Append up to four new buckets (one candidate per half per held slot) to the live list.
__device__ __forceinline__ void append_new(const TableDev& t, Ctl* ctl, long long fa, long long fb, int lane) {
    const unsigned ma = __ballot_sync(kFull, fa >= 0), mb = __ballot_sync(kFull, fb >= 0);
    const unsigned n = __popc(ma) + __popc(mb);
    if (!n) return;
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(&ctl->list_tail, (unsigned long long)n);
    base = shfl64(base, 0);
    const unsigned below = (1u << lane) - 1u;
    if (fa >= 0) t.list[base + __popc(ma & below)] = (unsigned)fa;
    if (fb >= 0) t.list[base + __popc(ma) + __popc(mb & below)] = (unsigned)fb;
}

__device__ __forceinline__ unsigned long long warp_sum(unsigned long long v) {
    for (int o = 16; o; o >>= 1) v += __shfl_down_sync(kFull, v, o);
    return v;
}

template <class T>
__device__ __forceinline__ void load_val_g(const TableDev& t, Val<T>& v, unsigned long long G, long long b, int j) {
    v.key = (G << kSlotBits) | (unsigned long long)j;
    v.b = b;
    v.dirty = false;
    v.pres = false;
    v.amp = czero<T>();
    if (b >= 0) {
        const size_t s = (size_t)b * kSlots + j;
        v.pres = slot_present(t.keys[s], j);
        if (v.pres) {
            const typename AmpT<T>::V x = reinterpret_cast<const typename AmpT<T>::V*>(t.amps)[s];
            v.amp = Cx<T>{x.x, x.y};
        }
    }
    v.pres0 = v.pres;
}

// Ownership of the units of the (up to) four list entries [e0, e0 + 4) ∩ [0, n) in one round
// of lookups: with K = 2^NX members per unit (NX <= 3, masks m1, m2, m3), lane l < 4K looks up
// member k = l % K of the unit of entry l / K. Returns the owner mask (bit e: entry e owns its unit, by unit_owner's
// rule); afterwards lane e*K + k holds member k's bucket (*mb, -1 when absent) and lane e*K
// the unit's base group (*G0).
template <int NX>
__device__ __forceinline__ unsigned units4(const TableDev& t, unsigned ep, unsigned long long e0, unsigned long long n,
                                           unsigned long long m1, unsigned long long m2, int lane, long long* mb,
                                           unsigned long long* G0, unsigned long long m3 = 0ULL) {
    constexpr int K = 1 << NX;
    const int e = lane / K, k = lane % K;
    bool valid = false;
    int idx = 0;
    *mb = -1;
    *G0 = 0;
    if (lane < 4 * K && e0 + e < n) {
        const long long b = (long long)t.list[e0 + e];
        const unsigned long long G = load_hdr(t.hdr + b).group;
        idx = ((G & m1) ? 1 : 0) | ((NX >= 2 && (G & m2)) ? 2 : 0) | ((NX == 3 && (G & m3)) ? 4 : 0);
        *G0 = G & ~(m1 | (NX >= 2 ? m2 : 0ULL) | (NX == 3 ? m3 : 0ULL));
        valid = true;
        *mb = k == idx ? b
                       : lookup_group(t, ep, *G0 | ((k & 1) ? m1 : 0ULL) | ((k & 2) ? m2 : 0ULL) |
                                                 ((k & 4) ? m3 : 0ULL));
    }
    const unsigned live = __ballot_sync(kFull, *mb >= 0);
    const bool own = valid && k == 0 && ((live >> (e * K)) & ((1u << idx) - 1u)) == 0;
    const unsigned om = __ballot_sync(kFull, own);
    unsigned res = 0;
#pragma unroll
    for (int i = 0; i < 4; ++i) res |= ((om >> (i * K)) & 1u) << i;
    return res;
}

// Process the owned units of a units4 round: pairs two per warp step (one per half), quads one
// per warp step (the half selects the q2 bit); each unit's groups are loaded straight from the
// table, the gates applied (from shared memory with SMEM), and the slots written back.
template <class T, int NX, bool SPEC = true, bool SMEM = false>
__device__ __forceinline__ void run_units4(const TableDev& t, unsigned ep, Ctl* ctl, const GateDesc* gates,
                                           const SmemGate* sg, uint32_t g0,
                                           uint32_t g1, unsigned long long m1, unsigned long long m2, unsigned om,
                                           long long mb, unsigned long long G0,
                                           int lane, const PruneBits& pb, Val<T>& va, Val<T>& vb,
                                           unsigned long long& cnt_nnz, unsigned long long& cnt_empty,
                                           unsigned long long& upd) {
    constexpr int K = NX == 2 ? 4 : 2;
    const int half = lane >> 4, j = lane & 15;
    while (om) {
        int u, src;
        if (NX == 1) {
            const int u0 = __ffs(om) - 1;
            om &= om - 1;
            int u1 = -1;
            if (om) { u1 = __ffs(om) - 1; om &= om - 1; }
            u = half ? u1 : u0;
            src = u >= 0 ? u : u0;
        } else {
            u = __ffs(om) - 1;
            om &= om - 1;
            src = u;
        }
        const bool hi = NX == 2 && half;
        // this half's two members: (0, 1), or (2, 3) for the upper half of a quad
        const long long xa = (long long)shfl64((unsigned long long)mb, src * K + (hi ? 2 : 0));
        const long long xb = (long long)shfl64((unsigned long long)mb, src * K + (hi ? 3 : 1));
        const unsigned long long uG0 = shfl64(G0, src * K);
        const unsigned long long Ga = uG0 | (hi ? m2 : 0ULL);
        const bool act = u >= 0;
        load_val_g<T>(t, va, Ga, act ? xa : -1, j);
        load_val_g<T>(t, vb, Ga | m1, act ? xb : -1, j);
        if constexpr (SMEM) run_gates_s<T, SPEC>(sg, gates, g0, g1, va, vb, lane, pb, upd);   // gates in shared memory
        else run_gates<T, SPEC>(gates, g0, g1, va, vb, lane, pb, upd);
        const long long fa = write_val<T>(t, ep, va, lane, &ctl->status, cnt_nnz, cnt_empty);
        const long long fb = write_val<T>(t, ep, vb, lane, &ctl->status, cnt_nnz, cnt_empty);
        append_new(t, ctl, fa, fb, lane);
    }
}


// ---- passes with three cross-group qubits (octets of groups) --------------------------------
// A unit is the eight groups G0 | i0*m1 | i1*m2 | i2*m3. One warp holds one unit: the half
// selects i1 (as in a quad), and each lane holds slot j of four groups: a = (0, 0), b = (1, 0),
// c = (0, 1), d = (1, 1) in (i0, i2). Gates on q1 pair a-b and c-d, gates on q3 pair a-c and
// b-d (lane-local); gates on q2 and on qubits 0..3 pair lanes (the target bit is shared by the
// four slots); diagonal gates are lane-local.
template <class T, uint32_t K, class G>
__device__ __forceinline__ void gate_on4(const G& g, const GateHead& h, Val<T>& a, Val<T>& b, Val<T>& c, Val<T>& d,
                                         const PruneBits& pb) {
    if constexpr (branch_kind(K) || swap_kind(K)) {
        if (h.op & kOpPair) {
            pair_step<T, K>(g, h, a, b, pb);
            pair_step<T, K>(g, h, c, d, pb);
        } else if (h.op & kOpPair3) {
            pair_step<T, K>(g, h, a, c, pb);
            pair_step<T, K>(g, h, b, d, pb);
        } else {
            const int off = 1 << ((h.op >> kOpOffShift) & 7u);
            const bool bit = slot_bit(h, a.key);
            shfl_step<T, K>(g, h, off, bit, a, pb);
            shfl_step<T, K>(g, h, off, bit, b, pb);
            shfl_step<T, K>(g, h, off, bit, c, pb);
            shfl_step<T, K>(g, h, off, bit, d, pb);
        }
    } else {
        diag_step<T, K>(g, h, a);
        diag_step<T, K>(g, h, b);
        diag_step<T, K>(g, h, c);
        diag_step<T, K>(g, h, d);
    }
}

template <class T>
__device__ __forceinline__ unsigned present4(const Val<T>& a, const Val<T>& b, const Val<T>& c, const Val<T>& d) {
    return (unsigned)a.pres + (unsigned)b.pres + (unsigned)c.pres + (unsigned)d.pres;
}

// Gates [g0, g1) on the lane's four slots (from shared memory with SMEM, sg[i] = gate g0 + i).
template <class T, bool SMEM>
__device__ __forceinline__ void run_gates4(const SmemGate* sg, const GateDesc* __restrict__ gates, uint32_t g0,
                                           uint32_t g1, Val<T>& a, Val<T>& b, Val<T>& c, Val<T>& d, int lane,
                                           const PruneBits& pb, unsigned long long& upd) {
    unsigned n = present4(a, b, c, d);
    bool recount = false;
    for (uint32_t gi = g0; gi < g1; ++gi) {
        GateHead h;
        if constexpr (SMEM) {
            const SmemGate& x = sg[gi - g0];
            const uint4 v0 = x.h0, v1 = x.h1;
            h.kind = v0.x;
            h.target = v0.y;
            h.ctrl = (unsigned long long)v0.z | ((unsigned long long)v0.w << 32);
            h.cval = (unsigned long long)v1.x | ((unsigned long long)v1.y << 32);
            h.op = v1.z;
            h.credit = v1.w;
        } else {
            h = gate_head(gates + gi);
        }
        if (recount) n = present4(a, b, c, d);
        recount = (h.op & kOpBranch) != 0;
        upd += (unsigned long long)n * (1ULL + h.credit);
        auto go = [&](const auto& g) {
            switch (h.kind) {
            case KX: gate_on4<T, KX>(g, h, a, b, c, d, pb); break;
            case KY: gate_on4<T, KY>(g, h, a, b, c, d, pb); break;
            case KZ: gate_on4<T, KZ>(g, h, a, b, c, d, pb); break;
            case KH: gate_on4<T, KH>(g, h, a, b, c, d, pb); break;
            case KPHASE:
            case KT:
            case KTDG: gate_on4<T, KPHASE>(g, h, a, b, c, d, pb); break;   // T, Tdg: Phase with their (c, s)
            case KRZ: gate_on4<T, KRZ>(g, h, a, b, c, d, pb); break;
            case KRX: gate_on4<T, KRX>(g, h, a, b, c, d, pb); break;
            case KRY: gate_on4<T, KRY>(g, h, a, b, c, d, pb); break;
            case KS:
            case KSDG: gate_on4<T, KS>(g, h, a, b, c, d, pb); break;   // Sdg: S negated
            case KU: gate_on4<T, KU>(g, h, a, b, c, d, pb); break;
            default: gate_on4<T, KYPH>(g, h, a, b, c, d, pb); break;
            }
        };
        if constexpr (SMEM) go(SmemPair<T>::of(sg[gi - g0], gates + gi));
        else go(gates + gi);
    }
}

// Process the owned octets of a units4<3> round, one per warp step: each half loads its four
// groups, applies the gates and writes the slots back.
template <class T, bool SMEM>
__device__ __forceinline__ void run_units8(const TableDev& t, unsigned ep, Ctl* ctl, const GateDesc* gates,
                                           const SmemGate* sg, uint32_t g0, uint32_t g1, unsigned long long m1,
                                           unsigned long long m2, unsigned long long m3, unsigned om, long long mb,
                                           unsigned long long G0, int lane, const PruneBits& pb,
                                           unsigned long long& cnt_nnz, unsigned long long& cnt_empty,
                                           unsigned long long& upd) {
    constexpr int K = 8;
    const int half = lane >> 4, j = lane & 15;
    Val<T> va, vb, vc, vd;
    while (om) {
        const int u = __ffs(om) - 1;
        om &= om - 1;
        // this half's members: (i0, i1 = half, i2) -> k = i0 + 2*i1 + 4*i2
        const int ka = 2 * half;
        const long long xa = (long long)shfl64((unsigned long long)mb, u * K + ka);
        const long long xb = (long long)shfl64((unsigned long long)mb, u * K + ka + 1);
        const long long xc = (long long)shfl64((unsigned long long)mb, u * K + ka + 4);
        const long long xd = (long long)shfl64((unsigned long long)mb, u * K + ka + 5);
        const unsigned long long Ga = shfl64(G0, u * K) | (half ? m2 : 0ULL);
        load_val_g<T>(t, va, Ga, xa, j);
        load_val_g<T>(t, vb, Ga | m1, xb, j);
        load_val_g<T>(t, vc, Ga | m3, xc, j);
        load_val_g<T>(t, vd, Ga | m1 | m3, xd, j);
        run_gates4<T, SMEM>(sg, gates, g0, g1, va, vb, vc, vd, lane, pb, upd);
        const long long fa = write_val<T>(t, ep, va, lane, &ctl->status, cnt_nnz, cnt_empty);
        const long long fb = write_val<T>(t, ep, vb, lane, &ctl->status, cnt_nnz, cnt_empty);
        const long long fc = write_val<T>(t, ep, vc, lane, &ctl->status, cnt_nnz, cnt_empty);
        const long long fd = write_val<T>(t, ep, vd, lane, &ctl->status, cnt_nnz, cnt_empty);
        append_new(t, ctl, fa, fb, lane);
        append_new(t, ctl, fc, fd, lane);
    }
}

}  // namespace
}  // namespace sqc
